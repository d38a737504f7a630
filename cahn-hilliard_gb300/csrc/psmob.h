// psmob.h — the `pseudospectral_mobility` step (psmob.cu).
#pragma once

#include <stdint.h>

#include <string>

#include "common.cuh"
#include "spectral.h"

namespace chgb {

struct PsMob;

int psmob_create(const chgb_params &p, const Geom &g, const ModelDev &m, PsMob **out, std::string &err);
void psmob_destroy(PsMob *s);
// rho_hat = R2C(rho) of the device field `rho` (the integrator's constructor).
cudaError_t psmob_set_rho(PsMob *s, const double *rho, cudaStream_t st, int64_t *launches);
// One step with the mobility field `mob` of this step; `rho` is read and rewritten in place.
cudaError_t psmob_step(PsMob *s, const double *mob, double *rho, cudaStream_t st, int64_t *launches);
int psmob_launches_per_step(const PsMob *s);
// GMRES path: kernels its device-side loops (restart cycles, Arnoldi steps)
// have launched so far; waits for `st` to read the device counters.
int64_t psmob_gmres_loop_launches(const PsMob *s, cudaStream_t st);

}  // namespace chgb
