// psmob_impl.h — state shared by psmob.cu (M0 splitting) and psmob_gmres.cu
// (the GMRES path) of the `pseudospectral_mobility` step.
#pragma once

#include <vector>

#include "psmob.h"

namespace chgb {

struct PsGmres;

struct PsMob {
    chgb_params p;
    Geom g;
    ModelDev m;
    int S = 1;
    long long bins = 0, hat = 0, hall = 0;
    SpectralState *eng = nullptr;
    double2 *rho_hat = nullptr, *fder_hat = nullptr, *mu_hat = nullptr, *tmp_hat = nullptr, *div_hat = nullptr;
    double *q2 = nullptr, *dealias = nullptr, *kc[3] = {nullptr, nullptr, nullptr};
    double *fder = nullptr, *tmp = nullptr;
    double *M0 = nullptr, *part = nullptr;
    unsigned *m0_count = nullptr;   // blocks of the M0 launch done, per species (zero between launches)
    bool constant = true;
    PsGmres *gm = nullptr;   // GMRES path: Krylov basis and work vectors, allocated on first use
};


// M0 = max mobility per species into s->M0; returns the launches made (one).
int psmob_m0(PsMob *s, const double *mob, cudaStream_t st);
// s->tmp_hat = D i k_d in  /  s->div_hat (= on d == 0, += after) i k_d D s->tmp_hat.
cudaError_t psmob_grad(PsMob *s, const double2 *in, int d, cudaStream_t st);
cudaError_t psmob_div(PsMob *s, int d, cudaStream_t st);
// q2 / dealias tables as the fused spectral stages take them.
PsmobTables psmob_tables(const PsMob *s);
cudaError_t psmob_step_gmres(PsMob *s, const double *mob, double *rho, cudaStream_t st, int64_t *launches);
void psmob_gmres_release(PsMob *s);

}  // namespace chgb
