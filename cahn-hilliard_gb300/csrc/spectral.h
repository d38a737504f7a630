// spectral.h — pseudospectral integrator state (spectral.cu).
#pragma once

#include <stdint.h>

#include <string>

#include "common.cuh"

namespace chgb {

struct SpectralState;

// Allocate the spectral state of one box (rho_hat, wave-vector tables, scratch).
int spectral_create(const chgb_params &p, const Geom &g, const ModelDev &m, SpectralState **out, std::string &err);
void spectral_destroy(SpectralState *s);
// rho_hat = FFT(rho) (src/integrators/PseudospectralCPU.cpp:95-101); rho is a device field.
int spectral_set_rho(SpectralState *s, const double *d_rho, cudaStream_t st, int64_t *launches, std::string &err);
// nsteps semi-implicit steps (src/integrators/PseudospectralCPU.cpp:112-136).
int spectral_step(SpectralState *s, int64_t nsteps, cudaStream_t st, int64_t *launches, std::string &err);
// Real-space density of the current state into d_rho.
int spectral_real(SpectralState *s, double *d_rho, cudaStream_t st, int64_t *launches, std::string &err);

}  // namespace chgb
