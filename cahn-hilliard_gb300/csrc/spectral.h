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

// ---- batched 2D steps over many boxes (batch.cu) ----------------------------
// One replica as the batched kernels see it; launch shapes are for 256-thread CTAs.
struct PsBatchRep {
    double2 *work, *psi_hat;
    const double *alpha, *beta;
    const double2 *tw;
    ModelDev m;
    int N, M, log2M, log2N, H;
    int row_rpc, row_tpl;   // rows per CTA, threads per row line
    int col_C, col_tpl;     // columns per CTA, threads per column line
    long long bins, hat;
};
constexpr int PS_BATCH_THREADS = 256;
// 2D, N in [8, 1024]: the state can join a batch.
bool spectral_batchable(const SpectralState *s);
// Fill the descriptor; returns the dynamic shared memory its row and column CTAs need.
void spectral_batch_rep(const SpectralState *s, PsBatchRep *r, size_t *row_smem, size_t *col_smem);
// Whether the next step can start from the half spectrum (false right after an upload).
bool spectral_hat_valid(const SpectralState *s);
// Record `nsteps` steps taken by batched kernels.
void spectral_mark_stepped(SpectralState *s);
cudaError_t configure_ps2d_batch(int kind, size_t row_smem, size_t col_smem);
cudaError_t launch_ps2d_batch(int kind, const PsBatchRep *reps, const int2 *row_items, int nrow, const int4 *col_items,
                              int ncol, size_t row_smem, size_t col_smem, cudaStream_t st);

}  // namespace chgb
