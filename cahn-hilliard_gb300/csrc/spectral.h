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

// Scaled half spectrum psi_t = rho_hat / N^dims of one species (the master state).
const double2 *spectral_psi_hat(const SpectralState *s, int species);
double2 *spectral_psi_hat_mut(SpectralState *s);
// FFTW-style unnormalised transforms of S-species fields on caller buffers
// (the half spectrum in the state's layout); c2r overwrites `hat`.
cudaError_t spectral_r2c(SpectralState *s, const double *real, double2 *hat, cudaStream_t st, int *launches);
cudaError_t spectral_c2r(SpectralState *s, double2 *hat, double *real, cudaStream_t st, int *launches);
long long spectral_hat_size(const SpectralState *s);   // complex values per species

// ---- the variable-mobility step's transforms with its pointwise stages fused
// (psmob.cu; dims >= 2).  Each gives the same bits as the plain transform plus
// the matching elementwise stage of src/integrators/PseudospectralMobilityCPU.cpp.
struct PsmobTables {
    const double *q2, *dealias;   // |k|^2 and the dealiasing mask, half-spectrum layout
    int use_dealias;
};
// fder_hat = R2C(f'(rho)); with mu non-null also mu = D (fder_hat + two_k q2 rho_hat) (:245-254).
cudaError_t spectral_psmob_fprime(SpectralState *s, const double *rho, double2 *fder_hat, double2 *mu,
                                  const double2 *rho_hat, const PsmobTables &t, double two_k, cudaStream_t st,
                                  int *launches);
// One axis of the flux divergence (:258-293): g = C2R(D i k_d src), g <- (M - M0) g / N^d
// (M g / N^d when M0 is null), div (= if first, += otherwise) i k_d D R2C(g).  scratch: a half spectrum.
cudaError_t spectral_psmob_flux(SpectralState *s, const double2 *src, const double *kd, const PsmobTables &t,
                                const double *mob, const double *M0, double2 *div, bool first, double2 *scratch,
                                cudaStream_t st, int *launches);
// The semi-implicit update of rho_hat (:296-306; div_hat null: constant mobility) and rho = C2R(rho_hat / N^d).
cudaError_t spectral_psmob_update(SpectralState *s, double2 *rho_hat, const double2 *fder_hat, const double2 *div_hat,
                                  const double *q2, const double *M0, double dt, double Ssplit, double k0,
                                  double2 *scratch, double *rho, cudaStream_t st, int *launches);

// ---- adjoint support (adjoint.cu) -------------------------------------------
// psi_hat <- hat and the transformed rows a step starts from.
cudaError_t spectral_load_hat(SpectralState *s, const double2 *hat, cudaStream_t st);
// One forward step from the half spectrum, also writing rho_n (real) to real_out.
cudaError_t spectral_step_record(SpectralState *s, double *real_out, cudaStream_t st);
// real_out = C2R(hat_scaled), unnormalised (a scaled state gives the field).
cudaError_t spectral_inverse(SpectralState *s, const double2 *hat_scaled, double *real_out, cudaStream_t st);

struct SpectralAdj;
bool spectral_adjoint_supported(const SpectralState *s);   // 2D, Landau, one species
SpectralAdj *spectral_adj_create(SpectralState *s, std::string &err);
void spectral_adj_destroy(SpectralAdj *a);
double2 *spectral_adj_lam(SpectralAdj *a);                  // lam_hat (R2C of the adjoint field)
cudaError_t spectral_adj_zero(SpectralAdj *a, const SpectralState *s, cudaStream_t st);
cudaError_t spectral_adj_add_seed(SpectralAdj *a, const SpectralState *s, const double2 *x, double scale,
                                  cudaStream_t st);
// mode 1: start a step (gradient sums, beta lam_hat, inverse y); 2: finish a step
// (forward y, lam_hat update); 3: finish one step and start the previous one.
cudaError_t spectral_adj_col(SpectralAdj *a, SpectralState *s, int mode, const double2 *psi_next,
                             const double2 *psi_cur, cudaStream_t st);
cudaError_t spectral_adj_row(SpectralAdj *a, SpectralState *s, const double *psi_n, cudaStream_t st);
// {dL/deps, dL/dk, dL/dM} from the fixed-order partial sums.
int spectral_adj_grads(SpectralAdj *a, double *g3);

// ---- batched 2D steps over many boxes (batch.cu) ----------------------------
// One replica as the batched kernels see it; launch shapes are for 256-thread CTAs.
struct PsBatchRep {
    double2 *work, *psi_hat;
    const double *alpha, *beta;
    const int4 *twf;        // fixed-point twiddles (bfp.cuh)
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
