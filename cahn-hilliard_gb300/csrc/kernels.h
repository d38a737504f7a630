// kernels.h — internal launchers shared by the translation units of libchgb.
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "common.cuh"

namespace chgb {

// One fused `euler` / `euler_mobility` time step, psi_in -> psi_out (euler.cu).
// With configure = true nothing is launched: the kernel that would run gets its
// shared-memory attribute set (done once per handle, outside graph capture).
cudaError_t launch_euler_step(int integrator, const Geom &g, const ModelDev &m, const EulerConsts &c,
                              const double *in, double *out, cudaStream_t st, bool configure = false);

// The same step as two kernels (mu/M for every cell into `mu`/`mob`, then the
// update): no halo recomputation, bit-identical results.  Needs dims >= 2 and
// N >= 32 (euler_split_supported).  `mob` is used by the free-energy mobility only.
bool euler_split_supported(const Geom &g);
// Two `euler` steps per launch (small 2D boxes): in -> out after two steps;
// `mid`, when given, receives the state after the first.
bool euler_two_supported(int integrator, const Geom &g);
cudaError_t launch_euler_two(const Geom &g, const ModelDev &m, const EulerConsts &c, const double *in, double *out,
                             cudaStream_t st, bool configure = false, double *mid = nullptr);
// The whole 2D `euler` box (N = 32 or 64) in one 16-CTA cluster's shared memory:
// `nsteps` (>= 1) steps in one launch, in -> out.  With configure = true the
// kernel opts in to the 16-CTA cluster and the call fails unless the GPU can
// hold one.
bool euler_cluster_supported(int integrator, const Geom &g);
cudaError_t launch_euler_cluster(const Geom &g, const ModelDev &m, const EulerConsts &c, const double *in,
                                 double *out, int nsteps, cudaStream_t st, bool configure = false);
cudaError_t launch_euler_split(int integrator, const Geom &g, const ModelDev &m, const EulerConsts &c,
                               const double *in, double *out, double *mu, double *mob, cudaStream_t st);

// Block fixed point (kernel_variant 5; euler.cu): plain `euler` with the
// Landau model, dims >= 2, N >= 32; in 3D the split pair (mu stored in `mu` as
// integers), in 2D one kernel per step (`mu` unused).  One exponent for the whole
// field per step; not the other variants' bits (within a few units of 2^-56 of
// the field's largest value per step).  BfpState lives in device memory and
// must hold the field's key before the first step of a sequence:
// launch_bfp_refresh (a memset and one kernel) sets it from psi.
constexpr int BFP_SLOTS = 32, BFP_SLOT_STRIDE = 16;   // key slots, one per 128-byte line
struct BfpState {
    // (generation << 16) | largest biased exponent of |psi|, over the slots
    // key[bank][j * BFP_SLOT_STRIDE] (each CTA folds into one of them).  The 3D
    // pair uses bank 0; the 2D kernel, which reads a key and folds the next in
    // one launch, reads the bank of the step's ping-pong parity and folds into
    // the other.
    unsigned long long key[2][BFP_SLOTS * BFP_SLOT_STRIDE];
    unsigned long long gen;   // generation this step's update kernel writes (set by the mu kernel)
    int lmu;                  // this step's mu is stored as integers in units of 2^lmu (mode 1)
    int mode;                 // 1 block fixed point; 0 FP64 sums (zero, subnormal, huge or non-finite fields)
};
struct BfpConsts {
    long long mc;   // c2's 53-bit mantissa times 2^10, signed
    int ec;         // c2's biased exponent (1 for zero and subnormals)
    int elin;       // |2 D c2 - eps| + 2 D |c2| < 2^elin
};
bool euler_bfp_supported(int integrator, int model_kind, const Geom &g);
// One step; `parity` is the ping-pong parity of `in` (the 2D kernel's key bank).
cudaError_t launch_euler_bfp(const Geom &g, const EulerConsts &c, const double *in, double *out, double *mu,
                             BfpState *st, int parity, cudaStream_t stream);
// The key of psi into key bank `bank` (bfp_key_bank of the box and parity).
cudaError_t launch_bfp_refresh(const double *psi, long long n, BfpState *st, int bank, cudaStream_t stream);
inline int bfp_key_bank(const Geom &g, int parity) { return g.dims == 2 ? parity : 0; }

// One 2D `euler` replica of a batch (batch.cu): buffers 0 and 1 and its constants.
struct EulerBatchRep {
    double *a, *b;
    Geom g;
    ModelDev m;
    EulerConsts c;
};
// One time step of every replica of a batch group: CTA i takes tile items[i].y of
// replica items[i].x; tile 16 (16x16), 32 (32x32) or 64 (64x16).  With
// configure = true only the kernel's shared-memory attribute is set.
cudaError_t launch_euler2d_batch(int kind, int tile, const EulerBatchRep *reps, const int2 *items, int nitems,
                                 int parity, bool configure, cudaStream_t st);

// Elementwise model hooks and reductions (fields.cu).
cudaError_t launch_der_bulk(const ModelDev &m, const double *rho, double *der, long long bins, cudaStream_t st);
cudaError_t launch_set_mobility(const ModelDev &m, const double *rho, double M0, double *mob, long long n,
                                cudaStream_t st);
cudaError_t launch_fill(double *p, double v, long long n, cudaStream_t st);
// p[i] = mean + amp * (a hash of i in [-1/2, 1/2)).
cudaError_t launch_fill_noise(double *p, double mean, double amp, long long n, cudaStream_t st);
// `regularised` / `gel` mobility of the coming step from rho (S species of
// `bins` cells): mob = M rho / (rho + rho_min) per species, or the gel order
// parameter advanced one explicit step and mob = exp(-c / c_0) for every species.
cudaError_t launch_mobility_update(const MobilityDev &md, const double *rho, double *gel, double *mob, int S,
                                   long long bins, cudaStream_t st);
// euler_mobility kernels' mobility kind (1 constant, 2 free energy, 3 field) of a CHGB_MOBILITY_* type.
int mobility_kind(int mobility_type);
// Partial sums of mass and free energy into `partials` (2 * nblocks doubles),
// then the final two values into out[0..1]; returns the launch status.
cudaError_t launch_observables(const Geom &g, const ModelDev &m, const double *k, double dx, const double *rho,
                               double *partials, int nblocks, double *out, cudaStream_t st);
int observables_blocks(const Geom &g);
// Landau pressure field (into `field`, S * bins doubles, when not null) and its
// average into out[0] (out[1] = 0), the same partials layout and block count
// as launch_observables; returns the launch status.
cudaError_t launch_pressure(const Geom &g, double epsilon, const double *k, double dx, const double *rho,
                            double *field, double *partials, int nblocks, double *out, cudaStream_t st);

#ifdef CHGB_BOUNDS_CHECK
// The transforms' record of the bounds-check build (spectral.cu; bounds.cuh).
cudaError_t bc_read_spectral(unsigned long long *first);
#endif

// Store `msg` as the message chgb_last_error(NULL) returns (api.cu).
void record_error(const std::string &msg);

}  // namespace chgb
