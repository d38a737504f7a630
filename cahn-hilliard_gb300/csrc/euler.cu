// euler.cu — fused explicit finite-difference steps (`euler`, `euler_mobility`).
//
// One kernel launch is one time step, one HBM pass: each CTA stages a tile of
// psi with a halo of 2 cells in shared memory, computes the chemical
// potential mu = f'(psi) - 2k lap(psi) on the tile plus a halo of 1 (and, for
// `euler_mobility`, the mobility M on the same cells), then writes
// psi + dt * div(M grad mu) for its tile.  Nothing but psi_in and psi_out
// touches HBM.  3D tiles march along z with rolling planes of psi (5) and
// mu (3) so the halo recomputation stays in x and y only.
//
// Reference: src/integrators/EulerCPU.cpp:18-36 (three passes, Laplacian
// :58-88) and src/integrators/EulerMobilityCPU.cpp:31-83 (face fluxes and the
// divergence of src/integrators/EulerCPU.cpp:114-128).  The 2D and 3D
// neighbour sums are formed in fixed point and rounded once (fxsum.cuh), not
// added in the reference's order (-x, +x, -y, +y, -z, +z); 1D keeps that order.
// Constants are folded (c2 = 2k/dx^2, c1 = dt M/dx^2).  Both move results by at
// most a few ulp per step.
#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "bounds.cuh"
#include "common.cuh"
#include "fxsum.cuh"
#include "kernels.h"

namespace cg = cooperative_groups;

namespace chgb {

// Index checks of the bounds-check build: CHGB_BC (bounds.cuh).

// euler_mobility kernels' mobility kind for a CHGB_MOBILITY_* type.
int mobility_kind(int mobility_type) {
    switch(mobility_type) {
        case CHGB_MOBILITY_FREE_ENERGY: return 2;
        case CHGB_MOBILITY_REGULARISED:
        case CHGB_MOBILITY_GEL: return 3;
        default: return 1;
    }
}

// f' of one cell; with the free-energy mobility of simple_wertheim it also
// returns X(rho), which the mobility of the same cell reuses.
template <int KIND, int MOB>
__device__ __forceinline__ double der_bulk_x(const ModelDev &m, const double *r, double *d) {
    if constexpr(KIND == CHGB_MODEL_SIMPLE_WERTHEIM && MOB == 2) {
        const double X = sw_X(m, r[0]);
        d[0] = sw_der_given_X(m, r[0], X);
        return X;
    }
    else {
        der_bulk<KIND>(m, r, d);
        return 0.0;
    }
}

// The mobility of one cell for the template mobility kind: 1 constant, 2 the
// free-energy mobility of the cell's density (X from der_bulk_x), 3 the field
// computed before the step (regularised / gel; `gi` is the cell's index in one
// species' field).
template <int MOB>
__device__ __forceinline__ double cell_mobility(const ModelDev &m, const EulerConsts &c, int s, double r, double X,
                                                size_t bins, size_t gi) {
    if constexpr(MOB == 2) return sw_mobility_given_X(m, c.M, r, X);
    else if constexpr(MOB == 3) return CHGB_BC(40, gi, bins) ? c.mobf[s * bins + gi] : 0.0;
    else return c.M;
}

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------

// Sum of the 2*DIMS neighbours of p and lap = sum - 2*DIMS*v (1D: the
// reference's FP64 sum; 2D and 3D: fx_sum).
template <int DIMS>
__device__ __forceinline__ double lap_sum(const double *p, int sx, int sy, int sz, double v) {
    if constexpr(DIMS == 1) return fma(-2.0, v, p[-sx] + p[sx]);
    else if constexpr(DIMS == 2) return lap4(p[-sx], p[sx], p[-sy], p[sy], v);
    else return lap6(p[-sx], p[sx], p[-sy], p[sy], p[-sz], p[sz], v);
}

// Sum of the 2*DIMS neighbours only (DIMS 1, 2).
template <int DIMS>
__device__ __forceinline__ double nb_sum(const double *p, int sx, int sy) {
    if constexpr(DIMS == 1) return p[-sx] + p[sx];
    else return nb_sum4(p[-sx], p[sx], p[-sy], p[sy]);
}

// Chemical potential of one cell and species from its value r, its model
// derivative d (unused for Landau) and the sum of its 2*DIMS neighbours:
//   mu = f'(r) - c2 (sum - 2 DIMS r).
// For Landau f' = r^3 - eps r is folded with the diagonal of the Laplacian,
//   mu = r (r^2 + (2 DIMS c2 - eps)) - c2 sum,
// one FP64 instruction fewer per cell; the FP64 pipe is this kernel's bound.
template <int KIND, int DIMS>
__device__ __forceinline__ double mu_cell(const ModelDev &m, const EulerConsts &c, int s, double r, double d,
                                          double sum) {
    if constexpr(KIND == CHGB_MODEL_LANDAU) {
        return fma(-c.c2[s], sum, r * fma(r, r, c.lshift[DIMS - 1]));
    }
    else {
        return fma(-c.c2[s], fma(-2.0 * DIMS, r, sum), d);
    }
}

// ---------------------------------------------------------------------------
// 1D: tiles of T cells
// ---------------------------------------------------------------------------
template <int KIND, int MOB, int T>
__global__ void __launch_bounds__(256) euler1d_kernel(const double *__restrict__ in, double *__restrict__ out, Geom g,
                                                      ModelDev m, EulerConsts c) {
    constexpr int S = NSpecies<KIND>::value;
    constexpr int P = T + 4, Q = T + 2;
    __shared__ double psi[S][P];
    __shared__ double mu[S][Q];
    __shared__ double mob[MOB ? S : 1][MOB ? Q : 1];
    const int x0 = blockIdx.x * T;
    const size_t bins = (size_t) g.bins;
    for(int i = threadIdx.x; i < P; i += blockDim.x) {
        int gx = (x0 - 2 + i) & g.mask;
#pragma unroll
        for(int s = 0; s < S; s++) psi[s][i] = CHGB_BC(41, gx, bins) ? in[s * bins + gx] : 0.0;
    }
    __syncthreads();
    for(int i = threadIdx.x; i < Q; i += blockDim.x) {
        double r[S], d[S];
#pragma unroll
        for(int s = 0; s < S; s++) r[s] = psi[s][i + 1];
        const double xsw = der_bulk_x<KIND, MOB>(m, r, d);
#pragma unroll
        for(int s = 0; s < S; s++) {
            mu[s][i] = mu_cell<KIND, 1>(m, c, s, r[s], d[s], nb_sum<1>(&psi[s][i + 1], 1, 0));
            if(MOB) mob[s][i] = cell_mobility<MOB>(m, c, s, r[s], xsw, bins, (size_t) ((x0 - 1 + i) & g.mask));
        }
    }
    __syncthreads();
    for(int i = threadIdx.x; i < T; i += blockDim.x) {
#pragma unroll
        for(int s = 0; s < S; s++) {
            const double *u = &mu[s][i + 1];
            double res;
            if(MOB) {
                const double *mm = &mob[s][i + 1];
                double jp = (mm[0] + mm[1]) * (u[1] - u[0]);
                double jm = (mm[-1] + mm[0]) * (u[0] - u[-1]);
                res = fma(c.dt * c.half_inv_dx2, jp - jm, psi[s][i + 2]);
            }
            else {
                res = fma(c.c1, lap_sum<1>(u, 1, 0, 0, u[0]), psi[s][i + 2]);
            }
            if(CHGB_BC(42, x0 + i, bins)) out[s * bins + x0 + i] = res;
        }
    }
}

// ---------------------------------------------------------------------------
// 2D: TX x TY tiles, 256 threads
// ---------------------------------------------------------------------------
// One TX x TY tile at (x0, y0); shared by the single-box and the batched kernels.
template <int KIND, int MOB, int TX, int TY>
__device__ __forceinline__ void euler2d_tile(const double *__restrict__ in, double *__restrict__ out, const Geom &g,
                                             const ModelDev &m, const EulerConsts &c, int x0, int y0, double *smem) {
    constexpr int S = NSpecies<KIND>::value;
    constexpr int PX = TX + 4, PY = TY + 4, PP = PX * PY;
    constexpr int MX = TX + 2, MY = TY + 2, MP = MX * MY;
    double *psi = smem;               // [S][PY][PX]
    double *mu = psi + S * PP;        // [S][MY][MX]
    double *mob = mu + S * MP;        // [S][MY][MX] (euler_mobility only)
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;
    const int nthr = blockDim.x * blockDim.y;
    const size_t bins = (size_t) g.bins;

    for(int i = tid; i < PP; i += nthr) {
        int ly = i / PX, lx = i - ly * PX;
        int gx = (x0 - 2 + lx) & g.mask, gy = (y0 - 2 + ly) & g.mask;
        int gi = gx + (gy << g.log2N);
#pragma unroll
        for(int s = 0; s < S; s++) psi[s * PP + i] = CHGB_BC(43, gi, bins) ? in[s * bins + gi] : 0.0;
    }
    __syncthreads();
    for(int i = tid; i < MP; i += nthr) {
        int ly = i / MX, lx = i - ly * MX;
        int p = (ly + 1) * PX + (lx + 1);
        if(!CHGB_BC(44, p - PX, PP) || !CHGB_BC(44, p + PX, PP)) continue;
        double r[S], d[S];
#pragma unroll
        for(int s = 0; s < S; s++) r[s] = psi[s * PP + p];
        const double xsw = der_bulk_x<KIND, MOB>(m, r, d);
#pragma unroll
        for(int s = 0; s < S; s++) {
            mu[s * MP + i] = mu_cell<KIND, 2>(m, c, s, r[s], d[s], nb_sum<2>(psi + s * PP + p, 1, PX));
            if(MOB) {
                const size_t gi = (size_t) ((x0 - 1 + lx) & g.mask) + ((size_t) ((y0 - 1 + ly) & g.mask) << g.log2N);
                mob[s * MP + i] = cell_mobility<MOB>(m, c, s, r[s], xsw, bins, gi);
            }
        }
    }
    __syncthreads();
    for(int i = tid; i < TX * TY; i += nthr) {
        int ly = i / TX, lx = i - ly * TX;
        int q = (ly + 1) * MX + (lx + 1);
        int gi = (x0 + lx) + ((y0 + ly) << g.log2N);
        if(!CHGB_BC(45, q - MX, MP) || !CHGB_BC(45, q + MX, MP) || !CHGB_BC(45, gi, bins)) continue;
#pragma unroll
        for(int s = 0; s < S; s++) {
            const double *u = mu + s * MP + q;
            double psi0 = psi[s * PP + (ly + 2) * PX + (lx + 2)];
            double res;
            if(MOB) {
                const double *mm = mob + s * MP + q;
                double jxp = (mm[0] + mm[1]) * (u[1] - u[0]);
                double jxm = (mm[-1] + mm[0]) * (u[0] - u[-1]);
                double jyp = (mm[0] + mm[MX]) * (u[MX] - u[0]);
                double jym = (mm[-MX] + mm[0]) * (u[0] - u[-MX]);
                double div = (jxp - jxm) + (jyp - jym);
                res = fma(c.dt * c.half_inv_dx2, div, psi0);
            }
            else {
                res = fma(c.c1, lap_sum<2>(u, 1, MX, 0, u[0]), psi0);
            }
            out[s * bins + gi] = res;
        }
    }
}

template <int KIND, int MOB, int TX, int TY>
__global__ void __launch_bounds__(256) euler2d_kernel(const double *__restrict__ in, double *__restrict__ out, Geom g,
                                                      ModelDev m, EulerConsts c) {
    extern __shared__ double smem[];
    euler2d_tile<KIND, MOB, TX, TY>(in, out, g, m, c, blockIdx.x * TX, blockIdx.y * TY, smem);
}

// Two time steps of plain `euler` per launch on a TX x TY tile, for small 2D
// boxes whose steps are too short to hide a launch: psi with a halo of 4 in
// shared memory, mu on the tile + 3, psi after one step on the tile + 2, mu
// again on the tile + 1, psi after two steps on the tile.  The halo costs
// extra FP64 work (16x16 tiles: 15.9 instructions per cell and step against
// 12.6), so it pays only where the launch, not the FP64 pipe, sets the pace.
// Every value comes from the same helpers as euler2d_tile's, so two steps here
// are the same bits as two launches of the one-step kernel.  With `mid` set,
// the state after the first step is stored too (the adjoint's recomputed
// segments keep every state).
template <int KIND, int TX, int TY>
__global__ void __launch_bounds__(256) euler2d_two_kernel(const double *__restrict__ in, double *__restrict__ out,
                                                          double *__restrict__ mid, Geom g, ModelDev m,
                                                          EulerConsts c) {
    constexpr int S = NSpecies<KIND>::value;
    constexpr int P0X = TX + 8, P0 = P0X * (TY + 8);
    constexpr int M0X = TX + 6, M0 = M0X * (TY + 6);
    constexpr int P1X = TX + 4, P1 = P1X * (TY + 4);
    constexpr int M1X = TX + 2, M1 = M1X * (TY + 2);
    extern __shared__ double smem[];
    double *p0 = smem;              // [S][TY + 8][TX + 8]  psi
    double *mu0 = p0 + S * P0;      // [S][TY + 6][TX + 6]  mu(psi)
    double *p1 = mu0 + S * M0;      // [S][TY + 4][TX + 4]  psi after one step
    double *mu1 = p1 + S * P1;      // [S][TY + 2][TX + 2]  mu of that
    const int tid = threadIdx.x + blockDim.x * threadIdx.y, nthr = blockDim.x * blockDim.y;
    const size_t bins = (size_t) g.bins;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
    for(int i = tid; i < P0; i += nthr) {
        int ly = i / P0X, lx = i - ly * P0X;
        int gx = (x0 - 4 + lx) & g.mask, gy = (y0 - 4 + ly) & g.mask;
        size_t gi = (size_t) gx + ((size_t) gy << g.log2N);
#pragma unroll
        for(int s = 0; s < S; s++) p0[s * P0 + i] = CHGB_BC(46, gi, bins) ? in[s * bins + gi] : 0.0;
    }
    __syncthreads();
    for(int i = tid; i < M0; i += nthr) {
        int ly = i / M0X, lx = i - ly * M0X;
        int p = (ly + 1) * P0X + (lx + 1);
        if(!CHGB_BC(47, p - P0X, P0) || !CHGB_BC(47, p + P0X, P0)) continue;
        double r[S], d[S];
#pragma unroll
        for(int s = 0; s < S; s++) r[s] = p0[s * P0 + p];
        der_bulk<KIND>(m, r, d);
#pragma unroll
        for(int s = 0; s < S; s++)
            mu0[s * M0 + i] = mu_cell<KIND, 2>(m, c, s, r[s], d[s], nb_sum<2>(p0 + s * P0 + p, 1, P0X));
    }
    __syncthreads();
    for(int i = tid; i < P1; i += nthr) {
        int ly = i / P1X, lx = i - ly * P1X;
        int q = (ly + 1) * M0X + (lx + 1);
        const bool inner = mid && lx >= 2 && lx < TX + 2 && ly >= 2 && ly < TY + 2;
        const size_t gi = (size_t) (x0 + lx - 2) + ((size_t) (y0 + ly - 2) << g.log2N);
        if(!CHGB_BC(48, q - M0X, M0) || !CHGB_BC(48, q + M0X, M0) || (inner && !CHGB_BC(48, gi, bins))) continue;
#pragma unroll
        for(int s = 0; s < S; s++) {
            const double *u = mu0 + s * M0 + q;
            const double v = fma(c.c1, lap_sum<2>(u, 1, M0X, 0, u[0]), p0[s * P0 + (ly + 2) * P0X + (lx + 2)]);
            p1[s * P1 + i] = v;
            if(inner) mid[s * bins + gi] = v;
        }
    }
    __syncthreads();
    for(int i = tid; i < M1; i += nthr) {
        int ly = i / M1X, lx = i - ly * M1X;
        int p = (ly + 1) * P1X + (lx + 1);
        if(!CHGB_BC(49, p - P1X, P1) || !CHGB_BC(49, p + P1X, P1)) continue;
        double r[S], d[S];
#pragma unroll
        for(int s = 0; s < S; s++) r[s] = p1[s * P1 + p];
        der_bulk<KIND>(m, r, d);
#pragma unroll
        for(int s = 0; s < S; s++)
            mu1[s * M1 + i] = mu_cell<KIND, 2>(m, c, s, r[s], d[s], nb_sum<2>(p1 + s * P1 + p, 1, P1X));
    }
    __syncthreads();
    for(int i = tid; i < TX * TY; i += nthr) {
        int ly = i / TX, lx = i - ly * TX;
        int q = (ly + 1) * M1X + (lx + 1);
        size_t gi = (size_t) (x0 + lx) + ((size_t) (y0 + ly) << g.log2N);
        if(!CHGB_BC(50, q - M1X, M1) || !CHGB_BC(50, q + M1X, M1) || !CHGB_BC(50, gi, bins)) continue;
#pragma unroll
        for(int s = 0; s < S; s++) {
            const double *u = mu1 + s * M1 + q;
            out[s * bins + gi] = fma(c.c1, lap_sum<2>(u, 1, M1X, 0, u[0]), p1[s * P1 + (ly + 2) * P1X + (lx + 2)]);
        }
    }
}

// 2D `euler` on a box small enough to live in the shared memory of one
// thread-block cluster (N = 4 T: 16 CTAs, one T x T tile each).  Each CTA keeps
// its tile in shared memory for the whole launch, double-buffered, and one
// launch runs many steps: global memory is read at the start and written at
// the end.  A step:
//   1. gathers the 2-cell halo ring of psi from the neighbouring CTAs' shared
//      memory (distributed shared memory; each thread's remote addresses are
//      resolved once per launch);
//   2. computes mu on the ring of the tile + 1 that needs the halo;
//   3. updates the tile into the other buffer;
//   4. arrives on the cluster barrier (publishing the new tile), computes mu on
//      the tile's interior for the next step -- local data only, which hides the
//      barrier's latency -- and waits on the barrier.
// The barrier also orders every remote read of a buffer before its next
// overwrite.  The values come from the same helpers as euler2d_tile's: the
// same bits as one launch per step.
constexpr int CLUSTER_TILES = 4;   // tiles per side of the box: 16 CTAs per cluster

// Position (ly, lx) in the (T + 4)^2 psi frame of halo-ring cell r (the frame
// minus its central T x T tile): two full rows on top and below, then two
// columns on each side.
__device__ __forceinline__ void cluster_ring_psi(int r, int T, int &ly, int &lx) {
    const int PX = T + 4;
    if(r < 2 * PX) {
        ly = r / PX;
        lx = r - ly * PX;
    }
    else if(r < 4 * PX) {
        r -= 2 * PX;
        ly = T + 2 + r / PX;
        lx = r % PX;
    }
    else if(r < 4 * PX + 2 * T) {
        r -= 4 * PX;
        ly = 2 + r / 2;
        lx = r % 2;
    }
    else {
        r -= 4 * PX + 2 * T;
        ly = 2 + r / 2;
        lx = T + 2 + r % 2;
    }
}

// Position (my, mx) in the (T + 2)^2 mu frame of ring cell r (8 T cells: the
// frame minus the (T - 2)^2 cells whose stencil stays on the tile).
__device__ __forceinline__ void cluster_ring_mu(int r, int T, int &my, int &mx) {
    const int MX = T + 2;
    if(r < 2 * MX) {
        my = r / MX;
        mx = r - my * MX;
    }
    else if(r < 4 * MX) {
        r -= 2 * MX;
        my = T + r / MX;
        mx = r % MX;
    }
    else if(r < 4 * MX + 2 * (T - 2)) {
        r -= 4 * MX;
        my = 2 + r / 2;
        mx = r % 2;
    }
    else {
        r -= 4 * MX + 2 * (T - 2);
        my = 2 + r / 2;
        mx = T + r % 2;
    }
}

template <int KIND, int T>
__device__ __forceinline__ void cluster_mu_cell(const ModelDev &m, const EulerConsts &c, const double (*P)[(T + 4) * (T + 4)],
                                                double (*MU)[(T + 2) * (T + 2)], int my, int mx) {
    constexpr int S = NSpecies<KIND>::value, PX = T + 4, MX = T + 2;
    const int p = (my + 1) * PX + (mx + 1);
    if(!CHGB_BC(51, p - PX, (T + 4) * (T + 4)) || !CHGB_BC(51, p + PX, (T + 4) * (T + 4)) ||
       !CHGB_BC(51, my * MX + mx, (T + 2) * (T + 2)))
        return;
    double r[S], d[S];
#pragma unroll
    for(int s = 0; s < S; s++) r[s] = P[s][p];
    der_bulk<KIND>(m, r, d);
#pragma unroll
    for(int s = 0; s < S; s++) MU[s][my * MX + mx] = mu_cell<KIND, 2>(m, c, s, r[s], d[s], nb_sum<2>(&P[s][p], 1, PX));
}

template <int KIND, int T, int NTHR>
__global__ void __launch_bounds__(NTHR) euler2d_cluster_kernel(const double *__restrict__ in,
                                                               double *__restrict__ out, Geom g, ModelDev m,
                                                               EulerConsts c, int nsteps) {
    static_assert(NTHR >= T * T, "one tile cell per thread");
    constexpr int S = NSpecies<KIND>::value;
    constexpr int TT = T * T, NT = CLUSTER_TILES * CLUSTER_TILES;
    constexpr int PX = T + 4, PP = PX * PX, MX = T + 2, MP = MX * MX;
    constexpr int NRING = PP - TT, NRING_MU = 8 * T, NINNER = (T - 2) * (T - 2);
    constexpr int KR = (NRING + NTHR - 1) / NTHR;   // halo-ring cells per thread
    __shared__ double own[2][S][TT];
    __shared__ double P[S][PP];        // psi on the tile + 2 (centre: this step's tile)
    __shared__ double MU[S][MP];       // mu on the tile + 1
    __shared__ unsigned rank_of[NT];   // cluster rank of the CTA that owns tile (tx, ty), at tx + 4 ty
    cg::cluster_group cluster = cg::this_cluster();
    const int tid = threadIdx.x;
    const bool cell = tid < TT;
    const int ly0 = (cell ? tid : 0) / T, lx0 = (cell ? tid : 0) % T;
    const int x0 = blockIdx.x * T, y0 = blockIdx.y * T;
    const size_t bins = (size_t) g.bins;
    const size_t gi0 = (size_t) (x0 + lx0) + ((size_t) (y0 + ly0) << g.log2N);
    const int pc = (ly0 + 2) * PX + (lx0 + 2);
    if(cell && CHGB_BC(52, gi0, bins)) {
#pragma unroll
        for(int s = 0; s < S; s++) {
            const double v = in[s * bins + gi0];
            own[0][s][tid] = v;
            P[s][pc] = v;
        }
    }
    // every CTA of the cluster is running past this barrier: publish this
    // CTA's rank into every CTA's table, then wait until all tables are full
    cluster.sync();
    if(tid < NT) {
        unsigned *dst = cluster.map_shared_rank(rank_of, (unsigned) tid);
        dst[blockIdx.x + CLUSTER_TILES * blockIdx.y] = cluster.block_rank();
    }
    cluster.sync();
    int rp[KR];
    const double *src[2][KR];
#pragma unroll
    for(int k = 0; k < KR; k++) {
        const int r = (tid + k * NTHR < NRING) ? tid + k * NTHR : 0;
        int ly, lx;
        cluster_ring_psi(r, T, ly, lx);
        rp[k] = ly * PX + lx;
        const int gx = (x0 - 2 + lx) & g.mask, gy = (y0 - 2 + ly) & g.mask;
        const int tx = gx / T, ty = gy / T;
        int off = (gx - tx * T) + (gy - ty * T) * T;
        int tile = tx + CLUSTER_TILES * ty;
        if(!CHGB_BC(53, off, TT) || !CHGB_BC(53, tile, NT) || !CHGB_BC(53, rp[k], PP)) {
            off = 0;
            tile = 0;
            rp[k] = 0;
        }
        src[0][k] = cluster.map_shared_rank(&own[0][0][0], rank_of[tile]) + off;
        src[1][k] = cluster.map_shared_rank(&own[1][0][0], rank_of[tile]) + off;
    }
    for(int j = tid; j < NINNER; j += NTHR) cluster_mu_cell<KIND, T>(m, c, P, MU, 2 + j / (T - 2), 2 + j % (T - 2));
    for(int step = 0; step < nsteps; step++) {
        const int cur = step & 1;
        double v[KR][S];
#pragma unroll
        for(int k = 0; k < KR; k++) {
            const double *q = cur ? src[1][k] : src[0][k];
#pragma unroll
            for(int s = 0; s < S; s++) v[k][s] = (tid + k * NTHR < NRING) ? q[s * TT] : 0.0;
        }
#pragma unroll
        for(int k = 0; k < KR; k++)
            if(tid + k * NTHR < NRING) {
#pragma unroll
                for(int s = 0; s < S; s++) P[s][rp[k]] = v[k][s];
            }
        __syncthreads();
        for(int r = tid; r < NRING_MU; r += NTHR) {
            int my, mx;
            cluster_ring_mu(r, T, my, mx);
            cluster_mu_cell<KIND, T>(m, c, P, MU, my, mx);
        }
        __syncthreads();
        if(cell) {
            const int q = (ly0 + 1) * MX + (lx0 + 1);
#pragma unroll
            for(int s = 0; s < S; s++) {
                const double nv = fma(c.c1, lap_sum<2>(&MU[s][q], 1, MX, 0, MU[s][q]), P[s][pc]);
                own[cur ^ 1][s][tid] = nv;
                P[s][pc] = nv;
            }
        }
        __syncthreads();
        asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
        for(int j = tid; j < NINNER; j += NTHR) cluster_mu_cell<KIND, T>(m, c, P, MU, 2 + j / (T - 2), 2 + j % (T - 2));
        asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
    }
    if(cell && CHGB_BC(54, gi0, bins)) {
#pragma unroll
        for(int s = 0; s < S; s++) out[s * bins + gi0] = own[nsteps & 1][s][tid];
    }
}

// Batched 2D `euler`: CTA b takes tile items[b].y of replica items[b].x; every
// replica steps a -> b (parity 0) or b -> a (parity 1).  All tiles have the
// same size, so the CTAs carry equal work whatever the replicas' N.
template <int KIND, int TX, int TY>
__global__ void __launch_bounds__(256) euler2d_batch_kernel(const EulerBatchRep *__restrict__ reps,
                                                            const int2 *__restrict__ items, int parity) {
    extern __shared__ double smem[];
    const int2 it = items[blockIdx.x];
    const EulerBatchRep &r = reps[it.x];
    const int tiles_x = r.g.N / TX;
    const int ty = it.y / tiles_x, tx = it.y - ty * tiles_x;
    const double *in = parity ? r.b : r.a;
    double *out = parity ? r.a : r.b;
    euler2d_tile<KIND, 0, TX, TY>(in, out, r.g, r.m, r.c, tx * TX, ty * TY, smem);
}

// ---------------------------------------------------------------------------
// 3D: TX x TY tiles marching over ZC planes, rolling windows in shared memory
// ---------------------------------------------------------------------------
template <int KIND, int MOB, int TX, int TY>
__global__ void __launch_bounds__(256) euler3d_kernel(const double *__restrict__ in, double *__restrict__ out, Geom g,
                                                      ModelDev m, EulerConsts c, int zc) {
    constexpr int S = NSpecies<KIND>::value;
    constexpr int PX = TX + 4, PY = TY + 4, PP = PX * PY;
    constexpr int MX = TX + 2, MY = TY + 2, MP = MX * MY;
    extern __shared__ double smem[];
    double *psi = smem;                    // [5][S][PP]
    double *mu = psi + 5 * S * PP;         // [3][S][MP]
    double *mob = mu + 3 * S * MP;         // [3][S][MP]
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;
    const int nthr = blockDim.x * blockDim.y;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = blockIdx.z * zc;
    const size_t bins = (size_t) g.bins;
    const int sh2 = 2 * g.log2N;

    auto load_plane = [&](int z) {
        double *dst = psi + ((z + 5) % 5) * S * PP;
        size_t zoff = (size_t) (z & g.mask) << sh2;
        for(int i = tid; i < PP; i += nthr) {
            int ly = i / PX, lx = i - ly * PX;
            int gx = (x0 - 2 + lx) & g.mask, gy = (y0 - 2 + ly) & g.mask;
            size_t gi = zoff + gx + (gy << g.log2N);
#pragma unroll
            for(int s = 0; s < S; s++) dst[s * PP + i] = CHGB_BC(55, gi, bins) ? in[s * bins + gi] : 0.0;
        }
    };
    auto mu_plane = [&](int z) {
        const double *pc = psi + ((z + 5) % 5) * S * PP;
        const double *pm = psi + ((z + 4) % 5) * S * PP;
        const double *pp = psi + ((z + 6) % 5) * S * PP;
        double *mdst = mu + ((z + 3) % 3) * S * MP;
        double *bdst = mob + ((z + 3) % 3) * S * MP;
        for(int i = tid; i < MP; i += nthr) {
            int ly = i / MX, lx = i - ly * MX;
            int p = (ly + 1) * PX + (lx + 1);
            if(!CHGB_BC(56, p - PX, PP) || !CHGB_BC(56, p + PX, PP)) continue;
            double r[S], d[S];
#pragma unroll
            for(int s = 0; s < S; s++) r[s] = pc[s * PP + p];
            const double xsw = der_bulk_x<KIND, MOB>(m, r, d);
#pragma unroll
            for(int s = 0; s < S; s++) {
                const double *q = pc + s * PP + p;
                const double sum = nb_sum6(q[-1], q[1], q[-PX], q[PX], pm[s * PP + p], pp[s * PP + p]);
                mdst[s * MP + i] = mu_cell<KIND, 3>(m, c, s, r[s], d[s], sum);
                if(MOB) {
                    const size_t gi = (size_t) ((x0 - 1 + lx) & g.mask) +
                                      ((size_t) ((y0 - 1 + ly) & g.mask) << g.log2N) +
                                      ((size_t) (z & g.mask) << sh2);
                    bdst[s * MP + i] = cell_mobility<MOB>(m, c, s, r[s], xsw, bins, gi);
                }
            }
        }
    };
    auto out_plane = [&](int z) {
        const double *uc = mu + ((z + 3) % 3) * S * MP;
        const double *um = mu + ((z + 2) % 3) * S * MP;
        const double *up = mu + ((z + 4) % 3) * S * MP;
        const double *bc = mob + ((z + 3) % 3) * S * MP;
        const double *bm = mob + ((z + 2) % 3) * S * MP;
        const double *bp = mob + ((z + 4) % 3) * S * MP;
        const double *pc = psi + ((z + 5) % 5) * S * PP;
        size_t zoff = (size_t) z << sh2;
        for(int i = tid; i < TX * TY; i += nthr) {
            int ly = i / TX, lx = i - ly * TX;
            int q = (ly + 1) * MX + (lx + 1);
            size_t gi = zoff + (x0 + lx) + ((y0 + ly) << g.log2N);
            if(!CHGB_BC(57, q - MX, MP) || !CHGB_BC(57, q + MX, MP) || !CHGB_BC(57, gi, bins)) continue;
#pragma unroll
            for(int s = 0; s < S; s++) {
                const double *u = uc + s * MP + q;
                double psi0 = pc[s * PP + (ly + 2) * PX + (lx + 2)];
                double res;
                if(MOB) {
                    const double *mm = bc + s * MP + q;
                    double mzm = bm[s * MP + q], mzp = bp[s * MP + q];
                    double uzm = um[s * MP + q], uzp = up[s * MP + q];
                    double jxp = (mm[0] + mm[1]) * (u[1] - u[0]);
                    double jxm = (mm[-1] + mm[0]) * (u[0] - u[-1]);
                    double jyp = (mm[0] + mm[MX]) * (u[MX] - u[0]);
                    double jym = (mm[-MX] + mm[0]) * (u[0] - u[-MX]);
                    double jzp = (mm[0] + mzp) * (uzp - u[0]);
                    double jzm = (mzm + mm[0]) * (u[0] - uzm);
                    double div = ((jxp - jxm) + (jyp - jym)) + (jzp - jzm);
                    res = fma(c.dt * c.half_inv_dx2, div, psi0);
                }
                else {
                    res = fma(c.c1, lap6(u[-1], u[1], u[-MX], u[MX], um[s * MP + q], up[s * MP + q], u[0]), psi0);
                }
                out[s * bins + gi] = res;
            }
        }
    };

    load_plane(z0 - 2);
    load_plane(z0 - 1);
    load_plane(z0);
    load_plane(z0 + 1);
    __syncthreads();
    mu_plane(z0 - 1);
    mu_plane(z0);
    for(int z = z0; z < z0 + zc; z++) {
        load_plane(z + 2);
        __syncthreads();
        mu_plane(z + 1);
        __syncthreads();
        out_plane(z);
    }
}

// ---------------------------------------------------------------------------
// Split step: kernel 1 writes mu (and the free-energy M) of every cell once,
// kernel 2 reads them back for the update.  No FP64 work is repeated on halo
// cells; the cost is 8 B (16 B with M) per cell and step of extra traffic,
// which is cheap next to the FP64 pipe on this part.  The arithmetic is the
// fused kernels' (the fixed-point sums do not depend on where the terms'
// fixed-point forms are made), so both variants give bit-identical results.
// Tiles are 32 x 8 cells per 256-thread block, one cell per thread; 3D
// marches over `zc` planes with a ring of three planes in shared memory.
// ---------------------------------------------------------------------------
// The plain (Landau, constant-mobility) split kernels are compiled for eight
// CTAs per SM (32 registers a thread): with the plane prefetch in registers
// they would otherwise take 40-46 and fit five or six (3D N=256 on GB300:
// 5.9e10 cell-steps/s at five, 6.5e10 at eight).  The other models' kernels
// need more registers than that and keep the default.
constexpr int STX = 32, STY = 8, SPX = STX + 2, SPY = STY + 2, SPP = SPX * SPY;

// Programmatic dependent launch of the split pair: each kernel waits for the
// previous kernel of the stream to finish (and its writes to land) before its
// first global access, then lets the next kernel's CTAs be placed on the SMs
// this grid no longer needs, which hides the launch gap between the two
// kernels of a step and between steps.  Without the launch attribute the wait
// returns at once.  (Measured on GB300: 2D N=1024 split step 25.9 -> 25.1 us,
// N=256 4.5 -> 4.2 us; the 3D N=256 step is unchanged.  The fused kernels,
// whose single wave would then hold idle waiting CTAs, do not use it.)
__device__ __forceinline__ void pdl_begin() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;");
}

template <int DIMS, int S>
__device__ __forceinline__ void split_load_plane(double (*dst)[SPP], const double *__restrict__ src, const Geom &g,
                                                 int x0, int y0, int z, size_t bins, int tid) {
    const size_t zoff = (DIMS == 3) ? ((size_t) (z & g.mask) << (2 * g.log2N)) : 0;
    for(int i = tid; i < SPP; i += STX * STY) {
        int ly = i / SPX, lx = i - ly * SPX;
        int gx = (x0 - 1 + lx) & g.mask, gy = (y0 - 1 + ly) & g.mask;
        size_t gi = zoff + gx + ((size_t) gy << g.log2N);
#pragma unroll
        for(int s = 0; s < S; s++)
            if(CHGB_BC(1, gi, bins)) dst[s][i] = src[s * bins + gi];
    }
}

// The same plane load for a single-species field, also storing each value's
// fixed-point form (fx_term) for the neighbour sums.
template <int DIMS>
__device__ __forceinline__ void split_load_plane_fx(double *dst, long long *dT, int *dE, const double *__restrict__ src,
                                                    const Geom &g, int x0, int y0, int z, int tid) {
    const size_t zoff = (DIMS == 3) ? ((size_t) (z & g.mask) << (2 * g.log2N)) : 0;
    for(int i = tid; i < SPP; i += STX * STY) {
        int ly = i / SPX, lx = i - ly * SPX;
        int gx = (x0 - 1 + lx) & g.mask, gy = (y0 - 1 + ly) & g.mask;
        const size_t gi = zoff + gx + ((size_t) gy << g.log2N);
        const double v = CHGB_BC(2, gi, g.bins) ? src[gi] : 0.0;
        dst[i] = v;
        fx_term(v, dT[i], dE[i]);
    }
}

// The same, in two halves: fetch a plane's values into registers (two per
// thread: 340 values, 256 threads), then store them with their fixed-point
// forms.  The 3D kernels fetch plane z + 2 while they compute plane z, so the
// global-memory latency of staging is not waited for at the barrier.
constexpr int SPF = (SPP + STX * STY - 1) / (STX * STY);

template <int DIMS>
__device__ __forceinline__ void split_fetch_plane(double (&v)[SPF], const double *__restrict__ src, const Geom &g,
                                                  int x0, int y0, int z, int tid) {
    const size_t zoff = (DIMS == 3) ? ((size_t) (z & g.mask) << (2 * g.log2N)) : 0;
#pragma unroll
    for(int k = 0; k < SPF; k++) {
        const int i = tid + k * STX * STY;
        if(i < SPP) {
            int ly = i / SPX, lx = i - ly * SPX;
            int gx = (x0 - 1 + lx) & g.mask, gy = (y0 - 1 + ly) & g.mask;
            const size_t gi = zoff + gx + ((size_t) gy << g.log2N);
            v[k] = CHGB_BC(3, gi, g.bins) ? src[gi] : 0.0;
        }
    }
}

__device__ __forceinline__ void split_commit_plane_fx(double *dst, long long *dT, int *dE, const double (&v)[SPF],
                                                      int tid) {
#pragma unroll
    for(int k = 0; k < SPF; k++) {
        const int i = tid + k * STX * STY;
        if(i < SPP) {
            dst[i] = v[k];
            fx_term(v[k], dT[i], dE[i]);
        }
    }
}

// Neighbour sum of the cell at p of a staged plane ring (fixed-point forms
// computed at staging): planes c (the cell's), zm and zp (3D).
template <int DIMS, bool INT_ROUND>
__device__ __forceinline__ double split_nb_sum_fx(const double (*ring)[SPP], const long long (*rT)[SPP],
                                                  const int (*rE)[SPP], int c, int zm, int zp, int p) {
    constexpr int K = 2 * DIMS;
    long long T[K];
    int ek[K];
    const int off[4] = {-1, 1, -SPX, SPX};
    if(!CHGB_BC(7, p - SPX, SPP) || !CHGB_BC(7, p + SPX, SPP)) return 0.0;
#pragma unroll
    for(int i = 0; i < 4; i++) {
        T[i] = rT[c][p + off[i]];
        ek[i] = rE[c][p + off[i]];
    }
    if constexpr(DIMS == 3) {
        T[4] = rT[zm][p];
        ek[4] = rE[zm][p];
        T[5] = rT[zp][p];
        ek[5] = rE[zp][p];
    }
    const int emax = fx_emax<K>(ek);
    if(!fx_in_range(emax)) {
        const double *q = &ring[c][p];
        return seq_sum(q[-1], q[1], q[-SPX], q[SPX], DIMS == 3 ? ring[zm][p] : 0.0, DIMS == 3 ? ring[zp][p] : 0.0, K);
    }
    return fx_total<K, INT_ROUND>(T, ek, emax);
}

// The Laplacian's numerator at p of a staged plane ring: the neighbour sum
// minus 2 dims times the centre, rounded once (fx_lap).
template <int DIMS>
__device__ __forceinline__ double split_lap_fx(const double (*ring)[SPP], const long long (*rT)[SPP],
                                               const int (*rE)[SPP], int c, int zm, int zp, int p) {
    constexpr int K = 2 * DIMS;
    long long T[K];
    int ek[K];
    const int off[4] = {-1, 1, -SPX, SPX};
    if(!CHGB_BC(7, p - SPX, SPP) || !CHGB_BC(7, p + SPX, SPP)) return 0.0;
#pragma unroll
    for(int i = 0; i < 4; i++) {
        T[i] = rT[c][p + off[i]];
        ek[i] = rE[c][p + off[i]];
    }
    if constexpr(DIMS == 3) {
        T[4] = rT[zm][p];
        ek[4] = rE[zm][p];
        T[5] = rT[zp][p];
        ek[5] = rE[zp][p];
    }
    const long long Tv = rT[c][p];
    const int ekv = rE[c][p];
    int emax = fx_emax<K>(ek);
    emax = ekv > emax ? ekv : emax;
    if(!fx_in_range(emax)) {
        const double *q = &ring[c][p];
        return fma(-2.0 * DIMS, q[0],
                   seq_sum(q[-1], q[1], q[-SPX], q[SPX], DIMS == 3 ? ring[zm][p] : 0.0, DIMS == 3 ? ring[zp][p] : 0.0, K));
    }
    return fx_total<K>(T, ek, emax, -(long long) K * Tv, ekv);
}

template <int KIND, int MOB, int DIMS>
__global__ void __launch_bounds__(256, (KIND == CHGB_MODEL_LANDAU && MOB == 0) ? 8 : 1) mu_kernel(const double *__restrict__ in, double *__restrict__ mu,
                                                 double *__restrict__ mob, Geom g, ModelDev m, EulerConsts c, int zc) {
    constexpr int S = NSpecies<KIND>::value;
    constexpr int R = (DIMS == 3) ? 3 : 1;
    // single species: each staged value's fixed-point form is computed once,
    // at staging, instead of at each of its seven uses
    constexpr bool PRE = S == 1;
    __shared__ double ring[R][S][SPP];
    __shared__ long long ringT[PRE ? R : 1][PRE ? SPP : 1];
    __shared__ int ringE[PRE ? R : 1][PRE ? SPP : 1];
    const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + STX * ty;
    const int x0 = blockIdx.x * STX, y0 = blockIdx.y * STY;
    const int z0 = (DIMS == 3) ? blockIdx.z * zc : 0;
    const int nz = (DIMS == 3) ? zc : 1;
    const size_t bins = (size_t) g.bins;
    const int p = (ty + 1) * SPX + (tx + 1);
    auto stage = [&](int slot, int z) {
        if constexpr(PRE) split_load_plane_fx<DIMS>(ring[slot][0], ringT[slot], ringE[slot], in, g, x0, y0, z, tid);
        else split_load_plane<DIMS, S>(ring[slot], in, g, x0, y0, z, bins, tid);
    };
    pdl_begin();
    double pf[SPF];   // plane z + 1, fetched during the previous plane (3D single species)
    if constexpr(DIMS == 3) {
        stage((z0 + 2) % 3, z0 - 1);
        stage(z0 % 3, z0);
        if constexpr(PRE) split_fetch_plane<DIMS>(pf, in, g, x0, y0, z0 + 1, tid);
    }
    for(int z = z0; z < z0 + nz; z++) {
        const int cz = (DIMS == 3) ? z % 3 : 0;
        if constexpr(DIMS == 3 && PRE) {
            split_commit_plane_fx(ring[(z + 1) % 3][0], ringT[(z + 1) % 3], ringE[(z + 1) % 3], pf, tid);
            if(z + 1 < z0 + nz) split_fetch_plane<DIMS>(pf, in, g, x0, y0, z + 2, tid);
        }
        else if constexpr(DIMS == 3) stage((z + 1) % 3, z + 1);
        else stage(0, 0);
        __syncthreads();
        double r[S], d[S];
#pragma unroll
        for(int s = 0; s < S; s++) r[s] = ring[cz][s][p];
        const double xsw = der_bulk_x<KIND, MOB>(m, r, d);
        const size_t gi = (size_t) (x0 + tx) + ((size_t) (y0 + ty) << g.log2N) +
                          ((DIMS == 3) ? ((size_t) z << (2 * g.log2N)) : 0);
#pragma unroll
        for(int s = 0; s < S; s++) {
            const double *q = &ring[cz][s][p];
            double sum;
            if constexpr(PRE)
                // 2D Landau: four neighbours leave the integer pipes room, while the
                // mu spends three FP64 instructions of its own -- round in integers
                // (measured on GB300: 2D N=1024 5.92e10 -> 6.23e10 cell-steps/s; in 3D
                // the six-neighbour sum already fills the integer pipe, 5.52e10 -> 5.11e10)
                sum = split_nb_sum_fx<DIMS, KIND == CHGB_MODEL_LANDAU && DIMS == 2>(
                    reinterpret_cast<const double (*)[SPP]>(&ring[0][0][0]), ringT, ringE, cz, (z + 2) % 3, (z + 1) % 3, p);
            else
                sum = (DIMS == 3) ? nb_sum6(q[-1], q[1], q[-SPX], q[SPX], ring[(z + 2) % 3][s][p], ring[(z + 1) % 3][s][p])
                                  : nb_sum4(q[-1], q[1], q[-SPX], q[SPX]);
            if(CHGB_BC(4, gi, bins)) mu[s * bins + gi] = mu_cell<KIND, DIMS>(m, c, s, r[s], d[s], sum);
            if(MOB == 2) mob[s * bins + gi] = sw_mobility_given_X(m, c.M, r[s], xsw);
        }
        __syncthreads();
    }
}

template <int S, int MOB, int DIMS>
__global__ void __launch_bounds__(256, (S == 1 && MOB == 0) ? 8 : 1) update_kernel(const double *__restrict__ psi_in, const double *__restrict__ mu,
                                                     const double *__restrict__ mob, double *__restrict__ out, Geom g,
                                                     EulerConsts c, int zc) {
    constexpr int R = (DIMS == 3) ? 3 : 1;
    constexpr bool MFIELD = MOB >= 2;   // per-cell mobility read from `mob` (written by mu_kernel or given)
    constexpr int MR = MFIELD ? R : 1;
    constexpr bool PRE = S == 1 && MOB == 0;   // fixed-point forms staged with mu (see mu_kernel)
    // single-species euler_mobility: each face flux (M_i + M_j)(mu_j - mu_i) is
    // formed once -- x and y faces of a plane in shared memory, the z face
    // carried from one plane to the next in a register -- instead of once by
    // each of its two cells.  Same expression, so the same bits.
    constexpr bool FACES = S == 1 && MOB != 0;
    constexpr int FXW = STX + 1, FXN = FXW * STY, FYN = STX * (STY + 1);
    __shared__ double ring[R][S][SPP];
    __shared__ double mring[MR][MFIELD ? S : 1][MFIELD ? SPP : 1];
    __shared__ double fx[FACES ? FXN : 1], fy[FACES ? FYN : 1];
    __shared__ long long ringT[PRE ? R : 1][PRE ? SPP : 1];
    __shared__ int ringE[PRE ? R : 1][PRE ? SPP : 1];
    const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + STX * ty;
    const int x0 = blockIdx.x * STX, y0 = blockIdx.y * STY;
    const int z0 = (DIMS == 3) ? blockIdx.z * zc : 0;
    const int nz = (DIMS == 3) ? zc : 1;
    const size_t bins = (size_t) g.bins;
    const int p = (ty + 1) * SPX + (tx + 1);
    auto stage = [&](int slot, int z) {
        if constexpr(PRE) split_load_plane_fx<DIMS>(ring[slot][0], ringT[slot], ringE[slot], mu, g, x0, y0, z, tid);
        else split_load_plane<DIMS, S>(ring[slot], mu, g, x0, y0, z, bins, tid);
    };
    pdl_begin();
    double pf[SPF];   // plane z + 1 of mu, fetched during the previous plane (3D single species)
    double jz_prev = 0.0;   // FACES, 3D: the z face below the next plane (this plane's upper face)
    if constexpr(DIMS == 3) {
        stage((z0 + 2) % 3, z0 - 1);
        stage(z0 % 3, z0);
        if constexpr(PRE) split_fetch_plane<DIMS>(pf, mu, g, x0, y0, z0 + 1, tid);
        if constexpr(MFIELD) {
            split_load_plane<DIMS, S>(mring[(z0 + 2) % 3], mob, g, x0, y0, z0 - 1, bins, tid);
            split_load_plane<DIMS, S>(mring[z0 % 3], mob, g, x0, y0, z0, bins, tid);
        }
    }
    for(int z = z0; z < z0 + nz; z++) {
        const int cz = (DIMS == 3) ? z % 3 : 0, zm = (z + 2) % 3, zp = (z + 1) % 3;
        const size_t gi = (size_t) (x0 + tx) + ((size_t) (y0 + ty) << g.log2N) +
                          ((DIMS == 3) ? ((size_t) z << (2 * g.log2N)) : 0);
        // the cell's psi is read before the plane is staged, so that its
        // latency overlaps the staging and the barrier
        double psi_cell[S];
#pragma unroll
        for(int s = 0; s < S; s++) psi_cell[s] = CHGB_BC(5, gi, bins) ? psi_in[s * bins + gi] : 0.0;
        if constexpr(DIMS == 3) {
            if constexpr(PRE) {
                split_commit_plane_fx(ring[zp][0], ringT[zp], ringE[zp], pf, tid);
                if(z + 1 < z0 + nz) split_fetch_plane<DIMS>(pf, mu, g, x0, y0, z + 2, tid);
            }
            else stage(zp, z + 1);
            if constexpr(MFIELD) split_load_plane<DIMS, S>(mring[zp], mob, g, x0, y0, z + 1, bins, tid);
        }
        else {
            stage(0, 0);
            if constexpr(MFIELD) split_load_plane<DIMS, S>(mring[0], mob, g, x0, y0, 0, bins, tid);
        }
        __syncthreads();
        if constexpr(FACES) {
            // x face f between tile columns lx - 1 and lx (lx in 0..STX), y face
            // between tile rows ly - 1 and ly (ly in 0..STY)
            for(int f = tid; f < FXN + FYN; f += STX * STY) {
                int a, b;
                if(f < FXN) {
                    const int ly = f / FXW, lx = f - ly * FXW;
                    a = (ly + 1) * SPX + lx;
                    b = a + 1;
                }
                else {
                    const int g2 = f - FXN, ly = g2 / STX, lx = g2 - ly * STX;
                    a = ly * SPX + lx + 1;
                    b = a + SPX;
                }
                const double ma = MFIELD ? mring[cz][0][a] : c.M, mb = MFIELD ? mring[cz][0][b] : c.M;
                const double j = (ma + mb) * (ring[cz][0][b] - ring[cz][0][a]);
                if(f < FXN) fx[f] = j;
                else fy[f - FXN] = j;
            }
            __syncthreads();
        }
#pragma unroll
        for(int s = 0; s < S; s++) {
            const double *u = &ring[cz][s][p];
            const double psi0 = psi_cell[s];
            double res;
            if(FACES) {
                const double jxm = fx[ty * FXW + tx], jxp = fx[ty * FXW + tx + 1];
                const double jym = fy[ty * STX + tx], jyp = fy[(ty + 1) * STX + tx];
                double div = (jxp - jxm) + (jyp - jym);
                if(DIMS == 3) {
                    const double m0 = MFIELD ? mring[cz][s][p] : c.M;
                    const double mzp = MFIELD ? mring[zp][s][p] : c.M;
                    const double jzp = (m0 + mzp) * (ring[zp][s][p] - u[0]);
                    double jzm;
                    if(z == z0) {
                        const double mzm = MFIELD ? mring[zm][s][p] : c.M;
                        jzm = (mzm + m0) * (u[0] - ring[zm][s][p]);
                    }
                    else {
                        jzm = jz_prev;
                    }
                    jz_prev = jzp;
                    div = div + (jzp - jzm);
                }
                res = fma(c.dt * c.half_inv_dx2, div, psi0);
            }
            else if(MOB) {
                double m0, mxm, mxp, mym, myp, mzm = 0, mzp = 0;
                if(MFIELD) {
                    const double *mm = &mring[cz][s][p];
                    m0 = mm[0];
                    mxm = mm[-1];
                    mxp = mm[1];
                    mym = mm[-SPX];
                    myp = mm[SPX];
                    if(DIMS == 3) {
                        mzm = mring[zm][s][p];
                        mzp = mring[zp][s][p];
                    }
                }
                else {
                    m0 = mxm = mxp = mym = myp = mzm = mzp = c.M;
                }
                double jxp = (m0 + mxp) * (u[1] - u[0]);
                double jxm = (mxm + m0) * (u[0] - u[-1]);
                double jyp = (m0 + myp) * (u[SPX] - u[0]);
                double jym = (mym + m0) * (u[0] - u[-SPX]);
                double div = (jxp - jxm) + (jyp - jym);
                if(DIMS == 3) {
                    double jzp = (m0 + mzp) * (ring[zp][s][p] - u[0]);
                    double jzm = (mzm + m0) * (u[0] - ring[zm][s][p]);
                    div = div + (jzp - jzm);
                }
                res = fma(c.dt * c.half_inv_dx2, div, psi0);
            }
            else {
                double lap;
                if constexpr(PRE)
                    lap = split_lap_fx<DIMS>(reinterpret_cast<const double (*)[SPP]>(&ring[0][0][0]), ringT, ringE, cz,
                                             zm, zp, p);
                else
                    lap = (DIMS == 3) ? lap6(u[-1], u[1], u[-SPX], u[SPX], ring[zm][s][p], ring[zp][s][p], u[0])
                                      : lap4(u[-1], u[1], u[-SPX], u[SPX], u[0]);
                res = fma(c.c1, lap, psi0);
            }
            if(CHGB_BC(6, gi, bins)) out[s * bins + gi] = res;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Block fixed point (kernel_variant 5: Landau `euler`): the split pair in 3D
// (mu_bfp_kernel, update_bfp_kernel), one kernel per step in 2D
// (euler2d_bfp_kernel, below), the same arithmetic
// ---------------------------------------------------------------------------
// The split pair above aligns the terms of each neighbour sum to the largest
// exponent of that stencil: per cell a maximum over seven exponents and seven
// variable shifts, about half of a step's integer work.  Here one exponent
// serves the whole field for a step (block floating point, the field being the
// block):
//   - psi: emax, the largest biased exponent of |psi| over the field, is read
//     from BfpState::key (below).  Each value becomes
//     X = floor(psi 2^(1080 - emax)), |X| < 2^58, once, when it is staged, and
//     a neighbour sum is a plain int64 sum.
//   - mu: from emax and the model's constants follows a bound |mu| < 2^Emu,
//     Emu = max(3 s, elin + s) + 2 with |psi| < 2^s and
//     |lshift| + 2 D c2 < 2^elin (|psi|^3 + |lshift psi| + c2 |sum|, one bit
//     spare).  mu goes to HBM in fixed point, M = floor(mu 2^(58 - Emu)),
//     |M| <= 2^57 + 1, so the update's sums need no conversion.  Its two parts
//     are formed apart and subtracted in integers: psi (psi^2 + lshift) in
//     FP64 (the step's only two FP64 instructions of mu), truncated to M's
//     unit, and c2 sum as the high half of the 64 x 64-bit product of the sum
//     with c2's mantissa, shifted to M's unit.
//   - the update: L = sum(M_nb) - 2 D M, exact (|L| < 2^61), and
//     psi' = psi + c1 (L 2^(Emu - 58)): one int64 -> double rounding (on the
//     FP64 pipe or in integers, see BFP_INT_ROUND_WARPS) and one FMA.  Each CTA
//     folds the largest exponent of its psi' into the key.
// Errors: the truncations of X, of psi (psi^2 + lshift) and of c2 sum, each
// below 2^-56 of the field's largest value or of mu's bound, where the
// reference's FP64 sums round relative to each cell's own terms.  The results
// are not the other variants' bits; they agree with the reference far below
// the parity tests' 1e-12 (relative to the field's largest value).
// The key is (generation << 16) | emax, the largest of BFP_SLOTS 64-bit slots.
// A step's mu kernel reads generation g and publishes g + 1 (BfpState::gen)
// with mu's exponent and the mode; the step's update kernel folds each CTA's
// exponent into one slot as ((g + 1) << 16) | e by atomicMax, so the newer
// generation supersedes the older with no reset between steps, and slots no
// CTA wrote in this step fall behind.  Each chgb_step call first sets the key
// from the field (a memset, then bfp_refresh_kernel).  A field whose emax is
// 0 (zeros and subnormals only) or 2047 (inf, NaN), or so large or small that
// mu's unit leaves [2^-1000, 2^900], takes plain FP64 sums in the reference's
// neighbour order for that step (mode 0, mu stored as FP64).

// floor(x 2^(1080 - u)) for a finite x whose biased exponent is at most u.
__device__ __forceinline__ long long bfp_fixed(double x, int u) {
    long long T;
    int ek;
    fx_term(x, T, ek);
    return fx_sar(T, u - ek);
}

// In-plane offsets of the values a thread stages (the same for every plane of a
// CTA's column): computed once instead of per plane.
__device__ __forceinline__ void bfp_plane_offsets(int (&o)[SPF], const Geom &g, int x0, int y0, int tid) {
#pragma unroll
    for(int k = 0; k < SPF; k++) {
        const int i = tid + k * STX * STY;
        const int ly = i / SPX, lx = i - ly * SPX;
        o[k] = ((x0 - 1 + lx) & g.mask) + (((y0 - 1 + ly) & g.mask) << g.log2N);
    }
}

template <int DIMS, typename T>
__device__ __forceinline__ void bfp_fetch_plane(T (&v)[SPF], const T *__restrict__ src, const Geom &g,
                                                const int (&o)[SPF], int z, int tid) {
    const size_t zoff = (DIMS == 3) ? ((size_t) (z & g.mask) << (2 * g.log2N)) : 0;
    const T *plane = src + zoff;
#pragma unroll
    for(int k = 0; k < SPF; k++)
        if(tid + k * STX * STY < SPP && CHGB_BC(11, zoff + o[k], g.bins)) v[k] = plane[o[k]];
}

// The same with the offsets formed per plane: fewer registers, more integer work
// (the update kernel, whose integer pipe has room and whose registers do not).
template <int DIMS, typename T>
__device__ __forceinline__ void bfp_fetch_plane_idx(T (&v)[SPF], const T *__restrict__ src, const Geom &g, int x0,
                                                    int y0, int z, int tid) {
    const T *plane = src + ((DIMS == 3) ? ((size_t) (z & g.mask) << (2 * g.log2N)) : 0);
#pragma unroll
    for(int k = 0; k < SPF; k++) {
        const int i = tid + k * STX * STY;
        if(i < SPP) {
            const int ly = i / SPX, lx = i - ly * SPX;
            const int o = ((x0 - 1 + lx) & g.mask) + (((y0 - 1 + ly) & g.mask) << g.log2N);
            if(CHGB_BC(12, (size_t) (plane - src) + o, g.bins)) v[k] = plane[o];
        }
    }
}

// The largest biased exponent of a block's per-thread values e, folded into
// key slot `slot` as ((gen << 16) | e) by one atomicMax (256-thread blocks).
// The CTAs of a launch spread over BFP_SLOTS slots, one 128-byte line each, so
// that their atomics do not queue on one address.
__device__ __forceinline__ void bfp_fold_key(int e, unsigned long long gen, unsigned long long *bank, int slot,
                                             int tid) {
    __shared__ int wmax[8];
    e = __reduce_max_sync(0xffffffffu, e);
    if((tid & 31) == 0) wmax[tid >> 5] = e;
    __syncthreads();
    if(tid == 0) {
        int m = wmax[0];
#pragma unroll
        for(int w = 1; w < 8; w++) m = wmax[w] > m ? wmax[w] : m;
        atomicMax(&bank[(slot % BFP_SLOTS) * BFP_SLOT_STRIDE], (gen << 16) | (unsigned long long) m);
    }
}

// The field's key: the largest of the slots (the newest generation, then the
// largest exponent), read by warp 0 and shared through shared memory, so that
// one load per CTA reaches each slot's line.
__device__ __forceinline__ unsigned long long bfp_read_key(const unsigned long long *bank, int tid) {
    __shared__ unsigned long long s_key;
    if(tid < 32) {
        unsigned long long k = *(const volatile unsigned long long *) &bank[tid * BFP_SLOT_STRIDE];
#pragma unroll
        for(int o = 16; o > 0; o >>= 1) {
            const unsigned long long t = __shfl_xor_sync(0xffffffffu, k, o);
            k = t > k ? t : k;
        }
        if(tid == 0) s_key = k;
    }
    __syncthreads();
    return s_key;
}

template <int DIMS, bool FAST>
__device__ __forceinline__ void mu_bfp_run(const double *__restrict__ in, long long *__restrict__ mu, const Geom &g,
                                           const EulerConsts &c, const BfpConsts &b, int emax, int lmu, int zc,
                                           double (*ring)[SPP], long long (*ringX)[SPP]) {
    const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + STX * ty;
    const int x0 = blockIdx.x * STX, y0 = blockIdx.y * STY;
    const int z0 = (DIMS == 3) ? blockIdx.z * zc : 0;
    const int nz = (DIMS == 3) ? zc : 1;
    const int p = (ty + 1) * SPX + (tx + 1);
    const int umu = lmu + 1080;                   // M = floor(mu 2^(1080 - umu))
    const int rc = umu + 1021 - emax - b.ec;      // c2 sum: high product -> M's unit
    const double ls = c.lshift[DIMS - 1];
    auto commit = [&](int slot, const double (&v)[SPF]) {
#pragma unroll
        for(int k = 0; k < SPF; k++) {
            const int i = tid + k * STX * STY;
            if(i < SPP && CHGB_BC(13, slot, (DIMS == 3) ? 3 : 1)) {
                ring[slot][i] = v[k];
                if constexpr(FAST) ringX[slot][i] = bfp_fixed(v[k], emax);
            }
        }
    };
    int off[SPF];
    bfp_plane_offsets(off, g, x0, y0, tid);
    double pf[SPF];
    if constexpr(DIMS == 3) {
        bfp_fetch_plane<DIMS>(pf, in, g, off, z0 - 1, tid);
        commit((z0 + 2) % 3, pf);
        bfp_fetch_plane<DIMS>(pf, in, g, off, z0, tid);
        commit(z0 % 3, pf);
        bfp_fetch_plane<DIMS>(pf, in, g, off, z0 + 1, tid);
    }
    for(int z = z0; z < z0 + nz; z++) {
        const int cz = (DIMS == 3) ? z % 3 : 0, zm = (z + 2) % 3, zp = (z + 1) % 3;
        if constexpr(DIMS == 3) {
            commit(zp, pf);
            if(z + 1 < z0 + nz) bfp_fetch_plane<DIMS>(pf, in, g, off, z + 2, tid);
        }
        else {
            bfp_fetch_plane<DIMS>(pf, in, g, off, 0, tid);
            commit(0, pf);
        }
        __syncthreads();
        const size_t gi = (size_t) (x0 + tx) + ((size_t) (y0 + ty) << g.log2N) +
                          ((DIMS == 3) ? ((size_t) z << (2 * g.log2N)) : 0);
        bool ok = CHGB_BC(14, p - SPX, SPP) && CHGB_BC(14, p + SPX, SPP) && CHGB_BC(15, gi, g.bins);
        if constexpr(DIMS == 3) ok = ok && CHGB_BC(14, cz, 3) && CHGB_BC(14, zm, 3) && CHGB_BC(14, zp, 3);
        if(ok) {
            const double r = ring[cz][p];
            if constexpr(FAST) {
                const long long *q = &ringX[cz][p];
                long long sum = (q[-1] + q[1]) + (q[-SPX] + q[SPX]);
                if constexpr(DIMS == 3) sum += ringX[zm][p] + ringX[zp][p];
                const long long F = bfp_fixed(r * fma(r, r, ls), umu);
                mu[gi] = F - fx_sar(__mul64hi(sum, b.mc), rc);
            }
            else {
                const double *q = &ring[cz][p];
                double sum;
                if constexpr(DIMS == 3) sum = seq_sum(q[-1], q[1], q[-SPX], q[SPX], ring[zm][p], ring[zp][p], 6);
                else sum = seq_sum(q[-1], q[1], q[-SPX], q[SPX], 0.0, 0.0, 4);
                reinterpret_cast<double *>(mu)[gi] = fma(-c.c2[0], sum, r * fma(r, r, ls));
            }
        }
        __syncthreads();
    }
}

template <int DIMS>
__global__ void __launch_bounds__(256, 8) mu_bfp_kernel(const double *__restrict__ in, long long *__restrict__ mu,
                                                        Geom g, EulerConsts c, BfpConsts b, BfpState *st, int zc) {
    constexpr int R = (DIMS == 3) ? 3 : 1;
    __shared__ double ring[R][SPP];
    __shared__ long long ringX[R][SPP];
    pdl_begin();
    const unsigned long long key = bfp_read_key(st->key[0], threadIdx.x + STX * threadIdx.y);
    const int emax = (int) (key & 0xFFFFu);
    const int s = emax - 1022;                    // |psi| < 2^s
    const int emu = max(3 * s, b.elin + s) + 2;   // |mu| < 2^emu
    const int lmu = emu - 58;                     // M's unit is 2^lmu
    const bool fast = emax >= 1 && emax <= 2046 && lmu >= -1000 && lmu <= 900;
    if(blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.x == 0 && threadIdx.y == 0) {
        st->gen = (key >> 16) + 1;
        st->lmu = lmu;
        st->mode = fast ? 1 : 0;
    }
    if(fast) mu_bfp_run<DIMS, true>(in, mu, g, c, b, emax, lmu, zc, ring, ringX);
    else mu_bfp_run<DIMS, false>(in, mu, g, c, b, emax, lmu, zc, ring, ringX);
}

// Returns the largest biased exponent of the thread's psi'.
// L 2^lmu (L != 0, |L| < 2^62) rounded to the nearest double, ties to even, in
// integer arithmetic: the value of __ll2double_rn(L) scaled by 2^lmu.
__device__ __forceinline__ double bfp_to_double_int(long long L, int lmu) {
    const unsigned long long a = L < 0 ? 0ull - (unsigned long long) L : (unsigned long long) L;
    const int top = 63 - __clzll((long long) a);   // the leading bit, <= 61
    int E = top;
    unsigned long long M;
    if(top > 52) {
        const int r = top - 52;
        const unsigned long long rem = a & ((1ull << r) - 1), half = 1ull << (r - 1);
        M = a >> r;
        if(rem > half || (rem == half && (M & 1))) {
            M++;
            if(M >> 53) {
                M >>= 1;
                E++;
            }
        }
    }
    else {
        M = a << (52 - top);
    }
    return __longlong_as_double((long long) (((unsigned long long) (L < 0) << 63) |
                                             ((unsigned long long) (E + 1023 + lmu) << 52) |
                                             (M & 0xFFFFFFFFFFFFFull)));
}

// Warps 0-3 of an update CTA round L with bfp_to_double_int, warps 4-7 with the
// FP64-pipe conversion: the same bits, and the FP64 pipe, the update's busier
// one, carries less (3D N=256 on GB300: 9.62e10 -> 9.69e10 cell-steps/s; 2 or 3
// of the 8 warps gave 9.68e10 and 9.69e10).
constexpr int BFP_INT_ROUND_WARPS = 4;

template <int DIMS, bool FAST>
__device__ __forceinline__ int update_bfp_run(const double *__restrict__ psi_in, const long long *__restrict__ mu,
                                              double *__restrict__ out, const Geom &g, const EulerConsts &c, int lmu,
                                              int zc, long long (*ringX)[SPP]) {
    const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + STX * ty;
    const int x0 = blockIdx.x * STX, y0 = blockIdx.y * STY;
    const int z0 = (DIMS == 3) ? blockIdx.z * zc : 0;
    const int nz = (DIMS == 3) ? zc : 1;
    const int p = (ty + 1) * SPX + (tx + 1);
    const long long escale = (long long) lmu * (1ll << 52);   // 2^lmu through the exponent field
    auto commit = [&](int slot, const long long (&v)[SPF]) {
#pragma unroll
        for(int k = 0; k < SPF; k++) {
            const int i = tid + k * STX * STY;
            if(i < SPP && CHGB_BC(16, slot, (DIMS == 3) ? 3 : 1)) ringX[slot][i] = v[k];
        }
    };
    int emx = 0;
    long long pf[SPF];
    if constexpr(DIMS == 3) {
        bfp_fetch_plane_idx<DIMS>(pf, mu, g, x0, y0, z0 - 1, tid);
        commit((z0 + 2) % 3, pf);
        bfp_fetch_plane_idx<DIMS>(pf, mu, g, x0, y0, z0, tid);
        commit(z0 % 3, pf);
        bfp_fetch_plane_idx<DIMS>(pf, mu, g, x0, y0, z0 + 1, tid);
    }
    for(int z = z0; z < z0 + nz; z++) {
        const int cz = (DIMS == 3) ? z % 3 : 0, zm = (z + 2) % 3, zp = (z + 1) % 3;
        const size_t gi = (size_t) (x0 + tx) + ((size_t) (y0 + ty) << g.log2N) +
                          ((DIMS == 3) ? ((size_t) z << (2 * g.log2N)) : 0);
        bool ok = CHGB_BC(17, gi, g.bins) && CHGB_BC(18, p - SPX, SPP) && CHGB_BC(18, p + SPX, SPP);
        if constexpr(DIMS == 3) ok = ok && CHGB_BC(18, cz, 3) && CHGB_BC(18, zm, 3) && CHGB_BC(18, zp, 3);
        const double psi0 = ok ? psi_in[gi] : 0.0;   // read before the staging barrier, to overlap its latency
        if constexpr(DIMS == 3) {
            commit(zp, pf);
            if(z + 1 < z0 + nz) bfp_fetch_plane_idx<DIMS>(pf, mu, g, x0, y0, z + 2, tid);
        }
        else {
            bfp_fetch_plane_idx<DIMS>(pf, mu, g, x0, y0, 0, tid);
            commit(0, pf);
        }
        __syncthreads();
        double res = 0.0;
        if(!ok) {
        }
        else if constexpr(FAST) {
            const long long *q = &ringX[cz][p];
            long long L = (q[-1] + q[1]) + (q[-SPX] + q[SPX]);
            if constexpr(DIMS == 3) L += ringX[zm][p] + ringX[zp][p];
            L -= (long long) (2 * DIMS) * q[0];
            const double ld = L == 0 ? 0.0
                              : ((int) threadIdx.y < BFP_INT_ROUND_WARPS)
                                  ? bfp_to_double_int(L, lmu)
                                  : __longlong_as_double(__double_as_longlong(__ll2double_rn(L)) + escale);
            res = fma(c.c1, ld, psi0);
        }
        else {
            const double *u = reinterpret_cast<const double *>(&ringX[cz][p]);
            double sum;
            if constexpr(DIMS == 3)
                sum = seq_sum(u[-1], u[1], u[-SPX], u[SPX], __longlong_as_double(ringX[zm][p]),
                              __longlong_as_double(ringX[zp][p]), 6);
            else sum = seq_sum(u[-1], u[1], u[-SPX], u[SPX], 0.0, 0.0, 4);
            res = fma(c.c1, fma(-2.0 * DIMS, u[0], sum), psi0);
        }
        if(ok) out[gi] = res;
        const int e = (int) ((unsigned long long) __double_as_longlong(res) >> 52) & 0x7FF;
        emx = e > emx ? e : emx;
        __syncthreads();
    }
    return emx;
}

template <int DIMS>
__global__ void __launch_bounds__(256, 8) update_bfp_kernel(const double *__restrict__ psi_in,
                                                            const long long *__restrict__ mu, double *__restrict__ out,
                                                            Geom g, EulerConsts c, BfpState *st, int zc) {
    constexpr int R = (DIMS == 3) ? 3 : 1;
    __shared__ long long ringX[R][SPP];   // M (mode 1) or mu's FP64 bits (mode 0)
    __shared__ unsigned long long s_gen;
    __shared__ int s_lmu, s_mode;
    const int tid = threadIdx.x + STX * threadIdx.y;
    pdl_begin();
    if(tid == 0) {   // one load per CTA of the step's state, shared
        s_gen = *(const volatile unsigned long long *) &st->gen;
        s_lmu = *(const volatile int *) &st->lmu;
        s_mode = *(const volatile int *) &st->mode;
    }
    __syncthreads();
    const int lmu = s_lmu;
    const int emx = s_mode ? update_bfp_run<DIMS, true>(psi_in, mu, out, g, c, lmu, zc, ringX)
                           : update_bfp_run<DIMS, false>(psi_in, mu, out, g, c, lmu, zc, ringX);
    bfp_fold_key(emx, s_gen, st->key[0], blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z), tid);
}

// The key of the field psi (n values, n even): (0 << 16) | its largest biased
// exponent, after the caller zeroed it.
__global__ void __launch_bounds__(256) bfp_refresh_kernel(const double2 *__restrict__ psi, long long n2,
                                                          unsigned long long *bank) {
    int e = 0;
    for(long long i = (long long) blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += (long long) gridDim.x * blockDim.x) {
        const double2 v = psi[i];
        const int a = (int) ((unsigned long long) __double_as_longlong(v.x) >> 52) & 0x7FF;
        const int b = (int) ((unsigned long long) __double_as_longlong(v.y) >> 52) & 0x7FF;
        e = max(e, max(a, b));
    }
    bfp_fold_key(e, 0ull, bank, blockIdx.x, threadIdx.x);
}

// 2D: one kernel per step.  A CTA stages a 32 x 16 tile of psi with a halo of
// 2 (and X of every staged value), forms M on the tile plus a halo of 1, then
// updates the tile, two cells per thread.  The halo's M is formed by each CTA
// that needs it from the same X, so the results are the pair's integers and
// bits; what changes is one launch per step instead of two, and no M round
// trip through memory.  The key is read from bank `parity` and the step's
// exponents fold into the other bank (CTAs of one launch both read and fold).
constexpr int F2X = 32;
constexpr int F2SX = F2X + 4;                       // psi with a halo of 2: 36 x (F2Y + 4)
constexpr int F2MX = F2X + 2;                       // M with a halo of 1: 34 x (F2Y + 2)
template <int F2Y> struct F2Tile {
    static constexpr int SP = F2SX * (F2Y + 4), MP = F2MX * (F2Y + 2);
};

template <int F2Y, bool FAST>
__device__ __forceinline__ int euler2d_bfp_run(const double *__restrict__ in, double *__restrict__ out, const Geom &g,
                                               const EulerConsts &c, const BfpConsts &b, int emax, int lmu,
                                               double *sp, long long *sx, long long *sm) {
    const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + STX * ty;
    const int x0 = blockIdx.x * F2X, y0 = blockIdx.y * F2Y;
    const int umu = lmu + 1080;                   // M = floor(mu 2^(1080 - umu))
    const int rc = umu + 1021 - emax - b.ec;      // c2 sum: high product -> M's unit
    const double ls = c.lshift[1];
    const long long escale = (long long) lmu * (1ll << 52);
    constexpr int F2SP = F2Tile<F2Y>::SP, F2MP = F2Tile<F2Y>::MP;
    for(int i = tid; i < F2SP; i += STX * STY) {
        const int ly = i / F2SX, lx = i - ly * F2SX;
        const size_t gi = ((x0 - 2 + lx) & g.mask) + ((size_t) ((y0 - 2 + ly) & g.mask) << g.log2N);
        const double v = CHGB_BC(21, gi, g.bins) ? in[gi] : 0.0;
        sp[i] = v;
        if constexpr(FAST) sx[i] = bfp_fixed(v, emax);
    }
    __syncthreads();
    for(int j = tid; j < F2MP; j += STX * STY) {
        const int my = j / F2MX, mx = j - my * F2MX;
        const int q = (my + 1) * F2SX + mx + 1;
        if(!CHGB_BC(22, q - F2SX, F2SP) || !CHGB_BC(22, q + F2SX, F2SP)) continue;
        const double r = sp[q];
        if constexpr(FAST) {
            const long long sum = (sx[q - 1] + sx[q + 1]) + (sx[q - F2SX] + sx[q + F2SX]);
            sm[j] = bfp_fixed(r * fma(r, r, ls), umu) - fx_sar(__mul64hi(sum, b.mc), rc);
        }
        else {
            const double sum = seq_sum(sp[q - 1], sp[q + 1], sp[q - F2SX], sp[q + F2SX], 0.0, 0.0, 4);
            reinterpret_cast<double *>(sm)[j] = fma(-c.c2[0], sum, r * fma(r, r, ls));
        }
    }
    __syncthreads();
    int emx = 0;
#pragma unroll
    for(int k = 0; k < F2Y / STY; k++) {
        const int ly = ty + STY * k;
        const int m = (ly + 1) * F2MX + tx + 1;
        const size_t gi = (size_t) (x0 + tx) + ((size_t) (y0 + ly) << g.log2N);
        if(!CHGB_BC(23, m - F2MX, F2MP) || !CHGB_BC(23, m + F2MX, F2MP) ||
           !CHGB_BC(23, (ly + 2) * F2SX + tx + 2, F2SP) || !CHGB_BC(24, gi, g.bins))
            continue;
        const double psi0 = sp[(ly + 2) * F2SX + tx + 2];
        double res;
        if constexpr(FAST) {
            long long L = (sm[m - 1] + sm[m + 1]) + (sm[m - F2MX] + sm[m + F2MX]);
            L -= 4ll * sm[m];
            const double ld = L == 0 ? 0.0
                              : ((int) threadIdx.y < BFP_INT_ROUND_WARPS)
                                  ? bfp_to_double_int(L, lmu)
                                  : __longlong_as_double(__double_as_longlong(__ll2double_rn(L)) + escale);
            res = fma(c.c1, ld, psi0);
        }
        else {
            const double *u = reinterpret_cast<const double *>(sm);
            res = fma(c.c1, fma(-4.0, u[m], seq_sum(u[m - 1], u[m + 1], u[m - F2MX], u[m + F2MX], 0.0, 0.0, 4)),
                      psi0);
        }
        out[gi] = res;
        const int e = (int) ((unsigned long long) __double_as_longlong(res) >> 52) & 0x7FF;
        emx = e > emx ? e : emx;
    }
    return emx;
}

template <int F2Y>
__global__ void __launch_bounds__(256, 8) euler2d_bfp_kernel(const double *__restrict__ in, double *__restrict__ out,
                                                             Geom g, EulerConsts c, BfpConsts b, BfpState *st,
                                                             int parity) {
    __shared__ double sp[F2Tile<F2Y>::SP];
    __shared__ long long sx[F2Tile<F2Y>::SP];
    __shared__ long long sm[F2Tile<F2Y>::MP];   // M (mode 1) or mu's FP64 bits (mode 0)
    const int tid = threadIdx.x + STX * threadIdx.y;
    pdl_begin();
    const unsigned long long key = bfp_read_key(st->key[parity], tid);
    const int emax = (int) (key & 0xFFFFu);
    const int s = emax - 1022;                    // |psi| < 2^s
    const int lmu = max(3 * s, b.elin + s) + 2 - 58;
    const bool fast = emax >= 1 && emax <= 2046 && lmu >= -1000 && lmu <= 900;
    const int emx = fast ? euler2d_bfp_run<F2Y, true>(in, out, g, c, b, emax, lmu, sp, sx, sm)
                         : euler2d_bfp_run<F2Y, false>(in, out, g, c, b, emax, lmu, sp, sx, sm);
    bfp_fold_key(emx, (key >> 16) + 1, st->key[parity ^ 1], blockIdx.x + gridDim.x * blockIdx.y, tid);
}

}  // namespace chgb

extern "C" int chgb_bounds_report(unsigned long long *first) {
    if(!first) return CHGB_ERR_INVALID;
#ifdef CHGB_BOUNDS_CHECK
    // the explicit kernels' record (this file), then the transforms' (spectral.cu)
    unsigned long long a = 0, b = 0;
    if(chgb::bc_read_tu(&a) != cudaSuccess || chgb::bc_read_spectral(&b) != cudaSuccess) return CHGB_ERR_CUDA;
    *first = a ? a : b;
    return CHGB_OK;
#else
    *first = 0;
    chgb::record_error("chgb_bounds_report: not a bounds-check build (-DCHGB_BOUNDS_CHECK, lib/libchgb_bc.so)");
    return CHGB_ERR_UNSUPPORTED;
#endif
}

namespace chgb {

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
namespace {

template <int KIND, int MOB>
cudaError_t launch_1d(const Geom &g, const ModelDev &m, const EulerConsts &c, const double *in, double *out,
                      cudaStream_t st, bool configure) {
    if(configure) return cudaSuccess;
    if(g.N >= 256) {
        euler1d_kernel<KIND, MOB, 256><<<g.N / 256, 256, 0, st>>>(in, out, g, m, c);
    }
    else if(g.N >= 64) {
        euler1d_kernel<KIND, MOB, 64><<<g.N / 64, 64, 0, st>>>(in, out, g, m, c);
    }
    else if(g.N >= 16) {
        euler1d_kernel<KIND, MOB, 16><<<g.N / 16, 32, 0, st>>>(in, out, g, m, c);
    }
    else {
        euler1d_kernel<KIND, MOB, 4><<<g.N / 4, 32, 0, st>>>(in, out, g, m, c);
    }
    return cudaGetLastError();
}

template <int KIND, int MOB, int TX, int TY>
cudaError_t launch_2d_tile(const Geom &g, const ModelDev &m, const EulerConsts &c, const double *in, double *out,
                           cudaStream_t st, bool configure) {
    constexpr int S = NSpecies<KIND>::value;
    size_t smem = sizeof(double) * S * ((TX + 4) * (TY + 4) + (MOB ? 2 : 1) * (TX + 2) * (TY + 2));
    auto kern = euler2d_kernel<KIND, MOB, TX, TY>;
    if(configure) {
        return smem > 48 * 1024 ? cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem)
                                : cudaSuccess;
    }
    dim3 grid(g.N / TX, g.N / TY);
    kern<<<grid, dim3(32, 8), smem, st>>>(in, out, g, m, c);
    return cudaGetLastError();
}

template <int KIND, int MOB>
cudaError_t launch_2d(const Geom &g, const ModelDev &m, const EulerConsts &c, const double *in, double *out,
                      cudaStream_t st, bool configure) {
    // the largest tile that still gives >= 1024 CTAs (about 7 per SM): halo
    // recomputation favours big tiles, filling 152 SMs favours many (N=256:
    // 16x16 tiles run a step in 4.1 us, 32x32 tiles -- 64 CTAs -- in 6.4 us)
    const long long cells = (long long) g.N * g.N;
    if(g.N >= 32 && cells / (32 * 32) >= 1024) return launch_2d_tile<KIND, MOB, 32, 32>(g, m, c, in, out, st, configure);
    if(g.N >= 32 && cells / (32 * 16) >= 1024) return launch_2d_tile<KIND, MOB, 32, 16>(g, m, c, in, out, st, configure);
    if(g.N >= 16) return launch_2d_tile<KIND, MOB, 16, 16>(g, m, c, in, out, st, configure);
    if(g.N >= 8) return launch_2d_tile<KIND, MOB, 8, 8>(g, m, c, in, out, st, configure);
    return launch_2d_tile<KIND, MOB, 4, 4>(g, m, c, in, out, st, configure);
}

template <int KIND, int MOB, int TX, int TY>
cudaError_t launch_3d_tile(const Geom &g, const ModelDev &m, const EulerConsts &c, const double *in, double *out,
                           cudaStream_t st, bool configure) {
    constexpr int S = NSpecies<KIND>::value;
    size_t smem = sizeof(double) * S * (5 * (TX + 4) * (TY + 4) + (MOB ? 6 : 3) * (TX + 2) * (TY + 2));
    auto kern = euler3d_kernel<KIND, MOB, TX, TY>;
    if(configure) {
        return smem > 48 * 1024 ? cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem)
                                : cudaSuccess;
    }
    int zc = g.N < 32 ? g.N : 32;
    dim3 grid(g.N / TX, g.N / TY, g.N / zc);
    kern<<<grid, dim3(32, 8), smem, st>>>(in, out, g, m, c, zc);
    return cudaGetLastError();
}

template <int KIND, int MOB>
cudaError_t launch_3d(const Geom &g, const ModelDev &m, const EulerConsts &c, const double *in, double *out,
                      cudaStream_t st, bool configure) {
    if(g.N >= 32) return launch_3d_tile<KIND, MOB, 32, 16>(g, m, c, in, out, st, configure);
    if(g.N >= 16) return launch_3d_tile<KIND, MOB, 16, 16>(g, m, c, in, out, st, configure);
    if(g.N >= 8) return launch_3d_tile<KIND, MOB, 8, 8>(g, m, c, in, out, st, configure);
    return launch_3d_tile<KIND, MOB, 4, 4>(g, m, c, in, out, st, configure);
}

template <int KIND, int MOB>
cudaError_t launch_dims(const Geom &g, const ModelDev &m, const EulerConsts &c, const double *in, double *out,
                        cudaStream_t st, bool configure) {
    switch(g.dims) {
        case 1: return launch_1d<KIND, MOB>(g, m, c, in, out, st, configure);
        case 2: return launch_2d<KIND, MOB>(g, m, c, in, out, st, configure);
        default: return launch_3d<KIND, MOB>(g, m, c, in, out, st, configure);
    }
}

template <int KIND>
cudaError_t launch_mob(int mob, const Geom &g, const ModelDev &m, const EulerConsts &c, const double *in,
                       double *out, cudaStream_t st, bool configure) {
    // mob: 0 = plain euler, 1 = euler_mobility with constant M, 2 = free-energy M
    if(mob == 0) return launch_dims<KIND, 0>(g, m, c, in, out, st, configure);
    if(mob == 1) return launch_dims<KIND, 1>(g, m, c, in, out, st, configure);
    if(mob == 3) return launch_dims<KIND, 3>(g, m, c, in, out, st, configure);
    if constexpr(KIND == CHGB_MODEL_SIMPLE_WERTHEIM) return launch_dims<KIND, 2>(g, m, c, in, out, st, configure);
    return cudaErrorInvalidValue;
}

}  // namespace

namespace {

template <int KIND, int MOB, int DIMS>
cudaError_t launch_split_kind(const Geom &g, const ModelDev &m, const EulerConsts &c, const double *in, double *out,
                              double *mu, double *mob, cudaStream_t st) {
    constexpr int S = NSpecies<KIND>::value;
    // 8-plane z-chunks: the extra halo planes per chunk are cheap L2 loads,
    // and the many small CTAs keep every SM's FP64 pipe fed to the end of the
    // launch (N=256: 8192 CTAs, 7% faster than 32-plane chunks on GB300)
    int zc = (DIMS == 3) ? 8 : 1;
    dim3 grid(g.N / STX, g.N / STY, (DIMS == 3) ? g.N / zc : 1);
    dim3 block(STX, STY);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e = cudaLaunchKernelEx(&cfg, mu_kernel<KIND, MOB, DIMS>, in, mu, mob, g, m, c, zc);
    if(e != cudaSuccess) return e;
    return cudaLaunchKernelEx(&cfg, update_kernel<S, MOB, DIMS>, in, (const double *) mu, (const double *) mob, out, g,
                              c, zc);
}

template <int KIND, int MOB>
cudaError_t launch_split_mob(const Geom &g, const ModelDev &m, const EulerConsts &c, const double *in, double *out,
                             double *mu, double *mob, cudaStream_t st) {
    if(g.dims == 2) return launch_split_kind<KIND, MOB, 2>(g, m, c, in, out, mu, mob, st);
    return launch_split_kind<KIND, MOB, 3>(g, m, c, in, out, mu, mob, st);
}

template <int KIND>
cudaError_t launch_split_model(int mob_kind, const Geom &g, const ModelDev &m, const EulerConsts &c,
                               const double *in, double *out, double *mu, double *mob, cudaStream_t st) {
    if(mob_kind == 0) return launch_split_mob<KIND, 0>(g, m, c, in, out, mu, mob, st);
    if(mob_kind == 1) return launch_split_mob<KIND, 1>(g, m, c, in, out, mu, mob, st);
    // kind 3 reads the given field; mu_kernel writes `mob` only for kind 2
    if(mob_kind == 3) return launch_split_mob<KIND, 3>(g, m, c, in, out, mu, const_cast<double *>(c.mobf), st);
    if constexpr(KIND == CHGB_MODEL_SIMPLE_WERTHEIM) return launch_split_mob<KIND, 2>(g, m, c, in, out, mu, mob, st);
    return cudaErrorInvalidValue;
}

}  // namespace

bool euler_split_supported(const Geom &g) { return g.dims >= 2 && g.N >= 32; }

// Two steps per launch: plain `euler` in 2D boxes of 32 <= N <= 512, 16 x 16 tiles.
bool euler_two_supported(int integrator, const Geom &g) {
    return integrator == CHGB_INTEGRATOR_EULER && g.dims == 2 && g.N >= 32 && g.N <= 512;
}

namespace {
template <int KIND>
cudaError_t launch_two_kind(const Geom &g, const ModelDev &m, const EulerConsts &c, const double *in, double *out,
                            double *mid, cudaStream_t st, bool configure) {
    constexpr int S = NSpecies<KIND>::value, T = 16;
    const size_t smem = sizeof(double) * S * ((T + 8) * (T + 8) + (T + 6) * (T + 6) + (T + 4) * (T + 4) +
                                              (T + 2) * (T + 2));
    auto kern = euler2d_two_kernel<KIND, T, T>;
    if(configure) {
        return smem > 48 * 1024 ? cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem)
                                : cudaSuccess;
    }
    kern<<<dim3(g.N / T, g.N / T), dim3(32, 8), smem, st>>>(in, out, mid, g, m, c);
    return cudaGetLastError();
}
}  // namespace

cudaError_t launch_euler_two(const Geom &g, const ModelDev &m, const EulerConsts &c, const double *in, double *out,
                             cudaStream_t st, bool configure, double *mid) {
    switch(m.kind) {
        case CHGB_MODEL_LANDAU: return launch_two_kind<CHGB_MODEL_LANDAU>(g, m, c, in, out, mid, st, configure);
        case CHGB_MODEL_SIMPLE_WERTHEIM:
            return launch_two_kind<CHGB_MODEL_SIMPLE_WERTHEIM>(g, m, c, in, out, mid, st, configure);
        default: return launch_two_kind<CHGB_MODEL_SALEH>(g, m, c, in, out, mid, st, configure);
    }
}

bool euler_cluster_supported(int integrator, const Geom &g) {
    return integrator == CHGB_INTEGRATOR_EULER && g.dims == 2 && (g.N == 32 || g.N == 64);
}

namespace {
template <int KIND, int T>
cudaError_t launch_cluster_kind(const Geom &g, const ModelDev &m, const EulerConsts &c, const double *in,
                                double *out, int nsteps, cudaStream_t st, bool configure) {
    // at least four warps, one per SM sub-partition: each has its own FP64 unit
    constexpr int NTHR = T * T < 128 ? 128 : T * T;
    auto kern = euler2d_cluster_kernel<KIND, T, NTHR>;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(CLUSTER_TILES, CLUSTER_TILES, 1);
    cfg.blockDim = dim3(NTHR, 1, 1);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = CLUSTER_TILES;
    attr[0].val.clusterDim.y = CLUSTER_TILES;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if(configure) {
        // 16 CTAs is above the portable cluster size of 8: opt in, then ask
        // whether the GPU can hold such a cluster at all
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if(e != cudaSuccess) return e;
        int clusters = 0;
        e = cudaOccupancyMaxActiveClusters(&clusters, kern, &cfg);
        if(e != cudaSuccess) return e;
        return clusters > 0 ? cudaSuccess : cudaErrorInvalidConfiguration;
    }
    if(nsteps < 1) return cudaErrorInvalidValue;
    return cudaLaunchKernelEx(&cfg, kern, in, out, g, m, c, nsteps);
}

template <int KIND>
cudaError_t launch_cluster_tile(const Geom &g, const ModelDev &m, const EulerConsts &c, const double *in, double *out,
                                int nsteps, cudaStream_t st, bool configure) {
    if(g.N == 64) return launch_cluster_kind<KIND, 16>(g, m, c, in, out, nsteps, st, configure);
    if(g.N == 32) return launch_cluster_kind<KIND, 8>(g, m, c, in, out, nsteps, st, configure);
    return cudaErrorInvalidValue;
}
}  // namespace

cudaError_t launch_euler_cluster(const Geom &g, const ModelDev &m, const EulerConsts &c, const double *in,
                                 double *out, int nsteps, cudaStream_t st, bool configure) {
    switch(m.kind) {
        case CHGB_MODEL_LANDAU: return launch_cluster_tile<CHGB_MODEL_LANDAU>(g, m, c, in, out, nsteps, st, configure);
        case CHGB_MODEL_SIMPLE_WERTHEIM:
            return launch_cluster_tile<CHGB_MODEL_SIMPLE_WERTHEIM>(g, m, c, in, out, nsteps, st, configure);
        default: return launch_cluster_tile<CHGB_MODEL_SALEH>(g, m, c, in, out, nsteps, st, configure);
    }
}

namespace {
template <int KIND, int TX, int TY>
cudaError_t launch_batch_tile(const EulerBatchRep *reps, const int2 *items, int nitems, int parity, bool configure,
                              cudaStream_t st) {
    constexpr int S = NSpecies<KIND>::value;
    size_t smem = sizeof(double) * S * ((TX + 4) * (TY + 4) + (TX + 2) * (TY + 2));
    auto kern = euler2d_batch_kernel<KIND, TX, TY>;
    if(configure) {
        return smem > 48 * 1024 ? cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem)
                                : cudaSuccess;
    }
    if(nitems == 0) return cudaSuccess;
    kern<<<nitems, dim3(32, TX * TY >= 1024 ? 8 : 4), smem, st>>>(reps, items, parity);
    return cudaGetLastError();
}

template <int KIND>
cudaError_t launch_batch_kind(int tile, const EulerBatchRep *reps, const int2 *items, int nitems, int parity,
                              bool configure, cudaStream_t st) {
    switch(tile) {
        case 32: return launch_batch_tile<KIND, 32, 32>(reps, items, nitems, parity, configure, st);
        case 16: return launch_batch_tile<KIND, 16, 16>(reps, items, nitems, parity, configure, st);
        default: return launch_batch_tile<KIND, 64, 16>(reps, items, nitems, parity, configure, st);
    }
}
}  // namespace

cudaError_t launch_euler2d_batch(int kind, int tile, const EulerBatchRep *reps, const int2 *items, int nitems,
                                 int parity, bool configure, cudaStream_t st) {
    switch(kind) {
        case CHGB_MODEL_LANDAU:
            return launch_batch_kind<CHGB_MODEL_LANDAU>(tile, reps, items, nitems, parity, configure, st);
        case CHGB_MODEL_SIMPLE_WERTHEIM:
            return launch_batch_kind<CHGB_MODEL_SIMPLE_WERTHEIM>(tile, reps, items, nitems, parity, configure, st);
        default: return launch_batch_kind<CHGB_MODEL_SALEH>(tile, reps, items, nitems, parity, configure, st);
    }
}

bool euler_bfp_supported(int integrator, int model_kind, const Geom &g) {
    return integrator == CHGB_INTEGRATOR_EULER && model_kind == CHGB_MODEL_LANDAU && g.dims >= 2 && g.N >= 32;
}

// c2's mantissa and exponent, and elin, for the mu kernel of a DIMS-dimensional box.
static BfpConsts bfp_consts(const EulerConsts &c, int dims) {
    BfpConsts b;
    const double c2 = c.c2[0];
    unsigned long long u;
    std::memcpy(&u, &c2, sizeof u);
    const int e = (int) (u >> 52) & 0x7FF;
    const long long mag = (long long) ((u & 0xFFFFFFFFFFFFFull) | (e ? 1ull << 52 : 0ull));
    b.mc = (long long) ((u >> 63) ? -mag : mag) * 1024;   // |mc| < 2^63
    b.ec = e ? e : 1;
    const double lin = std::fabs(c.lshift[dims - 1]) + 2.0 * dims * std::fabs(c2);
    b.elin = lin > 0.0 && std::isfinite(lin) ? std::ilogb(lin) + 1 : -4000;   // lin < 2^elin
    return b;
}

cudaError_t launch_euler_bfp(const Geom &g, const EulerConsts &c, const double *in, double *out, double *mu,
                             BfpState *st, int parity, cudaStream_t stream) {
    const BfpConsts b = bfp_consts(c, g.dims);
    // z-chunk planes per CTA, measured on GB300 (cell-steps/s with 2, 4, 8, 16, 32
    // planes): N=64 3.26, 3.07, 2.41, 1.43, 0.81e10; N=128 6.16, 7.27, 6.99,
    // 6.91, 5.64e10; N=256 8.32e10 (4), 9.33e10 (8), 9.61e10 (16), 9.45e10 (32);
    // N=512 7.07, 8.91, 10.1, 10.7, 11.0e10.  Small boxes want short columns
    // (more CTAs, a shorter path through each), large ones long (fewer halo planes).
    const int zc = (g.dims != 3) ? 1 : g.N <= 64 ? 2 : g.N == 128 ? 4 : g.N == 256 ? 16 : 32;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(g.N / STX, g.N / STY, (g.dims == 3) ? g.N / zc : 1);
    cfg.blockDim = dim3(STX, STY);
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    long long *m = reinterpret_cast<long long *>(mu);
    cudaError_t e;
    if(g.dims == 2) {
        // one kernel per step; 32 x 16 tiles up to N = 1024, 32 x 32 above (2D
        // on GB300, cell-steps/s: N=1024 8.29e10 against 8.12e10, N=2048
        // 1.05e11 against 1.09e11, N=4096 1.12e11 against 1.16e11; the split
        // pair ran 6.35e10, 7.49e10 and 7.50e10)
        if(g.N >= 2048) {
            cfg.gridDim = dim3(g.N / F2X, g.N / 32);
            e = cudaLaunchKernelEx(&cfg, euler2d_bfp_kernel<32>, in, out, g, c, b, st, parity);
        }
        else {
            cfg.gridDim = dim3(g.N / F2X, g.N / 16);
            e = cudaLaunchKernelEx(&cfg, euler2d_bfp_kernel<16>, in, out, g, c, b, st, parity);
        }
    }
    else {
        e = cudaLaunchKernelEx(&cfg, mu_bfp_kernel<3>, in, m, g, c, b, st, zc);
        if(e == cudaSuccess) e = cudaLaunchKernelEx(&cfg, update_bfp_kernel<3>, in, (const long long *) m, out, g, c, st, zc);
    }
    return e;
}

cudaError_t launch_bfp_refresh(const double *psi, long long n, BfpState *st, int bank, cudaStream_t stream) {
    // both banks: the 2D kernel folds into the other bank next, whose older
    // generations must not outrank the new sequence's
    cudaError_t e = cudaMemsetAsync(st->key, 0, sizeof st->key, stream);
    if(e != cudaSuccess) return e;
    const long long n2 = n / 2;
    const long long blocks = std::min<long long>((n2 + 255) / 256, 152 * 8);
    bfp_refresh_kernel<<<(unsigned) blocks, 256, 0, stream>>>(reinterpret_cast<const double2 *>(psi), n2, st->key[bank]);
    return cudaGetLastError();
}

cudaError_t launch_euler_split(int integrator, const Geom &g, const ModelDev &m, const EulerConsts &c,
                               const double *in, double *out, double *mu, double *mob, cudaStream_t st) {
    int mob_kind = 0;
    if(integrator == CHGB_INTEGRATOR_EULER_MOBILITY) mob_kind = mobility_kind(c.mobility_type);
    switch(m.kind) {
        case CHGB_MODEL_LANDAU: return launch_split_model<CHGB_MODEL_LANDAU>(mob_kind, g, m, c, in, out, mu, mob, st);
        case CHGB_MODEL_SIMPLE_WERTHEIM:
            return launch_split_model<CHGB_MODEL_SIMPLE_WERTHEIM>(mob_kind, g, m, c, in, out, mu, mob, st);
        default: return launch_split_model<CHGB_MODEL_SALEH>(mob_kind, g, m, c, in, out, mu, mob, st);
    }
}

cudaError_t launch_euler_step(int integrator, const Geom &g, const ModelDev &m, const EulerConsts &c,
                              const double *in, double *out, cudaStream_t st, bool configure) {
    int mob = 0;
    if(integrator == CHGB_INTEGRATOR_EULER_MOBILITY) mob = mobility_kind(c.mobility_type);
    switch(m.kind) {
        case CHGB_MODEL_LANDAU: return launch_mob<CHGB_MODEL_LANDAU>(mob, g, m, c, in, out, st, configure);
        case CHGB_MODEL_SIMPLE_WERTHEIM: return launch_mob<CHGB_MODEL_SIMPLE_WERTHEIM>(mob, g, m, c, in, out, st, configure);
        default: return launch_mob<CHGB_MODEL_SALEH>(mob, g, m, c, in, out, st, configure);
    }
}

}  // namespace chgb
