// adjoint.cu — gradients of a loss on the final state through T time steps
// (chgb_adjoint_*).  No counterpart in the reference.
//
// Scope: 2D Landau boxes, `euler` (N >= 32, a multiple of 32) and
// `pseudospectral` (8 <= N <= 1024).  The loss is given by its gradient with
// respect to the radially averaged S(q) of the final state (see
// chgb_structure_factor) and/or with respect to the final field itself.
// Gradients come back for the initial field and for (epsilon, k, M) in
// internal units.
//
// Checkpointing: the forward pass stores the state every K steps (K ~ sqrt T);
// the backward pass walks the segments from the last, recomputes each segment
// from its checkpoint (keeping its K states) and runs the adjoint steps over it.
// Memory is (T/K + K) states, work 3 forward steps per step.
//
// euler (psi' = psi + c1 D mu, mu = f'(psi) - c2 D psi, D the 5-point
// Laplacian without 1/dx^2, c1 = dt M / dx^2, c2 = 2 k / dx^2):
//     w = c1 D lam_{n+1},  lam_n = lam_{n+1} + f''(psi_n) w - c2 D w,
//     dL/deps += -<w, psi_n>,  dL/dk += -(2/dx^2) <w, D psi_n>,  dL/dM += <w, mu_n> / M.
// Both integrators: the backward pass recomputes segment j - 1 on a second
// stream while the adjoint sweep of segment j runs (two segment buffers,
// events between them); on small boxes neither fills the GPU, so the
// recomputation is mostly hidden.  On such boxes (euler, N <= 256 by default)
// the forward, recomputation and adjoint kernels take two steps per launch,
// storing the state in between, which halves the launches of every pass.
// pseudospectral: see the adjoint kernels in spectral.cu.
// The per-block partial sums are accumulated in a fixed order, so the
// gradients are bit-for-bit reproducible.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <map>
#include <vector>

#include "trace.h"
#include "fxsum.cuh"
#include "handle.h"
#include "kernels.h"
#include "spectral.h"
#include "sq.h"

using namespace chgb;

namespace {

// Adjoint tiles are 32 wide; 32 rows on large boxes, 8 rows when the box is
// small enough that 32x32 tiles would leave most SMs idle (N=256: 64 CTAs).
constexpr int ATX = 32;
inline int adj_tile_rows(int N) { return N <= 512 ? 8 : 32; }

// 5-point Laplacian without 1/dx^2; the neighbour sum is the forward step's
// fixed-point sum (fxsum.cuh), off the FP64 pipe.
__device__ __forceinline__ double lap5(const double *p, int sy, double v) {
    return fma(-4.0, v, nb_sum4(p[-1], p[1], p[-sy], p[sy]));
}

// Add the CTA's sums of three per-thread values to dst[0..2] (256 threads, a
// fixed order).  Warp k sums value k: each lane first adds its eight strided
// slots, then the warp folds its 32 lanes -- 12 FP64 adds per warp, where a
// shuffle tree in every warp would cost 15 in each of the 8 warps (as much as
// a one-cell-per-thread adjoint step itself).
__device__ __forceinline__ void add_block_sums(double sa, double sb, double sc, double (*red)[256], int tid,
                                               double *__restrict__ dst) {
    red[0][tid] = sa;
    red[1][tid] = sb;
    red[2][tid] = sc;
    __syncthreads();
    if(tid < 96) {
        const int k = tid >> 5, l = tid & 31;
        double t = red[k][l];
#pragma unroll
        for(int j = 1; j < 8; j++) t += red[k][l + 32 * j];
        for(int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if(l == 0) dst[k] += t;
    }
}

// One adjoint step on a 32 x ATY tile: lam_out = lam + f''(psi) w - c2 D w with
// w = c1 D lam.  The parameter gradients need <w, psi>, <w, D psi> and <w, mu>;
// with mu = psi^3 - eps psi - c2 D psi and D symmetric (periodic box) they
// follow from A = <w, psi>, B = <D w, psi> and C = <w, psi^3>, which reuse D w
// and need psi on the tile only (no psi halo, no second Laplacian).
template <int ATY>
__global__ void __launch_bounds__(256) euler_adj2d_kernel(const double *__restrict__ lam_in,
                                                          const double *__restrict__ psi,
                                                          double *__restrict__ lam_out, Geom g, EulerConsts c,
                                                          double eps, double *__restrict__ part) {
    constexpr int LX = ATX + 4, LY = ATY + 4, LP = LX * LY;
    constexpr int WX = ATX + 2, WY = ATY + 2, WP = WX * WY;
    __shared__ double L[LP];
    __shared__ double W[WP];
    __shared__ double red[3][256];
    const int tid = threadIdx.x + blockDim.x * threadIdx.y, nthr = blockDim.x * blockDim.y;
    const int x0 = blockIdx.x * ATX, y0 = blockIdx.y * ATY;
    for(int i = tid; i < LP; i += nthr) {
        int ly = i / LX, lx = i - ly * LX;
        int gx = (x0 - 2 + lx) & g.mask, gy = (y0 - 2 + ly) & g.mask;
        L[i] = lam_in[gx + (gy << g.log2N)];
    }
    __syncthreads();
    for(int i = tid; i < WP; i += nthr) {
        int ly = i / WX, lx = i - ly * WX;
        int p = (ly + 1) * LX + (lx + 1);
        W[i] = c.c1 * lap5(&L[p], LX, L[p]);
    }
    __syncthreads();
    double sa = 0.0, sb = 0.0, sc = 0.0;
    for(int i = tid; i < ATX * ATY; i += nthr) {
        int ly = i / ATX, lx = i - ly * ATX;
        int q = (ly + 1) * WX + (lx + 1);
        const int gi = (x0 + lx) + ((y0 + ly) << g.log2N);
        double w = W[q];
        double dw = lap5(&W[q], WX, w);
        double ps = psi[gi];
        double lam = L[(ly + 2) * LX + (lx + 2)];
        double p2 = ps * ps;
        double fpp = fma(3.0, p2, -eps);
        lam_out[gi] = fma(-c.c2[0], dw, fma(fpp, w, lam));
        double wp = w * ps;
        sa += wp;
        sb = fma(dw, ps, sb);
        sc = fma(wp, p2, sc);
    }
    add_block_sums(sa, sb, sc, red, tid, part + 3 * (blockIdx.x + gridDim.x * blockIdx.y));
}

// Two adjoint steps on a 16 x 16 tile, for boxes whose steps are too short to
// fill the GPU: lam_{n+1} (halo 4) -> w (halo 3) -> lam_n (halo 2, from psi_n)
// -> c1 D lam_n (halo 1) -> lam_{n-1} (the tile, from psi_{n-1}).  Every value
// is formed by the same operations as in euler_adj2d_kernel, so the fields are
// the same bits as two single steps; the partial sums of both steps go to the
// same slots, summed over the tile only.
constexpr int A2T = 16;

template <bool ACC>
__device__ __forceinline__ double adj_cell(const double *W, int q, int sy, double ps, double lam, double eps,
                                           const EulerConsts &c, double &sa, double &sb, double &sc) {
    double w = W[q];
    double dw = lap5(&W[q], sy, w);
    double p2 = ps * ps;
    double fpp = fma(3.0, p2, -eps);
    if(ACC) {
        double wp = w * ps;
        sa += wp;
        sb = fma(dw, ps, sb);
        sc = fma(wp, p2, sc);
    }
    return fma(-c.c2[0], dw, fma(fpp, w, lam));
}

__global__ void __launch_bounds__(256) euler_adj2d_two_kernel(const double *__restrict__ lam_in,
                                                              const double *__restrict__ psi_hi,
                                                              const double *__restrict__ psi_lo,
                                                              double *__restrict__ lam_out, Geom g, EulerConsts c,
                                                              double eps, double *__restrict__ part) {
    constexpr int T = A2T;
    constexpr int LX = T + 8, LP = LX * LX;       // lam_{n+1}
    constexpr int W1X = T + 6, W1P = W1X * W1X;   // c1 D lam_{n+1}
    constexpr int MX = T + 4, MP = MX * MX;       // lam_n
    constexpr int W2X = T + 2, W2P = W2X * W2X;   // c1 D lam_n
    __shared__ double L[LP];
    __shared__ double W1[W1P];
    __shared__ double Ln[MP];
    __shared__ double W2[W2P];
    __shared__ double red[3][256];
    const int tid = threadIdx.x + blockDim.x * threadIdx.y, nthr = blockDim.x * blockDim.y;
    const int x0 = blockIdx.x * T, y0 = blockIdx.y * T;
    for(int i = tid; i < LP; i += nthr) {
        int ly = i / LX, lx = i - ly * LX;
        int gx = (x0 - 4 + lx) & g.mask, gy = (y0 - 4 + ly) & g.mask;
        L[i] = lam_in[gx + (gy << g.log2N)];
    }
    __syncthreads();
    for(int i = tid; i < W1P; i += nthr) {
        int ly = i / W1X, lx = i - ly * W1X;
        int p = (ly + 1) * LX + (lx + 1);
        W1[i] = c.c1 * lap5(&L[p], LX, L[p]);
    }
    __syncthreads();
    double sa = 0.0, sb = 0.0, sc = 0.0;
    for(int i = tid; i < MP; i += nthr) {
        int ly = i / MX, lx = i - ly * MX;
        int gx = (x0 - 2 + lx) & g.mask, gy = (y0 - 2 + ly) & g.mask;
        double ps = psi_hi[gx + (gy << g.log2N)];
        double lam = L[(ly + 2) * LX + (lx + 2)];
        int q = (ly + 1) * W1X + (lx + 1);
        if(lx >= 2 && lx < T + 2 && ly >= 2 && ly < T + 2) Ln[i] = adj_cell<true>(W1, q, W1X, ps, lam, eps, c, sa, sb, sc);
        else Ln[i] = adj_cell<false>(W1, q, W1X, ps, lam, eps, c, sa, sb, sc);
    }
    __syncthreads();
    for(int i = tid; i < W2P; i += nthr) {
        int ly = i / W2X, lx = i - ly * W2X;
        int p = (ly + 1) * MX + (lx + 1);
        W2[i] = c.c1 * lap5(&Ln[p], MX, Ln[p]);
    }
    __syncthreads();
    for(int i = tid; i < T * T; i += nthr) {
        int ly = i / T, lx = i - ly * T;
        const int gi = (x0 + lx) + ((y0 + ly) << g.log2N);
        int q = (ly + 1) * W2X + (lx + 1);
        lam_out[gi] = adj_cell<true>(W2, q, W2X, psi_lo[gi], Ln[(ly + 2) * MX + (lx + 2)], eps, c, sa, sb, sc);
    }
    add_block_sums(sa, sb, sc, red, tid, part + 3 * (blockIdx.x + gridDim.x * blockIdx.y));
}

__global__ void add_field_kernel(double *__restrict__ y, const double *__restrict__ x, long long n) {
    for(long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x)
        y[i] += x[i];
}

__global__ void scale_hat_kernel(double2 *__restrict__ y, const double2 *__restrict__ x, double a, long long n) {
    for(long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
        double2 v = x[i];
        y[i] = make_double2(a * v.x, a * v.y);
    }
}

int grid_of(long long n) { return (int) std::min<long long>((n + 255) / 256, 152 * 8); }

}  // namespace

struct chgb_adjoint {
    chgb_params p;
    int64_t T = 0;
    int K = 1;
    int nseg = 0;
    chgb_handle *h = nullptr;
    bool spectral = false;
    size_t n = 0;                      // cells
    std::vector<double *> ckpt_real;   // euler: field at step j K
    std::vector<double2 *> ckpt_hat;   // pseudospectral: scaled half spectrum at step j K
    double *seg_real = nullptr;        // K + 1 fields
    double *seg_real2 = nullptr;       // the second segment buffers of the pipelined backward pass
    double2 *seg_hat2 = nullptr;
    cudaStream_t st2 = nullptr;        // recomputation stream
    cudaEvent_t ev_rec[2] = {nullptr, nullptr}, ev_adj[2] = {nullptr, nullptr}, ev_start = nullptr;
    double2 *seg_hat = nullptr;        // K + 1 half spectra (pseudospectral)
    double *lam[2] = {nullptr, nullptr};
    double *part = nullptr;            // euler: 3 partial sums per block
    int nblocks = 0;
    bool two = false;                  // euler: two steps per launch, forward and adjoint
    double2 *tmp_hat = nullptr;
    double *tmp_real = nullptr;
    SpectralAdj *adj = nullptr;
    bool forward_done = false;
    std::map<long long, cudaGraphExec_t> graphs;   // segment sweeps, captured once per shape
    std::string err;
};

static int afail(chgb_adjoint *a, int code, const std::string &msg) {
    if(a) a->err = msg;
    record_error(msg);
    return code;
}

#define ACK(a, call, what)                                                                            \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if(e_ != cudaSuccess) return afail(a, CHGB_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e_)); \
    } while(0)

static void adj_release(chgb_adjoint *a) {
    if(!a) return;
    if(a->h && a->h->stream) cudaStreamSynchronize(a->h->stream);
    for(auto *p : a->ckpt_real) cudaFree(p);
    for(auto *p : a->ckpt_hat) cudaFree(p);
    if(a->st2) cudaStreamSynchronize(a->st2);
    cudaFree(a->seg_real);
    cudaFree(a->seg_real2);
    cudaFree(a->seg_hat);
    cudaFree(a->seg_hat2);
    for(int i = 0; i < 2; i++) {
        if(a->ev_rec[i]) cudaEventDestroy(a->ev_rec[i]);
        if(a->ev_adj[i]) cudaEventDestroy(a->ev_adj[i]);
    }
    if(a->ev_start) cudaEventDestroy(a->ev_start);
    if(a->st2) cudaStreamDestroy(a->st2);
    cudaFree(a->lam[0]);
    cudaFree(a->lam[1]);
    cudaFree(a->part);
    cudaFree(a->tmp_hat);
    cudaFree(a->tmp_real);
    for(auto &kv : a->graphs) cudaGraphExecDestroy(kv.second);
    if(a->adj) spectral_adj_destroy(a->adj);
    if(a->h) chgb_destroy(a->h);
    delete a;
}

// Replay the work `record` enqueues, captured into a CUDA graph the first time
// a given `key` (sweep kind, length, parity) is seen.  The sweeps of every
// full segment have the same shape and the same buffers, so a run of T steps
// launches a handful of graphs instead of ~4 T kernels.
template <class F>
static cudaError_t run_graph(chgb_adjoint *a, long long key, cudaStream_t st, F record) {
    auto it = a->graphs.find(key);
    if(it == a->graphs.end()) {
        cudaGraph_t g;
        cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
        if(e != cudaSuccess) return e;
        cudaError_t re = record();
        cudaError_t ee = cudaStreamEndCapture(st, &g);
        if(re != cudaSuccess) return re;
        if(ee != cudaSuccess) return ee;
        cudaGraphExec_t ex;
        e = cudaGraphInstantiate(&ex, g, 0);
        cudaGraphDestroy(g);
        if(e != cudaSuccess) return e;
        it = a->graphs.emplace(key, ex).first;
    }
    return cudaGraphLaunch(it->second, st);
}

enum { G_EULER_FWD = 1, G_EULER_ADJ = 2, G_PS_FWD = 3, G_PS_REC = 4, G_PS_ADJ = 5 };
// flags: bit 0 the lambda ping-pong parity, bit 1 the segment buffer
static long long gkey(int kind, int nsteps, int flags) { return ((long long) kind << 40) | ((long long) nsteps << 4) | flags; }

// The launches of an euler segment of `steps` steps (forward, recomputation or
// adjoint sweep): one per step, or one per pair of steps plus one for an odd
// step when the box takes two steps per launch.
static int seg_launches(const chgb_adjoint *a, int steps) { return a->two ? (steps + 1) / 2 : steps; }

// Enqueue an euler segment from seg[0]: every state seg[1..steps] is stored.
static cudaError_t record_segment(chgb_adjoint *a, double *seg, int steps, cudaStream_t st) {
    chgb_handle *h = a->h;
    cudaError_t e = cudaSuccess;
    int i = 0;
    if(a->two)
        for(; i + 1 < steps && e == cudaSuccess; i += 2)
            e = launch_euler_two(h->g, h->m, h->ec, seg + (size_t) i * a->n, seg + (size_t) (i + 2) * a->n, st,
                                 false, seg + (size_t) (i + 1) * a->n);
    for(; i < steps && e == cudaSuccess; i++)
        e = launch_euler_step(h->p.integrator, h->g, h->m, h->ec, seg + (size_t) i * a->n,
                              seg + (size_t) (i + 1) * a->n, st);
    return e;
}

// Ensure the handle has its S(q) plan and, for euler boxes, the auxiliary
// transform state (h->fft) used for seeds and the final field gradient.
static int ensure_aux(chgb_adjoint *a) {
    chgb_handle *h = a->h;
    std::string err;
    if(!h->sq) {
        h->sq = sq_plan_create(h->g.N, err);
        if(!h->sq) return afail(a, CHGB_ERR_ALLOC, err);
    }
    if(!h->fft) {
        chgb_params q = h->p;
        q.integrator = CHGB_INTEGRATOR_PSEUDOSPECTRAL;
        q.mobility_type = CHGB_MOBILITY_CONSTANT;
        int r = spectral_create(q, h->g, h->m, &h->fft, err);
        if(r != CHGB_OK) return afail(a, r, err);
    }
    return CHGB_OK;
}

extern "C" {

int chgb_adjoint_create(const chgb_params *params, int64_t nsteps, int32_t checkpoint_every, chgb_adjoint **out) {
    CHGB_TRACE("chgb_adjoint_create");
    if(!params || !out || nsteps < 1) return afail(nullptr, CHGB_ERR_INVALID, "invalid argument");
    *out = nullptr;
    const chgb_params &p = *params;
    if(p.dims != 2 || p.model.kind != CHGB_MODEL_LANDAU || p.mobility_type != CHGB_MOBILITY_CONSTANT)
        return afail(nullptr, CHGB_ERR_UNSUPPORTED, "the adjoint supports 2D Landau boxes with constant mobility");
    if(p.integrator == CHGB_INTEGRATOR_EULER && (p.N < 32 || p.N % 32))
        return afail(nullptr, CHGB_ERR_UNSUPPORTED, "the euler adjoint needs N >= 32");
    if(p.integrator == CHGB_INTEGRATOR_EULER_MOBILITY)
        return afail(nullptr, CHGB_ERR_UNSUPPORTED, "the adjoint supports euler and pseudospectral");
    if(p.kernel_variant < 0 || p.kernel_variant > 4 ||
       (p.kernel_variant == 3 && (p.integrator != CHGB_INTEGRATOR_EULER || p.N < 32 || p.N > 512)) ||
       (p.kernel_variant == 4 && (p.integrator != CHGB_INTEGRATOR_EULER || (p.N != 32 && p.N != 64))))
        return afail(nullptr, CHGB_ERR_INVALID,
                     "kernel_variant must be 0..4; 3 needs a 2D `euler` box with 32 <= N <= 512, 4 one with N = 32 "
                     "or 64");
    chgb_adjoint *a = new chgb_adjoint();
    a->p = p;
    a->T = nsteps;
    a->K = checkpoint_every > 0 ? checkpoint_every : (int) std::ceil(std::sqrt((double) nsteps));
    a->nseg = (int) ((nsteps + a->K - 1) / a->K);
    // The adjoint launches its own kernels, and the box only lends its
    // constants and buffers, so it is created with the fused step (no timing).
    // kernel_variant picks the checkpointed passes' form instead: 3 two steps
    // per launch, 1 and 2 one, 0 (and 4, whose resident box has no use for
    // stored states) two on 2D boxes up to N = 256 (where a step is too short
    // to fill the GPU) -- a fixed rule, so that every adjoint of a box sums its
    // gradients in the same order.
    chgb_params q = p;
    if(q.kernel_variant != 1 && q.kernel_variant != 2) q.kernel_variant = 1;
    int r = chgb_create(&q, &a->h);
    if(r != CHGB_OK) {
        std::string msg = chgb_last_error(nullptr);
        adj_release(a);
        return afail(nullptr, r, msg);
    }
    chgb_handle *h = a->h;
    a->spectral = h->ps != nullptr;
    if(a->spectral && !spectral_adjoint_supported(h->ps)) {
        adj_release(a);
        return afail(nullptr, CHGB_ERR_UNSUPPORTED, "the pseudospectral adjoint needs 8 <= N <= 1024");
    }
    a->n = (size_t) h->g.bins;
    bool ok = true;
    size_t fbytes = a->n * sizeof(double);
    if(a->spectral) {
        long long hs = spectral_hat_size(h->ps);
        size_t hbytes = sizeof(double2) * (size_t) hs;
        a->ckpt_hat.assign(a->nseg + 1, nullptr);
        for(auto &c : a->ckpt_hat) ok = ok && cudaMalloc(&c, hbytes) == cudaSuccess;
        ok = ok && cudaMalloc(&a->seg_real, fbytes * (a->K + 1)) == cudaSuccess &&
             cudaMalloc(&a->seg_hat, hbytes * (a->K + 1)) == cudaSuccess &&
             cudaMalloc(&a->seg_real2, fbytes * (a->K + 1)) == cudaSuccess &&
             cudaMalloc(&a->seg_hat2, hbytes * (a->K + 1)) == cudaSuccess &&
             cudaMalloc(&a->tmp_hat, hbytes) == cudaSuccess && cudaMalloc(&a->tmp_real, fbytes) == cudaSuccess;
        if(ok) {
            std::string err;
            a->adj = spectral_adj_create(h->ps, err);
            ok = a->adj != nullptr;
        }
    }
    else {
        a->ckpt_real.assign(a->nseg + 1, nullptr);
        for(auto &c : a->ckpt_real) ok = ok && cudaMalloc(&c, fbytes) == cudaSuccess;
        a->two = p.kernel_variant == 3 ||
                 ((p.kernel_variant == 0 || p.kernel_variant == 4) && euler_two_supported(p.integrator, h->g) &&
                  h->g.N <= 256);
        a->nblocks = std::max((h->g.N / ATX) * (h->g.N / adj_tile_rows(h->g.N)), (h->g.N / A2T) * (h->g.N / A2T));
        ok = ok && cudaMalloc(&a->seg_real, fbytes * (a->K + 1)) == cudaSuccess &&
             cudaMalloc(&a->seg_real2, fbytes * (a->K + 1)) == cudaSuccess &&
             cudaMalloc(&a->lam[0], fbytes) == cudaSuccess && cudaMalloc(&a->lam[1], fbytes) == cudaSuccess &&
             cudaMalloc(&a->part, sizeof(double) * 3 * a->nblocks) == cudaSuccess &&
             cudaMalloc(&a->tmp_hat, sizeof(double2) * (size_t) h->g.N * (h->g.N / 2 + 1)) == cudaSuccess &&
             cudaMalloc(&a->tmp_real, fbytes) == cudaSuccess;
    }
    ok = ok && cudaStreamCreateWithFlags(&a->st2, cudaStreamNonBlocking) == cudaSuccess &&
         cudaEventCreateWithFlags(&a->ev_rec[0], cudaEventDisableTiming) == cudaSuccess &&
         cudaEventCreateWithFlags(&a->ev_rec[1], cudaEventDisableTiming) == cudaSuccess &&
         cudaEventCreateWithFlags(&a->ev_adj[0], cudaEventDisableTiming) == cudaSuccess &&
         cudaEventCreateWithFlags(&a->ev_adj[1], cudaEventDisableTiming) == cudaSuccess &&
         cudaEventCreateWithFlags(&a->ev_start, cudaEventDisableTiming) == cudaSuccess;
    if(!ok) {
        cudaGetLastError();
        adj_release(a);
        return afail(nullptr, CHGB_ERR_ALLOC, "adjoint allocation failed");
    }
    r = ensure_aux(a);
    if(r != CHGB_OK) {
        std::string msg = a->err;
        adj_release(a);
        return afail(nullptr, r, msg);
    }
    *out = a;
    return CHGB_OK;
}

int chgb_adjoint_destroy(chgb_adjoint *a) {
    adj_release(a);
    return CHGB_OK;
}

int chgb_adjoint_forward(chgb_adjoint *a, const double *rho0, double *sq, double *rho_T) {
    CHGB_TRACE("chgb_adjoint_forward");
    if(!a || !rho0) return afail(a, CHGB_ERR_INVALID, "NULL argument");
    chgb_handle *h = a->h;
    cudaStream_t st = h->stream;
    int r = chgb_upload(h, rho0, nullptr);
    if(r != CHGB_OK) return afail(a, r, chgb_last_error(h));
    std::string err;
    if(a->spectral) {
        // start from the half spectrum, as every recomputed segment does
        ACK(a, spectral_load_hat(h->ps, spectral_psi_hat_mut(h->ps), st), "load state");
        long long hs = spectral_hat_size(h->ps);
        ACK(a, cudaMemcpyAsync(a->ckpt_hat[0], spectral_psi_hat(h->ps, 0), sizeof(double2) * hs, cudaMemcpyDeviceToDevice, st), "checkpoint");
        for(int j = 0; j < a->nseg; j++) {
            const int steps = (int) std::min<int64_t>(a->K, a->T - (int64_t) j * a->K);
            SpectralState *ps = h->ps;
            int64_t dummy = 0;
            ACK(a, run_graph(a, gkey(G_PS_FWD, steps, 0), st, [&]() -> cudaError_t {
                    std::string e2;
                    return spectral_step(ps, steps, st, &dummy, e2) == CHGB_OK ? cudaSuccess : cudaErrorUnknown;
                }), "forward segment");
            h->launches += 2 * steps;
            ACK(a, cudaMemcpyAsync(a->ckpt_hat[j + 1], spectral_psi_hat(h->ps, 0), sizeof(double2) * hs,
                                   cudaMemcpyDeviceToDevice, st), "checkpoint");
        }
    }
    else {
        const size_t fbytes = a->n * sizeof(double);
        ACK(a, cudaMemcpyAsync(a->ckpt_real[0], h->d_rho[h->cur], fbytes, cudaMemcpyDeviceToDevice, st), "checkpoint");
        ACK(a, cudaMemcpyAsync(a->seg_real, h->d_rho[h->cur], fbytes, cudaMemcpyDeviceToDevice, st), "segment start");
        for(int j = 0; j < a->nseg; j++) {
            const int steps = (int) std::min<int64_t>(a->K, a->T - (int64_t) j * a->K);
            ACK(a, run_graph(a, gkey(G_EULER_FWD, steps, 0), st,
                             [&]() -> cudaError_t { return record_segment(a, a->seg_real, steps, st); }),
                "forward segment");
            h->launches += seg_launches(a, steps);
            double *end = a->seg_real + (size_t) steps * a->n;
            ACK(a, cudaMemcpyAsync(a->ckpt_real[j + 1], end, fbytes, cudaMemcpyDeviceToDevice, st), "checkpoint");
            ACK(a, cudaMemcpyAsync(a->seg_real, end, fbytes, cudaMemcpyDeviceToDevice, st), "segment start");
        }
        // the box holds the final state (S(q), download)
        ACK(a, cudaMemcpyAsync(h->d_rho[h->cur], a->ckpt_real[a->nseg], fbytes, cudaMemcpyDeviceToDevice, st), "final");
    }
    h->steps_done = a->T;
    if(sq) {
        r = chgb_structure_factor(h, 0, sq, sq_nbins(h->g.N));
        if(r != CHGB_OK) return afail(a, r, chgb_last_error(h));
    }
    if(rho_T) {
        r = chgb_download(h, rho_T, nullptr);
        if(r != CHGB_OK) return afail(a, r, chgb_last_error(h));
    }
    ACK(a, cudaStreamSynchronize(st), "forward");
    a->forward_done = true;
    return CHGB_OK;
}

int chgb_adjoint_backward(chgb_adjoint *a, const double *dl_dsq, const double *dl_drho_T, double *grad_rho0,
                          double *grad_params) {
    CHGB_TRACE("chgb_adjoint_backward");
    if(!a) return afail(a, CHGB_ERR_INVALID, "NULL adjoint");
    if(!a->forward_done) return afail(a, CHGB_ERR_INVALID, "chgb_adjoint_forward must run first");
    chgb_handle *h = a->h;
    cudaStream_t st = h->stream;
    const Geom &g = h->g;
    const double cells = (double) g.bins;
    std::string err;
    const long long hs = (long long) g.N * (g.N / 2 + 1);
    const size_t fbytes = a->n * sizeof(double);

    if(a->spectral) {
        SpectralState *ps = h->ps;
        ACK(a, spectral_adj_zero(a->adj, ps, st), "zero");
        const double2 *psiT = a->ckpt_hat[a->nseg];
        if(dl_dsq) {
            ACK(a, sq_seed(h->sq, psiT, cells, dl_dsq, a->tmp_hat, st), "S(q) seed");
            ACK(a, spectral_adj_add_seed(a->adj, ps, a->tmp_hat, 1.0, st), "seed");
        }
        if(dl_drho_T) {
            ACK(a, cudaMemcpyAsync(a->tmp_real, dl_drho_T, fbytes, cudaMemcpyHostToDevice, st), "seed upload");
            int64_t dummy = 0;
            int r = spectral_set_rho(h->fft, a->tmp_real, st, &dummy, err);   // R2C / cells
            if(r != CHGB_OK) return afail(a, r, err);
            ACK(a, spectral_adj_add_seed(a->adj, ps, spectral_psi_hat(h->fft, 0), cells, st), "seed");
        }
        double2 *hbuf[2] = {a->seg_hat, a->seg_hat2};
        double *rbuf[2] = {a->seg_real, a->seg_real2};
        auto seg_len = [&](int j) { return (int) std::min<int64_t>(a->K, a->T - (int64_t) j * a->K); };
        // recompute segment j (half spectra and real fields) into buffers j & 1 on
        // the second stream, after the sweep that last read them (segment j + 2)
        auto recompute = [&](int j) -> int {
            const int b = j & 1, nsteps = seg_len(j);
            double2 *sh = hbuf[b];
            double *sr = rbuf[b];
            cudaStream_t s2 = a->st2;
            ACK(a, cudaStreamWaitEvent(s2, a->ev_adj[b], 0), "wait");
            ACK(a, spectral_load_hat(ps, a->ckpt_hat[j], s2), "segment start");
            ACK(a, run_graph(a, gkey(G_PS_REC, nsteps, b << 1), s2, [&]() -> cudaError_t {
                    cudaError_t e = cudaSuccess;
                    for(int i = 0; i < nsteps && e == cudaSuccess; i++) {
                        e = cudaMemcpyAsync(sh + (size_t) i * hs, spectral_psi_hat(ps, 0), sizeof(double2) * hs,
                                            cudaMemcpyDeviceToDevice, s2);
                        if(e == cudaSuccess) e = spectral_step_record(ps, sr + (size_t) i * a->n, s2);
                    }
                    if(e == cudaSuccess)
                        e = cudaMemcpyAsync(sh + (size_t) nsteps * hs, spectral_psi_hat(ps, 0), sizeof(double2) * hs,
                                            cudaMemcpyDeviceToDevice, s2);
                    return e;
                }), "segment recompute");
            ACK(a, cudaEventRecord(a->ev_rec[b], s2), "event");
            h->launches += 2 * nsteps + 1;
            return CHGB_OK;
        };
        ACK(a, cudaEventRecord(a->ev_start, st), "event");
        ACK(a, cudaStreamWaitEvent(a->st2, a->ev_start, 0), "wait");
        int rr = recompute(a->nseg - 1);
        if(rr != CHGB_OK) return rr;
        for(int j = a->nseg - 1; j >= 0; j--) {
            if(j >= 1) {
                rr = recompute(j - 1);
                if(rr != CHGB_OK) return rr;
            }
            const int b = j & 1, nsteps = seg_len(j);
            const double2 *sh = hbuf[b];
            const double *sr = rbuf[b];
            ACK(a, cudaStreamWaitEvent(st, a->ev_rec[b], 0), "wait");
            ACK(a, run_graph(a, gkey(G_PS_ADJ, nsteps, b << 1), st, [&]() -> cudaError_t {
                    cudaError_t e = spectral_adj_col(a->adj, ps, 1, sh + (size_t) nsteps * hs,
                                                     sh + (size_t) (nsteps - 1) * hs, st);
                    for(int i = nsteps - 1; i >= 1 && e == cudaSuccess; i--) {
                        e = spectral_adj_row(a->adj, ps, sr + (size_t) i * a->n, st);
                        if(e == cudaSuccess)
                            e = spectral_adj_col(a->adj, ps, 3, sh + (size_t) i * hs, sh + (size_t) (i - 1) * hs, st);
                    }
                    if(e == cudaSuccess) e = spectral_adj_row(a->adj, ps, sr, st);
                    if(e == cudaSuccess) e = spectral_adj_col(a->adj, ps, 2, nullptr, nullptr, st);
                    return e;
                }), "adjoint segment");
            ACK(a, cudaEventRecord(a->ev_adj[b], st), "event");
            h->launches += 2 * nsteps + 1;
        }
        if(grad_rho0) {
            // lam_0 = C2R(lam_hat_0) / cells
            scale_hat_kernel<<<grid_of(hs), 256, 0, st>>>(a->tmp_hat, spectral_adj_lam(a->adj), 1.0 / cells, hs);
            ACK(a, cudaGetLastError(), "scale");
            ACK(a, spectral_inverse(h->fft, a->tmp_hat, a->tmp_real, st), "inverse");
            ACK(a, cudaMemcpyAsync(grad_rho0, a->tmp_real, fbytes, cudaMemcpyDeviceToHost, st), "download");
        }
        ACK(a, cudaStreamSynchronize(st), "backward");
        if(grad_params) {
            int r = spectral_adj_grads(a->adj, grad_params);
            if(r != CHGB_OK) return afail(a, r, "gradient download failed");
        }
        // the box's state was overwritten by the recomputation: restore the final state
        ACK(a, spectral_load_hat(ps, a->ckpt_hat[a->nseg], st), "restore");
        ACK(a, cudaStreamSynchronize(st), "restore");
        return CHGB_OK;
    }

    // euler
    double *lam = a->lam[0], *lam_other = a->lam[1];
    ACK(a, cudaMemsetAsync(lam, 0, fbytes, st), "zero");
    ACK(a, cudaMemsetAsync(a->part, 0, sizeof(double) * 3 * a->nblocks, st), "zero");
    if(dl_dsq) {
        int64_t dummy = 0;
        int r = spectral_set_rho(h->fft, a->ckpt_real[a->nseg], st, &dummy, err);   // psi_t of the final field
        if(r != CHGB_OK) return afail(a, r, err);
        ACK(a, sq_seed(h->sq, spectral_psi_hat(h->fft, 0), 1.0, dl_dsq, a->tmp_hat, st), "S(q) seed");   // lam_hat / cells
        ACK(a, spectral_inverse(h->fft, a->tmp_hat, lam, st), "inverse");
    }
    if(dl_drho_T) {
        ACK(a, cudaMemcpyAsync(a->tmp_real, dl_drho_T, fbytes, cudaMemcpyHostToDevice, st), "seed upload");
        add_field_kernel<<<grid_of((long long) a->n), 256, 0, st>>>(lam, a->tmp_real, (long long) a->n);
        ACK(a, cudaGetLastError(), "seed");
    }
    const int aty = adj_tile_rows(g.N);
    dim3 agrid(g.N / ATX, g.N / aty);
    double *segbuf[2] = {a->seg_real, a->seg_real2};
    auto seg_len = [&](int j) { return (int) std::min<int64_t>(a->K, a->T - (int64_t) j * a->K); };
    // recompute segment j into buffer j & 1 on the second stream, once the adjoint
    // sweep that last read that buffer (segment j + 2) has finished
    auto recompute = [&](int j) -> int {
        const int b = j & 1, nsteps = seg_len(j);
        double *buf = segbuf[b];
        ACK(a, cudaStreamWaitEvent(a->st2, a->ev_adj[b], 0), "wait");
        ACK(a, cudaMemcpyAsync(buf, a->ckpt_real[j], fbytes, cudaMemcpyDeviceToDevice, a->st2), "segment start");
        ACK(a, run_graph(a, gkey(G_EULER_FWD, nsteps, b << 1), a->st2,
                         [&]() -> cudaError_t { return record_segment(a, buf, nsteps, a->st2); }),
            "segment recompute");
        ACK(a, cudaEventRecord(a->ev_rec[b], a->st2), "event");
        h->launches += seg_launches(a, nsteps);
        return CHGB_OK;
    };
    ACK(a, cudaEventRecord(a->ev_start, st), "event");
    ACK(a, cudaStreamWaitEvent(a->st2, a->ev_start, 0), "wait");
    int r = recompute(a->nseg - 1);
    if(r != CHGB_OK) return r;
    for(int j = a->nseg - 1; j >= 0; j--) {
        if(j >= 1) {
            r = recompute(j - 1);
            if(r != CHGB_OK) return r;
        }
        const int b = j & 1, nsteps = seg_len(j);
        const double *buf = segbuf[b];
        ACK(a, cudaStreamWaitEvent(st, a->ev_rec[b], 0), "wait");
        const int parity = (lam == a->lam[0]) ? 0 : 1;
        ACK(a, run_graph(a, gkey(G_EULER_ADJ, nsteps, parity | (b << 1)), st, [&]() -> cudaError_t {
                double *li = a->lam[parity], *lo = a->lam[parity ^ 1];
                int i = nsteps - 1;
                if(a->two) {
                    for(; i >= 1; i -= 2) {
                        euler_adj2d_two_kernel<<<dim3(g.N / A2T, g.N / A2T), dim3(32, 8), 0, st>>>(
                            li, buf + (size_t) i * a->n, buf + (size_t) (i - 1) * a->n, lo, g, h->ec, h->m.epsilon,
                            a->part);
                        cudaError_t e = cudaGetLastError();
                        if(e != cudaSuccess) return e;
                        std::swap(li, lo);
                    }
                }
                for(; i >= 0; i--) {
                    const double *psi_i = buf + (size_t) i * a->n;
                    if(aty == 8)
                        euler_adj2d_kernel<8><<<agrid, dim3(32, 8), 0, st>>>(li, psi_i, lo, g, h->ec, h->m.epsilon,
                                                                             a->part);
                    else
                        euler_adj2d_kernel<32><<<agrid, dim3(32, 8), 0, st>>>(li, psi_i, lo, g, h->ec, h->m.epsilon,
                                                                              a->part);
                    cudaError_t e = cudaGetLastError();
                    if(e != cudaSuccess) return e;
                    std::swap(li, lo);
                }
                return cudaSuccess;
            }), "adjoint segment");
        ACK(a, cudaEventRecord(a->ev_adj[b], st), "event");
        if(seg_launches(a, nsteps) & 1) std::swap(lam, lam_other);
        h->launches += seg_launches(a, nsteps);
    }
    if(grad_rho0) ACK(a, cudaMemcpyAsync(grad_rho0, lam, fbytes, cudaMemcpyDeviceToHost, st), "download");
    std::vector<double> part(3 * a->nblocks);
    ACK(a, cudaMemcpyAsync(part.data(), a->part, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, st), "partials");
    ACK(a, cudaStreamSynchronize(st), "backward");
    if(grad_params) {
        // A = <w, psi>, B = <D w, psi> = <w, D psi>, C = <w, psi^3>, summed over steps
        double sa = 0, sb = 0, sc = 0;
        for(int b = 0; b < a->nblocks; b++) {
            sa += part[3 * b];
            sb += part[3 * b + 1];
            sc += part[3 * b + 2];
        }
        const double dx2 = h->p.dx * h->p.dx;
        grad_params[0] = -sa;
        grad_params[1] = -(2.0 / dx2) * sb;
        // <w, mu> with mu = psi^3 - eps psi - c2 D psi
        grad_params[2] = (sc - h->m.epsilon * sa - h->ec.c2[0] * sb) / h->p.M;
    }
    return CHGB_OK;
}

int64_t chgb_adjoint_launch_count(const chgb_adjoint *a) { return (a && a->h) ? a->h->launches : 0; }

}  // extern "C"
