// psmob_gmres.cu — the GMRES path of `pseudospectral_mobility`
// (pseudospectral.use_gmres = true).
//
// Reference: src/integrators/PseudospectralMobilityCPU.cpp, _evolve_full
// :312-427, _apply_Pinv :440-466, _apply_A :468-535, _gmres_solve :537-662.
// Each step solves
//     A rho' = b,   A x = x - dt div(M grad((S - 2k lap) x)),
//     b = rho + dt div(M grad(f'(rho) - S rho)),
// by restarted GMRES (restart length m, Saad & Schultz 1986), left-
// preconditioned by the diagonal k-space operator
// P^-1 = 1 / (1 + dt M0 (S q^2 + 2k q^4)), starting from rho.
//
// The whole solve of one time step is ONE CUDA graph launch, with no host
// round trip:
//   setup    M0, the right-hand side b, x = rho, P^-1 b, r = P^-1 b - P^-1 A x,
//            the norms |P^-1 b| and |r|;
//   WHILE    (restart cycles, a conditional node; the condition is set on the
//            device by the kernel that tests the true residual)
//     cycle start   V_0 = r / |r|, the Krylov residual vector g = |r| e_0;
//     WHILE  (Arnoldi steps of the cycle)
//        w = P^-1 A V_j; two passes of classical Gram-Schmidt against
//        V_0..V_j (5 kernels whatever j is, instead of 3(j+1) for modified
//        Gram-Schmidt; two passes orthogonalise at least as well as one
//        modified pass); h_{j+1} = |w|, V_{j+1} = w / h_{j+1};
//        one device thread then rotates the new Hessenberg column by the
//        cycle's earlier Givens rotations, forms the rotation that zeroes
//        h_{j+1}, updates g, tests |g_{j+1}| / |P^-1 b| against the tolerance
//        and the cycle and iteration limits, and, when the cycle ends, solves
//        the triangular system R y = g by back substitution;
//     cycle end     x += V y, r = P^-1 b - P^-1 A x, |r|: stop when
//                   |r| / |P^-1 b| < tol or the iteration limit is reached;
//   finish   rho = x and its transform.
// The stopping rules are the reference's (iteration counting, the 1e-30
// breakdown threshold, the true-residual test after each cycle).  The inner
// products are fixed-order block reductions and the orthogonalisation is
// classical Gram-Schmidt in two passes, so the iterates agree with the
// reference's to round-off rather than bit for bit.  Both loops are bounded on
// the device: a cycle takes at most m Arnoldi steps, and the restart loop at
// most gmres_max_iter + 1 cycles (the reference's loop has no such bound when a
// breakdown in the first column repeats without convergence).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "kernels.h"
#include "psmob_impl.h"

namespace chgb {

namespace {

constexpr int DOT_BLOCKS = 256;   // blocks of every reduction: the grouping of the sums never changes
constexpr int RT = 256;           // threads per block of the vector kernels

int vgrid(long long n) { return (int) std::min<long long>((n + 255) / 256, 152 * 8); }

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for(int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Sum over a block of RT threads in a fixed order; the result is valid in thread 0.
__device__ __forceinline__ double block_sum(double v, double *red) {
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if(lane == 0) red[w] = v;
    __syncthreads();
    if(w == 0) {
        v = (lane < RT / 32) ? red[lane] : 0.0;
        v = warp_sum(v);
    }
    __syncthreads();
    return v;
}

__global__ void dot_partial_kernel(const double *__restrict__ a, const double *__restrict__ b, long long n,
                                   double *__restrict__ part) {
    double acc = 0.0;
    for(long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x)
        acc += a[i] * b[i];
    __shared__ double red[256];
    red[threadIdx.x] = acc;
    __syncthreads();
    for(int o = blockDim.x / 2; o > 0; o >>= 1) {
        if(threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if(threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// out = sum of the partials (fixed order); sqrt of it when `root`
__global__ void dot_final_kernel(const double *__restrict__ part, int nb, int root, double *__restrict__ out) {
    if(threadIdx.x != 0 || blockIdx.x != 0) return;
    double s = 0.0;
    for(int b = 0; b < nb; b++) s += part[b];
    *out = root ? sqrt(s) : s;
}

__global__ void sub_kernel(const double *__restrict__ a, const double *__restrict__ b, long long n,
                           double *__restrict__ out) {
    for(long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x)
        out[i] = a[i] - b[i];
}

// out = a / N^d, as a * inv_bins (exact: N^d is a power of two)
__global__ void div_kernel(const double *__restrict__ a, double inv_bins, long long n, double *__restrict__ out) {
    for(long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x)
        out[i] = a[i] * inv_bins;
}

// q_hat = D (S + 2k q^2) x_hat in place (:485-491)
__global__ void qhat_kernel(double2 *__restrict__ h, const double *__restrict__ q2, const double *__restrict__ dealias,
                            int use_dealias, double Ssplit, double two_k, long long n) {
    for(long long k = blockIdx.x * (long long) blockDim.x + threadIdx.x; k < n; k += (long long) gridDim.x * blockDim.x) {
        double f = Ssplit + two_k * q2[k];
        double2 v = h[k];
        v.x = f * v.x;
        v.y = f * v.y;
        if(use_dealias) {
            double D = dealias[k];
            v.x *= D;
            v.y *= D;
        }
        h[k] = v;
    }
}

// J = M (C2R(...) / N^d) in place.  Here and below inv_bins = 1 / N^d, exact
// (a power of two): the product is the division, bit for bit.
__global__ void fluxM_kernel(double *__restrict__ g, const double *__restrict__ mob, long long n, double inv_bins) {
    for(long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
        double gv = g[i] * inv_bins;
        g[i] = mob[i] * gv;
    }
}

// Ax = x - dt (div / N^d)   (:527-533)
__global__ void applyA_final_kernel(const double *__restrict__ x, const double *__restrict__ div, double dt,
                                    double inv_bins, long long n, double *__restrict__ Ax) {
    for(long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
        double dr = div[i] * inv_bins;
        Ax[i] = x[i] - dt * dr;
    }
}

// hat /= 1 + dt M0 (S q^2 + 2k q^4)   (:452-459)
__global__ void pinv_kernel(double2 *__restrict__ h, const double *__restrict__ q2, const double *__restrict__ M0,
                            double dt, double Ssplit, double k0, long long hat, long long n) {
    for(long long k = blockIdx.x * (long long) blockDim.x + threadIdx.x; k < n; k += (long long) gridDim.x * blockDim.x) {
        const int s = (int) (k / hat);
        double k2v = q2[k];
        double k4v = k2v * k2v;
        double denom = 1.0 + dt * M0[s] * (Ssplit * k2v + 2.0 * k0 * k4v);
        double2 v = h[k];
        h[k] = make_double2(v.x / denom, v.y / denom);
    }
}

// tmp = f'(rho) - S rho  /  b = rho + dt (tmp / N^d)
__global__ void g_kernel(const double *__restrict__ fder, const double *__restrict__ rho, double Ssplit, long long n,
                         double *__restrict__ out) {
    for(long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x)
        out[i] = fder[i] - Ssplit * rho[i];
}

__global__ void rhs_kernel(const double *__restrict__ rho, const double *__restrict__ div, double dt, double inv_bins,
                           long long n, double *__restrict__ b) {
    for(long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
        double t = div[i] * inv_bins;
        b[i] = rho[i] + dt * t;
    }
}

// ---------------------------------------------------------------------------
// Device-resident GMRES state and the kernels of the Krylov iteration
// ---------------------------------------------------------------------------

// Scalars of the solve in progress (device memory), plus counters over the
// handle's life (for the launch count).
struct GmState {
    int j;          // Arnoldi column being formed in this cycle
    int iters;      // Arnoldi steps counted as the reference counts them (iter_total)
    int cycles;     // restart cycles run in this solve
    int jend;       // columns of the cycle that just ended
    double rhs_norm, beta;
    unsigned long long arnoldi_total, cycles_total;
};

// Everything a kernel of the iteration needs, passed by value.
struct GmDev {
    GmState *st;
    double *hcol;   // the new Hessenberg column h_0..h_{j+1} (m + 1)
    double *R;      // rotated Hessenberg matrix, column k at R + k (m + 1), rows 0..k
    double *cs, *sn;  // Givens rotations of the cycle (m each)
    double *gv;     // Krylov-coordinate residual (m + 1)
    double *y;      // solution of R y = g (m)
    double *V;      // Krylov basis, (m + 1) x n
    double *w, *vj, *x, *r;
    double *part;   // DOT_BLOCKS partial sums per basis vector: part[i * DOT_BLOCKS + b]
    double *part2;  // DOT_BLOCKS partial sums of |w|^2
    const double *slot;  // slot[0] = |P^-1 b|, slot[1] = |r|
    long long n;
    int m, max_iter;
    double tol;
    cudaGraphConditionalHandle outer, inner;
};

// The reference's std::max(norm, 1e-30), NaN kept as std::max keeps it.
__device__ __forceinline__ double floor_norm(double v) { return (v < 1e-30) ? 1e-30 : v; }

// Start of a solve: the norms of P^-1 b and of the first residual; enter the
// restart loop unless the start already meets the tolerance.
__global__ void gm_solve_begin_kernel(GmDev d) {
    GmState *st = d.st;
    st->rhs_norm = floor_norm(d.slot[0]);
    st->beta = d.slot[1];
    st->iters = 0;
    st->cycles = 0;
    const bool go = !(st->beta / st->rhs_norm < d.tol) && d.max_iter > 0;
    cudaGraphSetConditional(d.outer, go ? 1u : 0u);
}

// Start of a restart cycle: V_0 = r / beta, g = beta e_0, column 0.
__global__ void gm_cycle_begin_kernel(GmDev d) {
    const double beta = d.st->beta;
    for(long long k = blockIdx.x * (long long) blockDim.x + threadIdx.x; k < d.n; k += (long long) gridDim.x * blockDim.x)
        d.V[k] = d.r[k] / beta;
    if(blockIdx.x == 0 && threadIdx.x == 0) {
        GmState *st = d.st;
        d.gv[0] = beta;
        for(int i = 1; i <= d.m; i++) d.gv[i] = 0.0;
        st->j = 0;
        st->jend = 0;
        st->cycles_total++;
        cudaGraphSetConditional(d.inner, st->iters < d.max_iter ? 1u : 0u);
    }
}

// vj = V_j: the operator's input at a fixed address.
__global__ void gm_take_column_kernel(GmDev d) {
    const double *src = d.V + (size_t) d.st->j * d.n;
    for(long long k = blockIdx.x * (long long) blockDim.x + threadIdx.x; k < d.n; k += (long long) gridDim.x * blockDim.x)
        d.vj[k] = src[k];
}

// Gram-Schmidt, first half of a pass: per block, <w, V_i> for i = 0..j.
__global__ void __launch_bounds__(RT) gm_dots_kernel(GmDev d) {
    __shared__ double red[RT / 32];
    const int j = d.st->j;
    for(int i = 0; i <= j; i++) {
        const double *v = d.V + (size_t) i * d.n;
        double acc = 0.0;
        for(long long k = blockIdx.x * (long long) RT + threadIdx.x; k < d.n; k += (long long) gridDim.x * RT)
            acc += d.w[k] * v[k];
        acc = block_sum(acc, red);
        if(threadIdx.x == 0) d.part[(size_t) i * DOT_BLOCKS + blockIdx.x] = acc;
    }
}

// Gram-Schmidt, second half of a pass: every block folds the partials into
// c_i (groups of 8 threads per coefficient, a fixed order), block 0 records
// them in the Hessenberg column (pass 0 sets, pass 1 adds the correction),
// and w -= sum_i c_i V_i.  Pass 1 also leaves per-block partials of |w|^2.
__global__ void __launch_bounds__(RT) gm_orth_kernel(GmDev d, int pass) {
    extern __shared__ double c[];      // j + 1 coefficients
    __shared__ double red[RT / 32];
    const int j = d.st->j;
    const int sub = threadIdx.x & 7, grp = threadIdx.x >> 3;
    for(int i0 = 0; i0 <= j; i0 += RT / 8) {
        const int i = i0 + grp;
        double acc = 0.0;
        if(i <= j)
            for(int b = sub; b < DOT_BLOCKS; b += 8) acc += d.part[(size_t) i * DOT_BLOCKS + b];
        acc += __shfl_xor_sync(0xffffffffu, acc, 4);
        acc += __shfl_xor_sync(0xffffffffu, acc, 2);
        acc += __shfl_xor_sync(0xffffffffu, acc, 1);
        if(i <= j && sub == 0) c[i] = acc;
    }
    __syncthreads();
    if(blockIdx.x == 0)
        for(int i = threadIdx.x; i <= j; i += RT) d.hcol[i] = pass == 0 ? c[i] : d.hcol[i] + c[i];
    double sq = 0.0;
    for(long long k = blockIdx.x * (long long) RT + threadIdx.x; k < d.n; k += (long long) gridDim.x * RT) {
        double v = d.w[k];
        for(int i = 0; i <= j; i++) v -= c[i] * d.V[(size_t) i * d.n + k];
        d.w[k] = v;
        sq += v * v;
    }
    if(pass == 1) {
        sq = block_sum(sq, red);
        if(threadIdx.x == 0) d.part2[blockIdx.x] = sq;
    }
}

// h_{j+1} = |w| (every block folds the partials in the same order) and
// V_{j+1} = w / h_{j+1}.
__global__ void __launch_bounds__(RT) gm_norm_scale_kernel(GmDev d) {
    __shared__ double nrm;
    if(threadIdx.x < 32) {
        double acc = 0.0;
        for(int b = threadIdx.x; b < DOT_BLOCKS; b += 32) acc += d.part2[b];
        acc = warp_sum(acc);
        if(threadIdx.x == 0) nrm = sqrt(acc);
    }
    __syncthreads();
    const int j = d.st->j;
    const double h = nrm;
    if(blockIdx.x == 0 && threadIdx.x == 0) d.hcol[j + 1] = h;
    double *dst = d.V + (size_t) (j + 1) * d.n;
    for(long long k = blockIdx.x * (long long) RT + threadIdx.x; k < d.n; k += (long long) gridDim.x * RT)
        dst[k] = d.w[k] / h;
}

// One thread: fold the new column into the cycle's QR factorisation by Givens
// rotations (Saad & Schultz 1986), decide whether the cycle goes on, and at
// its end solve R y = g.  A breakdown (h_{j+1} <= 1e-30) ends the cycle with
// the column kept unrotated and this step not counted, and so does meeting the
// tolerance, as the reference's loop does (:589-634).
__global__ void gm_givens_kernel(GmDev d) {
    GmState *st = d.st;
    const int j = st->j, m = d.m;
    double *col = d.R + (size_t) j * (m + 1);
    bool more = false;
    st->arnoldi_total++;
    if(!(d.hcol[j + 1] > 1e-30)) {
        for(int i = 0; i <= j; i++) col[i] = d.hcol[i];
    }
    else {
        double hi = d.hcol[0];
        for(int i = 0; i < j; i++) {
            // rotation i acts on rows i and i + 1
            const double lo = d.hcol[i + 1];
            col[i] = d.cs[i] * hi + d.sn[i] * lo;
            hi = -d.sn[i] * hi + d.cs[i] * lo;
        }
        const double a = hi, b = d.hcol[j + 1];
        const double rr = sqrt(a * a + b * b);
        const double c = rr > 0 ? a / rr : 1.0, s = rr > 0 ? b / rr : 0.0;
        d.cs[j] = c;
        d.sn[j] = s;
        col[j] = c * a + s * b;
        const double gj = d.gv[j];
        d.gv[j] = c * gj;
        d.gv[j + 1] = -s * gj;
        if(!(fabs(d.gv[j + 1]) / st->rhs_norm < d.tol)) {
            st->iters++;
            st->j = j + 1;
            more = st->j < m && st->iters < d.max_iter;
        }
    }
    if(!more) {
        // back substitution by columns: y_k = t_k / R_kk, then t_i -= R_ik y_k for i < k
        const int n = j + 1;
        st->jend = n;
        for(int i = 0; i < n; i++) d.y[i] = d.gv[i];
        for(int k = n - 1; k >= 0; k--) {
            const double *rk = d.R + (size_t) k * (m + 1);
            const double yk = d.y[k] / rk[k];
            d.y[k] = yk;
            for(int i = 0; i < k; i++) d.y[i] -= rk[i] * yk;
        }
    }
    cudaGraphSetConditional(d.inner, more ? 1u : 0u);
}

// x[k] += V_i[k] y_i for i = 0 .. jend-1 in order (:644-646)
__global__ void gm_xupdate_kernel(GmDev d) {
    const int jend = d.st->jend;
    for(long long k = blockIdx.x * (long long) blockDim.x + threadIdx.x; k < d.n; k += (long long) gridDim.x * blockDim.x) {
        double acc = d.x[k];
        for(int i = 0; i < jend; i++) acc += d.V[(size_t) i * d.n + k] * d.y[i];
        d.x[k] = acc;
    }
}

// End of a restart cycle: the true residual's norm decides whether to restart
// (:648-656); at most max_iter + 1 cycles run.
__global__ void gm_cycle_end_kernel(GmDev d) {
    GmState *st = d.st;
    st->beta = d.slot[1];
    st->cycles++;
    const bool go = !(st->beta / st->rhs_norm < d.tol) && st->iters < d.max_iter && st->cycles <= d.max_iter;
    cudaGraphSetConditional(d.outer, go ? 1u : 0u);
}

}  // namespace

struct PsGmres {
    int m = 2;
    long long n = 0;
    double *b = nullptr, *x = nullptr, *rhs = nullptr, *Mx = nullptr, *r = nullptr, *w = nullptr, *Av = nullptr,
           *vj = nullptr;
    double *V = nullptr;       // (m + 1) x n
    double *part = nullptr;    // DOT_BLOCKS x (m + 1)
    double *part2 = nullptr;   // DOT_BLOCKS
    double *slot = nullptr;    // |P^-1 b|, |r|
    double *arr = nullptr;     // hcol (m + 2), R (m (m + 1)), cs (m), sn (m), g (m + 1), y (m)
    GmState *state = nullptr;
    double2 *hat = nullptr;    // scratch half spectrum
    // the solve of one step as one graph (conditional WHILE nodes for the
    // restart cycles and the Arnoldi steps), built for one (mobility, density)
    // pair of buffers
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    const double *graph_mob = nullptr;
    const double *graph_rho = nullptr;
    int setup_launches = 0, cycle_launches = 0, arnoldi_launches = 0;
};

void psmob_gmres_release(PsMob *s) {
    PsGmres *g = s->gm;
    if(!g) return;
    if(g->exec) cudaGraphExecDestroy(g->exec);
    if(g->graph) cudaGraphDestroy(g->graph);
    for(double *p : {g->b, g->x, g->rhs, g->Mx, g->r, g->w, g->Av, g->vj, g->V, g->part, g->part2, g->slot, g->arr})
        cudaFree(p);
    cudaFree(g->state);
    cudaFree(g->hat);
    delete g;
    s->gm = nullptr;
}

int64_t psmob_gmres_loop_launches(const PsMob *s, cudaStream_t st) {
    const PsGmres *g = s->gm;
    if(!g || !g->state) return 0;
    GmState h{};
    if(cudaStreamSynchronize(st) != cudaSuccess ||
       cudaMemcpy(&h, g->state, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return (int64_t) h.cycles_total * g->cycle_launches + (int64_t) h.arnoldi_total * g->arnoldi_launches;
}

namespace {

struct Ctx {
    PsMob *s;
    PsGmres *g;
    const double *mob;
    cudaStream_t st;
    int nl = 0;
    cudaError_t e = cudaSuccess;
};

// dot(a, b) (or its square root) into the device slot `out`
void dot_dev(Ctx &c, const double *a, const double *b, double *out, bool root) {
    if(c.e != cudaSuccess) return;
    dot_partial_kernel<<<DOT_BLOCKS, 256, 0, c.st>>>(a, b, c.g->n, c.g->part);
    dot_final_kernel<<<1, 32, 0, c.st>>>(c.g->part, DOT_BLOCKS, root ? 1 : 0, out);
    c.nl += 2;
    c.e = cudaGetLastError();
}

// out = D i k_d-gradients of `in_hat`, fluxes M grad, divergence, C2R: out_real = C2R(div_hat) (unnormalised)
void div_M_grad(Ctx &c, const double2 *in_hat, double *out_real) {
    PsMob *s = c.s;
    const long long rn = s->bins * s->S;
    if(s->g.dims >= 2) {   // the stages on the transforms' passes (spectral_psmob_flux, M0 null: flux M g)
        const PsmobTables t = psmob_tables(s);
        for(int d = 0; d < s->g.dims && c.e == cudaSuccess; d++)
            c.e = spectral_psmob_flux(s->eng, in_hat, s->kc[d], t, c.mob, nullptr, s->div_hat, d == 0, s->tmp_hat,
                                      c.st, &c.nl);
        if(c.e == cudaSuccess) c.e = spectral_c2r(s->eng, s->div_hat, out_real, c.st, &c.nl);
        return;
    }
    for(int d = 0; d < s->g.dims && c.e == cudaSuccess; d++) {
        c.e = psmob_grad(s, in_hat, d, c.st);
        c.nl++;
        if(c.e == cudaSuccess) c.e = spectral_c2r(s->eng, s->tmp_hat, s->tmp, c.st, &c.nl);
        if(c.e == cudaSuccess) {
            fluxM_kernel<<<vgrid(rn), 256, 0, c.st>>>(s->tmp, c.mob, rn, 1.0 / (double) s->bins);
            c.nl++;
            c.e = cudaGetLastError();
        }
        if(c.e == cudaSuccess) c.e = spectral_r2c(s->eng, s->tmp, s->tmp_hat, c.st, &c.nl);
        if(c.e == cudaSuccess) {
            c.e = psmob_div(s, d, c.st);
            c.nl++;
        }
    }
    if(c.e == cudaSuccess) c.e = spectral_c2r(s->eng, s->div_hat, out_real, c.st, &c.nl);
}

// Ax = A x  (_apply_A)
void apply_A(Ctx &c, const double *x, double *Ax) {
    PsMob *s = c.s;
    const long long rn = c.g->n;
    if(c.e == cudaSuccess) c.e = spectral_r2c(s->eng, x, c.g->hat, c.st, &c.nl);
    if(c.e == cudaSuccess) {
        qhat_kernel<<<vgrid(s->hall), 256, 0, c.st>>>(c.g->hat, s->q2, s->dealias, s->p.use_dealias ? 1 : 0,
                                                       s->p.splitting_S, 2.0 * s->p.k[0], s->hall);
        c.nl++;
        c.e = cudaGetLastError();
    }
    div_M_grad(c, c.g->hat, s->fder);   // s->fder is free scratch here
    if(c.e == cudaSuccess) {
        applyA_final_kernel<<<vgrid(rn), 256, 0, c.st>>>(x, s->fder, s->p.dt, 1.0 / (double) s->bins, rn, Ax);
        c.nl++;
        c.e = cudaGetLastError();
    }
}

// z = P^-1 r  (_apply_Pinv)
void apply_Pinv(Ctx &c, const double *r, double *z) {
    PsMob *s = c.s;
    if(c.e == cudaSuccess) c.e = spectral_r2c(s->eng, r, c.g->hat, c.st, &c.nl);
    if(c.e == cudaSuccess) {
        pinv_kernel<<<vgrid(s->hall), 256, 0, c.st>>>(c.g->hat, s->q2, s->M0, s->p.dt, s->p.splitting_S, s->p.k[0],
                                                       s->hat, s->hall);
        c.nl++;
        c.e = cudaGetLastError();
    }
    if(c.e == cudaSuccess) c.e = spectral_c2r(s->eng, c.g->hat, z, c.st, &c.nl);
    if(c.e == cudaSuccess) {
        div_kernel<<<vgrid(c.g->n), 256, 0, c.st>>>(z, 1.0 / (double) s->bins, c.g->n, z);
        c.nl++;
        c.e = cudaGetLastError();
    }
}

void apply_M(Ctx &c, const double *v, double *out) {
    apply_A(c, v, c.g->Av);
    apply_Pinv(c, c.g->Av, out);
}

void launched(Ctx &c) {
    c.nl++;
    if(c.e == cudaSuccess) c.e = cudaGetLastError();
}

// Insert a WHILE conditional node at the capture point of `st` and make it the
// capture's only dependency; *body receives the node's body graph.
cudaError_t add_while(cudaStream_t st, cudaGraphConditionalHandle h, cudaGraph_t *body) {
    cudaStreamCaptureStatus status;
    cudaGraph_t cg = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    size_t nd = 0;
    cudaError_t e = cudaStreamGetCaptureInfo(st, &status, nullptr, &cg, &deps, nullptr, &nd);
    if(e != cudaSuccess) return e;
    if(status != cudaStreamCaptureStatusActive) return cudaErrorStreamCaptureInvalidated;
    cudaGraphNodeParams prm = {cudaGraphNodeTypeConditional};
    prm.conditional.handle = h;
    prm.conditional.type = cudaGraphCondTypeWhile;
    prm.conditional.size = 1;
    cudaGraphNode_t node = nullptr;
    e = cudaGraphAddNode(&node, cg, deps, nullptr, nd, &prm);
    if(e != cudaSuccess) return e;
    *body = prm.conditional.phGraph_out[0];
    return cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
}

// Capture into `graph` (appending) what `fill` enqueues on `st`.
template <class F>
cudaError_t capture_into(cudaGraph_t graph, cudaStream_t st, Ctx &c, F fill) {
    cudaError_t e = cudaStreamBeginCaptureToGraph(st, graph, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if(e != cudaSuccess) return e;
    fill();
    cudaGraph_t out = nullptr;
    cudaError_t ee = cudaStreamEndCapture(st, &out);
    return c.e != cudaSuccess ? c.e : ee;
}

cudaError_t build_solve_graph(PsMob *s, const double *mob, double *rho, cudaStream_t st) {
    PsGmres *g = s->gm;
    if(g->exec) cudaGraphExecDestroy(g->exec);
    if(g->graph) cudaGraphDestroy(g->graph);
    g->exec = nullptr;
    g->graph = nullptr;
    cudaError_t e = cudaGraphCreate(&g->graph, 0);
    if(e != cudaSuccess) return e;
    const long long n = g->n;
    const int m = g->m, vg = vgrid(n);
    GmDev d;
    d.st = g->state;
    d.hcol = g->arr;
    d.R = d.hcol + (m + 2);
    d.cs = d.R + (size_t) m * (m + 1);
    d.sn = d.cs + m;
    d.gv = d.sn + m;
    d.y = d.gv + (m + 1);
    d.V = g->V;
    d.w = g->w;
    d.vj = g->vj;
    d.x = g->x;
    d.r = g->r;
    d.part = g->part;
    d.part2 = g->part2;
    d.slot = g->slot;
    d.n = n;
    d.m = m;
    d.max_iter = s->p.gmres_max_iter;
    d.tol = s->p.gmres_tol;
    e = cudaGraphConditionalHandleCreate(&d.outer, g->graph, 0, 0);
    if(e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&d.inner, g->graph, 0, 0);
    if(e != cudaSuccess) return e;
    const size_t orth_smem = sizeof(double) * (size_t) (m + 1);

    // top level: setup, the restart loop, finish
    Ctx c{s, g, mob, st};
    cudaGraph_t outer_body = nullptr, inner_body = nullptr;
    int finish_launches = 0;
    e = capture_into(g->graph, st, c, [&]() {
        c.nl += psmob_m0(s, mob, st);   // M0 for the preconditioner
        c.e = launch_der_bulk(s->m, rho, s->fder, s->bins, st);
        c.nl++;
        if(c.e == cudaSuccess) {
            g_kernel<<<vg, 256, 0, st>>>(s->fder, rho, s->p.splitting_S, n, s->tmp);
            launched(c);
        }
        if(c.e == cudaSuccess) c.e = spectral_r2c(s->eng, s->tmp, s->mu_hat, st, &c.nl);
        div_M_grad(c, s->mu_hat, s->fder);
        if(c.e == cudaSuccess) {
            rhs_kernel<<<vg, 256, 0, st>>>(rho, s->fder, s->p.dt, 1.0 / (double) s->bins, n, g->b);
            launched(c);
        }
        if(c.e == cudaSuccess) c.e = cudaMemcpyAsync(g->x, rho, sizeof(double) * n, cudaMemcpyDeviceToDevice, st);
        apply_Pinv(c, g->b, g->rhs);
        apply_M(c, g->x, g->Mx);
        if(c.e == cudaSuccess) {
            sub_kernel<<<vg, 256, 0, st>>>(g->rhs, g->Mx, n, g->r);
            launched(c);
        }
        dot_dev(c, g->rhs, g->rhs, g->slot, true);
        dot_dev(c, g->r, g->r, g->slot + 1, true);
        if(c.e == cudaSuccess) {
            gm_solve_begin_kernel<<<1, 1, 0, st>>>(d);
            launched(c);
        }
        if(c.e == cudaSuccess) c.e = add_while(st, d.outer, &outer_body);
        const int before = c.nl;
        if(c.e == cudaSuccess) c.e = cudaMemcpyAsync(rho, g->x, sizeof(double) * n, cudaMemcpyDeviceToDevice, st);
        if(c.e == cudaSuccess) c.e = spectral_r2c(s->eng, rho, s->rho_hat, st, &c.nl);
        finish_launches = c.nl - before;
    });
    if(e != cudaSuccess) return e;
    g->setup_launches = c.nl;
    (void) finish_launches;

    // a restart cycle: start, the Arnoldi loop, x update and the true residual
    Ctx co{s, g, mob, st};
    e = capture_into(outer_body, st, co, [&]() {
        gm_cycle_begin_kernel<<<vg, 256, 0, st>>>(d);
        launched(co);
        if(co.e == cudaSuccess) co.e = add_while(st, d.inner, &inner_body);
        if(co.e == cudaSuccess) {
            gm_xupdate_kernel<<<vg, 256, 0, st>>>(d);
            launched(co);
        }
        apply_M(co, g->x, g->Mx);
        if(co.e == cudaSuccess) {
            sub_kernel<<<vg, 256, 0, st>>>(g->rhs, g->Mx, n, g->r);
            launched(co);
        }
        dot_dev(co, g->r, g->r, g->slot + 1, true);
        if(co.e == cudaSuccess) {
            gm_cycle_end_kernel<<<1, 1, 0, st>>>(d);
            launched(co);
        }
    });
    if(e != cudaSuccess) return e;
    g->cycle_launches = co.nl;

    // an Arnoldi step: w = P^-1 A V_j, two Gram-Schmidt passes, norm and
    // scaling, the Givens update
    Ctx ca{s, g, mob, st};
    e = capture_into(inner_body, st, ca, [&]() {
        gm_take_column_kernel<<<vg, 256, 0, st>>>(d);
        launched(ca);
        apply_M(ca, g->vj, g->w);
        for(int pass = 0; pass < 2 && ca.e == cudaSuccess; pass++) {
            gm_dots_kernel<<<DOT_BLOCKS, RT, 0, st>>>(d);
            launched(ca);
            gm_orth_kernel<<<DOT_BLOCKS, RT, orth_smem, st>>>(d, pass);
            launched(ca);
        }
        if(ca.e == cudaSuccess) {
            gm_norm_scale_kernel<<<DOT_BLOCKS, RT, 0, st>>>(d);
            launched(ca);
        }
        if(ca.e == cudaSuccess) {
            gm_givens_kernel<<<1, 1, 0, st>>>(d);
            launched(ca);
        }
    });
    if(e != cudaSuccess) return e;
    g->arnoldi_launches = ca.nl;

    e = cudaGraphInstantiate(&g->exec, g->graph, 0);
    if(e != cudaSuccess) {
        g->exec = nullptr;
        return e;
    }
    g->graph_mob = mob;
    g->graph_rho = rho;
    return cudaSuccess;
}

}  // namespace

cudaError_t psmob_step_gmres(PsMob *s, const double *mob, double *rho, cudaStream_t st, int64_t *launches) {
    const long long n = s->bins * s->S;
    const int m = std::max(2, s->p.gmres_restart);
    if(!s->gm) {
        PsGmres *g = new PsGmres();
        g->m = m;
        g->n = n;
        const size_t vb = sizeof(double) * (size_t) n;
        const size_t arr = (size_t) (m + 2) + (size_t) m * (m + 1) + 2 * (size_t) m + (size_t) (m + 1) + (size_t) m;
        bool ok = cudaMalloc(&g->b, vb) == cudaSuccess && cudaMalloc(&g->x, vb) == cudaSuccess &&
                  cudaMalloc(&g->rhs, vb) == cudaSuccess && cudaMalloc(&g->Mx, vb) == cudaSuccess &&
                  cudaMalloc(&g->r, vb) == cudaSuccess && cudaMalloc(&g->w, vb) == cudaSuccess &&
                  cudaMalloc(&g->Av, vb) == cudaSuccess && cudaMalloc(&g->vj, vb) == cudaSuccess &&
                  cudaMalloc(&g->V, vb * (m + 1)) == cudaSuccess &&
                  cudaMalloc(&g->part, sizeof(double) * DOT_BLOCKS * (size_t) (m + 1)) == cudaSuccess &&
                  cudaMalloc(&g->part2, sizeof(double) * DOT_BLOCKS) == cudaSuccess &&
                  cudaMalloc(&g->slot, sizeof(double) * 2) == cudaSuccess &&
                  cudaMalloc(&g->arr, sizeof(double) * arr) == cudaSuccess &&
                  cudaMalloc(&g->state, sizeof(GmState)) == cudaSuccess &&
                  cudaMalloc(&g->hat, sizeof(double2) * (size_t) s->hall) == cudaSuccess;
        s->gm = g;
        if(!ok) {
            cudaGetLastError();
            psmob_gmres_release(s);
            return cudaErrorMemoryAllocation;
        }
        cudaError_t e = cudaMemsetAsync(g->state, 0, sizeof(GmState), st);
        if(e == cudaSuccess) e = cudaMemsetAsync(g->arr, 0, sizeof(double) * arr, st);
        if(e != cudaSuccess) return e;
    }
    PsGmres *g = s->gm;
    if(!g->exec || g->graph_mob != mob || g->graph_rho != rho) {
        cudaError_t e = build_solve_graph(s, mob, rho, st);
        if(e != cudaSuccess) return e;
    }
    cudaError_t e = cudaGraphLaunch(g->exec, st);
    *launches += g->setup_launches;
    return e;
}

}  // namespace chgb
