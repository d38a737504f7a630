// spectral.cu — the `pseudospectral` semi-implicit step, FP64, own FFT.
//
// Reference: src/integrators/PseudospectralCPU.cpp:13-136 (FFTW r2c/c2r,
// per-mode update) and its CUDA mirror src/CUDA/integrators/PseudospectralCUDA.cu
// (single-precision cuFFT for f'; not followed).
//
// State.  The master copy is the half spectrum psi_t = rho_hat / N^dims in the
// reference's layout [species][n0]..[n_{d-2}][N/2+1] (the last, fastest axis x
// halved, as FFTW's r2c).  Storing it pre-divided by N^dims makes the inverse
// transform produce rho directly, so the per-mode update of
// PseudospectralCPU.cpp:119-131 folds to
//     psi_t' = alpha * psi_t - beta * F[f'(rho)],
//     alpha = (1 + c S) / denom,  beta = c * dealias / denom / N^dims,
//     c = dt M q^2,  denom = 1 + dt M (S q^2 + 2 k q^4),
// with q^2 and the dealiasing mask tabulated on the host exactly as the
// reference computes them (their 1D/2D/3D formulas differ in rounding and in
// `<` vs `<=` at the cut).
//
// One time step is:
//   ROW  (x, contiguous rows): half spectrum row -> c2r -> rho row -> f'(rho)
//        -> r2c -> half spectrum row, all in shared memory (one kernel);
//   COL  (each slower axis): complex FFT along the axis of column bundles in
//        shared memory; on the slowest axis the forward transform, the per-mode
//        update and the inverse transform run in one kernel.
// 2D: ROW + COL_y(fwd, update, inv).  3D: ROW + COL_y(fwd) + COL_z(fwd, update,
// inv) + COL_y(inv).  1D: ROW + an elementwise update.
// The real r2c/c2r of a row of L = 2M values is a complex FFT of length M on
// the even/odd packing z[n] = x[2n] + i x[2n+1] plus one pre/post-processing
// sweep.  FFT passes are Stockham autosort, radix 4 (one radix-2 pass first
// when log2 of the length is odd), twiddles from one exactly symmetric
// table W[q] = exp(-2 pi i q / N).  The transforms run in 64-bit block
// floating point (bfp.cuh): each line is converted to fixed point with one
// exponent, transformed with integer arithmetic and converted back; the state,
// f' and the mode update stay FP64.
#include <cmath>
#include <vector>

#include "bfp.cuh"
#include "bounds.cuh"
#include "kernels.h"
#include "spectral.h"

namespace chgb {

#ifdef CHGB_BOUNDS_CHECK
cudaError_t bc_read_spectral(unsigned long long *first) { return bc_read_tu(first); }
#endif

namespace {

// ---------------------------------------------------------------------------
// Fixed-point (block floating point) Stockham FFT of one line, bfp.cuh.
// ---------------------------------------------------------------------------
constexpr int FX_NAN_SCALE = 1 << 30;   // output scale of a line that held a NaN or an infinity

__device__ __forceinline__ double2 fx_out(fx2 v, int sh) {
    if(sh == FX_NAN_SCALE) return make_double2(__longlong_as_double(0x7FF8000000000000ll),
                                               __longlong_as_double(0x7FF8000000000000ll));
    return fx_store(v, sh);
}

// One pass of fx_fft_line: radix 2 (R == 2, the first pass of an odd log2 L)
// or radix 4, Ns the length of the sub-transforms already formed.  in_d /
// out_d: the pass reads FP64 values (scaled by 2^sh_in into fixed point) /
// writes FP64 values (scaled back by 2^-sh_out) instead of fixed point; the
// template flags IN_D / OUT_D say whether that conversion code is compiled at
// all.  One body serves the first, middle and last passes of a line: with
// small boxes every SM runs a kernel's code about once, and instruction
// fetch, not arithmetic, is what a longer unrolled body costs.  DIR = -1
// forward (twiddles w), +1 inverse (conj w).
template <int DIR, int R, bool IN_D, bool OUT_D>
__device__ __forceinline__ void fx_pass(const void *src_, void *dst_, int L, int Ns, int lane, int tpl,
                                        const int4 *__restrict__ tw, int wstep, int sh_in, int sh_out, bool in_d,
                                        bool out_d) {
    const double2 *srcd = static_cast<const double2 *>(src_);
    const fx2 *srcf = static_cast<const fx2 *>(src_);
    double2 *dstd = static_cast<double2 *>(dst_);
    fx2 *dstf = static_cast<fx2 *>(dst_);
    if(R == 2) {
        for(int j = lane; j < L / 2; j += tpl) {
            if(!CHGB_BC(104, 2 * j + 1, L)) continue;
            fx2 v0, v1;
            if(IN_D && in_d) {
                v0 = fx_load(srcd[j], sh_in);
                v1 = fx_load(srcd[j + L / 2], sh_in);
            }
            else {
                v0 = srcf[j];
                v1 = srcf[j + L / 2];
            }
            const fx2 r0 = fx_add(v0, v1), r1 = fx_sub(v0, v1);
            if(OUT_D && out_d) {
                dstd[2 * j] = fx_out(r0, sh_out);
                dstd[2 * j + 1] = fx_out(r1, sh_out);
            }
            else {
                dstf[2 * j] = r0;
                dstf[2 * j + 1] = r1;
            }
        }
        return;
    }
    const int Q = L / 4;
    const int tstride = (Q / Ns) * wstep;
    for(int j = lane; j < Q; j += tpl) {
        const int k = j & (Ns - 1);
        if(!CHGB_BC(105, j + 3 * Q, L) || !CHGB_BC(105, (j - k) * 4 + k + 3 * Ns, L)) continue;
        fx2 v0, v1, v2, v3;
        if(IN_D && in_d) {
            v0 = fx_load(srcd[j], sh_in);
            v1 = fx_load(srcd[j + Q], sh_in);
            v2 = fx_load(srcd[j + 2 * Q], sh_in);
            v3 = fx_load(srcd[j + 3 * Q], sh_in);
        }
        else {
            v0 = srcf[j];
            v1 = srcf[j + Q];
            v2 = srcf[j + 2 * Q];
            v3 = srcf[j + 3 * Q];
        }
        fx2 s0, d0, s1, d1;
        if(Ns > 1) {
            const int m = k * tstride;
            const fx2 t2 = fx_cmul<(DIR > 0)>(v2, tw[2 * m]);
            s0 = fx_add(v0, t2);
            d0 = fx_sub(v0, t2);
            const fx2 t1 = fx_cmul<(DIR > 0)>(v1, tw[m]);
            const fx2 t3 = fx_cmul<(DIR > 0)>(v3, tw[3 * m]);
            s1 = fx_add(t1, t3);
            d1 = fx_sub(t1, t3);
        }
        else {
            s0 = fx_add(v0, v2);
            d0 = fx_sub(v0, v2);
            s1 = fx_add(v1, v3);
            d1 = fx_sub(v1, v3);
        }
        const fx2 mi_d1 = fx2{d1.y, -d1.x};   // -i * d1
        const int o = (j - k) * 4 + k;
        const fx2 r0 = fx_add(s0, s1), r2 = fx_sub(s0, s1);
        const fx2 r1 = DIR < 0 ? fx_add(d0, mi_d1) : fx_sub(d0, mi_d1);
        const fx2 r3 = DIR < 0 ? fx_sub(d0, mi_d1) : fx_add(d0, mi_d1);
        if(OUT_D && out_d) {
            dstd[o] = fx_out(r0, sh_out);
            dstd[o + Ns] = fx_out(r1, sh_out);
            dstd[o + 2 * Ns] = fx_out(r2, sh_out);
            dstd[o + 3 * Ns] = fx_out(r3, sh_out);
        }
        else {
            dstf[o] = r0;
            dstf[o + Ns] = r1;
            dstf[o + 2 * Ns] = r2;
            dstf[o + 3 * Ns] = r3;
        }
    }
}

// Fixed-point Stockham FFT of line li (length L >= 2, 16-byte elements, LS
// elements between lines) in the shared buffers a/b, the counterpart of
// fft_line.  The input is FP64 (IN_D, scaled by 2^sh_in) or fixed point; the
// output FP64 (OUT_D, scaled by 2^-sh_out; FX_NAN_SCALE writes NaN) or fixed
// point.  Every thread of the block must call it (it synchronises after each
// pass).  Returns the buffer holding the result.
template <int DIR, bool IN_D, bool OUT_D>
__device__ void *fx_fft_line(void *a, void *b, int L, int log2L, int LS, int li, int lane, int tpl, bool active,
                             const int4 *__restrict__ tw, int wstep, int sh_in, int sh_out) {
    char *in = static_cast<char *>(a), *out = static_cast<char *>(b);
    const size_t off = (size_t) li * LS * 16;
    const int passes = (log2L & 1) + log2L / 2;
    int p = 0, Ns = 1;
    if(log2L & 1) {
        if(active)
            fx_pass<DIR, 2, IN_D, OUT_D>(in + off, out + off, L, 1, lane, tpl, tw, wstep, sh_in, sh_out, true,
                                         passes == 1);
        char *t = in;
        in = out;
        out = t;
        Ns = 2;
        p = 1;
        __syncthreads();
    }
    for(; Ns < L; Ns *= 4, p++) {
        if(active)
            fx_pass<DIR, 4, IN_D, OUT_D>(in + off, out + off, L, Ns, lane, tpl, tw, wstep, sh_in, sh_out, p == 0,
                                         p == passes - 1);
        char *t = in;
        in = out;
        out = t;
        __syncthreads();
    }
    return in;
}

// Largest exponent field over elements [0, n) of line li (lines LS apart) of
// an FP64 buffer, reduced over the line's threads into sm_e[li] (see
// fx_line_max); the caller synchronises before reading it.
__device__ __forceinline__ void fx_line_exponent(const double2 *buf, int n, int LS, int li, int lane, int tpl,
                                                 bool active, int *sm_e) {
    int e = 0;
    if(active) {
        const double2 *src = buf + (size_t) li * LS;
        for(int j = lane; j < n; j += tpl) {
            const double2 v = src[j];
            e = max(e, max(fx_expo(v.x), fx_expo(v.y)));
        }
    }
    fx_line_max(e, tpl, li, lane, active, sm_e);
}

enum { ROW_IN_REAL = 0, ROW_IN_HAT = 1 };
// Flux stage of the variable-mobility step between a row's c2r and r2c:
// g <- (M - M0[s]) (g / N^d) (FLUX_DM) or M (g / N^d) (FLUX_M).
enum { FLUX_NONE = 0, FLUX_DM = 1, FLUX_M = 2 };

// ROW kernel: `lines` = rows_per_cta * S lines per CTA, line li -> species
// li % S of row blockIdx.x * rows_per_cta + li / S.  Half-spectrum rows live at
// work[s * hat + row * H]; real rows at real[s * bins + row * N].  The shared
// memory holds two buffers of lines * (M + 1) 16-byte elements, then 2 * lines
// ints for the lines' exponents.  The transforms run in fixed point
// (fx_fft_line); f' and the stored values are FP64.  Headroom: the c2r
// pre-processing and the r2c post-processing each grow magnitudes by up to 4,
// so both transforms take G = log2 M + 3.  FLUX: the mobility stage applied to
// the real row between the two transforms (mob, M0 as psm_flux_kernel's).
template <int KIND, int IN, bool FPRIME, bool WRITE_REAL, bool R2C, int FLUX = FLUX_NONE>
__device__ __forceinline__ void row_body(double2 *__restrict__ work, const double *__restrict__ real_in,
                                         double *__restrict__ real_out, int N, int M, int log2M, int rows_per_cta,
                                         int tpl, long long bins, long long hat, const int4 *__restrict__ twf,
                                         const ModelDev &m, long long row0, double2 *sm2,
                                         const double *__restrict__ mob = nullptr,
                                         const double *__restrict__ M0 = nullptr) {
    constexpr int S = NSpecies<KIND>::value;
    const int LS = M + 1;
    const int lines = rows_per_cta * S;
    double2 *A = sm2;
    double2 *B = sm2 + lines * LS;
    int *sm_e = reinterpret_cast<int *>(sm2 + 2 * lines * LS);   // [0, lines): c2r input, [lines, 2 lines): r2c input
    const int li = threadIdx.x / tpl, lane = threadIdx.x - li * tpl;
    const bool active = li < lines;
    const int s = active ? li % S : 0;
    const long long row = row0 + (active ? li / S : 0);
    const int H = M + 1;
    const int G = log2M + 3;
    if(active && lane == 0) {
        sm_e[li] = 0;
        sm_e[lines + li] = 0;
    }
    double2 *cur;

    if(IN == ROW_IN_REAL) {
        if(active && CHGB_BC(106, row * N + N - 1, bins)) {
            const double2 *src = reinterpret_cast<const double2 *>(real_in + s * bins + row * N);
            for(int n = lane; n < M; n += tpl) A[li * LS + n] = src[n];
        }
        __syncthreads();
        cur = A;
    }
    else {
        int e = 0;
        if(active && CHGB_BC(107, row * H + H - 1, hat)) {
            // c2r of a half spectrum: the imaginary parts of the k = 0 and k = M
            // bins do not reach the real row (FFTW's c2r contract; they are
            // not round-off zeros when the spectrum is i k times a field)
            const double2 *src = work + s * hat + row * H;
            for(int k = lane; k < H; k += tpl) {
                double2 v = src[k];
                if(k == 0 || k == M) v.y = 0.0;
                B[li * LS + k] = v;
                e = max(e, max(fx_expo(v.x), fx_expo(v.y)));
            }
        }
        __syncthreads();
        fx_line_max(e, tpl, li, lane, active, sm_e);
        __syncthreads();
        const int emax = active ? sm_e[li] : 0;
        const int sh = fx_scale(emax, G);
        // c2r pre-processing in fixed point:
        //   Z[k] = (X[k] + conj X[M-k]) + i conj(w^k) (X[k] - conj X[M-k])
        if(active) {
            const double2 *X = B + li * LS;
            fx2 *Z = reinterpret_cast<fx2 *>(A + li * LS);
            for(int k = lane; k < M; k += tpl) {
                const fx2 xk = fx_load(X[k], sh);
                fx2 xc = fx_load(X[M - k], sh);
                xc.y = -xc.y;
                const fx2 e2 = fx_add(xk, xc);
                const fx2 t = fx_cmul<true>(fx_sub(xk, xc), twf[k]);
                Z[k] = fx2{e2.x - t.y, e2.y + t.x};
            }
        }
        __syncthreads();
        cur = static_cast<double2 *>(
            fx_fft_line<+1, false, true>(A, B, M, log2M, LS, li, lane, tpl, active, twf, 2, 0,
                                         emax == 2047 ? FX_NAN_SCALE : sh));
    }
    double2 *other = (cur == A) ? B : A;

    if(WRITE_REAL && active && CHGB_BC(106, row * N + N - 1, bins)) {
        double2 *dst = reinterpret_cast<double2 *>(real_out + s * bins + row * N);
        for(int n = lane; n < M; n += tpl) dst[n] = cur[li * LS + n];
    }
    if(FLUX != FLUX_NONE) {
        if(active) {
            const double2 *mrow = reinterpret_cast<const double2 *>(mob + s * bins + row * N);
            const double inv_bins = 1.0 / (double) bins;   // exact: N^d is a power of two
            const double m0 = (FLUX == FLUX_DM) ? M0[s] : 0.0;
            for(int n = lane; n < M; n += tpl) {
                double2 v = cur[li * LS + n];
                const double2 mm = mrow[n];
                const double g0 = v.x * inv_bins, g1 = v.y * inv_bins;
                if(FLUX == FLUX_DM) {
                    v.x = (mm.x - m0) * g0;
                    v.y = (mm.y - m0) * g1;
                }
                else {
                    v.x = mm.x * g0;
                    v.y = mm.y * g1;
                }
                cur[li * LS + n] = v;
            }
        }
        __syncthreads();
    }
    if(FPRIME) {
        // f'(rho) of the row's cells; species-0 lines do the work for all species
        if(active && s == 0) {
            for(int n = lane; n < M; n += tpl) {
                double r0[S], r1[S], d0[S], d1[S];
#pragma unroll
                for(int q = 0; q < S; q++) {
                    double2 v = cur[(li + q) * LS + n];
                    r0[q] = v.x;
                    r1[q] = v.y;
                }
                der_bulk<KIND>(m, r0, d0);
                der_bulk<KIND>(m, r1, d1);
#pragma unroll
                for(int q = 0; q < S; q++) cur[(li + q) * LS + n] = make_double2(d0[q], d1[q]);
            }
        }
        __syncthreads();
    }
    if(R2C) {
        fx_line_exponent(cur, M, LS, li, lane, tpl, active, sm_e + lines);
        __syncthreads();
        const int emax = active ? sm_e[lines + li] : 0;
        const int sh = fx_scale(emax, G);
        const fx2 *Z = static_cast<const fx2 *>(
                           fx_fft_line<-1, true, false>(cur, other, M, log2M, LS, li, lane, tpl, active, twf, 2, sh, 0)) +
                       li * LS;
        // post-processing: X[k] = (a + w^k (-i b)) / 2 with a = Zk + conj Z_{M-k},
        // b = Zk - conj Z_{M-k}; the halving is folded into the output scale
        if(active && CHGB_BC(107, row * H + H - 1, hat)) {
            const int sh_out = emax == 2047 ? FX_NAN_SCALE : sh + 1;
            double2 *dst = work + s * hat + row * H;
            for(int k = lane; k <= M; k += tpl) {
                const fx2 zk = Z[k == M ? 0 : k];
                fx2 zc = Z[k == 0 ? 0 : M - k];
                zc.y = -zc.y;
                const fx2 a = fx_add(zk, zc), bb = fx_sub(zk, zc);
                const fx2 t = fx_cmul<false>(fx2{bb.y, -bb.x}, twf[k]);
                double2 xk = fx_out(fx_add(a, t), sh_out);
                if(k == 0 || k == M) xk.y = 0.0;
                dst[k] = xk;
            }
        }
    }
}

template <int KIND, int IN, bool FPRIME, bool WRITE_REAL, bool R2C, int FLUX = FLUX_NONE>
__global__ void __launch_bounds__(1024) row_kernel(double2 *__restrict__ work, const double *__restrict__ real_in,
                                                   double *__restrict__ real_out, int N, int M, int log2M,
                                                   int rows_per_cta, int tpl, long long bins, long long hat,
                                                   const int4 *__restrict__ twf, ModelDev m,
                                                   const double *__restrict__ mob, const double *__restrict__ M0) {
    extern __shared__ double2 sm2[];
    row_body<KIND, IN, FPRIME, WRITE_REAL, R2C, FLUX>(work, real_in, real_out, N, M, log2M, rows_per_cta, tpl, bins,
                                                      hat, twf, m, (long long) blockIdx.x * rows_per_cta, sm2, mob, M0);
}

// Batched row pass of one time step: CTA b takes rows items[b].y.. of replica items[b].x.
template <int KIND>
__global__ void __launch_bounds__(256) row_batch_kernel(const PsBatchRep *__restrict__ reps,
                                                        const int2 *__restrict__ items) {
    extern __shared__ double2 sm2[];
    const int2 it = items[blockIdx.x];
    const PsBatchRep &r = reps[it.x];
    row_body<KIND, ROW_IN_HAT, true, false, true>(r.work, nullptr, nullptr, r.N, r.M, r.log2M, r.row_rpc, r.row_tpl,
                                                  r.bins, r.hat, r.twf, r.m, it.y, sm2);
}

enum { COL_FWD = 0, COL_INV = 1, COL_STEP = 2, COL_INIT = 3, COL_GRAD_INV = 4, COL_FWD_DIV = 5, COL_FWD_MU = 6,
       COL_UPD_INV = 7 };

// The pointwise stages of the variable-mobility step that ride on a column
// pass (src/integrators/PseudospectralMobilityCPU.cpp:249-306), each in the
// order of operations of the matching psmob.cu kernel, so either path gives
// the same bits.  All arrays share the half-spectrum layout (species-major);
// fields a mode does not use stay null.
//   COL_GRAD_INV (load):  D i k_d src                            (:258-263)
//   COL_FWD_DIV (store):  div (= if first, += otherwise) i k_d D f (:284-293)
//   COL_FWD_MU (store):   work = f, mu = D (f + two_k q2 rho_hat)  (:249-254)
//   COL_UPD_INV (load):   the semi-implicit update of rho_hat, inverse
//                         transform of rho_hat / N^d               (:296-306)
struct ColOps {
    const double *kd, *dealias, *q2, *M0;
    const double2 *src, *fder, *div_in;
    double2 *out, *rho;
    int use_dealias, first, with_div;
    double two_k, dt, Ssplit, k0, inv_bins;   // inv_bins = 1 / N^d, exact (a power of two)
};

// (column, position) of element e of a CTA's ncols lines stored position-major
// (e = pos * ncols + c): a mask and a shift when ncols is a power of two (every
// CTA but a ragged last one, lg = log2 ncols), integer division otherwise.
__device__ __forceinline__ void col_split(int e, int ncols, int lg, int &c, int &pos) {
    if(lg >= 0) {
        c = e & (ncols - 1);
        pos = e >> lg;
    }
    else {
        c = e % ncols;
        pos = e / ncols;
    }
}

__device__ __forceinline__ int col_log2(int ncols) { return (ncols & (ncols - 1)) == 0 ? __ffs(ncols) - 1 : -1; }

// COL pass: C lines (adjacent half-spectrum columns kx0..) of one species and
// one plane per CTA; element pos of line li at
//   off = species * hat + plane * plane_stride + (kx0 + li) + pos * elem_stride.
// The shared memory holds two buffers of C * L elements, then 2 * C ints for
// the lines' exponents.  Transforms in fixed point, G = log2 L + 1.
template <int MODE>
__device__ __forceinline__ void col_body(double2 *__restrict__ work, double2 *__restrict__ psi_hat,
                                         const double *__restrict__ alpha, const double *__restrict__ beta, int L,
                                         int log2L, int H, int C, int tpl, long long elem_stride,
                                         long long plane_stride, long long hat, const int4 *__restrict__ twf,
                                         int wstep, double scale, int kx0, long long plane, long long species,
                                         double2 *sm2, const ColOps &ops = ColOps()) {
    const int LS = L;
    double2 *A = sm2;
    double2 *B = sm2 + C * LS;
    int *sm_e = reinterpret_cast<int *>(sm2 + 2 * C * LS);
    const int li = threadIdx.x / tpl, lane = threadIdx.x - li * tpl;
    const long long base = species * hat + plane * plane_stride + kx0;
    const int ncols = min(C, H - kx0);
    const int lg = col_log2(ncols);
    const bool active = li < ncols;
    const int nthr = blockDim.x;
    const int G = log2L + 1;
    if(active && lane == 0) {
        sm_e[li] = 0;
        sm_e[C + li] = 0;
    }

    // coalesced load: consecutive threads take adjacent columns of one row
    for(int e = threadIdx.x; e < ncols * L; e += nthr) {
        int c, pos;
        col_split(e, ncols, lg, c, pos);
        const long long off = base + c + pos * elem_stride;
        if(!CHGB_BC(101, off - species * hat, hat) || !CHGB_BC(102, c * LS + pos, C * LS)) continue;
        double2 v;
        if(MODE == COL_GRAD_INV) {
            v = mul_ik(ops.kd[off], ops.src[off]);
            if(ops.use_dealias) {
                const double D = ops.dealias[off];
                v.x *= D;
                v.y *= D;
            }
        }
        else if(MODE == COL_UPD_INV) {
            const double k2 = ops.q2[off];
            const double k4 = k2 * k2;
            const double m0 = ops.M0[species];
            const double denom = 1.0 + ops.dt * m0 * (ops.Ssplit * k2 + 2.0 * ops.k0 * k4);
            const double cc = ops.dt * m0 * k2;
            const double2 r = ops.rho[off], f = ops.fder[off];
            double ar = r.x, ai = r.y;
            if(ops.with_div) {
                const double2 d = ops.div_in[off];
                ar = r.x + ops.dt * d.x;
                ai = r.y + ops.dt * d.y;
            }
            const double nr = (ar - cc * (f.x - ops.Ssplit * r.x)) / denom;
            const double ni = (ai - cc * (f.y - ops.Ssplit * r.y)) / denom;
            ops.rho[off] = make_double2(nr, ni);
            v = make_double2(nr * ops.inv_bins, ni * ops.inv_bins);
        }
        else {
            v = work[off];
        }
        A[c * LS + pos] = v;
    }
    __syncthreads();
    fx_line_exponent(A, L, LS, li, lane, tpl, active, sm_e);
    __syncthreads();
    int emax = active ? sm_e[li] : 0;
    int sh = fx_scale(emax, G);
    double2 *cur;
    if(MODE == COL_INV || MODE == COL_GRAD_INV || MODE == COL_UPD_INV) {
        cur = static_cast<double2 *>(fx_fft_line<+1, true, true>(A, B, L, log2L, LS, li, lane, tpl, active, twf,
                                                                 wstep, sh, emax == 2047 ? FX_NAN_SCALE : sh));
    }
    else {
        cur = static_cast<double2 *>(fx_fft_line<-1, true, true>(A, B, L, log2L, LS, li, lane, tpl, active, twf,
                                                                 wstep, sh, emax == 2047 ? FX_NAN_SCALE : sh));
    }
    if(MODE == COL_INIT) {
        for(int e = threadIdx.x; e < ncols * L; e += nthr) {
            int c, pos;
            col_split(e, ncols, lg, c, pos);
            if(!CHGB_BC(101, base + c + pos * elem_stride - species * hat, hat) || !CHGB_BC(102, c * LS + pos, C * LS))
                continue;
            double2 v = cur[c * LS + pos];
            psi_hat[base + c + pos * elem_stride] = make_double2(v.x * scale, v.y * scale);
        }
        return;
    }
    if(MODE == COL_STEP) {
        for(int e = threadIdx.x; e < ncols * L; e += nthr) {
            int c, pos;
            col_split(e, ncols, lg, c, pos);
            long long off = base + c + pos * elem_stride;
            if(!CHGB_BC(101, off - species * hat, hat) || !CHGB_BC(102, c * LS + pos, C * LS)) continue;
            double2 ph = psi_hat[off];
            double al = alpha[off], be = beta[off];
            double2 f = cur[c * LS + pos];
            double2 nv = make_double2(fma(al, ph.x, -be * f.x), fma(al, ph.y, -be * f.y));
            psi_hat[off] = nv;
            cur[c * LS + pos] = nv;
        }
        __syncthreads();
        fx_line_exponent(cur, L, LS, li, lane, tpl, active, sm_e + C);
        __syncthreads();
        emax = active ? sm_e[C + li] : 0;
        sh = fx_scale(emax, G);
        double2 *other = (cur == A) ? B : A;
        cur = static_cast<double2 *>(fx_fft_line<+1, true, true>(cur, other, L, log2L, LS, li, lane, tpl, active,
                                                                 twf, wstep, sh,
                                                                 emax == 2047 ? FX_NAN_SCALE : sh));
    }
    for(int e = threadIdx.x; e < ncols * L; e += nthr) {
        int c, pos;
        col_split(e, ncols, lg, c, pos);
        const long long off = base + c + pos * elem_stride;
        if(!CHGB_BC(101, off - species * hat, hat) || !CHGB_BC(102, c * LS + pos, C * LS)) continue;
        double2 f = cur[c * LS + pos];
        if(MODE == COL_FWD_DIV) {
            if(ops.use_dealias) {
                const double D = ops.dealias[off];
                f.x *= D;
                f.y *= D;
            }
            const double2 t = mul_ik(ops.kd[off], f);
            if(ops.first) {
                ops.out[off] = make_double2(0.0 + t.x, 0.0 + t.y);
            }
            else {
                const double2 d = ops.out[off];
                ops.out[off] = make_double2(d.x + t.x, d.y + t.y);
            }
        }
        else {
            work[off] = f;
            if(MODE == COL_FWD_MU) {
                const double t = ops.two_k * ops.q2[off];
                const double2 r = ops.rho[off];
                double2 v = make_double2(f.x + t * r.x, f.y + t * r.y);
                if(ops.use_dealias) {
                    const double D = ops.dealias[off];
                    v.x *= D;
                    v.y *= D;
                }
                ops.out[off] = v;
            }
        }
    }
}

template <int MODE>
__global__ void __launch_bounds__(1024) col_kernel(double2 *__restrict__ work, double2 *__restrict__ psi_hat,
                                                   const double *__restrict__ alpha, const double *__restrict__ beta,
                                                   int L, int log2L, int H, int C, int tpl, long long elem_stride,
                                                   long long plane_stride, long long hat,
                                                   const int4 *__restrict__ twf, int wstep, double scale, ColOps ops) {
    extern __shared__ double2 sm2[];
    col_body<MODE>(work, psi_hat, alpha, beta, L, log2L, H, C, tpl, elem_stride, plane_stride, hat, twf, wstep, scale,
                   blockIdx.x * C, blockIdx.y, blockIdx.z, sm2, ops);
}

// Batched 2D column pass (forward, update, inverse) of one time step:
// CTA b takes columns items[b].z.. of species items[b].y of replica items[b].x.
__global__ void __launch_bounds__(256) col_batch_kernel(const PsBatchRep *__restrict__ reps,
                                                        const int4 *__restrict__ items) {
    extern __shared__ double2 sm2[];
    const int4 it = items[blockIdx.x];
    const PsBatchRep &r = reps[it.x];
    col_body<COL_STEP>(r.work, r.psi_hat, r.alpha, r.beta, r.N, r.log2N, r.H, r.col_C, r.col_tpl, r.H, 0, r.hat, r.twf,
                       1, 0.0, it.z, 0, it.y, sm2);
}

// 1D: elementwise init (psi_t = F[rho] / N) or update on the half spectrum.
__global__ void update1d_kernel(double2 *__restrict__ work, double2 *__restrict__ psi_hat,
                                const double *__restrict__ alpha, const double *__restrict__ beta, long long n,
                                int init, double scale) {
    for(long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
        double2 f = work[i];
        if(init) {
            psi_hat[i] = make_double2(f.x * scale, f.y * scale);
        }
        else {
            double2 ph = psi_hat[i];
            double al = alpha[i], be = beta[i];
            double2 nv = make_double2(fma(al, ph.x, -be * f.x), fma(al, ph.y, -be * f.y));
            psi_hat[i] = nv;
            work[i] = nv;
        }
    }
}

int ilog2(int n) {
    int l = 0;
    while((1 << l) < n) l++;
    return l;
}

}  // namespace

struct SpectralState {
    chgb_params p;
    Geom g;
    ModelDev m;
    int H = 0;
    long long hat = 0;       // complex values per species
    double2 *psi_hat = nullptr, *work = nullptr;
    int4 *twf = nullptr;      // the twiddles in fixed point (bfp.cuh): limbs of round(w 2^61)
    double *alpha = nullptr, *beta = nullptr;
    const double *real_buf = nullptr;  // the handle's real-space density buffer
    bool real_valid = false;  // the real buffer holds the current rho
    bool hat_valid = false;   // work holds the x-half-spectrum rows of the current rho
    // launch shapes
    int row_rpc = 1, row_tpl = 1, row_threads = 1;
    size_t row_smem = 0;
    int col_C = 1, col_tpl = 1, col_threads = 1;
    size_t col_smem = 0;
};

// Wave-vector tables of src/integrators/PseudospectralCPU.cpp:32-86, folded
// into the update coefficients.
static void build_tables(const SpectralState &s, std::vector<double> &alpha, std::vector<double> &beta) {
    const int N = s.g.N, dims = s.g.dims, S = s.g.S;
    const double dx = s.p.dx, dt = s.p.dt, M = s.p.M, Ssplit = s.p.splitting_S;
    const double bins = (double) s.g.bins;
    std::vector<double> k2v(s.hat), mask(s.hat);
    double k_cut = N * M_PI / (N * dx) * 2.0 / 3.0;
    long long idx = 0;
    if(dims == 1) {
        for(int i = 0; i < s.H; i++, idx++) {
            double k = 2.0 * M_PI * i / (N * dx);
            mask[idx] = (k <= k_cut) ? 1.0 : 0.0;
            k2v[idx] = k * k;
        }
    }
    else if(dims == 2) {
        for(int kx_idx = 0; kx_idx < N; kx_idx++) {
            int kx = (kx_idx < N / 2) ? kx_idx : N - kx_idx;
            for(int ky = 0; ky < N / 2 + 1; ky++, idx++) {
                double k = 2.0 * M_PI * std::sqrt((double) (kx * kx + ky * ky)) / (N * dx);
                mask[idx] = (k < k_cut) ? 1.0 : 0.0;
                k2v[idx] = k * k;
            }
        }
    }
    else {
        for(int kx_idx = 0; kx_idx < N; kx_idx++) {
            int kx_i = (kx_idx < N / 2) ? kx_idx : (kx_idx - N);
            double kx = 2.0 * M_PI * kx_i / (N * dx);
            for(int ky_idx = 0; ky_idx < N; ky_idx++) {
                int ky_i = (ky_idx < N / 2) ? ky_idx : (ky_idx - N);
                double ky = 2.0 * M_PI * ky_i / (N * dx);
                for(int kz_idx = 0; kz_idx < N / 2 + 1; kz_idx++, idx++) {
                    double kz = 2.0 * M_PI * kz_idx / (N * dx);
                    double k2 = kx * kx + ky * ky + kz * kz;
                    double k = std::sqrt(k2);
                    mask[idx] = (k <= k_cut) ? 1.0 : 0.0;
                    k2v[idx] = k2;
                }
            }
        }
    }
    alpha.resize((size_t) S * s.hat);
    beta.resize((size_t) S * s.hat);
    for(int sp = 0; sp < S; sp++) {
        for(long long i = 0; i < s.hat; i++) {
            double k2 = k2v[i], k4 = k2 * k2;
            double denom = 1.0 + dt * M * (Ssplit * k2 + 2.0 * s.p.k[sp] * k4);
            double c = dt * M * k2;
            double dm = s.p.use_dealias ? mask[i] : 1.0;
            alpha[sp * s.hat + i] = (1.0 + c * Ssplit) / denom;
            beta[sp * s.hat + i] = c * dm / denom / bins;
        }
    }
}

// One fixed-point twiddle component: W = round(v 2^61) as limbs (W >> 31, W mod 2^31).
static void fx_limbs(long double v, int &hi, int &lo) {
    const long long W = llroundl(v * 2305843009213693952.0L);   // 2^61
    hi = (int) (W >> 31);
    lo = (int) (W & 0x7FFFFFFFll);
}

// W[q] = exp(-2 pi i q / N), q < N, in fixed point for the transforms of
// bfp.cuh: built from one octant in long double so that the table is exactly
// symmetric (W[N/4] = -i, W[N/2] = -1 exactly), then rounded to 2^-61.
static void build_twiddles(int N, std::vector<int4> &wf) {
    wf.resize(N);
    for(int q = 0; q < N; q++) {
        // reduce q to the first octant with exact symmetries
        long double c, s;
        int oct = (int) (((long long) q * 8) / N);
        int r = q - oct * (N / 8);
        auto cs = [&](long double num, long double &co, long double &si) {
            long double a = 2.0L * 3.141592653589793238462643383279502884L * num / (long double) N;
            co = cosl(a);
            si = sinl(a);
        };
        long double co, si;
        if(N < 8) {
            cs((long double) q, co, si);
            c = co;
            s = si;
            if(q * 4 == N) { c = 0; s = 1; }
            if(q * 2 == N) { c = -1; s = 0; }
            if(q * 4 == 3 * N) { c = 0; s = -1; }
        }
        else {
            int e = N / 8;
            // angle = (oct * e + r) * 2pi/N = oct * pi/4 + r * 2pi/N
            switch(oct) {
                case 0: cs(r, co, si); c = co; s = si; break;
                case 1: cs(e - r, co, si); c = si; s = co; break;       // pi/2 - t
                case 2: cs(r, co, si); c = -si; s = co; break;          // pi/2 + t
                case 3: cs(e - r, co, si); c = -co; s = si; break;      // pi - t
                case 4: cs(r, co, si); c = -co; s = -si; break;         // pi + t
                case 5: cs(e - r, co, si); c = -si; s = -co; break;     // 3pi/2 - t
                case 6: cs(r, co, si); c = si; s = -co; break;          // 3pi/2 + t
                default: cs(e - r, co, si); c = co; s = -si; break;     // 2pi - t
            }
        }
        int4 f;
        fx_limbs(c, f.x, f.y);
        fx_limbs(-s, f.z, f.w);
        wf[q] = f;
    }
}

static void tune_col_shape(SpectralState *s);

// Dynamic shared memory limit of every column-pass kernel.
static void set_col_smem(size_t smem) {
    for(const void *f : {(const void *) col_kernel<COL_FWD>, (const void *) col_kernel<COL_INV>,
                         (const void *) col_kernel<COL_STEP>, (const void *) col_kernel<COL_INIT>,
                         (const void *) col_kernel<COL_GRAD_INV>, (const void *) col_kernel<COL_FWD_DIV>,
                         (const void *) col_kernel<COL_FWD_MU>, (const void *) col_kernel<COL_UPD_INV>})
        cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
}

int spectral_create(const chgb_params &p, const Geom &g, const ModelDev &m, SpectralState **out, std::string &err) {
    *out = nullptr;
    if(g.N > 4096) {
        err = "pseudospectral supports N <= 4096";
        return CHGB_ERR_INVALID;
    }
    SpectralState *s = new SpectralState();
    s->p = p;
    s->g = g;
    s->m = m;
    s->H = g.N / 2 + 1;
    s->hat = s->H;
    for(int d = 1; d < g.dims; d++) s->hat *= g.N;
    size_t hat_bytes = sizeof(double2) * (size_t) s->hat * g.S;
    bool ok = cudaMalloc(&s->psi_hat, hat_bytes) == cudaSuccess && cudaMalloc(&s->work, hat_bytes) == cudaSuccess &&
              cudaMalloc(&s->alpha, sizeof(double) * (size_t) s->hat * g.S) == cudaSuccess &&
              cudaMalloc(&s->beta, sizeof(double) * (size_t) s->hat * g.S) == cudaSuccess &&
              cudaMalloc(&s->twf, sizeof(int4) * g.N) == cudaSuccess;
    if(!ok) {
        cudaGetLastError();
        spectral_destroy(s);
        err = "device allocation failed";
        return CHGB_ERR_ALLOC;
    }
    std::vector<double> a, b;
    build_tables(*s, a, b);
    std::vector<int4> wf;
    build_twiddles(g.N, wf);
    ok = cudaMemcpy(s->alpha, a.data(), sizeof(double) * a.size(), cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(s->beta, b.data(), sizeof(double) * b.size(), cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(s->twf, wf.data(), sizeof(int4) * wf.size(), cudaMemcpyHostToDevice) == cudaSuccess;
    if(!ok) {
        spectral_destroy(s);
        err = "table upload failed";
        return CHGB_ERR_CUDA;
    }
    // launch shapes
    const int M = g.N / 2;
    const long long rows = (long long) g.bins / g.N;
    s->row_tpl = std::max(1, std::min(M / 4, 256));
    // rows per CTA: up to 128 threads, but never below ~2 CTAs per SM -- the
    // FP64 pipe of each SM is the shared resource, so small boxes want their
    // few rows spread over as many SMs as possible (2D N=256: 256 one-warp
    // CTAs rather than 64 four-warp ones)
    constexpr long long kSpreadCtas = 2 * 152;
    s->row_rpc = 1;
    while(s->row_rpc * 2 * s->row_tpl * g.S <= 128 && s->row_rpc * 2 <= rows &&
          rows / (s->row_rpc * 2) >= kSpreadCtas)
        s->row_rpc *= 2;
    s->row_threads = s->row_rpc * g.S * s->row_tpl;
    s->row_smem = sizeof(double2) * 2 * (size_t) s->row_rpc * g.S * (M + 1) + sizeof(int) * 2 * s->row_rpc * g.S;
    const int L = g.N;
    s->col_tpl = std::max(1, std::min(L / 4, 256));
    // columns per CTA: the same rule (2D N=256: 129 CTAs of one column each)
    const long long col_lines = (long long) s->H * (g.dims == 3 ? g.N : 1) * g.S;
    s->col_C = 1;
    while(s->col_C * 2 * s->col_tpl <= 256 && s->col_C * 2 <= 8 && col_lines / (s->col_C * 2) >= kSpreadCtas)
        s->col_C *= 2;
    s->col_threads = s->col_C * s->col_tpl;
    s->col_smem = sizeof(double2) * 2 * (size_t) s->col_C * L + sizeof(int) * 2 * s->col_C;
    // shared-memory attributes, once
    auto setattr = [&](const void *f, size_t smem) {
        if(smem > 48 * 1024) cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
    };
#define SETROW(K)                                                                                   \
    setattr((const void *) row_kernel<K, ROW_IN_REAL, false, false, true>, s->row_smem);            \
    setattr((const void *) row_kernel<K, ROW_IN_REAL, true, false, true>, s->row_smem);             \
    setattr((const void *) row_kernel<K, ROW_IN_HAT, true, false, true>, s->row_smem);              \
    setattr((const void *) row_kernel<K, ROW_IN_HAT, false, true, false>, s->row_smem);             \
    setattr((const void *) row_kernel<K, ROW_IN_HAT, true, true, true>, s->row_smem);              \
    setattr((const void *) row_kernel<K, ROW_IN_HAT, false, false, true, FLUX_DM>, s->row_smem);    \
    setattr((const void *) row_kernel<K, ROW_IN_HAT, false, false, true, FLUX_M>, s->row_smem);
    SETROW(CHGB_MODEL_LANDAU)
    SETROW(CHGB_MODEL_SIMPLE_WERTHEIM)
    SETROW(CHGB_MODEL_SALEH)
#undef SETROW
    if(s->col_smem > 48 * 1024) set_col_smem(s->col_smem);
    cudaError_t e = cudaGetLastError();
    if(e != cudaSuccess) {
        spectral_destroy(s);
        err = std::string("kernel configuration: ") + cudaGetErrorString(e);
        return CHGB_ERR_CUDA;
    }
    tune_col_shape(s);
    *out = s;
    return CHGB_OK;
}

void spectral_destroy(SpectralState *s) {
    if(!s) return;
    if(s->psi_hat) cudaFree(s->psi_hat);
    if(s->work) cudaFree(s->work);
    if(s->alpha) cudaFree(s->alpha);
    if(s->beta) cudaFree(s->beta);
    if(s->twf) cudaFree(s->twf);
    delete s;
}

namespace {

template <int KIND, int IN, bool FPRIME, bool WRITE_REAL, bool R2C>
cudaError_t launch_row_kind(SpectralState *s, const double *real_in, double *real_out, cudaStream_t st) {
    const int M = s->g.N / 2;
    const long long rows = (long long) s->g.bins / s->g.N;
    dim3 grid((unsigned) (rows / s->row_rpc));
    row_kernel<KIND, IN, FPRIME, WRITE_REAL, R2C><<<grid, s->row_threads, s->row_smem, st>>>(
        s->work, real_in, real_out, s->g.N, M, ilog2(M), s->row_rpc, s->row_tpl, s->g.bins, s->hat, s->twf, s->m,
        nullptr, nullptr);
    return cudaGetLastError();
}

// Row pass of the variable-mobility flux: c2r of work's rows, the flux stage, r2c back into work.
template <int KIND, int FLUX>
cudaError_t launch_row_flux_kind(SpectralState *s, const double *mob, const double *M0, cudaStream_t st) {
    const int M = s->g.N / 2;
    const long long rows = (long long) s->g.bins / s->g.N;
    dim3 grid((unsigned) (rows / s->row_rpc));
    row_kernel<KIND, ROW_IN_HAT, false, false, true, FLUX><<<grid, s->row_threads, s->row_smem, st>>>(
        s->work, nullptr, nullptr, s->g.N, M, ilog2(M), s->row_rpc, s->row_tpl, s->g.bins, s->hat, s->twf, s->m, mob,
        M0);
    return cudaGetLastError();
}

template <int FLUX>
cudaError_t launch_row_flux(SpectralState *s, const double *mob, const double *M0, cudaStream_t st) {
    switch(s->m.kind) {
        case CHGB_MODEL_LANDAU: return launch_row_flux_kind<CHGB_MODEL_LANDAU, FLUX>(s, mob, M0, st);
        case CHGB_MODEL_SIMPLE_WERTHEIM: return launch_row_flux_kind<CHGB_MODEL_SIMPLE_WERTHEIM, FLUX>(s, mob, M0, st);
        default: return launch_row_flux_kind<CHGB_MODEL_SALEH, FLUX>(s, mob, M0, st);
    }
}

template <int IN, bool FPRIME, bool WRITE_REAL, bool R2C>
cudaError_t launch_row(SpectralState *s, const double *real_in, double *real_out, cudaStream_t st) {
    switch(s->m.kind) {
        case CHGB_MODEL_LANDAU:
            return launch_row_kind<CHGB_MODEL_LANDAU, IN, FPRIME, WRITE_REAL, R2C>(s, real_in, real_out, st);
        case CHGB_MODEL_SIMPLE_WERTHEIM:
            return launch_row_kind<CHGB_MODEL_SIMPLE_WERTHEIM, IN, FPRIME, WRITE_REAL, R2C>(s, real_in, real_out, st);
        default: return launch_row_kind<CHGB_MODEL_SALEH, IN, FPRIME, WRITE_REAL, R2C>(s, real_in, real_out, st);
    }
}

// axis: 1 = y, 2 = z (3D only).  planes/strides follow the [z][y][kx] layout.
template <int MODE>
cudaError_t launch_col(SpectralState *s, int axis, cudaStream_t st, const ColOps &ops = ColOps()) {
    const int N = s->g.N, H = s->H;
    long long elem_stride, plane_stride;
    int planes;
    if(s->g.dims == 2) {
        elem_stride = H;
        plane_stride = 0;
        planes = 1;
    }
    else if(axis == 1) {
        elem_stride = H;
        plane_stride = (long long) N * H;
        planes = N;
    }
    else {
        elem_stride = (long long) N * H;
        plane_stride = H;
        planes = N;
    }
    dim3 grid((unsigned) ((H + s->col_C - 1) / s->col_C), (unsigned) planes, (unsigned) s->g.S);
    col_kernel<MODE><<<grid, s->col_threads, s->col_smem, st>>>(s->work, s->psi_hat, s->alpha, s->beta, N, ilog2(N),
                                                               H, s->col_C, s->col_tpl, elem_stride, plane_stride,
                                                               s->hat, s->twf, 1, 1.0 / (double) s->g.bins, ops);
    return cudaGetLastError();
}

}  // namespace

// Columns per CTA of the column passes, timed at create.  Adjacent columns in
// one CTA use whole 32-byte sectors of the strided column loads, while fewer,
// larger CTAs spread the lines over fewer SMs; which wins depends on the box
// (measured on GB300: 2 for 2D N=1024 and 3D N=128, 1 for 2D N=256 and
// N=2048).  So boxes of 2^18 cells and more time one column step with 1, 2
// and 4 columns per CTA (those that fit 1024 threads and the shared memory) on
// a state filled with noise, and keep the fastest.  Every shape gives the same
// bits: a line's transform does not depend on its CTA.  The state is zeroed
// afterwards (an upload sets it).
static void tune_col_shape(SpectralState *s) {
    if(s->g.dims < 2 || (long long) s->g.bins < (1ll << 18)) return;
    cudaStream_t st = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    if(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
       cudaEventCreate(&ev0) != cudaSuccess || cudaEventCreate(&ev1) != cudaSuccess) {
        cudaGetLastError();
        if(ev0) cudaEventDestroy(ev0);
        if(st) cudaStreamDestroy(st);
        return;
    }
    const int L = s->g.N, axis = s->g.dims - 1;
    const long long nd = s->hat * s->g.S * 2;   // doubles of psi_hat / work
    const int C0 = s->col_C, T0 = s->col_threads;
    const size_t M0 = s->col_smem;
    int bestC = C0, bestT = T0;
    size_t bestM = M0;
    float best = 0.0f;
    bool ok = launch_fill_noise(reinterpret_cast<double *>(s->psi_hat), 0.0, 1e-2, nd, st) == cudaSuccess &&
              launch_fill_noise(reinterpret_cast<double *>(s->work), 0.0, 1e-2, nd, st) == cudaSuccess;
    for(int C : {1, 2, 4}) {
        if(!ok) break;
        const int threads = C * s->col_tpl;
        const size_t smem = sizeof(double2) * 2 * (size_t) C * L + sizeof(int) * 2 * C;
        if(threads > 1024 || smem > 227 * 1024) continue;
        if(smem > 48 * 1024 &&
           cudaFuncSetAttribute(col_kernel<COL_STEP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem) !=
               cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        s->col_C = C;
        s->col_threads = threads;
        s->col_smem = smem;
        cudaError_t e = launch_col<COL_STEP>(s, axis, st);   // warm-up
        if(e == cudaSuccess) e = cudaEventRecord(ev0, st);
        for(int r = 0; r < 5 && e == cudaSuccess; r++) e = launch_col<COL_STEP>(s, axis, st);
        if(e == cudaSuccess) e = cudaEventRecord(ev1, st);
        if(e == cudaSuccess) e = cudaEventSynchronize(ev1);
        float ms = 0.0f;
        if(e == cudaSuccess) e = cudaEventElapsedTime(&ms, ev0, ev1);
        if(e != cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        if(best == 0.0f || ms < best) {
            best = ms;
            bestC = C;
            bestT = threads;
            bestM = smem;
        }
    }
    s->col_C = bestC;
    s->col_threads = bestT;
    s->col_smem = bestM;
    if(bestM > 48 * 1024) set_col_smem(bestM);
    cudaMemsetAsync(s->psi_hat, 0, sizeof(double) * nd, st);
    cudaMemsetAsync(s->work, 0, sizeof(double) * nd, st);
    cudaStreamSynchronize(st);
    cudaGetLastError();
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    cudaStreamDestroy(st);
}

namespace {

cudaError_t launch_update1d(SpectralState *s, int init, cudaStream_t st) {
    long long n = s->hat * s->g.S;
    int grid = (int) std::min<long long>((n + 255) / 256, 152 * 8);
    update1d_kernel<<<grid, 256, 0, st>>>(s->work, s->psi_hat, s->alpha, s->beta, n, init, 1.0 / (double) s->g.bins);
    return cudaGetLastError();
}

}  // namespace

int spectral_set_rho(SpectralState *s, const double *d_rho, cudaStream_t st, int64_t *launches, std::string &err) {
    s->real_buf = d_rho;
    cudaError_t e = launch_row<ROW_IN_REAL, false, false, true>(s, d_rho, nullptr, st);
    int n = 1;
    if(e == cudaSuccess) {
        if(s->g.dims == 1) {
            e = launch_update1d(s, 1, st);
            n++;
        }
        else if(s->g.dims == 2) {
            e = launch_col<COL_INIT>(s, 1, st);
            n++;
        }
        else {
            e = launch_col<COL_FWD>(s, 1, st);
            if(e == cudaSuccess) e = launch_col<COL_INIT>(s, 2, st);
            n += 2;
        }
    }
    *launches += n;
    if(e != cudaSuccess) {
        err = std::string("pseudospectral init: ") + cudaGetErrorString(e);
        return CHGB_ERR_CUDA;
    }
    s->real_valid = true;
    s->hat_valid = false;
    return CHGB_OK;
}

int spectral_step(SpectralState *s, int64_t nsteps, cudaStream_t st, int64_t *launches, std::string &err) {
    // The real buffer is only an input of the first step after an upload.
    for(int64_t t = 0; t < nsteps; t++) {
        cudaError_t e;
        if(s->hat_valid) e = launch_row<ROW_IN_HAT, true, false, true>(s, nullptr, nullptr, st);
        else e = launch_row<ROW_IN_REAL, true, false, true>(s, s->real_buf, nullptr, st);
        int n = 1;
        if(e == cudaSuccess) {
            if(s->g.dims == 1) {
                e = launch_update1d(s, 0, st);
                n++;
            }
            else if(s->g.dims == 2) {
                e = launch_col<COL_STEP>(s, 1, st);
                n++;
            }
            else {
                e = launch_col<COL_FWD>(s, 1, st);
                if(e == cudaSuccess) e = launch_col<COL_STEP>(s, 2, st);
                if(e == cudaSuccess) e = launch_col<COL_INV>(s, 1, st);
                n += 3;
            }
        }
        *launches += n;
        if(e != cudaSuccess) {
            err = std::string("pseudospectral step: ") + cudaGetErrorString(e);
            return CHGB_ERR_CUDA;
        }
        s->hat_valid = true;
        s->real_valid = false;
    }
    return CHGB_OK;
}

int spectral_real(SpectralState *s, double *d_rho, cudaStream_t st, int64_t *launches, std::string &err) {
    if(s->real_valid) return CHGB_OK;
    cudaError_t e = launch_row<ROW_IN_HAT, false, true, false>(s, nullptr, d_rho, st);
    *launches += 1;
    if(e != cudaSuccess) {
        err = std::string("pseudospectral real field: ") + cudaGetErrorString(e);
        return CHGB_ERR_CUDA;
    }
    s->real_valid = true;
    return CHGB_OK;
}

}  // namespace chgb

// ---------------------------------------------------------------------------
// batched 2D steps
// ---------------------------------------------------------------------------
namespace chgb {

bool spectral_batchable(const SpectralState *s) { return s->g.dims == 2 && s->g.N >= 8 && s->g.N <= 1024; }

bool spectral_hat_valid(const SpectralState *s) { return s->hat_valid; }

void spectral_mark_stepped(SpectralState *s) {
    s->hat_valid = true;
    s->real_valid = false;
}

void spectral_batch_rep(const SpectralState *s, PsBatchRep *r, size_t *row_smem, size_t *col_smem) {
    const int N = s->g.N, M = N / 2, S = s->g.S;
    r->work = s->work;
    r->psi_hat = s->psi_hat;
    r->alpha = s->alpha;
    r->beta = s->beta;
    r->twf = s->twf;
    r->m = s->m;
    r->N = N;
    r->M = M;
    r->log2M = ilog2(M);
    r->log2N = ilog2(N);
    r->H = s->H;
    r->bins = s->g.bins;
    r->hat = s->hat;
    r->row_tpl = std::max(1, std::min(M / 4, 64));
    r->row_rpc = 1;
    while(r->row_rpc * 2 * r->row_tpl * S <= PS_BATCH_THREADS && r->row_rpc * 2 <= N) r->row_rpc *= 2;
    r->col_tpl = std::max(1, std::min(N / 4, 64));
    r->col_C = std::max(1, std::min(PS_BATCH_THREADS / r->col_tpl, 16));
    *row_smem = sizeof(double2) * 2 * (size_t) r->row_rpc * S * (M + 1) + sizeof(int) * 2 * r->row_rpc * S;
    *col_smem = sizeof(double2) * 2 * (size_t) r->col_C * N + sizeof(int) * 2 * r->col_C;
}

namespace {
template <int KIND>
cudaError_t configure_kind(size_t row_smem, size_t col_smem) {
    cudaError_t e = cudaSuccess;
    if(row_smem > 48 * 1024)
        e = cudaFuncSetAttribute(row_batch_kernel<KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) row_smem);
    if(e == cudaSuccess && col_smem > 48 * 1024)
        e = cudaFuncSetAttribute(col_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) col_smem);
    return e;
}
}  // namespace

cudaError_t configure_ps2d_batch(int kind, size_t row_smem, size_t col_smem) {
    switch(kind) {
        case CHGB_MODEL_LANDAU: return configure_kind<CHGB_MODEL_LANDAU>(row_smem, col_smem);
        case CHGB_MODEL_SIMPLE_WERTHEIM: return configure_kind<CHGB_MODEL_SIMPLE_WERTHEIM>(row_smem, col_smem);
        default: return configure_kind<CHGB_MODEL_SALEH>(row_smem, col_smem);
    }
}

cudaError_t launch_ps2d_batch(int kind, const PsBatchRep *reps, const int2 *row_items, int nrow, const int4 *col_items,
                              int ncol, size_t row_smem, size_t col_smem, cudaStream_t st) {
    if(nrow > 0) {
        switch(kind) {
            case CHGB_MODEL_LANDAU:
                row_batch_kernel<CHGB_MODEL_LANDAU><<<nrow, PS_BATCH_THREADS, row_smem, st>>>(reps, row_items);
                break;
            case CHGB_MODEL_SIMPLE_WERTHEIM:
                row_batch_kernel<CHGB_MODEL_SIMPLE_WERTHEIM><<<nrow, PS_BATCH_THREADS, row_smem, st>>>(reps, row_items);
                break;
            default: row_batch_kernel<CHGB_MODEL_SALEH><<<nrow, PS_BATCH_THREADS, row_smem, st>>>(reps, row_items); break;
        }
        cudaError_t e = cudaGetLastError();
        if(e != cudaSuccess) return e;
    }
    if(ncol > 0) col_batch_kernel<<<ncol, PS_BATCH_THREADS, col_smem, st>>>(reps, col_items);
    return cudaGetLastError();
}

}  // namespace chgb

namespace chgb {
const double2 *spectral_psi_hat(const SpectralState *s, int species) { return s->psi_hat + (size_t) species * s->hat; }
}  // namespace chgb

// ---------------------------------------------------------------------------
// Adjoint of the 2D Landau pseudospectral step (backward pass of chgb_adjoint_*)
//
// Forward, in real space: psi' = A psi - B f'(psi), A = C2R diag(alpha) R2C / N^2,
// B = C2R diag(beta) R2C (both symmetric).  Adjoint, kept in Fourier space
// (lam_hat = R2C(lam)):
//     lam_hat_n = alpha lam_hat_{n+1} - R2C( f''(psi_n) * C2R(beta lam_hat_{n+1}) ),
// the same two-kernel structure as the forward step, with the same
// fixed-point transforms.  Parameter gradients,
// with <u, C2R(X)> = sum_full X_k conj(R2C(u)_k):
//   dL/deps += <B lam_{n+1}, psi_n>                          (row pass)
//   dL/dk   += sum_k w_k Re(conj lam_hat_{n+1} * tk * psi_t_{n+1})
//   dL/dM   += sum_k w_k Re(conj lam_hat_{n+1} * (tm1 psi_t_{n+1} - tm2 psi_t_n))
// with tk = -2 dt M q^4 / den, tm1 = 1 / (M den), tm2 = 2 k q^4 dt / den^2 + alpha / (M den)
// (dalpha/dk, dbeta/dk are -2 dt M q^4/den times alpha, beta; dbeta/dM = beta/(M den)
// and beta f_hat_n = alpha psi_t_n - psi_t_{n+1}).
// ---------------------------------------------------------------------------
namespace chgb {

namespace {

// Sum over the block; the result is valid in thread 0.
__device__ __forceinline__ double block_sum(double v, double *red) {
    for(int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if(lane == 0) red[w] = v;
    __syncthreads();
    double t = 0.0;
    if(threadIdx.x == 0)
        for(int i = 0; i < nw; i++) t += red[i];
    return t;
}

// Row pass of the adjoint step: work rows (x half spectrum of beta lam_hat after
// the inverse y transform) -> C2R -> B lam; geps += <B lam, psi_n>; * f''(psi_n) -> R2C.
__global__ void __launch_bounds__(1024) row_adj_kernel(double2 *__restrict__ work, const double *__restrict__ psi_n,
                                                      int N, int M, int log2M, int rows_per_cta, int tpl,
                                                      const int4 *__restrict__ twf, double eps,
                                                      double *__restrict__ geps) {
    extern __shared__ double2 sm2[];
    __shared__ double red[32];
    const int LS = M + 1, H = M + 1;
    const int lines = rows_per_cta;
    double2 *A = sm2;
    double2 *B = sm2 + lines * LS;
    int *sm_e = reinterpret_cast<int *>(sm2 + 2 * lines * LS);   // exponents: c2r input, r2c input
    const int li = threadIdx.x / tpl, lane = threadIdx.x - li * tpl;
    const bool active = li < lines;
    const long long row = (long long) blockIdx.x * rows_per_cta + (active ? li : 0);
    const int G = log2M + 3;
    if(active && lane == 0) {
        sm_e[li] = 0;
        sm_e[lines + li] = 0;
    }
    int e = 0;
    if(active) {
        const double2 *src = work + row * H;
        for(int k = lane; k < H; k += tpl) {
            const double2 v = src[k];
            B[li * LS + k] = v;
            e = max(e, max(fx_expo(v.x), fx_expo(v.y)));
        }
    }
    __syncthreads();
    fx_line_max(e, tpl, li, lane, active, sm_e);
    __syncthreads();
    int emax = active ? sm_e[li] : 0;
    int sh = fx_scale(emax, G);
    // c2r pre-processing in fixed point, as the forward row pass
    if(active) {
        const double2 *X = B + li * LS;
        fx2 *Z = reinterpret_cast<fx2 *>(A + li * LS);
        for(int k = lane; k < M; k += tpl) {
            const fx2 xk = fx_load(X[k], sh);
            fx2 xc = fx_load(X[M - k], sh);
            xc.y = -xc.y;
            const fx2 e2 = fx_add(xk, xc);
            const fx2 t = fx_cmul<true>(fx_sub(xk, xc), twf[k]);
            Z[k] = fx2{e2.x - t.y, e2.y + t.x};
        }
    }
    __syncthreads();
    double2 *cur = static_cast<double2 *>(fx_fft_line<+1, false, true>(A, B, M, log2M, LS, li, lane, tpl, active, twf,
                                                                       2, 0, emax == 2047 ? FX_NAN_SCALE : sh));
    double2 *other = (cur == A) ? B : A;
    double acc = 0.0;
    if(active) {
        const double2 *pr = reinterpret_cast<const double2 *>(psi_n + row * N);
        for(int n = lane; n < M; n += tpl) {
            double2 b = cur[li * LS + n];
            double2 p = pr[n];
            acc = fma(b.x, p.x, acc);
            acc = fma(b.y, p.y, acc);
            cur[li * LS + n] = make_double2(b.x * fma(3.0 * p.x, p.x, -eps), b.y * fma(3.0 * p.y, p.y, -eps));
        }
    }
    double t = block_sum(acc, red);
    if(threadIdx.x == 0) geps[blockIdx.x] += t;
    __syncthreads();
    fx_line_exponent(cur, M, LS, li, lane, tpl, active, sm_e + lines);
    __syncthreads();
    emax = active ? sm_e[lines + li] : 0;
    sh = fx_scale(emax, G);
    const fx2 *Z = static_cast<const fx2 *>(
                       fx_fft_line<-1, true, false>(cur, other, M, log2M, LS, li, lane, tpl, active, twf, 2, sh, 0)) +
                   li * LS;
    if(active) {
        const int sh_out = emax == 2047 ? FX_NAN_SCALE : sh + 1;
        double2 *dst = work + row * H;
        for(int k = lane; k <= M; k += tpl) {
            const fx2 zk = Z[k == M ? 0 : k];
            fx2 zc = Z[k == 0 ? 0 : M - k];
            zc.y = -zc.y;
            const fx2 a = fx_add(zk, zc), bb = fx_sub(zk, zc);
            const fx2 tt = fx_cmul<false>(fx2{bb.y, -bb.x}, twf[k]);
            double2 xk = fx_out(fx_add(a, tt), sh_out);
            if(k == 0 || k == M) xk.y = 0.0;
            dst[k] = xk;
        }
    }
}

enum { ADJ_A = 1, ADJ_B = 2, ADJ_BA = 3 };

// Column pass of the adjoint: B part (forward y FFT of the row result, lam_hat
// update) and/or A part (gradient sums with psi_next = psi_t_{n+1} and
// psi_cur = psi_t_n, then beta * lam_hat and the inverse y FFT into work).
template <int MODE>
__global__ void __launch_bounds__(1024) col_adj_kernel(double2 *__restrict__ work, double2 *__restrict__ lam,
                                                      const double *__restrict__ alpha, const double *__restrict__ beta,
                                                      const double *__restrict__ tk, const double *__restrict__ tm1,
                                                      const double *__restrict__ tm2,
                                                      const double2 *__restrict__ psi_next,
                                                      const double2 *__restrict__ psi_cur, int L, int log2L, int H,
                                                      int C, int tpl, const int4 *__restrict__ twf,
                                                      double *__restrict__ gk, double *__restrict__ gm) {
    extern __shared__ double2 sm2[];
    __shared__ double red[32];
    const int LS = L;
    double2 *A = sm2;
    double2 *B = sm2 + C * LS;
    int *sm_e = reinterpret_cast<int *>(sm2 + 2 * C * LS);   // exponents: forward input, inverse input
    const int li = threadIdx.x / tpl, lane = threadIdx.x - li * tpl;
    const int kx0 = blockIdx.x * C;
    const int ncols = min(C, H - kx0);
    const int lg = col_log2(ncols);
    const bool active = li < ncols;
    const int nthr = blockDim.x;
    const int G = log2L + 1;
    if(active && lane == 0) {
        sm_e[li] = 0;
        sm_e[C + li] = 0;
    }
    double2 *cur = A;
    if(MODE & ADJ_B) {
        for(int e = threadIdx.x; e < ncols * L; e += nthr) {
            int c, pos;
            col_split(e, ncols, lg, c, pos);
            A[c * LS + pos] = work[kx0 + c + (long long) pos * H];
        }
        __syncthreads();
        fx_line_exponent(A, L, LS, li, lane, tpl, active, sm_e);
        __syncthreads();
        const int emax = active ? sm_e[li] : 0;
        const int sh = fx_scale(emax, G);
        cur = static_cast<double2 *>(fx_fft_line<-1, true, true>(A, B, L, log2L, LS, li, lane, tpl, active, twf, 1,
                                                                 sh, emax == 2047 ? FX_NAN_SCALE : sh));
        for(int e = threadIdx.x; e < ncols * L; e += nthr) {
            int c, pos;
            col_split(e, ncols, lg, c, pos);
            long long off = kx0 + c + (long long) pos * H;
            double2 q = cur[c * LS + pos];
            double2 l = lam[off];
            double al = alpha[off];
            double2 nv = make_double2(fma(al, l.x, -q.x), fma(al, l.y, -q.y));
            lam[off] = nv;
            cur[c * LS + pos] = nv;
        }
        __syncthreads();
    }
    else {
        for(int e = threadIdx.x; e < ncols * L; e += nthr) {
            int c, pos;
            col_split(e, ncols, lg, c, pos);
            A[c * LS + pos] = lam[kx0 + c + (long long) pos * H];
        }
        __syncthreads();
    }
    if(MODE & ADJ_A) {
        double ak = 0.0, am = 0.0;
        for(int e = threadIdx.x; e < ncols * L; e += nthr) {
            int c, pos;
            col_split(e, ncols, lg, c, pos);
            int kx = kx0 + c;
            long long off = kx + (long long) pos * H;
            double2 l = cur[c * LS + pos];
            double2 pn = psi_next[off], pc = psi_cur[off];
            double w = (kx == 0 || kx == L / 2) ? 1.0 : 2.0;
            double dn = fma(l.x, pn.x, l.y * pn.y);
            double dc = fma(l.x, pc.x, l.y * pc.y);
            ak = fma(w * tk[off], dn, ak);
            am = fma(w, fma(tm1[off], dn, -tm2[off] * dc), am);
            double be = beta[off];
            cur[c * LS + pos] = make_double2(be * l.x, be * l.y);
        }
        double t = block_sum(ak, red);
        if(threadIdx.x == 0) gk[blockIdx.x] += t;
        t = block_sum(am, red);
        if(threadIdx.x == 0) gm[blockIdx.x] += t;
        __syncthreads();
        fx_line_exponent(cur, L, LS, li, lane, tpl, active, sm_e + C);
        __syncthreads();
        const int emax = active ? sm_e[C + li] : 0;
        const int sh = fx_scale(emax, G);
        double2 *other = (cur == A) ? B : A;
        cur = static_cast<double2 *>(fx_fft_line<+1, true, true>(cur, other, L, log2L, LS, li, lane, tpl, active, twf,
                                                                 1, sh, emax == 2047 ? FX_NAN_SCALE : sh));
        for(int e = threadIdx.x; e < ncols * L; e += nthr) {
            int c, pos;
            col_split(e, ncols, lg, c, pos);
            work[kx0 + c + (long long) pos * H] = cur[c * LS + pos];
        }
    }
}

__global__ void axpy_hat_kernel(double2 *__restrict__ y, const double2 *__restrict__ x, double a, long long n) {
    for(long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
        double2 v = x[i], w = y[i];
        y[i] = make_double2(fma(a, v.x, w.x), fma(a, v.y, w.y));
    }
}

}  // namespace

struct SpectralAdj {
    double *tk = nullptr, *tm1 = nullptr, *tm2 = nullptr;
    double2 *lam = nullptr;
    double2 *work = nullptr;   // the adjoint sweep's own transform scratch (the state's stays free for recomputation)
    double *geps = nullptr, *gk = nullptr, *gm = nullptr;   // per-CTA partial sums
    int n_row_cta = 0, n_col_cta = 0;
};

bool spectral_adjoint_supported(const SpectralState *s) {
    return s->g.dims == 2 && s->g.S == 1 && s->m.kind == CHGB_MODEL_LANDAU && s->g.N >= 8;
}

SpectralAdj *spectral_adj_create(SpectralState *s, std::string &err) {
    SpectralAdj *a = new SpectralAdj();
    const int N = s->g.N;
    const double dx = s->p.dx, dt = s->p.dt, M = s->p.M, Ssplit = s->p.splitting_S, k = s->p.k[0];
    std::vector<double> tk(s->hat), tm1(s->hat), tm2(s->hat);
    long long idx = 0;
    // the same wave vectors as build_tables (src/integrators/PseudospectralCPU.cpp:44-57)
    for(int kx_idx = 0; kx_idx < N; kx_idx++) {
        int kx = (kx_idx < N / 2) ? kx_idx : N - kx_idx;
        for(int ky = 0; ky < N / 2 + 1; ky++, idx++) {
            double kk = 2.0 * M_PI * std::sqrt((double) (kx * kx + ky * ky)) / (N * dx);
            double k2 = kk * kk, k4 = k2 * k2;
            double denom = 1.0 + dt * M * (Ssplit * k2 + 2.0 * k * k4);
            double c = dt * M * k2;
            double alpha = (1.0 + c * Ssplit) / denom;
            tk[idx] = -2.0 * dt * M * k4 / denom;
            tm1[idx] = 1.0 / (M * denom);
            tm2[idx] = 2.0 * k * k4 * dt / (denom * denom) + alpha / (M * denom);
        }
    }
    a->n_row_cta = (int) (((long long) s->g.bins / N) / s->row_rpc);
    a->n_col_cta = (s->H + s->col_C - 1) / s->col_C;
    bool ok = cudaMalloc(&a->tk, sizeof(double) * s->hat) == cudaSuccess &&
              cudaMalloc(&a->tm1, sizeof(double) * s->hat) == cudaSuccess &&
              cudaMalloc(&a->tm2, sizeof(double) * s->hat) == cudaSuccess &&
              cudaMalloc(&a->lam, sizeof(double2) * s->hat) == cudaSuccess &&
              cudaMalloc(&a->work, sizeof(double2) * s->hat) == cudaSuccess &&
              cudaMalloc(&a->geps, sizeof(double) * a->n_row_cta) == cudaSuccess &&
              cudaMalloc(&a->gk, sizeof(double) * a->n_col_cta) == cudaSuccess &&
              cudaMalloc(&a->gm, sizeof(double) * a->n_col_cta) == cudaSuccess;
    ok = ok && cudaMemcpy(a->tk, tk.data(), sizeof(double) * s->hat, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(a->tm1, tm1.data(), sizeof(double) * s->hat, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(a->tm2, tm2.data(), sizeof(double) * s->hat, cudaMemcpyHostToDevice) == cudaSuccess;
    if(ok) {
        size_t rs = s->row_smem, cs = s->col_smem;
        if(rs > 48 * 1024) cudaFuncSetAttribute(row_adj_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) rs);
        if(cs > 48 * 1024) {
            cudaFuncSetAttribute(col_adj_kernel<ADJ_A>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) cs);
            cudaFuncSetAttribute(col_adj_kernel<ADJ_B>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) cs);
            cudaFuncSetAttribute(col_adj_kernel<ADJ_BA>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) cs);
        }
        ok = cudaGetLastError() == cudaSuccess;
    }
    if(!ok) {
        cudaGetLastError();
        spectral_adj_destroy(a);
        err = "adjoint allocation failed";
        return nullptr;
    }
    return a;
}

void spectral_adj_destroy(SpectralAdj *a) {
    if(!a) return;
    cudaFree(a->tk);
    cudaFree(a->tm1);
    cudaFree(a->tm2);
    cudaFree(a->lam);
    cudaFree(a->work);
    cudaFree(a->geps);
    cudaFree(a->gk);
    cudaFree(a->gm);
    delete a;
}

double2 *spectral_adj_lam(SpectralAdj *a) { return a->lam; }

cudaError_t spectral_adj_zero(SpectralAdj *a, const SpectralState *s, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(a->geps, 0, sizeof(double) * a->n_row_cta, st);
    if(e == cudaSuccess) e = cudaMemsetAsync(a->gk, 0, sizeof(double) * a->n_col_cta, st);
    if(e == cudaSuccess) e = cudaMemsetAsync(a->gm, 0, sizeof(double) * a->n_col_cta, st);
    if(e == cudaSuccess) e = cudaMemsetAsync(a->lam, 0, sizeof(double2) * s->hat, st);
    return e;
}

cudaError_t spectral_adj_add_seed(SpectralAdj *a, const SpectralState *s, const double2 *x, double scale,
                                  cudaStream_t st) {
    int grid = (int) std::min<long long>((s->hat + 255) / 256, 152 * 8);
    axpy_hat_kernel<<<grid, 256, 0, st>>>(a->lam, x, scale, s->hat);
    return cudaGetLastError();
}

// mode: 1 = A only (start of a segment), 2 = B only (end), 3 = B then A
cudaError_t spectral_adj_col(SpectralAdj *a, SpectralState *s, int mode, const double2 *psi_next,
                             const double2 *psi_cur, cudaStream_t st) {
    const int N = s->g.N;
    dim3 grid((unsigned) a->n_col_cta);
#define ADJ_COL_ARGS                                                                                                   \
    a->work, a->lam, s->alpha, s->beta, a->tk, a->tm1, a->tm2, psi_next, psi_cur, N, ilog2(N), s->H, s->col_C,         \
        s->col_tpl, s->twf, a->gk, a->gm
    if(mode == ADJ_A) col_adj_kernel<ADJ_A><<<grid, s->col_threads, s->col_smem, st>>>(ADJ_COL_ARGS);
    else if(mode == ADJ_B) col_adj_kernel<ADJ_B><<<grid, s->col_threads, s->col_smem, st>>>(ADJ_COL_ARGS);
    else col_adj_kernel<ADJ_BA><<<grid, s->col_threads, s->col_smem, st>>>(ADJ_COL_ARGS);
#undef ADJ_COL_ARGS
    return cudaGetLastError();
}

cudaError_t spectral_adj_row(SpectralAdj *a, SpectralState *s, const double *psi_n, cudaStream_t st) {
    const int M = s->g.N / 2;
    row_adj_kernel<<<a->n_row_cta, s->row_threads, s->row_smem, st>>>(a->work, psi_n, s->g.N, M, ilog2(M), s->row_rpc,
                                                                       s->row_tpl, s->twf, s->m.epsilon, a->geps);
    return cudaGetLastError();
}

// Sum the per-CTA partials in a fixed order: g3 = {sum geps, sum gk, sum gm}.
int spectral_adj_grads(SpectralAdj *a, double *g3) {
    std::vector<double> ge(a->n_row_cta), gk(a->n_col_cta), gm(a->n_col_cta);
    if(cudaMemcpy(ge.data(), a->geps, sizeof(double) * ge.size(), cudaMemcpyDeviceToHost) != cudaSuccess ||
       cudaMemcpy(gk.data(), a->gk, sizeof(double) * gk.size(), cudaMemcpyDeviceToHost) != cudaSuccess ||
       cudaMemcpy(gm.data(), a->gm, sizeof(double) * gm.size(), cudaMemcpyDeviceToHost) != cudaSuccess)
        return CHGB_ERR_CUDA;
    double s0 = 0, s1 = 0, s2 = 0;
    for(double v : ge) s0 += v;
    for(double v : gk) s1 += v;
    for(double v : gm) s2 += v;
    g3[0] = s0;
    g3[1] = s1;
    g3[2] = s2;
    return CHGB_OK;
}

// psi_hat <- hat; work <- inverse y transform of hat (the state a step starts from).
cudaError_t spectral_load_hat(SpectralState *s, const double2 *hat, cudaStream_t st) {
    size_t bytes = sizeof(double2) * (size_t) s->hat * s->g.S;
    cudaError_t e = cudaSuccess;
    if(hat != s->psi_hat) e = cudaMemcpyAsync(s->psi_hat, hat, bytes, cudaMemcpyDeviceToDevice, st);
    if(e == cudaSuccess) e = cudaMemcpyAsync(s->work, hat, bytes, cudaMemcpyDeviceToDevice, st);
    if(e == cudaSuccess) e = launch_col<COL_INV>(s, 1, st);
    s->hat_valid = true;
    s->real_valid = false;
    return e;
}

// One forward step from the half-spectrum state that also writes rho_n (real) to real_out.
cudaError_t spectral_step_record(SpectralState *s, double *real_out, cudaStream_t st) {
    cudaError_t e = launch_row<ROW_IN_HAT, true, true, true>(s, nullptr, real_out, st);
    if(e == cudaSuccess) e = launch_col<COL_STEP>(s, 1, st);
    s->hat_valid = true;
    s->real_valid = false;
    return e;
}

// real_out = C2R(hat_scaled) (unnormalised: a scaled state gives the field).
cudaError_t spectral_inverse(SpectralState *s, const double2 *hat_scaled, double *real_out, cudaStream_t st) {
    size_t bytes = sizeof(double2) * (size_t) s->hat * s->g.S;
    cudaError_t e = cudaMemcpyAsync(s->work, hat_scaled, bytes, cudaMemcpyDeviceToDevice, st);
    if(e == cudaSuccess) e = launch_col<COL_INV>(s, 1, st);
    if(e == cudaSuccess) e = launch_row<ROW_IN_HAT, false, true, false>(s, nullptr, real_out, st);
    s->hat_valid = false;
    return e;
}

double2 *spectral_psi_hat_mut(SpectralState *s) { return s->psi_hat; }

// Plain transforms on caller buffers, FFTW's unnormalised r2c / c2r in the
// half-spectrum layout, S species: the row and column passes of a step without
// the model or the update.  `hat` stands in for the state's work array for the
// duration of the call (the kernels take it as an argument at launch).
cudaError_t spectral_r2c(SpectralState *s, const double *real, double2 *hat, cudaStream_t st, int *launches) {
    double2 *saved = s->work;
    s->work = hat;
    cudaError_t e = launch_row<ROW_IN_REAL, false, false, true>(s, real, nullptr, st);
    int n = 1;
    if(e == cudaSuccess && s->g.dims >= 2) {
        e = launch_col<COL_FWD>(s, 1, st);
        n++;
    }
    if(e == cudaSuccess && s->g.dims == 3) {
        e = launch_col<COL_FWD>(s, 2, st);
        n++;
    }
    s->work = saved;
    *launches += n;
    return e;
}

cudaError_t spectral_c2r(SpectralState *s, double2 *hat, double *real, cudaStream_t st, int *launches) {
    double2 *saved = s->work;
    s->work = hat;
    cudaError_t e = cudaSuccess;
    int n = 0;
    if(s->g.dims == 3) {
        e = launch_col<COL_INV>(s, 2, st);
        n++;
    }
    if(e == cudaSuccess && s->g.dims >= 2) {
        e = launch_col<COL_INV>(s, 1, st);
        n++;
    }
    if(e == cudaSuccess) {
        e = launch_row<ROW_IN_HAT, false, true, false>(s, nullptr, real, st);
        n++;
    }
    s->work = saved;
    *launches += n;
    return e;
}
long long spectral_hat_size(const SpectralState *s) { return s->hat; }

// ---- the variable-mobility step with its pointwise stages on the passes -----
// dims >= 2.  The stage rides on the slowest axis's column pass (y in 2D, z in
// 3D): the first inverse pass of a c2r loads through it, the last forward pass
// of an r2c stores through it.  `scratch` stands in for the state's work array.

cudaError_t spectral_psmob_fprime(SpectralState *s, const double *rho, double2 *fder_hat, double2 *mu,
                                  const double2 *rho_hat, const PsmobTables &t, double two_k, cudaStream_t st,
                                  int *launches) {
    double2 *saved = s->work;
    s->work = fder_hat;
    const int last = s->g.dims - 1;
    cudaError_t e = launch_row<ROW_IN_REAL, true, false, true>(s, rho, nullptr, st);
    int n = 1;
    if(e == cudaSuccess && s->g.dims == 3) {
        e = launch_col<COL_FWD>(s, 1, st);
        n++;
    }
    if(e == cudaSuccess) {
        if(mu) {
            ColOps o{};
            o.q2 = t.q2;
            o.dealias = t.dealias;
            o.use_dealias = t.use_dealias;
            o.rho = const_cast<double2 *>(rho_hat);   // read only in this mode
            o.out = mu;
            o.two_k = two_k;
            e = launch_col<COL_FWD_MU>(s, last, st, o);
        }
        else {
            e = launch_col<COL_FWD>(s, last, st);
        }
        n++;
    }
    s->work = saved;
    *launches += n;
    return e;
}

cudaError_t spectral_psmob_flux(SpectralState *s, const double2 *src, const double *kd, const PsmobTables &t,
                                const double *mob, const double *M0, double2 *div, bool first, double2 *scratch,
                                cudaStream_t st, int *launches) {
    double2 *saved = s->work;
    s->work = scratch;
    const int last = s->g.dims - 1;
    ColOps o{};
    o.kd = kd;
    o.dealias = t.dealias;
    o.use_dealias = t.use_dealias;
    o.src = src;
    o.out = div;
    o.first = first ? 1 : 0;
    cudaError_t e = launch_col<COL_GRAD_INV>(s, last, st, o);
    int n = 1;
    if(e == cudaSuccess && s->g.dims == 3) {
        e = launch_col<COL_INV>(s, 1, st);
        n++;
    }
    if(e == cudaSuccess) {
        e = M0 ? launch_row_flux<FLUX_DM>(s, mob, M0, st) : launch_row_flux<FLUX_M>(s, mob, nullptr, st);
        n++;
    }
    if(e == cudaSuccess && s->g.dims == 3) {
        e = launch_col<COL_FWD>(s, 1, st);
        n++;
    }
    if(e == cudaSuccess) {
        e = launch_col<COL_FWD_DIV>(s, last, st, o);
        n++;
    }
    s->work = saved;
    *launches += n;
    return e;
}

cudaError_t spectral_psmob_update(SpectralState *s, double2 *rho_hat, const double2 *fder_hat, const double2 *div_hat,
                                  const double *q2, const double *M0, double dt, double Ssplit, double k0,
                                  double2 *scratch, double *rho, cudaStream_t st, int *launches) {
    double2 *saved = s->work;
    s->work = scratch;
    ColOps o{};
    o.q2 = q2;
    o.M0 = M0;
    o.rho = rho_hat;
    o.fder = fder_hat;
    o.div_in = div_hat;
    o.with_div = div_hat ? 1 : 0;
    o.dt = dt;
    o.Ssplit = Ssplit;
    o.k0 = k0;
    o.inv_bins = 1.0 / (double) s->g.bins;
    cudaError_t e = launch_col<COL_UPD_INV>(s, s->g.dims - 1, st, o);
    int n = 1;
    if(e == cudaSuccess && s->g.dims == 3) {
        e = launch_col<COL_INV>(s, 1, st);
        n++;
    }
    if(e == cudaSuccess) {
        e = launch_row<ROW_IN_HAT, false, true, false>(s, nullptr, rho, st);
        n++;
    }
    s->work = saved;
    *launches += n;
    return e;
}

}  // namespace chgb
