// psmob.cu — the `pseudospectral_mobility` step (variable mobility), FP64.
//
// Reference: src/integrators/PseudospectralMobilityCPU.cpp (constructor
// :13-160 for the tables, _evolve_simple :236-310 for the step).  With M0 the
// largest mobility of each species, the constant part M0 of the mobility is
// treated semi-implicitly and the remainder (M - M0) explicitly through
// real-space fluxes:
//   mu_hat  = f'_hat + 2 k q^2 rho_hat                     (dealiased)
//   J_d     = (M - M0) C2R(i k_d mu_hat) / N^d             (d = each axis)
//   div_hat = sum_d i k_d R2C(J_d)                         (dealiased)
//   rho_hat = (rho_hat + dt div_hat - dt M0 q^2 (f'_hat - S rho_hat))
//             / (1 + dt M0 (S q^2 + 2 k q^4))
//   rho     = C2R(rho_hat / N^d)
// rho_hat is the unnormalised transform, as FFTW's r2c gives it.  The
// transforms are the pseudospectral engine's row and column passes.  In 2D and
// 3D each pointwise stage rides on one of them (spectral_psmob_*): f' on the
// r2c's row pass, mu on its last column pass, i k_d on the first inverse column
// pass of a flux's c2r, the flux itself between the c2r and r2c of one row
// pass, the divergence on the last forward column pass, the update on the
// final c2r's first column pass -- 2D: 12 launches a step instead of 22.  1D
// uses the elementwise kernels below.  Both are written in the reference's
// order of operations and give the same bits.  A constant mobility makes every
// flux exactly zero, so those stages are skipped.
#include <cmath>
#include <vector>

#include "kernels.h"
#include "psmob.h"
#include "psmob_impl.h"

namespace chgb {

namespace {

constexpr int M0_BLOCKS = 4 * 152;   // most partial maxima per species (4 blocks per SM)

// M0 = max(0, max M) per species in one launch (PseudospectralMobilityCPU.cpp:
// 434-442): each block reduces a grid-stride share of the species' mobility
// into part[s * nblk + b]; the last block to finish, counted per species,
// reduces the partials and resets its counter for the next launch.  A maximum
// is exact, so the grouping does not change the result; every comparison is
// the reference's m < v ? v : m from m = 0, which passes over NaN.
__device__ __forceinline__ double m0_block_max(double m, double *red) {
    red[threadIdx.x] = m;
    __syncthreads();
    for(int o = blockDim.x / 2; o > 0; o >>= 1) {
        if(threadIdx.x < o) red[threadIdx.x] = (red[threadIdx.x] < red[threadIdx.x + o]) ? red[threadIdx.x + o]
                                                                                      : red[threadIdx.x];
        __syncthreads();
    }
    return red[0];
}

__global__ void __launch_bounds__(256) m0_kernel(const double *__restrict__ mob, long long bins,
                                                 double *__restrict__ part, unsigned *__restrict__ count,
                                                 double *__restrict__ M0) {
    const int s = blockIdx.y;
    __shared__ double red[256];
    __shared__ bool last;
    double m = 0.0;
    for(long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < bins;
        i += (long long) gridDim.x * blockDim.x) {
        const double v = mob[s * bins + i];
        m = (m < v) ? v : m;
    }
    m = m0_block_max(m, red);
    if(threadIdx.x == 0) {
        part[s * gridDim.x + blockIdx.x] = m;
        __threadfence();   // the partial is visible before the count says so
        last = atomicAdd(&count[s], 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if(!last) return;
    __threadfence();
    m = 0.0;
    for(int b = threadIdx.x; b < (int) gridDim.x; b += blockDim.x) {
        const double v = __ldcg(&part[s * gridDim.x + b]);
        m = (m < v) ? v : m;
    }
    __syncthreads();   // red is reused
    m = m0_block_max(m, red);
    if(threadIdx.x == 0) {
        M0[s] = m;
        count[s] = 0;
    }
}

// mu_hat = f'_hat + 2 k q^2 rho_hat (:249-254)
__global__ void psm_mu_kernel(const double2 *__restrict__ fder, const double2 *__restrict__ rho,
                              const double *__restrict__ q2, const double *__restrict__ dealias, double two_k,
                              int use_dealias, long long n, double2 *__restrict__ mu) {
    for(long long k = blockIdx.x * (long long) blockDim.x + threadIdx.x; k < n; k += (long long) gridDim.x * blockDim.x) {
        double t = two_k * q2[k];
        double2 f = fder[k], r = rho[k];
        double2 v = make_double2(f.x + t * r.x, f.y + t * r.y);
        if(use_dealias) {
            double D = dealias[k];
            v.x *= D;
            v.y *= D;
        }
        mu[k] = v;
    }
}

// out = i k_d mu_hat (:258-263)
__global__ void psm_grad_kernel(const double2 *__restrict__ mu, const double *__restrict__ kd,
                                const double *__restrict__ dealias, int use_dealias, long long n,
                                double2 *__restrict__ out) {
    for(long long k = blockIdx.x * (long long) blockDim.x + threadIdx.x; k < n; k += (long long) gridDim.x * blockDim.x) {
        double2 v = mul_ik(kd[k], mu[k]);
        if(use_dealias) {
            double D = dealias[k];
            v.x *= D;
            v.y *= D;
        }
        out[k] = v;
    }
}

// J = (M - M0) * (C2R(...) / N^d) in place (:267-281).  N^d is a power of two,
// so the product with its (exact) reciprocal is the division, bit for bit.
__global__ void psm_flux_kernel(double *__restrict__ g, const double *__restrict__ mob, const double *__restrict__ M0,
                                long long bins, int S, double inv_bins) {
    const long long n = bins * S;
    for(long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
        const int s = (int) (i / bins);
        double gv = g[i] * inv_bins;
        double dM = mob[i] - M0[s];
        g[i] = dM * gv;
    }
}

// div_hat (=|+=) i k_d R2C(J_d) (:284-293)
__global__ void psm_div_kernel(const double2 *__restrict__ fh, const double *__restrict__ kd,
                               const double *__restrict__ dealias, int use_dealias, int first, long long n,
                               double2 *__restrict__ div) {
    for(long long k = blockIdx.x * (long long) blockDim.x + threadIdx.x; k < n; k += (long long) gridDim.x * blockDim.x) {
        double2 f = fh[k];
        if(use_dealias) {
            double D = dealias[k];
            f.x *= D;
            f.y *= D;
        }
        double2 t = mul_ik(kd[k], f);
        if(first) {
            div[k] = make_double2(0.0 + t.x, 0.0 + t.y);
        }
        else {
            double2 d = div[k];
            div[k] = make_double2(d.x + t.x, d.y + t.y);
        }
    }
}

// the stabilised semi-implicit update (:296-306); copy = rho_hat / N^d
__global__ void psm_update_kernel(double2 *__restrict__ rho, const double2 *__restrict__ fder,
                                  const double2 *__restrict__ div, const double *__restrict__ q2,
                                  const double *__restrict__ M0, double dt, double Ssplit, double k0, long long hat,
                                  long long n, double inv_bins, int with_div, double2 *__restrict__ copy) {
    for(long long k = blockIdx.x * (long long) blockDim.x + threadIdx.x; k < n; k += (long long) gridDim.x * blockDim.x) {
        const int s = (int) (k / hat);
        double k2 = q2[k];
        double k4 = k2 * k2;
        double m0 = M0[s];
        double denom = 1.0 + dt * m0 * (Ssplit * k2 + 2.0 * k0 * k4);
        double c = dt * m0 * k2;
        double2 r = rho[k], f = fder[k];
        double ar = r.x, ai = r.y;
        if(with_div) {
            double2 d = div[k];
            ar = r.x + dt * d.x;
            ai = r.y + dt * d.y;
        }
        double nr = (ar - c * (f.x - Ssplit * r.x)) / denom;
        double ni = (ai - c * (f.y - Ssplit * r.y)) / denom;
        rho[k] = make_double2(nr, ni);
        copy[k] = make_double2(nr * inv_bins, ni * inv_bins);
    }
}

int grid_of(long long n) { return (int) std::min<long long>((n + 255) / 256, 152 * 8); }

}  // namespace

void psmob_destroy(PsMob *s) {
    if(!s) return;
    if(s->eng) spectral_destroy(s->eng);
    for(double2 *p : {s->rho_hat, s->fder_hat, s->mu_hat, s->tmp_hat, s->div_hat}) cudaFree(p);
    for(double *p : {s->q2, s->dealias, s->kc[0], s->kc[1], s->kc[2], s->fder, s->tmp, s->M0, s->part}) cudaFree(p);
    cudaFree(s->m0_count);
    psmob_gmres_release(s);
    delete s;
}

int psmob_create(const chgb_params &p, const Geom &g, const ModelDev &m, PsMob **out, std::string &err) {
    *out = nullptr;
    PsMob *s = new PsMob();
    s->p = p;
    s->g = g;
    s->m = m;
    s->S = g.S;
    s->bins = g.bins;
    chgb_params q = p;
    q.integrator = CHGB_INTEGRATOR_PSEUDOSPECTRAL;   // the engine's own update tables go unused
    int r = spectral_create(q, g, m, &s->eng, err);
    if(r != CHGB_OK) {
        psmob_destroy(s);
        return r;
    }
    s->hat = spectral_hat_size(s->eng);
    s->hall = s->hat * s->S;
    s->constant = p.mobility_type == CHGB_MOBILITY_CONSTANT;
    // wave vectors and dealiaser, PseudospectralMobilityCPU.cpp:56-118
    const int N = g.N, dims = g.dims;
    const double dx = p.dx;
    std::vector<double> q2(s->hall), dl(s->hall), kc[3];
    for(int d = 0; d < dims; d++) kc[d].assign(s->hall, 0.0);
    const double k_cut = N * M_PI / (N * dx) * 2.0 / 3.0;
    long long k_idx = 0;
    for(int sp = 0; sp < s->S; sp++) {
        if(dims == 1) {
            for(long long i = 0; i < s->hat; i++, k_idx++) {
                double kx = 2.0 * M_PI * i / (N * dx);
                dl[k_idx] = (std::abs(kx) <= k_cut) ? 1.0 : 0.0;
                kc[0][k_idx] = kx;
                q2[k_idx] = kx * kx;
            }
        }
        else if(dims == 2) {
            for(int a = 0; a < N; a++) {
                int ai = (a < N / 2) ? a : (a - N);
                double kx = 2.0 * M_PI * ai / (N * dx);
                for(int b = 0; b < N / 2 + 1; b++, k_idx++) {
                    double ky = 2.0 * M_PI * b / (N * dx);
                    double k2 = kx * kx + ky * ky;
                    dl[k_idx] = (std::sqrt(k2) <= k_cut) ? 1.0 : 0.0;
                    kc[0][k_idx] = kx;
                    kc[1][k_idx] = ky;
                    q2[k_idx] = k2;
                }
            }
        }
        else {
            for(int a = 0; a < N; a++) {
                int ai = (a < N / 2) ? a : (a - N);
                double kx = 2.0 * M_PI * ai / (N * dx);
                for(int b = 0; b < N; b++) {
                    int bi = (b < N / 2) ? b : (b - N);
                    double ky = 2.0 * M_PI * bi / (N * dx);
                    for(int c = 0; c < N / 2 + 1; c++, k_idx++) {
                        double kz = 2.0 * M_PI * c / (N * dx);
                        double k2 = kx * kx + ky * ky + kz * kz;
                        dl[k_idx] = (std::sqrt(k2) <= k_cut) ? 1.0 : 0.0;
                        kc[0][k_idx] = kx;
                        kc[1][k_idx] = ky;
                        kc[2][k_idx] = kz;
                        q2[k_idx] = k2;
                    }
                }
            }
        }
    }
    const size_t hb = sizeof(double2) * (size_t) s->hall, tb = sizeof(double) * (size_t) s->hall;
    const size_t rb = sizeof(double) * (size_t) s->bins * s->S;
    bool ok = cudaMalloc(&s->rho_hat, hb) == cudaSuccess && cudaMalloc(&s->fder_hat, hb) == cudaSuccess &&
              cudaMalloc(&s->mu_hat, hb) == cudaSuccess && cudaMalloc(&s->tmp_hat, hb) == cudaSuccess &&
              cudaMalloc(&s->div_hat, hb) == cudaSuccess && cudaMalloc(&s->q2, tb) == cudaSuccess &&
              cudaMalloc(&s->dealias, tb) == cudaSuccess && cudaMalloc(&s->fder, rb) == cudaSuccess &&
              cudaMalloc(&s->tmp, rb) == cudaSuccess && cudaMalloc(&s->M0, sizeof(double) * s->S) == cudaSuccess &&
              cudaMalloc(&s->part, sizeof(double) * s->S * M0_BLOCKS) == cudaSuccess &&
              cudaMalloc(&s->m0_count, sizeof(unsigned) * s->S) == cudaSuccess &&
              cudaMemset(s->m0_count, 0, sizeof(unsigned) * s->S) == cudaSuccess;
    for(int d = 0; d < dims && ok; d++) ok = cudaMalloc(&s->kc[d], tb) == cudaSuccess;
    ok = ok && cudaMemcpy(s->q2, q2.data(), tb, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(s->dealias, dl.data(), tb, cudaMemcpyHostToDevice) == cudaSuccess;
    for(int d = 0; d < dims && ok; d++) ok = cudaMemcpy(s->kc[d], kc[d].data(), tb, cudaMemcpyHostToDevice) == cudaSuccess;
    if(!ok) {
        cudaGetLastError();
        psmob_destroy(s);
        err = "pseudospectral_mobility allocation failed";
        return CHGB_ERR_ALLOC;
    }
    *out = s;
    return CHGB_OK;
}

int psmob_m0(PsMob *s, const double *mob, cudaStream_t st) {
    const int nblk = (int) std::min<long long>(M0_BLOCKS, std::max<long long>(1, (s->bins + 2047) / 2048));
    m0_kernel<<<dim3(nblk, s->S), 256, 0, st>>>(mob, s->bins, s->part, s->m0_count, s->M0);
    return 1;
}

// The pointwise stages the GMRES path shares with the simple one.
cudaError_t psmob_grad(PsMob *s, const double2 *in, int d, cudaStream_t st) {
    psm_grad_kernel<<<grid_of(s->hall), 256, 0, st>>>(in, s->kc[d], s->dealias, s->p.use_dealias ? 1 : 0, s->hall,
                                                       s->tmp_hat);
    return cudaGetLastError();
}

cudaError_t psmob_div(PsMob *s, int d, cudaStream_t st) {
    psm_div_kernel<<<grid_of(s->hall), 256, 0, st>>>(s->tmp_hat, s->kc[d], s->dealias, s->p.use_dealias ? 1 : 0,
                                                      d == 0 ? 1 : 0, s->hall, s->div_hat);
    return cudaGetLastError();
}

cudaError_t psmob_set_rho(PsMob *s, const double *rho, cudaStream_t st, int64_t *launches) {
    int n = 0;
    cudaError_t e = spectral_r2c(s->eng, rho, s->rho_hat, st, &n);
    *launches += n;
    return e;
}

PsmobTables psmob_tables(const PsMob *s) { return PsmobTables{s->q2, s->dealias, s->p.use_dealias ? 1 : 0}; }

// 2D and 3D: the pointwise stages ride on the transforms' column and row passes
// (spectral_psmob_*), the same arithmetic in the same order.
static cudaError_t psmob_step_fused(PsMob *s, const double *mob, double *rho, cudaStream_t st, int64_t *launches) {
    const PsmobTables t = psmob_tables(s);
    int nl = 0;
    nl += psmob_m0(s, mob, st);
    cudaError_t e = spectral_psmob_fprime(s->eng, rho, s->fder_hat, s->constant ? nullptr : s->mu_hat, s->rho_hat, t,
                                          2.0 * s->p.k[0], st, &nl);
    for(int d = 0; d < s->g.dims && e == cudaSuccess && !s->constant; d++)
        e = spectral_psmob_flux(s->eng, s->mu_hat, s->kc[d], t, mob, s->M0, s->div_hat, d == 0, s->tmp_hat, st, &nl);
    if(e == cudaSuccess)
        e = spectral_psmob_update(s->eng, s->rho_hat, s->fder_hat, s->constant ? nullptr : s->div_hat, s->q2, s->M0,
                                  s->p.dt, s->p.splitting_S, s->p.k[0], s->tmp_hat, rho, st, &nl);
    *launches += nl;
    return e;
}

cudaError_t psmob_step(PsMob *s, const double *mob, double *rho, cudaStream_t st, int64_t *launches) {
    if(s->p.use_gmres) return psmob_step_gmres(s, mob, rho, st, launches);
    if(s->g.dims >= 2) return psmob_step_fused(s, mob, rho, st, launches);
    const long long n = s->hall;
    const int grid = grid_of(n);
    const int dl = s->p.use_dealias ? 1 : 0;
    int nl = 0;
    cudaError_t e;
    // reference mobility M0 per species
    nl += psmob_m0(s, mob, st);
    // bulk chemical potential and its transform
    e = launch_der_bulk(s->m, rho, s->fder, s->bins, st);
    nl++;
    if(e == cudaSuccess) e = spectral_r2c(s->eng, s->fder, s->fder_hat, st, &nl);
    if(e == cudaSuccess && !s->constant) {
        psm_mu_kernel<<<grid, 256, 0, st>>>(s->fder_hat, s->rho_hat, s->q2, s->dealias, 2.0 * s->p.k[0], dl, n,
                                            s->mu_hat);
        nl++;
        e = cudaGetLastError();
        for(int d = 0; d < s->g.dims && e == cudaSuccess; d++) {
            psm_grad_kernel<<<grid, 256, 0, st>>>(s->mu_hat, s->kc[d], s->dealias, dl, n, s->tmp_hat);
            nl++;
            e = cudaGetLastError();
            if(e == cudaSuccess) e = spectral_c2r(s->eng, s->tmp_hat, s->tmp, st, &nl);
            if(e == cudaSuccess) {
                const long long rn = s->bins * s->S;
                psm_flux_kernel<<<grid_of(rn), 256, 0, st>>>(s->tmp, mob, s->M0, s->bins, s->S, 1.0 / (double) s->bins);
                nl++;
                e = cudaGetLastError();
            }
            if(e == cudaSuccess) e = spectral_r2c(s->eng, s->tmp, s->tmp_hat, st, &nl);
            if(e == cudaSuccess) {
                psm_div_kernel<<<grid, 256, 0, st>>>(s->tmp_hat, s->kc[d], s->dealias, dl, d == 0 ? 1 : 0, n,
                                                     s->div_hat);
                nl++;
                e = cudaGetLastError();
            }
        }
    }
    if(e == cudaSuccess) {
        psm_update_kernel<<<grid, 256, 0, st>>>(s->rho_hat, s->fder_hat, s->div_hat, s->q2, s->M0, s->p.dt,
                                                s->p.splitting_S, s->p.k[0], s->hat, n, 1.0 / (double) s->bins,
                                                s->constant ? 0 : 1, s->tmp_hat);
        nl++;
        e = cudaGetLastError();
    }
    if(e == cudaSuccess) e = spectral_c2r(s->eng, s->tmp_hat, rho, st, &nl);
    *launches += nl;
    return e;
}

int psmob_launches_per_step(const PsMob *s) {
    const int t = s->g.dims;   // kernels per transform: row pass + one column pass per further axis
    if(t >= 2) {               // M0, f' + r2c (+ mu), update + c2r, per axis a c2r and r2c sharing the row pass
        int n = 1 + t + t;
        if(!s->constant) n += s->g.dims * (2 * t - 1);
        return n;
    }
    int n = 1 + 1 + t + 1 + t;  // M0, f', r2c, update, c2r
    if(!s->constant) n += 1 + s->g.dims * (1 + t + 1 + t + 1);
    return n;
}

}  // namespace chgb
