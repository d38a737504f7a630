// psmob_gmres.cu — the GMRES path of `pseudospectral_mobility`
// (pseudospectral.use_gmres = true).
//
// Reference: src/integrators/PseudospectralMobilityCPU.cpp, _evolve_full
// :312-427, _apply_Pinv :440-466, _apply_A :468-535, _gmres_solve :537-662.
// Each step solves
//     A rho' = b,   A x = x - dt div(M grad((S - 2k lap) x)),
//     b = rho + dt div(M grad(f'(rho) - S rho)),
// with restarted GMRES (restart m), left-preconditioned by the diagonal
// k-space operator P^-1 = 1 / (1 + dt M0 (S q^2 + 2k q^4)), from rho.  The
// vectors (species-major fields) and every operator application live on the
// device; the Arnoldi step is modified Gram-Schmidt whose inner products are
// deterministic two-level reductions written into device slots that the next
// update reads, so one step of the Arnoldi process needs one host round trip
// (the new Hessenberg column, for the Givens rotations and the stopping test,
// done on the host in the reference's order).  The sums run in a different
// order than the reference's sequential loops, so iterates agree to round-off
// rather than bit for bit.
#include <algorithm>
#include <cmath>
#include <vector>

#include "kernels.h"
#include "psmob_impl.h"

namespace chgb {

namespace {

constexpr int DOT_BLOCKS = 256;

int vgrid(long long n) { return (int) std::min<long long>((n + 255) / 256, 152 * 8); }

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

// out = a / *den  (device scalar)  or a / den_h
__global__ void div_kernel(const double *__restrict__ a, const double *__restrict__ den, double den_h, long long n,
                           double *__restrict__ out) {
    const double d = den ? *den : den_h;
    for(long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x)
        out[i] = a[i] / d;
}

// w -= (*h) v
__global__ void axpy_dev_kernel(double *__restrict__ w, const double *__restrict__ h, const double *__restrict__ v,
                                long long n) {
    const double c = *h;
    for(long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x)
        w[i] -= c * v[i];
}

// x[k] += V[i][k] y[i] for i = 0 .. j-1 in order (:644-646)
__global__ void xupdate_kernel(double *__restrict__ x, const double *__restrict__ V, const double *__restrict__ y,
                               int j, long long n) {
    for(long long k = blockIdx.x * (long long) blockDim.x + threadIdx.x; k < n; k += (long long) gridDim.x * blockDim.x) {
        double acc = x[k];
        for(int i = 0; i < j; i++) acc += V[(size_t) i * n + k] * y[i];
        x[k] = acc;
    }
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

// J = M (C2R(...) / N^d) in place
__global__ void fluxM_kernel(double *__restrict__ g, const double *__restrict__ mob, long long n, double bins) {
    for(long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
        double gv = g[i] / bins;
        g[i] = mob[i] * gv;
    }
}

// Ax = x - dt (div / N^d)   (:527-533)
__global__ void applyA_final_kernel(const double *__restrict__ x, const double *__restrict__ div, double dt,
                                    double bins, long long n, double *__restrict__ Ax) {
    for(long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
        double dr = div[i] / bins;
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

__global__ void rhs_kernel(const double *__restrict__ rho, const double *__restrict__ div, double dt, double bins,
                           long long n, double *__restrict__ b) {
    for(long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
        double t = div[i] / bins;
        b[i] = rho[i] + dt * t;
    }
}

}  // namespace

struct PsGmres {
    int m = 2;
    long long n = 0;
    double *b = nullptr, *x = nullptr, *rhs = nullptr, *Mx = nullptr, *r = nullptr, *w = nullptr, *Av = nullptr;
    double *V = nullptr;       // (m + 1) x n
    double *part = nullptr;    // DOT_BLOCKS partial sums
    double *h = nullptr;       // Hessenberg column slots (m + 2) and scalars
    double *y = nullptr;       // m
    double2 *hat = nullptr;    // scratch half spectrum
    // Arnoldi step j (operator, Gram-Schmidt, norm, scaling) captured as a CUDA
    // graph the first time it runs: its buffers are the same at every step.
    std::vector<cudaGraphExec_t> arnoldi;
    std::vector<int> arnoldi_launches;
    const double *arnoldi_mob = nullptr;   // the mobility field the graphs read
};

void psmob_gmres_release(PsMob *s) {
    PsGmres *g = s->gm;
    if(!g) return;
    for(double *p : {g->b, g->x, g->rhs, g->Mx, g->r, g->w, g->Av, g->V, g->part, g->h, g->y}) cudaFree(p);
    cudaFree(g->hat);
    for(cudaGraphExec_t x : g->arnoldi)
        if(x) cudaGraphExecDestroy(x);
    delete g;
    s->gm = nullptr;
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

double read_slot(Ctx &c, const double *slot) {
    double v = 0.0;
    if(c.e == cudaSuccess) c.e = cudaMemcpyAsync(&v, slot, sizeof(double), cudaMemcpyDeviceToHost, c.st);
    if(c.e == cudaSuccess) c.e = cudaStreamSynchronize(c.st);
    return v;
}

// out = D i k_d-gradients of `in_hat`, fluxes M grad, divergence, C2R: out_real = C2R(div_hat) (unnormalised)
void div_M_grad(Ctx &c, const double2 *in_hat, double *out_real) {
    PsMob *s = c.s;
    const long long rn = s->bins * s->S;
    for(int d = 0; d < s->g.dims && c.e == cudaSuccess; d++) {
        c.e = psmob_grad(s, in_hat, d, c.st);
        c.nl++;
        if(c.e == cudaSuccess) c.e = spectral_c2r(s->eng, s->tmp_hat, s->tmp, c.st, &c.nl);
        if(c.e == cudaSuccess) {
            fluxM_kernel<<<vgrid(rn), 256, 0, c.st>>>(s->tmp, c.mob, rn, (double) s->bins);
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
        applyA_final_kernel<<<vgrid(rn), 256, 0, c.st>>>(x, s->fder, s->p.dt, (double) s->bins, rn, Ax);
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
        div_kernel<<<vgrid(c.g->n), 256, 0, c.st>>>(z, nullptr, (double) s->bins, c.g->n, z);
        c.nl++;
        c.e = cudaGetLastError();
    }
}

void apply_M(Ctx &c, const double *v, double *out) {
    apply_A(c, v, c.g->Av);
    apply_Pinv(c, c.g->Av, out);
}

// Arnoldi step j: w = M V_j, modified Gram-Schmidt against V_0..V_j (each
// coefficient read on the device by the next update), h_{j+1} = |w|,
// V_{j+1} = w / h_{j+1}.  Enqueued as one graph launch instead of 30-odd
// kernel launches.
void arnoldi_record(Ctx &c, int j) {
    PsGmres *g = c.g;
    const long long n = g->n;
    const int vg = vgrid(n);
    apply_M(c, g->V + (size_t) j * n, g->w);
    for(int i = 0; i <= j && c.e == cudaSuccess; i++) {
        dot_dev(c, g->w, g->V + (size_t) i * n, g->h + i, false);
        axpy_dev_kernel<<<vg, 256, 0, c.st>>>(g->w, g->h + i, g->V + (size_t) i * n, n);
        c.nl++;
    }
    dot_dev(c, g->w, g->w, g->h + j + 1, true);
    div_kernel<<<vg, 256, 0, c.st>>>(g->w, g->h + j + 1, 0.0, n, g->V + (size_t) (j + 1) * n);
    c.nl++;
    if(c.e == cudaSuccess) c.e = cudaGetLastError();
}

void arnoldi_step(Ctx &c, int j) {
    PsGmres *g = c.g;
    if(c.e != cudaSuccess) return;
    if(g->arnoldi_mob != c.mob) {   // a new mobility buffer: record afresh
        for(cudaGraphExec_t &x : g->arnoldi)
            if(x) {
                cudaGraphExecDestroy(x);
                x = nullptr;
            }
        g->arnoldi_mob = c.mob;
    }
    if((int) g->arnoldi.size() < g->m) {
        g->arnoldi.resize(g->m, nullptr);
        g->arnoldi_launches.resize(g->m, 0);
    }
    if(!g->arnoldi[j]) {
        Ctx rc{c.s, g, c.mob, c.st};
        cudaGraph_t graph = nullptr;
        rc.e = cudaStreamBeginCapture(c.st, cudaStreamCaptureModeThreadLocal);
        if(rc.e != cudaSuccess) {
            c.e = rc.e;
            return;
        }
        arnoldi_record(rc, j);
        cudaError_t ee = cudaStreamEndCapture(c.st, &graph);
        if(rc.e == cudaSuccess) rc.e = ee;
        if(rc.e == cudaSuccess) rc.e = cudaGraphInstantiate(&g->arnoldi[j], graph, 0);
        if(graph) cudaGraphDestroy(graph);
        if(rc.e != cudaSuccess) {
            g->arnoldi[j] = nullptr;
            c.e = rc.e;
            return;
        }
        g->arnoldi_launches[j] = rc.nl;
    }
    c.e = cudaGraphLaunch(g->arnoldi[j], c.st);
    c.nl += g->arnoldi_launches[j];
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
        bool ok = cudaMalloc(&g->b, vb) == cudaSuccess && cudaMalloc(&g->x, vb) == cudaSuccess &&
                  cudaMalloc(&g->rhs, vb) == cudaSuccess && cudaMalloc(&g->Mx, vb) == cudaSuccess &&
                  cudaMalloc(&g->r, vb) == cudaSuccess && cudaMalloc(&g->w, vb) == cudaSuccess &&
                  cudaMalloc(&g->Av, vb) == cudaSuccess && cudaMalloc(&g->V, vb * (m + 1)) == cudaSuccess &&
                  cudaMalloc(&g->part, sizeof(double) * DOT_BLOCKS) == cudaSuccess &&
                  cudaMalloc(&g->h, sizeof(double) * (m + 4)) == cudaSuccess &&
                  cudaMalloc(&g->y, sizeof(double) * m) == cudaSuccess &&
                  cudaMalloc(&g->hat, sizeof(double2) * (size_t) s->hall) == cudaSuccess;
        s->gm = g;
        if(!ok) {
            cudaGetLastError();
            psmob_gmres_release(s);
            return cudaErrorMemoryAllocation;
        }
    }
    PsGmres *g = s->gm;
    Ctx c{s, g, mob, st};
    const int vg = vgrid(n);
    const double dt = s->p.dt, tol = s->p.gmres_tol;
    // 0) M0 for the preconditioner; 1-3) the right-hand side
    psmob_m0(s, mob, st);
    c.nl += 2;
    c.e = launch_der_bulk(s->m, rho, s->fder, s->bins, st);
    c.nl++;
    if(c.e == cudaSuccess) {
        g_kernel<<<vg, 256, 0, st>>>(s->fder, rho, s->p.splitting_S, n, s->tmp);
        c.nl++;
        c.e = cudaGetLastError();
    }
    if(c.e == cudaSuccess) c.e = spectral_r2c(s->eng, s->tmp, s->mu_hat, st, &c.nl);
    div_M_grad(c, s->mu_hat, s->fder);
    if(c.e == cudaSuccess) {
        rhs_kernel<<<vg, 256, 0, st>>>(rho, s->fder, dt, (double) s->bins, n, g->b);
        c.nl++;
        c.e = cudaGetLastError();
    }
    if(c.e == cudaSuccess) c.e = cudaMemcpyAsync(g->x, rho, sizeof(double) * n, cudaMemcpyDeviceToDevice, st);

    // 4) left-preconditioned restarted GMRES (:537-662)
    double *slot_beta = g->h + m + 1, *slot_rhs = g->h + m + 2;
    apply_Pinv(c, g->b, g->rhs);
    apply_M(c, g->x, g->Mx);
    if(c.e == cudaSuccess) {
        sub_kernel<<<vg, 256, 0, st>>>(g->rhs, g->Mx, n, g->r);
        c.nl++;
        c.e = cudaGetLastError();
    }
    dot_dev(c, g->rhs, g->rhs, slot_rhs, true);
    const double rhs_norm = std::max(read_slot(c, slot_rhs), 1e-30);
    dot_dev(c, g->r, g->r, slot_beta, true);
    double beta = read_slot(c, slot_beta);
    double rel = beta / rhs_norm;
    int iter_total = 0;
    if(!(rel < tol)) {
        std::vector<double> H((size_t) (m + 1) * m), cs(m), sn(m), gv(m + 1), y(m), col(m + 2);
        while(iter_total < s->p.gmres_max_iter && c.e == cudaSuccess) {
            std::fill(H.begin(), H.end(), 0.0);
            std::fill(cs.begin(), cs.end(), 0.0);
            std::fill(sn.begin(), sn.end(), 0.0);
            std::fill(gv.begin(), gv.end(), 0.0);
            div_kernel<<<vg, 256, 0, st>>>(g->r, nullptr, beta, n, g->V);
            c.nl++;
            gv[0] = beta;
            int j_end = 0;
            for(int j = 0; j < m && iter_total < s->p.gmres_max_iter; j++, iter_total++) {
                arnoldi_step(c, j);
                if(c.e == cudaSuccess)
                    c.e = cudaMemcpyAsync(col.data(), g->h, sizeof(double) * (j + 2), cudaMemcpyDeviceToHost, st);
                if(c.e == cudaSuccess) c.e = cudaStreamSynchronize(st);
                if(c.e != cudaSuccess) break;
                for(int i = 0; i <= j + 1; i++) H[(size_t) i * m + j] = col[i];
                if(!(H[(size_t) (j + 1) * m + j] > 1e-30)) {
                    j_end = j + 1;   // happy breakdown
                    break;
                }
                for(int i = 0; i < j; i++) {
                    double t1 = cs[i] * H[(size_t) i * m + j] + sn[i] * H[(size_t) (i + 1) * m + j];
                    double t2 = -sn[i] * H[(size_t) i * m + j] + cs[i] * H[(size_t) (i + 1) * m + j];
                    H[(size_t) i * m + j] = t1;
                    H[(size_t) (i + 1) * m + j] = t2;
                }
                double a = H[(size_t) j * m + j], b2 = H[(size_t) (j + 1) * m + j];
                double den = std::sqrt(a * a + b2 * b2);
                cs[j] = (den > 0) ? (a / den) : 1.0;
                sn[j] = (den > 0) ? (b2 / den) : 0.0;
                H[(size_t) j * m + j] = cs[j] * a + sn[j] * b2;
                H[(size_t) (j + 1) * m + j] = 0.0;
                double gj = gv[j];
                gv[j] = cs[j] * gj;
                gv[j + 1] = -sn[j] * gj;
                rel = std::abs(gv[j + 1]) / rhs_norm;
                if(rel < tol) {
                    j_end = j + 1;
                    break;
                }
                j_end = j + 1;
            }
            if(c.e != cudaSuccess) break;
            for(int i = j_end - 1; i >= 0; i--) {
                double sum = gv[i];
                for(int k = i + 1; k < j_end; k++) sum -= H[(size_t) i * m + k] * y[k];
                y[i] = sum / H[(size_t) i * m + i];
            }
            c.e = cudaMemcpyAsync(g->y, y.data(), sizeof(double) * std::max(1, j_end), cudaMemcpyHostToDevice, st);
            if(c.e == cudaSuccess) {
                xupdate_kernel<<<vg, 256, 0, st>>>(g->x, g->V, g->y, j_end, n);
                c.nl++;
                c.e = cudaGetLastError();
            }
            apply_M(c, g->x, g->Mx);
            if(c.e == cudaSuccess) {
                sub_kernel<<<vg, 256, 0, st>>>(g->rhs, g->Mx, n, g->r);
                c.nl++;
                c.e = cudaGetLastError();
            }
            dot_dev(c, g->r, g->r, slot_beta, true);
            beta = read_slot(c, slot_beta);   // also orders the host y buffer's reuse after the copy
            rel = beta / rhs_norm;
            if(rel < tol) break;
        }
    }
    // 5-6) rho = x, and its transform for a later simple step
    if(c.e == cudaSuccess) c.e = cudaMemcpyAsync(rho, g->x, sizeof(double) * n, cudaMemcpyDeviceToDevice, st);
    if(c.e == cudaSuccess) c.e = spectral_r2c(s->eng, rho, s->rho_hat, st, &c.nl);
    *launches += c.nl;
    return c.e;
}

}  // namespace chgb
