// sq.cu — radially averaged structure factor S(q) of a 2D box on the device.
//
// Definition of the reference's analysis script (utils/sq_from_traj.py:72-103):
// subtract the mean, S(k) = |FFT2(phi)|^2 / N_cells over the full spectrum,
// shell index rint(|k| / dq) with dq = 2 pi / (L dx), S(q) = shell mean.
// Here the spectrum is the half spectrum psi_t = rho_hat / N_cells the
// pseudospectral state already holds (euler boxes get one forward transform),
// so S(k) = N_cells |psi_t(k)|^2 with weight 2 for the modes whose mirror is
// not stored and the mean removed by dropping k = 0.  Shell indices are exact
// integers (rint(sqrt(i^2 + j^2)) never ties); modes are pre-sorted by shell
// and each shell is one CTA's fixed-order reduction, so S(q) is bit-for-bit
// reproducible.
#include <cmath>
#include <vector>

#include "kernels.h"
#include "sq.h"

namespace chgb {

namespace {

__global__ void __launch_bounds__(256) sq_shell_kernel(const double2 *__restrict__ hat, const int *__restrict__ order,
                                                       const int *__restrict__ offsets, const double *__restrict__ wcount,
                                                       double scale, double *__restrict__ sq) {
    const int b = blockIdx.x;
    const int lo = offsets[b], hi = offsets[b + 1];
    double acc = 0.0;
    for(int i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        int e = order[i];
        int mode = e >> 1;
        if(mode == 0) continue;   // k = 0: the mean, removed before the transform in the reference
        double w = (e & 1) ? 2.0 : 1.0;
        double2 f = hat[mode];
        acc += w * (f.x * f.x + f.y * f.y);
    }
    __shared__ double red[256];
    red[threadIdx.x] = acc;
    __syncthreads();
    for(int s = blockDim.x / 2; s > 0; s >>= 1) {
        if(threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if(threadIdx.x == 0) sq[b] = (wcount[b] > 0.0) ? red[0] * scale / wcount[b] : 0.0;
}

// lambda_t-seed of a loss on S(q): out_hat[k] = 2 N_cells (dL/dS_b / n_b) psi_t[k]
// for k != 0 (the mean of the field does not enter S(q)).
__global__ void sq_seed_kernel(const double2 *__restrict__ hat, const int *__restrict__ shell,
                               const double *__restrict__ coef, long long n, double2 *__restrict__ out) {
    for(long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
        int b = shell[i];
        double c = (i == 0) ? 0.0 : coef[b];
        double2 f = hat[i];
        out[i] = make_double2(c * f.x, c * f.y);
    }
}

}  // namespace

int sq_nbins(int N) {
    // shell of the corner mode (N/2, N/2) + 1
    long long s = 2LL * (N / 2) * (N / 2);
    long long r = (long long) std::floor(std::sqrt((double) s));
    while(r * r > s) r--;
    while((r + 1) * (r + 1) <= s) r++;
    long long shell = (s - r * r > r) ? r + 1 : r;   // rint(sqrt(s)); sqrt(s) is never a half-integer
    return (int) shell + 1;
}

int sq_shell_of(int kx, int ky) {
    long long s = (long long) kx * kx + (long long) ky * ky;
    long long r = (long long) std::floor(std::sqrt((double) s));
    while(r * r > s) r--;
    while((r + 1) * (r + 1) <= s) r++;
    return (int) ((s - r * r > r) ? r + 1 : r);
}

SqPlan *sq_plan_create(int N, std::string &err) {
    const int H = N / 2 + 1;
    const long long modes = (long long) N * H;
    const int nb = sq_nbins(N);
    std::vector<int> shell(modes), order, offsets(nb + 1, 0);
    std::vector<double> wcount(nb, 0.0);
    std::vector<std::vector<int>> per(nb);
    for(int yi = 0; yi < N; yi++) {
        int ky = (yi < N / 2) ? yi : yi - N;
        for(int kx = 0; kx < H; kx++) {
            long long m = (long long) yi * H + kx;
            int b = sq_shell_of(kx, ky);
            bool twice = (kx != 0 && kx != N / 2);
            shell[m] = b;
            per[b].push_back((int) (m * 2 + (twice ? 1 : 0)));
            wcount[b] += twice ? 2.0 : 1.0;
        }
    }
    for(int b = 0; b < nb; b++) {
        offsets[b] = (int) order.size();
        order.insert(order.end(), per[b].begin(), per[b].end());
    }
    offsets[nb] = (int) order.size();
    SqPlan *p = new SqPlan();
    p->N = N;
    p->nbins = nb;
    p->modes = modes;
    p->wcount = wcount;
    bool ok = cudaMalloc(&p->d_order, sizeof(int) * order.size()) == cudaSuccess &&
              cudaMalloc(&p->d_offsets, sizeof(int) * offsets.size()) == cudaSuccess &&
              cudaMalloc(&p->d_wcount, sizeof(double) * nb) == cudaSuccess &&
              cudaMalloc(&p->d_shell, sizeof(int) * modes) == cudaSuccess &&
              cudaMalloc(&p->d_sq, sizeof(double) * nb) == cudaSuccess &&
              cudaMalloc(&p->d_coef, sizeof(double) * nb) == cudaSuccess;
    ok = ok && cudaMemcpy(p->d_order, order.data(), sizeof(int) * order.size(), cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(p->d_offsets, offsets.data(), sizeof(int) * offsets.size(), cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(p->d_wcount, wcount.data(), sizeof(double) * nb, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(p->d_shell, shell.data(), sizeof(int) * modes, cudaMemcpyHostToDevice) == cudaSuccess;
    if(!ok) {
        cudaGetLastError();
        sq_plan_destroy(p);
        err = "S(q) plan allocation failed";
        return nullptr;
    }
    return p;
}

void sq_plan_destroy(SqPlan *p) {
    if(!p) return;
    cudaFree(p->d_order);
    cudaFree(p->d_offsets);
    cudaFree(p->d_wcount);
    cudaFree(p->d_shell);
    cudaFree(p->d_sq);
    cudaFree(p->d_coef);
    delete p;
}

cudaError_t sq_compute(const SqPlan *p, const double2 *hat, double cells, cudaStream_t st) {
    // S(k) = |F|^2 / cells with F = cells * psi_t  ->  cells * |psi_t|^2
    sq_shell_kernel<<<p->nbins, 256, 0, st>>>(hat, p->d_order, p->d_offsets, p->d_wcount, cells, p->d_sq);
    return cudaGetLastError();
}

cudaError_t sq_seed(const SqPlan *p, const double2 *hat, double cells, const double *dl_dsq, double2 *out,
                    cudaStream_t st) {
    // dS_b / d psi = (2 / cells) sum_k (1/n_b) Re(F_k e^{ik.x}); in the scaled half
    // spectrum of lambda (lambda_hat = R2C(lambda)) that is 2 cells psi_t[k] / n_b.
    std::vector<double> coef(p->nbins);
    for(int b = 0; b < p->nbins; b++) coef[b] = (p->wcount[b] > 0.0) ? 2.0 * cells * dl_dsq[b] / p->wcount[b] : 0.0;
    cudaError_t e = cudaMemcpyAsync(p->d_coef, coef.data(), sizeof(double) * p->nbins, cudaMemcpyHostToDevice, st);
    if(e != cudaSuccess) return e;
    e = cudaStreamSynchronize(st);   // coef is a host temporary
    if(e != cudaSuccess) return e;
    int grid = (int) std::min<long long>((p->modes + 255) / 256, 152 * 8);
    sq_seed_kernel<<<grid, 256, 0, st>>>(hat, p->d_shell, p->d_coef, p->modes, out);
    return cudaGetLastError();
}

}  // namespace chgb
