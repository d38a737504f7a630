// sq.h — structure factor S(q) of 2D boxes (sq.cu).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

namespace chgb {

// Shells of the half spectrum of an N x N box, sorted for fixed-order reductions.
struct SqPlan {
    int N = 0, nbins = 0;
    long long modes = 0;              // N * (N/2 + 1)
    std::vector<double> wcount;       // full-spectrum modes per shell
    int *d_order = nullptr;           // (mode << 1 | counted twice), sorted by shell
    int *d_offsets = nullptr;         // nbins + 1
    double *d_wcount = nullptr;
    int *d_shell = nullptr;           // shell of every half-spectrum mode
    double *d_sq = nullptr;           // nbins results
    double *d_coef = nullptr;         // nbins seed coefficients
};

int sq_nbins(int N);
int sq_shell_of(int kx, int ky);
SqPlan *sq_plan_create(int N, std::string &err);
void sq_plan_destroy(SqPlan *p);
// S(q) of the scaled half spectrum `hat` (psi_t = rho_hat / cells) into p->d_sq.
cudaError_t sq_compute(const SqPlan *p, const double2 *hat, double cells, cudaStream_t st);
// R2C of dL/drho for a loss on S(q) with gradient dl_dsq (host, nbins): into `out` (half spectrum).
cudaError_t sq_seed(const SqPlan *p, const double2 *hat, double cells, const double *dl_dsq, double2 *out,
                    cudaStream_t st);

}  // namespace chgb
