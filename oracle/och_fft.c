/*
 * och_fft.c — plain-C FP64 multi-dimensional real FFT for the oracle.
 *
 * TEST INFRASTRUCTURE ONLY: this file is part of the CPU oracle that checks
 * the CUDA path.  Nothing in the product links or calls it.
 *
 * It reproduces the transform semantics that the reference's pseudospectral
 * integrator asks of FFTW (src/integrators/PseudospectralCPU.cpp:90-99):
 *   - fftw_plan_many_dft_r2c: rank-d forward real transform, sign -1,
 *     unnormalised, row-major, the LAST (fastest) dimension halved to n/2+1;
 *   - fftw_plan_many_dft_c2r: the inverse, sign +1, unnormalised;
 *   - `howmany` contiguous transforms, input distance idist, output odist,
 *     unit stride.
 * FFTW3 itself is not available; the algorithm here is the textbook
 * iterative radix-2 decimation-in-time Cooley–Tukey FFT with directly
 * evaluated twiddles (no recurrences), which keeps the error at a few ulp.
 */
#include "och_fft.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

static int ilog2_exact(int n) {
    int l = 0;
    while((1 << l) < n) l++;
    return ((1 << l) == n) ? l : -1;
}

/* In-place complex FFT of n (power of two) interleaved values, sign = -1 or +1. */
void och_fft_c2c_inplace(double *a, int n, int sign) {
    int logn = ilog2_exact(n);
    if(logn < 0 || n < 2) return;
    /* bit reversal permutation */
    for(int i = 1, j = 0; i < n; i++) {
        int bit = n >> 1;
        for(; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if(i < j) {
            double tr = a[2 * i], ti = a[2 * i + 1];
            a[2 * i] = a[2 * j];
            a[2 * i + 1] = a[2 * j + 1];
            a[2 * j] = tr;
            a[2 * j + 1] = ti;
        }
    }
    for(int len = 2; len <= n; len <<= 1) {
        int half = len >> 1;
        for(int k = 0; k < half; k++) {
            double ang = 2.0 * M_PI * (double) k / (double) len;
            double wr = cos(ang);
            double wi = sign * sin(ang);
            for(int i = 0; i < n; i += len) {
                double *u = a + 2 * (i + k);
                double *v = a + 2 * (i + k + half);
                double vr = v[0] * wr - v[1] * wi;
                double vi = v[0] * wi + v[1] * wr;
                v[0] = u[0] - vr;
                v[1] = u[1] - vi;
                u[0] += vr;
                u[1] += vi;
            }
        }
    }
}

/* Complex FFT along one axis of a row-major complex array with `dims`
 * extents; every other axis is iterated over. */
static void fft_axis(double *data, int rank, const int *ext, int axis, int sign, double *line) {
    size_t inner = 1;
    for(int d = axis + 1; d < rank; d++) inner *= (size_t) ext[d];
    size_t outer = 1;
    for(int d = 0; d < axis; d++) outer *= (size_t) ext[d];
    int n = ext[axis];
    for(size_t o = 0; o < outer; o++) {
        for(size_t in = 0; in < inner; in++) {
            double *base = data + 2 * (o * (size_t) n * inner + in);
            for(int i = 0; i < n; i++) {
                line[2 * i] = base[2 * (size_t) i * inner];
                line[2 * i + 1] = base[2 * (size_t) i * inner + 1];
            }
            och_fft_c2c_inplace(line, n, sign);
            for(int i = 0; i < n; i++) {
                base[2 * (size_t) i * inner] = line[2 * i];
                base[2 * (size_t) i * inner + 1] = line[2 * i + 1];
            }
        }
    }
}

static size_t prod(int rank, const int *n) {
    size_t p = 1;
    for(int d = 0; d < rank; d++) p *= (size_t) n[d];
    return p;
}

void och_rfftn(int rank, const int *n, int howmany, const double *in, size_t idist,
               double *out, size_t odist) {
    int last = n[rank - 1];
    int hl = last / 2 + 1;
    size_t rows = prod(rank - 1, n);
    int maxn = 1;
    for(int d = 0; d < rank; d++) if(n[d] > maxn) maxn = n[d];
    double *line = (double *) malloc(sizeof(double) * 2 * (size_t) maxn);
    int *hext = (int *) malloc(sizeof(int) * (size_t) rank);
    for(int d = 0; d < rank; d++) hext[d] = n[d];
    hext[rank - 1] = hl;
    for(int b = 0; b < howmany; b++) {
        const double *src = in + (size_t) b * idist;
        double *dst = out + 2 * (size_t) b * odist;
        /* real rows along the last axis */
        for(size_t r = 0; r < rows; r++) {
            for(int i = 0; i < last; i++) {
                line[2 * i] = src[r * (size_t) last + i];
                line[2 * i + 1] = 0.0;
            }
            och_fft_c2c_inplace(line, last, -1);
            memcpy(dst + 2 * r * (size_t) hl, line, sizeof(double) * 2 * (size_t) hl);
        }
        for(int axis = rank - 2; axis >= 0; axis--) {
            fft_axis(dst, rank, hext, axis, -1, line);
        }
    }
    free(hext);
    free(line);
}

void och_irfftn(int rank, const int *n, int howmany, const double *in, size_t idist,
                double *out, size_t odist) {
    int last = n[rank - 1];
    int hl = last / 2 + 1;
    size_t rows = prod(rank - 1, n);
    size_t hsize = rows * (size_t) hl;
    int maxn = 1;
    for(int d = 0; d < rank; d++) if(n[d] > maxn) maxn = n[d];
    double *line = (double *) malloc(sizeof(double) * 2 * (size_t) maxn);
    double *tmp = (double *) malloc(sizeof(double) * 2 * hsize);
    int *hext = (int *) malloc(sizeof(int) * (size_t) rank);
    for(int d = 0; d < rank; d++) hext[d] = n[d];
    hext[rank - 1] = hl;
    for(int b = 0; b < howmany; b++) {
        const double *src = in + 2 * (size_t) b * idist;
        double *dst = out + (size_t) b * odist;
        memcpy(tmp, src, sizeof(double) * 2 * hsize);
        for(int axis = 0; axis <= rank - 2; axis++) {
            fft_axis(tmp, rank, hext, axis, +1, line);
        }
        for(size_t r = 0; r < rows; r++) {
            const double *h = tmp + 2 * r * (size_t) hl;
            /* Hermitian extension of the half spectrum along the last axis;
             * the imaginary parts of the k=0 and k=n/2 bins do not reach the
             * real output. */
            for(int k = 0; k < hl; k++) {
                line[2 * k] = h[2 * k];
                line[2 * k + 1] = h[2 * k + 1];
            }
            for(int k = hl; k < last; k++) {
                line[2 * k] = h[2 * (last - k)];
                line[2 * k + 1] = -h[2 * (last - k) + 1];
            }
            och_fft_c2c_inplace(line, last, +1);
            for(int i = 0; i < last; i++) dst[r * (size_t) last + i] = line[2 * i];
        }
    }
    free(hext);
    free(tmp);
    free(line);
}
