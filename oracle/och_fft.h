/*
 * och_fft.h — oracle FFT (test infrastructure only; never linked into the product).
 */
#ifndef OCH_FFT_H
#define OCH_FFT_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* In-place complex FFT of n interleaved (re, im) values, n a power of two. */
void och_fft_c2c_inplace(double *a, int n, int sign);

/*
 * Rank-d forward real-to-complex transform, FFTW r2c semantics: row-major,
 * last dimension halved to n[rank-1]/2+1, sign -1, unnormalised.  `howmany`
 * transforms, real inputs `idist` doubles apart, complex outputs `odist`
 * complex values apart.  `out` holds interleaved (re, im).
 */
void och_rfftn(int rank, const int *n, int howmany, const double *in, size_t idist,
               double *out, size_t odist);

/* The matching complex-to-real inverse, sign +1, unnormalised.  `in` is not modified. */
void och_irfftn(int rank, const int *n, int howmany, const double *in, size_t idist,
                double *out, size_t odist);

#ifdef __cplusplus
}
#endif

#endif
