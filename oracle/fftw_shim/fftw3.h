/*
 * fftw3.h — FFTW-API shim used only to compile the reference's CPU sources
 * into the test oracle (oracle/_ref).  FFTW3 is not installed on this
 * machine; the reference's pseudospectral integrators use exactly the
 * symbols declared here (src/integrators/PseudospectralCPU.cpp:93-108,
 * src/integrators/PseudospectralMobilityCPU.cpp), with the signatures of the
 * public FFTW 3 API so that the reference sources compile unmodified.
 * The transforms are the oracle's own FFT (oracle/och_fft.c).
 *
 * TEST INFRASTRUCTURE ONLY.
 */
#ifndef CHGB_FFTW_SHIM_H
#define CHGB_FFTW_SHIM_H

#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef struct chgb_fftw_shim_plan *fftw_plan;

#define FFTW_ESTIMATE (1U << 6)

fftw_plan fftw_plan_many_dft_r2c(int rank, const int *n, int howmany, double *in, const int *inembed,
                                 int istride, int idist, fftw_complex *out, const int *onembed, int ostride,
                                 int odist, unsigned flags);

fftw_plan fftw_plan_many_dft_c2r(int rank, const int *n, int howmany, fftw_complex *in, const int *inembed,
                                 int istride, int idist, double *out, const int *onembed, int ostride, int odist,
                                 unsigned flags);

void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);
void fftw_cleanup(void);

#ifdef __cplusplus
}
#endif

#endif
