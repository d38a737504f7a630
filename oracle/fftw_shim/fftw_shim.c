/*
 * fftw_shim.c — the FFTW-API shim's implementation on top of the oracle FFT.
 * Supports what the reference uses: unit strides, no embedding, `howmany`
 * contiguous transforms (src/integrators/PseudospectralCPU.cpp:91-99).
 *
 * TEST INFRASTRUCTURE ONLY.
 */
#include "fftw3.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../och_fft.h"

struct chgb_fftw_shim_plan {
    int r2c;
    int rank;
    int n[8];
    int howmany;
    void *in, *out;
    int idist, odist;
};

static fftw_plan make_plan(int r2c, int rank, const int *n, int howmany, void *in, const int *inembed,
                           int istride, int idist, void *out, const int *onembed, int ostride, int odist) {
    if(rank < 1 || rank > 8 || inembed || onembed || istride != 1 || ostride != 1) {
        fprintf(stderr, "fftw shim: unsupported plan (rank %d, strides %d/%d)\n", rank, istride, ostride);
        abort();
    }
    fftw_plan p = (fftw_plan) calloc(1, sizeof(*p));
    p->r2c = r2c;
    p->rank = rank;
    memcpy(p->n, n, sizeof(int) * (size_t) rank);
    p->howmany = howmany;
    p->in = in;
    p->out = out;
    p->idist = idist;
    p->odist = odist;
    return p;
}

fftw_plan fftw_plan_many_dft_r2c(int rank, const int *n, int howmany, double *in, const int *inembed,
                                 int istride, int idist, fftw_complex *out, const int *onembed, int ostride,
                                 int odist, unsigned flags) {
    (void) flags;
    return make_plan(1, rank, n, howmany, in, inembed, istride, idist, out, onembed, ostride, odist);
}

fftw_plan fftw_plan_many_dft_c2r(int rank, const int *n, int howmany, fftw_complex *in, const int *inembed,
                                 int istride, int idist, double *out, const int *onembed, int ostride, int odist,
                                 unsigned flags) {
    (void) flags;
    return make_plan(0, rank, n, howmany, in, inembed, istride, idist, out, onembed, ostride, odist);
}

void fftw_execute(const fftw_plan p) {
    if(p->r2c) {
        och_rfftn(p->rank, p->n, p->howmany, (const double *) p->in, (size_t) p->idist, (double *) p->out,
                  (size_t) p->odist);
    }
    else {
        och_irfftn(p->rank, p->n, p->howmany, (const double *) p->in, (size_t) p->idist, (double *) p->out,
                   (size_t) p->odist);
    }
}

void fftw_destroy_plan(fftw_plan p) { free(p); }

void fftw_cleanup(void) {}
