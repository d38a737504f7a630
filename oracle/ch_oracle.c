/*
 * ch_oracle.c — CPU oracle: plain-C restatement of the reference's FP64 CPU
 * hot path.  TEST INFRASTRUCTURE ONLY (see ch_oracle.h).
 *
 * Every function follows the reference file:line it names; the loop order and
 * the order of floating-point operations are kept where they decide the last
 * bits (neighbour summation order of the Laplacian, the three separate passes
 * of the explicit integrators).  Built with -ffp-contract=off so that the
 * result is the same on x86-64 and aarch64 hosts.
 */
#include "ch_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "och_fft.h"

#define SQR(x) ((x) * (x))
#define CUB(x) ((x) * (x) * (x))

/* ------------------------------------------------------------------------- */
/* drand48: POSIX.1 48-bit LCG, X' = (a X + c) mod 2^48, a = 0x5DEECE66D,    */
/* c = 0xB; srand48 sets the high 32 bits of X to the seed and the low 16 to */
/* 0x330E; drand48 returns X' / 2^48.  The reference seeds it once in        */
/* src/main.cpp:36 and draws from it in src/CahnHilliard.cpp:141.           */
/* ------------------------------------------------------------------------- */
void och_srand48(och_rand48 *r, int64_t seed) {
    r->x = (((uint64_t) seed & 0xFFFFFFFFull) << 16) | 0x330Eull;
}

double och_drand48(och_rand48 *r) {
    r->x = (0x5DEECE66Dull * r->x + 0xBull) & 0xFFFFFFFFFFFFull;
    return ldexp((double) r->x, -48);
}

/* src/CahnHilliard.cpp:133-161 */
void och_init_density(int dims, int N, int n_species, const double *densities, double initial_A,
                      int initial_N_peaks, double user_to_internal, och_rand48 *rng, double *rho) {
    int grid_size = N;
    for(int i = 1; i < dims; i++) grid_size *= N;
    double initial_k = 2 * M_PI * initial_N_peaks / (double) N;
    for(int bin = 0; bin < grid_size; bin++) {
        double modulation = initial_A * cos(initial_k * bin);
        for(int i = 0; i < n_species; i++) {
            double random_factor = (initial_N_peaks == 0) ? (och_drand48(rng) - 0.5)
                                                          : 1.0 + 0.02 * (och_drand48(rng) - 0.5);
            double average_rho = densities[i];
            if(average_rho != 0.0) {
                rho[i * grid_size + bin] = average_rho * (1.0 + 2.0 * modulation * random_factor);
            }
            else {
                rho[i * grid_size + bin] = 2.0 * modulation * random_factor;
            }
        }
    }
    double u3 = CUB(user_to_internal);
    for(int idx = 0; idx < grid_size; idx++) {
        for(int s = 0; s < n_species; s++) rho[s * grid_size + idx] /= u3;
    }
}

/* ------------------------------------------------------------------------- */
/* Models                                                                    */
/* ------------------------------------------------------------------------- */

/* src/models/SimpleWertheim.cpp:88-90 */
static double sw_X(const chgb_model_params *m, double rho) {
    double two_valence_delta = 2.0 * m->valence * m->delta;
    return (-1.0 + sqrt(1.0 + 2.0 * two_valence_delta * rho)) / (two_valence_delta * rho);
}

/* src/models/SalehWertheim.cpp:80-85 */
static double saleh_der_contribution(const chgb_model_params *m, const double *r, int species) {
    int half = m->saleh_valence[2] / 2;
    double delta = (species == 0) ? m->delta_AA : m->delta_BB;
    double rho_factor = delta * (m->saleh_valence[species] * r[species] + half * r[2]);
    double X = (-1.0 + sqrt(1.0 + 4.0 * rho_factor)) / (2.0 * rho_factor);
    return (rho_factor >= 0) ? log(X) : 0.0;
}

void och_der_bulk_free_energy(const chgb_model_params *m, int bins, const double *rho, double *rho_der) {
    if(m->kind == CHGB_MODEL_LANDAU) {
        /* src/models/Landau.cpp:46-53 */
        for(int idx = 0; idx < bins; idx++) {
            double op = rho[idx];
            rho_der[idx] = -m->epsilon * op + op * op * op;
        }
    }
    else if(m->kind == CHGB_MODEL_SIMPLE_WERTHEIM) {
        /* src/models/SimpleWertheim.cpp:40-53 */
        double reg = m->regularisation_delta;
        double log_delta = log(reg);
        for(int idx = 0; idx < bins; idx++) {
            double rho_tot = rho[idx];
            double der_f_ref = 2 * m->B2 * rho_tot;
            if(rho_tot < reg) {
                der_f_ref += log_delta + (rho_tot - reg) / reg;
            }
            else {
                der_f_ref += log(rho_tot);
            }
            double der_f_bond = (rho_tot > 0.) ? m->valence * log(sw_X(m, rho_tot)) : 0.0;
            rho_der[idx] = der_f_ref + der_f_bond;
        }
    }
    else if(m->kind == CHGB_MODEL_SALEH) {
        /* src/models/SalehWertheim.cpp:87-109; a species whose density is
         * exactly zero keeps the previous content of rho_der, as there. */
        int half = m->saleh_valence[2] / 2;
        for(int idx = 0; idx < bins; idx++) {
            double r[3] = {rho[idx], rho[bins + idx], rho[2 * bins + idx]};
            for(int s = 0; s < 3; s++) {
                if(r[s] != 0.) {
                    double rho_tot = 0.;
                    for(int t = 0; t < 3; t++) rho_tot += r[t];
                    double der_f_ref = log(r[s]) + 2.0 * m->B2 * rho_tot + 3.0 * m->B3 * SQR(rho_tot);
                    double der_f_bond;
                    if(s == 0) der_f_bond = m->saleh_valence[0] * saleh_der_contribution(m, r, 0);
                    else if(s == 1) der_f_bond = m->saleh_valence[1] * saleh_der_contribution(m, r, 1);
                    else der_f_bond = half * (saleh_der_contribution(m, r, 0) + saleh_der_contribution(m, r, 1));
                    rho_der[s * bins + idx] = der_f_ref + der_f_bond;
                }
            }
        }
    }
}

double och_bulk_free_energy(const chgb_model_params *m, int bins, const double *rho, int idx) {
    if(m->kind == CHGB_MODEL_LANDAU) {
        /* src/models/Landau.cpp:55-58 */
        double op = rho[idx];
        return -0.5 * m->epsilon * SQR(op) + 0.25 * SQR(SQR(op));
    }
    else if(m->kind == CHGB_MODEL_SIMPLE_WERTHEIM) {
        /* src/models/SimpleWertheim.cpp:71-86 */
        double r = rho[idx];
        double reg = m->regularisation_delta;
        double log_delta = log(reg);
        double f_ref = m->B2 * SQR(r);
        if(r < reg) {
            double a = 1 / (2.0 * reg);
            double b = log_delta - 1.0;
            double c = reg * (log_delta - 1.0) - a * SQR(reg) - b * reg;
            f_ref += a * SQR(r) + b * r + c;
        }
        else {
            f_ref += r * (log(r * m->density_conversion_factor) - 1.0);
        }
        double f_bond = (r > 0.) ? m->valence * r * (log(sw_X(m, r)) + 0.5 * (1. - sw_X(m, r))) : 0.0;
        return f_ref + f_bond;
    }
    else {
        /* src/models/SalehWertheim.cpp:47-78 */
        double r[3] = {rho[idx], rho[bins + idx], rho[2 * bins + idx]};
        int half = m->saleh_valence[2] / 2;
        double rho_tot = 0.;
        for(int t = 0; t < 3; t++) rho_tot += r[t];
        double mixing_S = 0.;
        for(int i = 0; i < 3; i++) {
            double x_i = r[i] / rho_tot;
            mixing_S += (x_i > 0) ? x_i * log(x_i) : 0;
        }
        double B2_contrib = m->B2 * rho_tot;
        double B3_contrib = 0.5 * m->B3 * SQR(rho_tot);
        double f_ref = rho_tot * (log(rho_tot * m->density_conversion_factor) - 1.0 + mixing_S + B2_contrib + B3_contrib);

        double rho_factor = m->delta_AA * (m->saleh_valence[0] * r[0] + half * r[2]);
        double X_1A = (-1.0 + sqrt(1.0 + 4.0 * rho_factor)) / (2.0 * rho_factor);
        double fe_part_1 = log(X_1A) - X_1A / 2.0 + 0.5;
        rho_factor = m->delta_BB * (m->saleh_valence[1] * r[1] + half * r[2]);
        double X_2B = (-1.0 + sqrt(1.0 + 4.0 * rho_factor)) / (2.0 * rho_factor);
        double fe_part_2 = log(X_2B) - X_2B / 2.0 + 0.5;
        double bonding = r[0] * m->saleh_valence[0] * fe_part_1 + r[1] * m->saleh_valence[1] * fe_part_2 +
                         r[2] * half * (fe_part_1 + fe_part_2);
        return f_ref + bonding;
    }
}

/* src/models/SimpleWertheim.cpp:104-111 */
void och_set_mobility(const chgb_model_params *m, int bins, const double *rho, double M0, double *mobility) {
    for(int idx = 0; idx < bins; idx++) {
        double rho_tot = rho[idx];
        double my_X = sw_X(m, rho_tot);
        double D = M0 * pow(my_X, (double) m->valence);
        mobility[idx] = rho_tot * D;
    }
}

/* ------------------------------------------------------------------------- */
/* Grid helpers: src/integrators/EulerCPU.cpp:39-55                          */
/* ------------------------------------------------------------------------- */
typedef struct grid {
    int dims, N, mask, bits, bins;
} grid;

static void fill_coords(const grid *g, int *coords, int idx) {
    for(int d = 0; d < g->dims; d++) {
        coords[d] = idx & g->mask;
        idx >>= g->bits;
    }
}

static int cell_idx(const grid *g, const int *coords) {
    int idx = 0, mul = 1;
    for(int d = 0; d < g->dims; d++) {
        idx += coords[d] * mul;
        mul <<= g->bits;
    }
    return idx;
}

/* src/integrators/EulerCPU.cpp:58-88.  The _k form takes the dimension as an
 * argument that the callers below pass as a constant, so that, inlined, its
 * loops unroll as the reference's template on `dims` does; the operations and
 * their order are the same for every caller. */
#define OCH_INLINE static inline __attribute__((always_inline))

OCH_INLINE double cell_laplacian_k(const grid *g, const double *f, int idx, double dx, int dims) {
    if(dims == 1) {
        int idx_m = (idx - 1 + g->N) & g->mask;
        int idx_p = (idx + 1) & g->mask;
        return (f[idx_m] + f[idx_p] - 2.0 * f[idx]) / SQR(dx);
    }
    int coords[3], cn[3];
    int t = idx;
    for(int d = 0; d < dims; d++) {
        coords[d] = t & g->mask;
        t >>= g->bits;
    }
    memcpy(cn, coords, sizeof(coords));
    double sum = 0.0;
    for(int d = 0; d < dims; d++) {
        int id;
        cn[d] = (coords[d] - 1 + g->N) & g->mask;
        id = 0;
        for(int e = dims - 1; e >= 0; e--) id = (id << g->bits) + cn[e];
        sum += f[id];
        cn[d] = (coords[d] + 1) & g->mask;
        id = 0;
        for(int e = dims - 1; e >= 0; e--) id = (id << g->bits) + cn[e];
        sum += f[id];
        cn[d] = coords[d];
    }
    return (sum - 2.0 * dims * f[idx]) / SQR(dx);
}

static double cell_laplacian(const grid *g, const double *f, int idx, double dx) {
    return cell_laplacian_k(g, f, idx, dx, g->dims);
}

OCH_INLINE void fill_coords_k(const grid *g, int *coords, int idx, int dims) {
    for(int d = 0; d < dims; d++) {
        coords[d] = idx & g->mask;
        idx >>= g->bits;
    }
}

OCH_INLINE int cell_idx_k(const grid *g, const int *coords, int dims) {
    int idx = 0;
    for(int e = dims - 1; e >= 0; e--) idx = (idx << g->bits) + coords[e];
    return idx;
}

/* ------------------------------------------------------------------------- */
/* Simulation box                                                            */
/* ------------------------------------------------------------------------- */
struct och_sim {
    chgb_params p;
    grid g;
    int S;
    double *rho, *mobility;
    double *gel;         /* gel mobility: the order parameter, one value per cell */
    double *scratch;     /* euler: rho_der; euler_mobility: mu */
    double *flux;        /* euler_mobility: dims values per cell and species */
    /* pseudospectral */
    int hat_grid_size;
    double *rho_hat, *rho_hat_copy, *f_der_hat; /* interleaved complex */
    double *sqr_wave_vectors, *dealiaser;
    double ps_M;
    int ps_M_set;
    /* pseudospectral_mobility */
    double *kcomp[3];                      /* signed wave-vector components per mode */
    double *mu_hat, *tmp_hat, *div_hat;    /* interleaved complex */
    double *tmp_real;                      /* bins x species */
    double M0[CHGB_MAX_SPECIES];
};

static void ps_rfft(och_sim *s, const double *in, double *out) {
    int n[3] = {s->g.N, s->g.N, s->g.N};
    och_rfftn(s->g.dims, n, s->S, in, (size_t) s->g.bins, out, (size_t) s->hat_grid_size);
}

static void ps_irfft(och_sim *s, const double *in, double *out) {
    int n[3] = {s->g.N, s->g.N, s->g.N};
    och_irfftn(s->g.dims, n, s->S, in, (size_t) s->hat_grid_size, out, (size_t) s->g.bins);
}

/* src/integrators/PseudospectralCPU.cpp:13-102 (wave vectors, dealiaser, initial rho_hat) */
static void ps_setup(och_sim *s) {
    int N = s->g.N, dims = s->g.dims;
    double dx = s->p.dx;
    s->hat_grid_size = N / 2 + 1;
    for(int i = 0; i < dims - 1; i++) s->hat_grid_size *= N;
    int hvs = s->hat_grid_size * s->S;
    s->rho_hat = (double *) calloc(2 * (size_t) hvs, sizeof(double));
    s->rho_hat_copy = (double *) calloc(2 * (size_t) hvs, sizeof(double));
    s->f_der_hat = (double *) calloc(2 * (size_t) hvs, sizeof(double));
    s->sqr_wave_vectors = (double *) calloc((size_t) hvs, sizeof(double));
    s->dealiaser = (double *) calloc((size_t) hvs, sizeof(double));
    double k_cut = N * M_PI / (N * dx) * 2.0 / 3.0;
    int k_idx = 0;
    for(int sp = 0; sp < s->S; sp++) {
        if(dims == 1) {
            for(int i = 0; i < s->hat_grid_size; i++) {
                double k = 2.0 * M_PI * i / (N * dx);
                s->dealiaser[k_idx] = (k <= k_cut) ? 1.0 : 0.0;
                s->sqr_wave_vectors[k_idx] = SQR(k);
                k_idx++;
            }
        }
        else if(dims == 2) {
            for(int kx_idx = 0; kx_idx < N; kx_idx++) {
                int kx = (kx_idx < N / 2) ? kx_idx : N - kx_idx;
                for(int ky = 0; ky < (N / 2 + 1); ky++) {
                    double k = 2.0 * M_PI * sqrt((double) (SQR(kx) + SQR(ky))) / (N * dx);
                    s->dealiaser[k_idx] = (k < k_cut) ? 1.0 : 0.0;
                    s->sqr_wave_vectors[k_idx] = SQR(k);
                    k_idx++;
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
                    for(int kz_idx = 0; kz_idx < (N / 2 + 1); kz_idx++) {
                        double kz = 2.0 * M_PI * kz_idx / (N * dx);
                        double k2 = SQR(kx) + SQR(ky) + SQR(kz);
                        double k = sqrt(k2);
                        s->dealiaser[k_idx] = (k <= k_cut) ? 1.0 : 0.0;
                        s->sqr_wave_vectors[k_idx] = k2;
                        k_idx++;
                    }
                }
            }
        }
    }
}

static void ps_forward_state(och_sim *s) {
    ps_rfft(s, s->rho, s->rho_hat);
    memcpy(s->rho_hat_copy, s->rho_hat, sizeof(double) * 2 * (size_t) s->hat_grid_size * s->S);
}

/* src/integrators/PseudospectralMobilityCPU.cpp:13-160: the same half-spectrum
 * layout as `pseudospectral`, signed wave-vector components per axis
 * (kcomp[0] along the slowest axis), k^2, and the dealiaser with k <= k_cut. */
static void psm_setup(och_sim *s) {
    int N = s->g.N, dims = s->g.dims;
    double dx = s->p.dx;
    s->hat_grid_size = N / 2 + 1;
    for(int i = 0; i < dims - 1; i++) s->hat_grid_size *= N;
    size_t hvs = (size_t) s->hat_grid_size * s->S;
    s->rho_hat = (double *) calloc(2 * hvs, sizeof(double));
    s->rho_hat_copy = (double *) calloc(2 * hvs, sizeof(double));
    s->f_der_hat = (double *) calloc(2 * hvs, sizeof(double));
    s->mu_hat = (double *) calloc(2 * hvs, sizeof(double));
    s->tmp_hat = (double *) calloc(2 * hvs, sizeof(double));
    s->div_hat = (double *) calloc(2 * hvs, sizeof(double));
    s->tmp_real = (double *) calloc((size_t) s->g.bins * s->S, sizeof(double));
    s->sqr_wave_vectors = (double *) calloc(hvs, sizeof(double));
    s->dealiaser = (double *) calloc(hvs, sizeof(double));
    for(int d = 0; d < dims; d++) s->kcomp[d] = (double *) calloc(hvs, sizeof(double));
    double k_cut = N * M_PI / (N * dx) * 2.0 / 3.0;
    size_t k_idx = 0;
    for(int sp = 0; sp < s->S; sp++) {
        if(dims == 1) {
            for(int i = 0; i < s->hat_grid_size; i++, k_idx++) {
                double kx = 2.0 * M_PI * i / (N * dx);
                s->dealiaser[k_idx] = (fabs(kx) <= k_cut) ? 1.0 : 0.0;
                s->kcomp[0][k_idx] = kx;
                s->sqr_wave_vectors[k_idx] = SQR(kx);
            }
        }
        else if(dims == 2) {
            for(int a = 0; a < N; a++) {
                int ai = (a < N / 2) ? a : (a - N);
                double kx = 2.0 * M_PI * ai / (N * dx);
                for(int b = 0; b < N / 2 + 1; b++, k_idx++) {
                    double ky = 2.0 * M_PI * b / (N * dx);
                    double k2 = SQR(kx) + SQR(ky);
                    s->dealiaser[k_idx] = (sqrt(k2) <= k_cut) ? 1.0 : 0.0;
                    s->kcomp[0][k_idx] = kx;
                    s->kcomp[1][k_idx] = ky;
                    s->sqr_wave_vectors[k_idx] = k2;
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
                        double k2 = SQR(kx) + SQR(ky) + SQR(kz);
                        s->dealiaser[k_idx] = (sqrt(k2) <= k_cut) ? 1.0 : 0.0;
                        s->kcomp[0][k_idx] = kx;
                        s->kcomp[1][k_idx] = ky;
                        s->kcomp[2][k_idx] = kz;
                        s->sqr_wave_vectors[k_idx] = k2;
                    }
                }
            }
        }
    }
}

/* (0 + i k) * z */
static inline void cmul_ik(double k, const double *z, double *out) {
    double re = 0.0 * z[0] - k * z[1];
    double im = 0.0 * z[1] + k * z[0];
    out[0] = re;
    out[1] = im;
}

/* src/integrators/PseudospectralMobilityCPU.cpp:236-310 (_evolve_simple) */
static void psm_evolve(och_sim *s) {
    const int dims = s->g.dims, S = s->S;
    const size_t bins = (size_t) s->g.bins, hgs = (size_t) s->hat_grid_size, hvs = hgs * S;
    const double dt = s->p.dt, Ssplit = s->p.splitting_S, k0 = s->p.k[0];
    const int dealias = s->p.use_dealias;
    /* reference mobility M0 = max over space, per species (:437-445) */
    for(int sp = 0; sp < S; sp++) {
        double m = 0.0;
        for(size_t i = 0; i < bins; i++) {
            double v = s->mobility[sp * bins + i];
            m = (m > v) ? m : v;
        }
        s->M0[sp] = m;
    }
    /* 1-2) bulk chemical potential and its transform */
    och_der_bulk_free_energy(&s->p.model, (int) bins, s->rho, s->scratch);
    ps_rfft(s, s->scratch, s->f_der_hat);
    /* 3) mu_hat = f_der_hat + 2 k q^2 rho_hat */
    for(size_t k = 0; k < hvs; k++) {
        double t = 2.0 * k0 * s->sqr_wave_vectors[k];
        double *mh = s->mu_hat + 2 * k;
        mh[0] = s->f_der_hat[2 * k] + t * s->rho_hat[2 * k];
        mh[1] = s->f_der_hat[2 * k + 1] + t * s->rho_hat[2 * k + 1];
        if(dealias) {
            mh[0] *= s->dealiaser[k];
            mh[1] *= s->dealiaser[k];
        }
    }
    memset(s->div_hat, 0, sizeof(double) * 2 * hvs);
    for(int d = 0; d < dims; d++) {
        /* 4) grad mu along d in real space */
        for(size_t k = 0; k < hvs; k++) {
            double *gh = s->tmp_hat + 2 * k;
            cmul_ik(s->kcomp[d][k], s->mu_hat + 2 * k, gh);
            if(dealias) {
                gh[0] *= s->dealiaser[k];
                gh[1] *= s->dealiaser[k];
            }
        }
        ps_irfft(s, s->tmp_hat, s->tmp_real);
        /* 5) flux (M - M0) grad mu */
        for(int sp = 0; sp < S; sp++) {
            for(size_t i = 0; i < bins; i++) {
                double g = s->tmp_real[sp * bins + i] / (double) bins;
                double dM = s->mobility[sp * bins + i] - s->M0[sp];
                s->tmp_real[sp * bins + i] = dM * g;
            }
        }
        /* 6) its transform and divergence */
        ps_rfft(s, s->tmp_real, s->tmp_hat);
        for(size_t k = 0; k < hvs; k++) {
            double *fh = s->tmp_hat + 2 * k;
            if(dealias) {
                fh[0] *= s->dealiaser[k];
                fh[1] *= s->dealiaser[k];
            }
            double t[2];
            cmul_ik(s->kcomp[d][k], fh, t);
            s->div_hat[2 * k] += t[0];
            s->div_hat[2 * k + 1] += t[1];
        }
    }
    /* 7) stabilised semi-implicit update (k_laplacian of species 0 for all, :302) */
    for(size_t k = 0; k < hvs; k++) {
        int sp = (int) (k / hgs);
        double k2 = s->sqr_wave_vectors[k];
        double k4 = SQR(k2);
        double M0 = s->M0[sp];
        double denom = 1.0 + dt * M0 * (Ssplit * k2 + 2.0 * k0 * k4);
        double c = dt * M0 * k2;
        double *rh = s->rho_hat + 2 * k, *rc = s->rho_hat_copy + 2 * k;
        const double *fh = s->f_der_hat + 2 * k, *dv = s->div_hat + 2 * k;
        double nr = ((rh[0] + dt * dv[0]) - c * (fh[0] - Ssplit * rh[0])) / denom;
        double ni = ((rh[1] + dt * dv[1]) - c * (fh[1] - Ssplit * rh[1])) / denom;
        rh[0] = nr;
        rh[1] = ni;
        rc[0] = nr / (double) bins;
        rc[1] = ni / (double) bins;
    }
    /* 8) back to real space */
    ps_irfft(s, s->rho_hat_copy, s->rho);
}

/* ---- pseudospectral_mobility, GMRES path (PseudospectralMobilityCPU.cpp:312-665) ---- */

/* out = C2R(i k_d * D * in_hat) / N for every axis, into grads[d] (bins x S each) */
static void psm_grad_real(och_sim *s, const double *in_hat, double **grads) {
    const size_t hvs = (size_t) s->hat_grid_size * s->S, n = (size_t) s->g.bins * s->S;
    for(int d = 0; d < s->g.dims; d++) {
        for(size_t k = 0; k < hvs; k++) {
            double *gh = s->tmp_hat + 2 * k;
            cmul_ik(s->kcomp[d][k], in_hat + 2 * k, gh);
            if(s->p.use_dealias) {
                gh[0] *= s->dealiaser[k];
                gh[1] *= s->dealiaser[k];
            }
        }
        ps_irfft(s, s->tmp_hat, grads[d]);
        for(size_t i = 0; i < n; i++) grads[d][i] /= (double) s->g.bins;
    }
}

/* div_hat = sum_d i k_d * D * R2C(M * grads[d]) (grads overwritten by the fluxes) */
static void psm_div_hat(och_sim *s, double **grads) {
    const size_t hvs = (size_t) s->hat_grid_size * s->S, n = (size_t) s->g.bins * s->S;
    for(int d = 0; d < s->g.dims; d++)
        for(size_t i = 0; i < n; i++) grads[d][i] = s->mobility[i] * grads[d][i];
    memset(s->div_hat, 0, sizeof(double) * 2 * hvs);
    for(int d = 0; d < s->g.dims; d++) {
        ps_rfft(s, grads[d], s->tmp_hat);
        for(size_t k = 0; k < hvs; k++) {
            double *fh = s->tmp_hat + 2 * k;
            if(s->p.use_dealias) {
                fh[0] *= s->dealiaser[k];
                fh[1] *= s->dealiaser[k];
            }
            double t[2];
            cmul_ik(s->kcomp[d][k], fh, t);
            s->div_hat[2 * k] += t[0];
            s->div_hat[2 * k + 1] += t[1];
        }
    }
}

/* _apply_Pinv (:440-466) */
static void psm_apply_pinv(och_sim *s, const double *r, double *z) {
    const size_t hgs = (size_t) s->hat_grid_size, hvs = hgs * s->S, n = (size_t) s->g.bins * s->S;
    ps_rfft(s, r, s->tmp_hat);
    for(size_t k = 0; k < hvs; k++) {
        int sp = (int) (k / hgs);
        double k2 = s->sqr_wave_vectors[k], k4 = k2 * k2;
        double denom = 1.0 + s->p.dt * s->M0[sp] * (s->p.splitting_S * k2 + 2.0 * s->p.k[0] * k4);
        s->tmp_hat[2 * k] /= denom;
        s->tmp_hat[2 * k + 1] /= denom;
    }
    ps_irfft(s, s->tmp_hat, z);
    for(size_t i = 0; i < n; i++) z[i] = z[i] / (double) s->g.bins;
}

/* _apply_A (:468-535): Ax = x - dt div(M grad((S - 2k lap) x)) */
static void psm_apply_A(och_sim *s, const double *x, double *Ax, double **grads) {
    const size_t hvs = (size_t) s->hat_grid_size * s->S, n = (size_t) s->g.bins * s->S;
    double *xh = s->mu_hat;   /* q_hat */
    ps_rfft(s, x, xh);
    for(size_t k = 0; k < hvs; k++) {
        double f = s->p.splitting_S + 2.0 * s->p.k[0] * s->sqr_wave_vectors[k];
        xh[2 * k] = f * xh[2 * k];
        xh[2 * k + 1] = f * xh[2 * k + 1];
        if(s->p.use_dealias) {
            xh[2 * k] *= s->dealiaser[k];
            xh[2 * k + 1] *= s->dealiaser[k];
        }
    }
    psm_grad_real(s, xh, grads);
    psm_div_hat(s, grads);
    ps_irfft(s, s->div_hat, s->tmp_real);
    for(size_t i = 0; i < n; i++) {
        double div_real = s->tmp_real[i] / (double) s->g.bins;
        Ax[i] = x[i] - s->p.dt * div_real;
    }
}

static double vdot(const double *a, const double *b, size_t n) {
    double sum = 0.0;
    for(size_t i = 0; i < n; i++) sum += a[i] * b[i];
    return sum;
}

/* _gmres_solve (:537-662), left-preconditioned restarted GMRES */
static int psm_gmres(och_sim *s, const double *b, double *x, double **grads) {
    const size_t n = (size_t) s->g.bins * s->S;
    const int m = s->p.gmres_restart > 2 ? s->p.gmres_restart : 2;
    const double tol = s->p.gmres_tol;
    double *rhs = (double *) malloc(n * sizeof(double));
    double *Mx = (double *) malloc(n * sizeof(double));
    double *r = (double *) malloc(n * sizeof(double));
    double *w = (double *) malloc(n * sizeof(double));
    double *Av = (double *) malloc(n * sizeof(double));
    double *V = (double *) malloc((size_t) (m + 1) * n * sizeof(double));
    double *H = (double *) malloc((size_t) (m + 1) * m * sizeof(double));
    double *cs = (double *) malloc(m * sizeof(double)), *sn = (double *) malloc(m * sizeof(double));
    double *g = (double *) malloc((m + 1) * sizeof(double)), *y = (double *) malloc(m * sizeof(double));
#define APPLY_M(v, out) do { psm_apply_A(s, (v), Av, grads); psm_apply_pinv(s, Av, (out)); } while(0)
    psm_apply_pinv(s, b, rhs);
    APPLY_M(x, Mx);
    for(size_t i = 0; i < n; i++) r[i] = rhs[i] - Mx[i];
    double rhs_norm = sqrt(vdot(rhs, rhs, n));
    if(rhs_norm < 1e-30) rhs_norm = 1e-30;
    double beta = sqrt(vdot(r, r, n));
    double rel = beta / rhs_norm;
    int iter_total = 0;
    if(!(rel < tol)) {
        while(iter_total < s->p.gmres_max_iter) {
            memset(H, 0, (size_t) (m + 1) * m * sizeof(double));
            memset(cs, 0, m * sizeof(double));
            memset(sn, 0, m * sizeof(double));
            memset(g, 0, (m + 1) * sizeof(double));
            for(size_t i = 0; i < n; i++) V[i] = r[i] / beta;
            g[0] = beta;
            int j_end = 0;
            for(int j = 0; j < m && iter_total < s->p.gmres_max_iter; j++, iter_total++) {
                APPLY_M(V + (size_t) j * n, w);
                for(int i = 0; i <= j; i++) {
                    double h = vdot(w, V + (size_t) i * n, n);
                    H[i * m + j] = h;
                    const double *vi = V + (size_t) i * n;
                    for(size_t k = 0; k < n; k++) w[k] -= h * vi[k];
                }
                H[(j + 1) * m + j] = sqrt(vdot(w, w, n));
                if(H[(j + 1) * m + j] > 1e-30) {
                    double *vn = V + (size_t) (j + 1) * n;
                    for(size_t k = 0; k < n; k++) vn[k] = w[k] / H[(j + 1) * m + j];
                }
                else {
                    j_end = j + 1;
                    break;
                }
                for(int i = 0; i < j; i++) {
                    double t1 = cs[i] * H[i * m + j] + sn[i] * H[(i + 1) * m + j];
                    double t2 = -sn[i] * H[i * m + j] + cs[i] * H[(i + 1) * m + j];
                    H[i * m + j] = t1;
                    H[(i + 1) * m + j] = t2;
                }
                double a = H[j * m + j], b2 = H[(j + 1) * m + j];
                double den = sqrt(a * a + b2 * b2);
                cs[j] = (den > 0) ? (a / den) : 1.0;
                sn[j] = (den > 0) ? (b2 / den) : 0.0;
                H[j * m + j] = cs[j] * a + sn[j] * b2;
                H[(j + 1) * m + j] = 0.0;
                double gj = g[j];
                g[j] = cs[j] * gj;
                g[j + 1] = -sn[j] * gj;
                rel = fabs(g[j + 1]) / rhs_norm;
                if(rel < tol) {
                    j_end = j + 1;
                    break;
                }
                j_end = j + 1;
            }
            for(int i = j_end - 1; i >= 0; i--) {
                double sum = g[i];
                for(int k = i + 1; k < j_end; k++) sum -= H[i * m + k] * y[k];
                y[i] = sum / H[i * m + i];
            }
            for(int i = 0; i < j_end; i++) {
                const double *vi = V + (size_t) i * n;
                for(size_t k = 0; k < n; k++) x[k] += vi[k] * y[i];
            }
            APPLY_M(x, Mx);
            for(size_t i = 0; i < n; i++) r[i] = rhs[i] - Mx[i];
            beta = sqrt(vdot(r, r, n));
            rel = beta / rhs_norm;
            if(rel < tol) break;
        }
    }
#undef APPLY_M
    free(rhs); free(Mx); free(r); free(w); free(Av); free(V); free(H); free(cs); free(sn); free(g); free(y);
    return iter_total;
}

/* _evolve_full (:312-427) */
static void psm_evolve_full(och_sim *s) {
    const int S = s->S;
    const size_t bins = (size_t) s->g.bins, n = bins * S;
    for(int sp = 0; sp < S; sp++) {
        double mx = 0.0;
        for(size_t i = 0; i < bins; i++) {
            double v = s->mobility[sp * bins + i];
            mx = (mx > v) ? mx : v;
        }
        s->M0[sp] = mx;
    }
    double *grads[3], *b = (double *) malloc(n * sizeof(double)), *x = (double *) malloc(n * sizeof(double));
    for(int d = 0; d < s->g.dims; d++) grads[d] = (double *) malloc(n * sizeof(double));
    och_der_bulk_free_energy(&s->p.model, (int) bins, s->rho, s->scratch);
    for(size_t i = 0; i < n; i++) s->tmp_real[i] = s->scratch[i] - s->p.splitting_S * s->rho[i];
    double *gh = s->mu_hat;
    ps_rfft(s, s->tmp_real, gh);
    psm_grad_real(s, gh, grads);
    psm_div_hat(s, grads);
    ps_irfft(s, s->div_hat, s->tmp_real);
    for(size_t i = 0; i < n; i++) s->tmp_real[i] /= (double) bins;
    for(size_t i = 0; i < n; i++) {
        b[i] = s->rho[i] + s->p.dt * s->tmp_real[i];
        x[i] = s->rho[i];
    }
    psm_gmres(s, b, x, grads);
    memcpy(s->rho, x, n * sizeof(double));
    ps_rfft(s, s->rho, s->rho_hat);
    memcpy(s->rho_hat_copy, s->rho_hat, sizeof(double) * 2 * (size_t) s->hat_grid_size * S);
    for(int d = 0; d < s->g.dims; d++) free(grads[d]);
    free(b);
    free(x);
}

och_sim *och_create(const chgb_params *p, const double *rho_init) {
    och_sim *s = (och_sim *) calloc(1, sizeof(och_sim));
    s->p = *p;
    s->S = p->model.n_species;
    s->g.dims = p->dims;
    s->g.N = p->N;
    s->g.mask = p->N - 1;
    s->g.bits = 0;
    while((1 << s->g.bits) < p->N) s->g.bits++;
    s->g.bins = p->N;
    for(int i = 1; i < p->dims; i++) s->g.bins *= p->N;
    size_t n = (size_t) s->g.bins * s->S;
    s->rho = (double *) malloc(n * sizeof(double));
    memcpy(s->rho, rho_init, n * sizeof(double));
    s->mobility = (double *) malloc(n * sizeof(double));
    /* src/mobility/ConstantMobility.h:18-22 fills M once; the free-energy
     * mobility is recomputed before every step. */
    for(size_t i = 0; i < n; i++) s->mobility[i] = p->M;
    if(p->mobility_type == CHGB_MOBILITY_GEL) {
        s->gel = (double *) malloc((size_t) s->g.bins * sizeof(double));
        och_gel_init(s->gel, (size_t) s->g.bins);
    }
    s->scratch = (double *) calloc(n, sizeof(double));
    if(p->integrator == CHGB_INTEGRATOR_EULER_MOBILITY) {
        s->flux = (double *) calloc(n * (size_t) p->dims, sizeof(double));
    }
    if(p->integrator == CHGB_INTEGRATOR_PSEUDOSPECTRAL) {
        ps_setup(s);
        ps_forward_state(s);
    }
    if(p->integrator == CHGB_INTEGRATOR_PSEUDOSPECTRAL_MOBILITY) {
        psm_setup(s);
        ps_forward_state(s);
    }
    return s;
}

void och_destroy(och_sim *s) {
    if(!s) return;
    free(s->rho);
    free(s->mobility);
    free(s->gel);
    free(s->scratch);
    free(s->flux);
    free(s->rho_hat);
    free(s->rho_hat_copy);
    free(s->f_der_hat);
    free(s->sqr_wave_vectors);
    free(s->dealiaser);
    for(int d = 0; d < 3; d++) free(s->kcomp[d]);
    free(s->mu_hat);
    free(s->tmp_hat);
    free(s->div_hat);
    free(s->tmp_real);
    free(s);
}

void och_set_rho(och_sim *s, const double *rho) {
    memcpy(s->rho, rho, sizeof(double) * (size_t) s->g.bins * s->S);
    if(s->p.integrator == CHGB_INTEGRATOR_PSEUDOSPECTRAL ||
       s->p.integrator == CHGB_INTEGRATOR_PSEUDOSPECTRAL_MOBILITY)
        ps_forward_state(s);
}

/* src/integrators/EulerCPU.cpp:18-36 */
OCH_INLINE void euler_evolve_k(och_sim *s, int dims) {
    const grid *g = &s->g;
    int bins = g->bins;
    double *rho_der = s->scratch;
    och_der_bulk_free_energy(&s->p.model, bins, s->rho, rho_der);
    for(int idx = 0; idx < bins; idx++) {
        for(int sp = 0; sp < s->S; sp++) {
            rho_der[sp * bins + idx] -= 2 * s->p.k[sp] * cell_laplacian_k(g, s->rho + sp * bins, idx, s->p.dx, dims);
        }
    }
    double M = s->mobility[0];
    for(int idx = 0; idx < bins; idx++) {
        for(int sp = 0; sp < s->S; sp++) {
            double total_derivative = M * cell_laplacian_k(g, rho_der + sp * bins, idx, s->p.dx, dims);
            s->rho[sp * bins + idx] += total_derivative * s->p.dt;
        }
    }
}

static void euler_evolve(och_sim *s) {
    switch(s->g.dims) {
        case 1: euler_evolve_k(s, 1); break;
        case 2: euler_evolve_k(s, 2); break;
        default: euler_evolve_k(s, 3); break;
    }
}

/* src/integrators/EulerMobilityCPU.cpp:31-83 (noise off) and the divergence of
 * src/integrators/EulerCPU.cpp:114-128 */
OCH_INLINE void euler_mobility_evolve_k(och_sim *s, int dims) {
    const grid *g = &s->g;
    int bins = g->bins;
    double dx = s->p.dx;
    double *mu = s->scratch;
    double *flux = s->flux;
    och_der_bulk_free_energy(&s->p.model, bins, s->rho, mu);
    for(int idx = 0; idx < bins; idx++) {
        for(int sp = 0; sp < s->S; sp++) {
            mu[sp * bins + idx] -= 2.0 * s->p.k[sp] * cell_laplacian_k(g, s->rho + sp * bins, idx, dx, dims);
        }
    }
    for(int idx = 0; idx < bins; idx++) {
        for(int sp = 0; sp < s->S; sp++) {
            int coords[3], cp[3];
            fill_coords_k(g, coords, idx, dims);
            for(int d = 0; d < dims; d++) {
                memcpy(cp, coords, sizeof(coords));
                cp[d] = (coords[d] + 1) & g->mask;
                int idx_p = cell_idx_k(g, cp, dims);
                double M_idx = s->mobility[sp * bins + idx];
                double M_p = s->mobility[sp * bins + idx_p];
                double M_face = 0.5 * (M_idx + M_p);
                flux[((size_t) sp * bins + idx) * dims + d] = M_face * (mu[sp * bins + idx_p] - mu[sp * bins + idx]) / dx;
            }
        }
    }
    for(int idx = 0; idx < bins; idx++) {
        for(int sp = 0; sp < s->S; sp++) {
            double res = 0;
            int coords[3], cm[3];
            fill_coords_k(g, coords, idx, dims);
            memcpy(cm, coords, sizeof(coords));
            for(int d = 0; d < dims; d++) {
                cm[d] = (coords[d] - 1 + g->N) & g->mask;
                int idx_m = cell_idx_k(g, cm, dims);
                res += (flux[((size_t) sp * bins + idx) * dims + d] - flux[((size_t) sp * bins + idx_m) * dims + d]) / dx;
                cm[d] = coords[d];
            }
            double div_sto = 0.0;
            s->rho[sp * bins + idx] += (res + div_sto) * s->p.dt;
        }
    }
}

static void euler_mobility_evolve(och_sim *s) {
    switch(s->g.dims) {
        case 1: euler_mobility_evolve_k(s, 1); break;
        case 2: euler_mobility_evolve_k(s, 2); break;
        default: euler_mobility_evolve_k(s, 3); break;
    }
}

/* src/integrators/PseudospectralCPU.cpp:112-136 */
static void pseudospectral_evolve(och_sim *s) {
    if(!s->ps_M_set) { /* `static double M` is frozen at the first call */
        s->ps_M = s->mobility[0];
        s->ps_M_set = 1;
    }
    double M = s->ps_M;
    int bins = s->g.bins;
    double dt = s->p.dt, S = s->p.splitting_S;
    och_der_bulk_free_energy(&s->p.model, bins, s->rho, s->scratch);
    ps_rfft(s, s->scratch, s->f_der_hat);
    int hvs = s->hat_grid_size * s->S;
    for(int k_idx = 0; k_idx < hvs; k_idx++) {
        double *fh = s->f_der_hat + 2 * k_idx;
        double *rh = s->rho_hat + 2 * k_idx;
        double *rc = s->rho_hat_copy + 2 * k_idx;
        if(s->p.use_dealias) {
            fh[0] *= s->dealiaser[k_idx];
            fh[1] *= s->dealiaser[k_idx];
        }
        double k2 = s->sqr_wave_vectors[k_idx];
        double k4 = SQR(k2);
        int species = k_idx / s->hat_grid_size;
        double denom = 1.0 + dt * M * (S * k2 + 2.0 * s->p.k[species] * k4);
        double c = dt * M * k2;
        double nr = (rh[0] - c * (fh[0] - S * rh[0])) / denom;
        double ni = (rh[1] - c * (fh[1] - S * rh[1])) / denom;
        rh[0] = rc[0] = nr;
        rh[1] = rc[1] = ni;
        rc[0] /= bins;
        rc[1] /= bins;
    }
    ps_irfft(s, s->rho_hat_copy, s->rho);
}

static void update_mobility(och_sim *s) {
    const size_t bins = (size_t) s->g.bins;
    if(s->p.mobility_type == CHGB_MOBILITY_FREE_ENERGY) {
        /* src/mobility/FreeEnergyMobility.h:25-34 */
        och_set_mobility(&s->p.model, s->g.bins * s->S, s->rho, s->p.M, s->mobility);
    }
    else if(s->p.mobility_type == CHGB_MOBILITY_REGULARISED) {
        /* src/mobility/RegularisedMobility.h:26-33 */
        for(size_t idx = 0; idx < bins; idx++) {
            for(int sp = 0; sp < s->S; sp++) {
                double r = s->rho[sp * bins + idx];
                s->mobility[sp * bins + idx] = s->p.M * r / (r + s->p.rho_min);
            }
        }
    }
    else if(s->p.mobility_type == CHGB_MOBILITY_GEL) {
        /* src/mobility/GelMobility.h:20 (p_gel) and :41-58 */
        double e = exp(s->p.gel_beta_delta_F);
        double p_gel = e / (1.0 + e);
        double phi_c = s->p.gel_phi_critical;
        for(size_t idx = 0; idx < bins; idx++) {
            double rho_tot = 0.0;
            for(int sp = 0; sp < s->S; sp++) rho_tot += s->rho[sp * bins + idx];
            double c = s->gel[idx];
            double phi = (rho_tot + 1.0) / 2.0;
            double g = (p_gel * phi - phi_c) / (1.0 - phi_c);
            double c_der = s->p.gel_M_c * (g * c - c * c);
            s->gel[idx] += c_der * s->p.dt;
            for(int sp = 0; sp < s->S; sp++) s->mobility[sp * bins + idx] = exp(-s->gel[idx] / s->p.gel_c0);
        }
    }
}

void och_step(och_sim *s, int64_t nsteps) {
    for(int64_t t = 0; t < nsteps; t++) {
        update_mobility(s);
        if(s->p.integrator == CHGB_INTEGRATOR_EULER) euler_evolve(s);
        else if(s->p.integrator == CHGB_INTEGRATOR_EULER_MOBILITY) euler_mobility_evolve(s);
        else if(s->p.integrator == CHGB_INTEGRATOR_PSEUDOSPECTRAL_MOBILITY) {
            if(s->p.use_gmres) psm_evolve_full(s);
            else psm_evolve(s);
        }
        else pseudospectral_evolve(s);
    }
}

void och_get_rho(const och_sim *s, double *out) {
    memcpy(out, s->rho, sizeof(double) * (size_t) s->g.bins * s->S);
}

void och_get_mobility(const och_sim *s, double *out) {
    memcpy(out, s->mobility, sizeof(double) * (size_t) s->g.bins * s->S);
}

/* src/CahnHilliard.cpp:285-297 */
double och_average_mass(const och_sim *s, int *nan) {
    int bins = s->g.bins;
    double mass = 0.;
    *nan = 0;
    for(int i = 0; i < bins; i++) {
        double tot = 0.;
        for(int sp = 0; sp < s->S; sp++) tot += s->rho[sp * bins + i];
        mass += tot;
        if(isnan(mass)) *nan = 1;
    }
    double V_bin = CUB(s->p.dx);
    return mass * V_bin / bins;
}

/* src/CahnHilliard.cpp:255-276,300-319 */
double och_average_free_energy(const och_sim *s, int *nan) {
    const grid *g = &s->g;
    int bins = g->bins, dims = g->dims;
    double dx = s->p.dx;
    double fe = 0.;
    *nan = 0;
    for(int i = 0; i < bins; i++) {
        double interfacial = 0.;
        for(int sp = 0; sp < s->S; sp++) {
            const double *f = s->rho + sp * bins;
            double grad[3];
            if(dims == 1) {
                int ip = (i + 1) & g->mask;
                grad[0] = (f[ip] - f[i]) / dx;
            }
            else {
                int coords[3], cp[3];
                fill_coords(g, coords, i);
                for(int d = 0; d < dims; d++) {
                    memcpy(cp, coords, sizeof(coords));
                    cp[d] = (coords[d] + 1) & g->mask;
                    grad[d] = (f[cell_idx(g, cp)] - f[i]) / dx;
                }
            }
            for(int d = 0; d < dims; d++) interfacial += s->p.k[sp] * grad[d] * grad[d];
        }
        fe += och_bulk_free_energy(&s->p.model, bins, s->rho, i) + interfacial;
        if(isnan(fe)) *nan = 1;
    }
    double V_bin = CUB(dx);
    return fe * V_bin / bins;
}

/* Landau pressure of one species, src/models/Landau.cpp:66-71: op * mu - f with
 * mu = f'(op) and f the bulk free energy, each written as the model writes it. */
static double landau_pressure(const chgb_model_params *m, double op) {
    double mu = -m->epsilon * op + op * op * op;
    double f = -0.5 * m->epsilon * SQR(op) + 0.25 * SQR(SQR(op));
    return op * mu - f;
}

/* Forward-difference gradient of species `sp` at cell i, src/CahnHilliard.cpp:255-276. */
static void forward_gradient(const och_sim *s, int sp, int i, double grad[3]) {
    const grid *g = &s->g;
    const double *f = s->rho + (size_t) sp * g->bins;
    double dx = s->p.dx;
    if(g->dims == 1) {
        int ip = (i + 1) & g->mask;
        grad[0] = (f[ip] - f[i]) / dx;
        return;
    }
    int coords[3], cp[3];
    fill_coords(g, coords, i);
    for(int d = 0; d < g->dims; d++) {
        memcpy(cp, coords, sizeof(coords));
        cp[d] = (coords[d] + 1) & g->mask;
        grad[d] = (f[cell_idx(g, cp)] - f[i]) / dx;
    }
}

int och_pressure_field(const och_sim *s, double *out) {
    /* src/CahnHilliard.cpp:340-356; FreeEnergyModel::pressure is critical() for
     * every model but Landau (src/models/FreeEnergyModel.h:43-44) */
    if(s->p.model.kind != CHGB_MODEL_LANDAU) return 1;
    const grid *g = &s->g;
    for(int i = 0; i < g->bins; i++) {
        for(int sp = 0; sp < s->S; sp++) {
            double grad[3];
            double v = landau_pressure(&s->p.model, s->rho[(size_t) sp * g->bins + i]);
            forward_gradient(s, sp, i, grad);
            for(int d = 0; d < g->dims; d++) v -= 0.5 * s->p.k[sp] * grad[d] * grad[d];
            out[(size_t) sp * g->bins + i] = v;
        }
    }
    return 0;
}

double och_average_pressure(const och_sim *s, int *unsupported) {
    /* src/CahnHilliard.cpp:321-337: no V_bin factor and no NaN check, as there */
    *unsupported = s->p.model.kind != CHGB_MODEL_LANDAU;
    if(*unsupported) return 0.0;
    const grid *g = &s->g;
    double pressure = 0.;
    for(int i = 0; i < g->bins; i++) {
        for(int sp = 0; sp < s->S; sp++) {
            double grad[3];
            pressure += landau_pressure(&s->p.model, s->rho[(size_t) sp * g->bins + i]);
            forward_gradient(s, sp, i, grad);
            for(int d = 0; d < g->dims; d++) pressure -= 0.5 * s->p.k[sp] * grad[d] * grad[d];
        }
    }
    return pressure / g->bins;
}
