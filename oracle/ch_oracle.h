/*
 * ch_oracle.h — CPU oracle of the Cahn–Hilliard time-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference's
 * FP64 CPU path (lorenzo-rovigatti/cahn-hilliard, src/integrators/ (the *CPU integrators),
 * src/models, src/CahnHilliard.cpp) used as the checker of the CUDA
 * library.  Only the tests, the smoke check and the CPU-baseline leg of the
 * benchmark may load it; the product never links, calls or falls back to it.
 *
 * Pinning: the restatement is checked against the reference's golden files
 * (tests/data/reference/landau_{euler,pseudospectral}_{1D,2D,3D}.dat, six
 * significant digits) and against full-precision dumps of the reference's own
 * CPU integrators compiled from its sources (oracle/Makefile -> oracle/_ref).
 *
 * Parameters use the product's C ABI structs (include/chgb.h) so that a test
 * can hand the same numbers to both sides.
 */
#ifndef CH_ORACLE_H
#define CH_ORACLE_H

#include <stdint.h>

#include "../include/chgb.h"

#ifdef __cplusplus
extern "C" {
#endif

/* POSIX drand48 generator state (48-bit linear congruential). */
typedef struct och_rand48 {
    uint64_t x;
} och_rand48;

void och_srand48(och_rand48 *r, int64_t seed);
double och_drand48(och_rand48 *r);

/* Initial density of src/CahnHilliard.cpp:133-161 (drand48 draws, then rho /= u^3). */
void och_init_density(int dims, int N, int n_species, const double *densities, double initial_A,
                      int initial_N_peaks, double user_to_internal, och_rand48 *rng, double *rho);

/* rho_der = f'(rho) over `bins` cells; species-major layout. */
void och_der_bulk_free_energy(const chgb_model_params *m, int bins, const double *rho, double *rho_der);
/* f(rho) of one cell `idx`. */
double och_bulk_free_energy(const chgb_model_params *m, int bins, const double *rho, int idx);
/* Initial gel order parameter (och_gel.cpp): the reference's default-seeded
 * std::mt19937 uniform [0, 1) draws times 1e-4, src/mobility/GelMobility.h:28-33. */
void och_gel_init(double *op, size_t n);

/* mobility = M0 * rho * X^valence (simple_wertheim). */
void och_set_mobility(const chgb_model_params *m, int bins, const double *rho, double M0, double *mobility);

typedef struct och_sim och_sim;

/* A simulation box owning rho, the mobility field and the integrator scratch. */
och_sim *och_create(const chgb_params *p, const double *rho_init);
void och_destroy(och_sim *s);
/* nsteps x (update_mobility + evolve), src/CahnHilliard.cpp:278-282. */
void och_step(och_sim *s, int64_t nsteps);
void och_get_rho(const och_sim *s, double *out);
void och_get_mobility(const och_sim *s, double *out);
/* Replace the density (pseudospectral: also recomputes rho_hat). */
void och_set_rho(och_sim *s, const double *rho);
/* average_mass / average_free_energy; *nan set to 1 when a NaN is met. */
double och_average_mass(const och_sim *s, int *nan);
double och_average_free_energy(const och_sim *s, int *nan);
/* pressure() / average_pressure() (src/CahnHilliard.cpp:321-356), Landau only:
 * the field returns 1 and the average sets *unsupported for other models. */
int och_pressure_field(const och_sim *s, double *out);
double och_average_pressure(const och_sim *s, int *unsupported);

#ifdef __cplusplus
}
#endif

#endif
