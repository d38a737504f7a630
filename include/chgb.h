/*
 * chgb.h — C ABI of the GB300 (sm_103a) Cahn–Hilliard time-step engine.
 *
 * The reference (lorenzo-rovigatti/cahn-hilliard) exposes its hot path as a C++
 * plugin API: the abstract integrator `Integrator<dims>` with `evolve()` and
 * `sync()` (src/integrators/Integrator.h:10-41), selected by `integrator` ×
 * `use_CUDA` in src/CahnHilliard.cpp:169-223, plus the device hooks of the
 * free-energy model `FreeEnergyModel::der_bulk_free_energy(field_type*, float*,
 * int)` and `set_mobility(field_type*, double, field_type*, int)`
 * (src/models/FreeEnergyModel.h:29,48), and the host reductions
 * `CahnHilliard::average_mass()` / `average_free_energy()`
 * (src/CahnHilliard.cpp:285-319).
 *
 * This header replaces that boundary with plain C: an opaque handle, plain
 * pointers and sizes, `int` status codes instead of `exit()`.  Every field is
 * FP64 and uses the reference's species-major layout
 *     data[s * N^dims + idx],  idx = x + N*y + N*N*z,
 * with periodic boundaries and N a power of two (src/utils/MultiField.h:59-63,
 * src/CahnHilliard.cpp:50-53,244-253).  All parameters are in the reference's
 * internal units, i.e. after the `distance_scaling_factor` rescaling that
 * src/CahnHilliard.cpp:153-163 and the model constructors apply.
 */
#ifndef CHGB_H
#define CHGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CHGB_ABI_VERSION 5
#define CHGB_MAX_SPECIES 3

/* Status codes returned by every entry point. */
enum {
    CHGB_OK = 0,
    CHGB_ERR_INVALID = 1,     /* bad argument or unsupported combination */
    CHGB_ERR_CUDA = 2,        /* a CUDA runtime call failed; see chgb_last_error */
    CHGB_ERR_NAN = 3,         /* a reduction met a NaN (reference: critical() -> exit(1)) */
    CHGB_ERR_UNSUPPORTED = 4, /* the reference would call critical() for this setup */
    CHGB_ERR_ALLOC = 5,       /* device or host allocation failed */
    CHGB_ERR_TIMEOUT = 6      /* a bounded device wait gave up */
};

/* `integrator` names of the reference (src/CahnHilliard.cpp:169-198). */
enum {
    CHGB_INTEGRATOR_EULER = 0,
    CHGB_INTEGRATOR_EULER_MOBILITY = 1,
    CHGB_INTEGRATOR_PSEUDOSPECTRAL = 2,
    /* variable-mobility pseudospectral step with the constant reference mobility
     * M0 = max M treated semi-implicitly (src/integrators/PseudospectralMobilityCPU.cpp:236-310);
     * `splitting_S` is `pseudospectral.S` as given, without the unit scaling of
     * `pseudospectral` (the reference's constructor does not scale it, :22) */
    CHGB_INTEGRATOR_PSEUDOSPECTRAL_MOBILITY = 3
};

/* `free_energy` names of the reference (src/main.cpp:44-53). */
enum {
    CHGB_MODEL_LANDAU = 0,
    CHGB_MODEL_SIMPLE_WERTHEIM = 1,
    CHGB_MODEL_SALEH = 2
};

/* `mobility.type` names of the reference (src/mobility/IMobility.cpp:18-57).
 * `regularised` and `gel` are computed on the device before every step, as
 * the reference's update_mobility() does on the host, and need an integrator
 * that supports a non-constant mobility (`euler_mobility`). */
enum {
    CHGB_MOBILITY_CONSTANT = 0,
    CHGB_MOBILITY_FREE_ENERGY = 1,
    CHGB_MOBILITY_REGULARISED = 2,   /* M rho / (rho + rho_min)  (src/mobility/RegularisedMobility.h:26-33) */
    CHGB_MOBILITY_GEL = 3            /* exp(-c / c_0), c the gel order parameter (src/mobility/GelMobility.h:41-58) */
};

/*
 * Free-energy model parameters, internal units.
 *   landau          : epsilon                       (src/models/Landau.cpp:16-36)
 *   simple_wertheim : valence, B2, delta,
 *                     regularisation_delta          (src/models/SimpleWertheim.cpp:20-34)
 *   saleh           : saleh_valence[3], B2, B3,
 *                     delta_AA, delta_BB            (src/models/SalehWertheim.cpp:19-41)
 * density_conversion_factor = (1/distance_scaling_factor)^3 enters only the
 * bulk free energy (src/models/FreeEnergyModel.h:18-22).
 */
typedef struct chgb_model_params {
    int32_t kind;                 /* CHGB_MODEL_* */
    int32_t n_species;            /* 1 (landau, simple_wertheim) or 3 (saleh) */
    double epsilon;
    int32_t valence;
    int32_t saleh_valence[3];
    double B2;
    double B3;
    double delta;
    double regularisation_delta;
    double delta_AA;
    double delta_BB;
    double density_conversion_factor;
} chgb_model_params;

/*
 * One simulation box.  `M` is the constant mobility (`mobility.M` divided by
 * user_to_internal, src/mobility/ConstantMobility.h:18-22) or M0 of the
 * free-energy mobility (src/mobility/FreeEnergyMobility.h:18-22).
 * `splitting_S` / `use_dealias` are `pseudospectral.S` (already scaled by
 * user_to_internal^3) and `pseudospectral.use_dealias`
 * (src/integrators/PseudospectralCPU.cpp:24-25).
 */
typedef struct chgb_params {
    int32_t dims;                 /* 1, 2 or 3 */
    int32_t N;                    /* cells per side, power of two, 4..4096 */
    int32_t integrator;           /* CHGB_INTEGRATOR_* */
    int32_t mobility_type;        /* CHGB_MOBILITY_* */
    double dt;
    double dx;
    double k[CHGB_MAX_SPECIES];   /* k_laplacian per species */
    double M;
    double splitting_S;
    int32_t use_dealias;
    int32_t kernel_variant;       /* euler / euler_mobility in 2D/3D with N >= 32:
                                     0 = pick the fastest at chgb_create (timed once),
                                     1 = one fused kernel per step (mu recomputed on tile halos),
                                     2 = two kernels per step (mu stored once per cell),
                                     3 = two fused steps per launch (2D `euler`, 32 <= N <= 512),
                                     4 = the whole box in one 16-CTA cluster's shared memory, many
                                         steps per launch (2D `euler`, N = 32 or 64);
                                     1-4 give bit-identical results;
                                     5 = block fixed point: one exponent for the whole field
                                         per step (2D/3D Landau `euler`, N >= 32; two kernels
                                         per step in 3D, mu stored as integers, one in 2D);
                                         agrees with 1-4 to round-off (below 2^-56 of the
                                         field's largest value per step), not bit for bit.
                                         Variant 0 picks it by a fixed rule, without timing,
                                         for 2D N >= 512 and 3D N >= 64, and times 1-4
                                         elsewhere, so a configuration always runs the same
                                         arithmetic. */
    chgb_model_params model;
    /* `regularised` mobility: mobility.rho_min / user_to_internal (M is `M` above). */
    double rho_min;
    /* `gel` mobility (src/mobility/IMobility.cpp:30-47): mobility.phi_critical,
     * mobility.c_0, mobility.M_c / user_to_internal and beta_delta_F =
     * 10 / (1 - landau.epsilon) - ln 24000.  The order parameter starts from
     * the reference's std::mt19937 (default seed) uniform [0, 1) draws times 1e-4
     * and advances by explicit Euler with `dt` before every step. */
    double gel_phi_critical;
    double gel_c0;
    double gel_M_c;
    double gel_beta_delta_F;
    /* `pseudospectral_mobility` with pseudospectral.use_gmres = true
     * (src/integrators/PseudospectralMobilityCPU.cpp:204-208, defaults 30, 200,
     * 1e-10): each step solves (1 - dt div M grad (S - 2k lap)) rho' = rhs with
     * left-preconditioned restarted GMRES instead of the M0 splitting. */
    int32_t use_gmres;
    int32_t gmres_restart;
    int32_t gmres_max_iter;
    double gmres_tol;
} chgb_params;

typedef struct chgb_handle chgb_handle;

/* ABI version of the loaded library (CHGB_ABI_VERSION of its build). */
int chgb_abi_version(void);

/*
 * Allocate the device state of one box on the current CUDA device and on
 * the handle's own stream.  Replaces the constructors of the CUDA
 * integrators (src/CUDA/integrators/CUDAIntegrator.cu:13-53, EulerCUDA.cu:37-52,
 * EulerMobilityCUDA.cu, PseudospectralCUDA.cu:104-224) and the factory that
 * picks them (src/CahnHilliard.cpp:169-223).  Rejects what the reference
 * rejects with critical(): non power-of-two N, a non-constant mobility with
 * `euler` / `pseudospectral` (src/integrators/Integrator.cpp:38-42), a
 * free-energy mobility with a model that has no set_mobility
 * (src/models/FreeEnergyModel.h:48-53).
 */
int chgb_create(const chgb_params *params, chgb_handle **out);

/* Free everything the handle owns (src/CUDA/integrators/CUDAIntegrator.cu:36-40). */
int chgb_destroy(chgb_handle *h);

/*
 * Copy a host density field (n_species * N^dims doubles) to the device and
 * make it the current state; for `pseudospectral` this also computes the
 * initial rho_hat as the reference constructor does
 * (src/integrators/PseudospectralCPU.cpp:95-101).  Synchronous.
 * Replaces CUDAIntegrator::_CPU_GPU (src/CUDA/integrators/CUDAIntegrator.cu:43-53),
 * which also uploads the host mobility field.  `mobility` may be NULL.  If it
 * is given it must be the field the mobility type defines, as it is in the
 * reference: for `constant`, M everywhere (checked to 1e-12 relative; any
 * other field returns CHGB_ERR_UNSUPPORTED, since a per-cell static mobility
 * is not a type of this path); for `free_energy` it is accepted and unused,
 * because the reference recomputes it from rho before every step
 * (src/mobility/FreeEnergyMobility.h:23-31).
 */
int chgb_upload(chgb_handle *h, const double *rho, const double *mobility);

/*
 * Advance the state by `nsteps` time steps, each one the reference's
 * CahnHilliard::evolve() = mobility->update_mobility() + integrator->evolve()
 * (src/CahnHilliard.cpp:278-282).  Asynchronous on the handle's stream.
 */
int chgb_step(chgb_handle *h, int64_t nsteps);

/*
 * Copy the current density (and, if `mobility` is not NULL, the mobility
 * field the reference would hold after its last update_mobility()) to host
 * memory.  Synchronous.  Replaces CUDAIntegrator::sync()
 * (src/CUDA/integrators/CUDAIntegrator.cu:56-70).
 */
int chgb_download(chgb_handle *h, double *rho, double *mobility);

/*
 * Device reductions of the current state: the reference's
 * average_mass() and average_free_energy() (src/CahnHilliard.cpp:285-319),
 * FP64, with the forward-difference gradient of src/CahnHilliard.cpp:255-276
 * and V_bin = dx^3.  `nan_flag` is set when either sum meets a NaN, and the
 * call then returns CHGB_ERR_NAN (the reference calls critical()).  Any
 * output pointer may be NULL.  Synchronous.
 */
int chgb_observables(chgb_handle *h, double *mass, double *free_energy, int32_t *nan_flag);

/*
 * Pressure of the current state, Landau only: the field of
 * CahnHilliard::pressure() (src/CahnHilliard.cpp:340-356), per cell and
 * species p_s(rho) - sum_d k_s/2 (grad_d rho_s)^2 with p = rho f'(rho) - f(rho)
 * (src/models/Landau.cpp:66-71) and the forward difference of
 * src/CahnHilliard.cpp:255-276, into the host buffer `field`
 * (n_species * N^dims doubles), and average_pressure()
 * (src/CahnHilliard.cpp:321-337), the sum over cells and species divided by
 * N^dims without the V_bin factor of the other averages, into `average`.
 * Either output may be NULL; both come from one pass over the field.  No NaN
 * check, as in the reference.  Other models return CHGB_ERR_UNSUPPORTED (the
 * reference's FreeEnergyModel::pressure() calls critical(),
 * src/models/FreeEnergyModel.h:43-44).  Synchronous.
 */
int chgb_pressure(chgb_handle *h, double *field, double *average);

/* Use an existing CUDA stream (cudaStream_t passed as void*); NULL = the handle's own. */
int chgb_set_stream(chgb_handle *h, void *stream);

/* Wait for all work queued on the handle's stream. */
int chgb_synchronize(chgb_handle *h);

/*
 * Device pointer to the current real-space density (n_species * N^dims
 * doubles).  Valid until the next chgb_step / chgb_upload / chgb_destroy.
 * For `pseudospectral` the real-space field is regenerated from rho_hat on
 * demand, as the reference's inverse transform does every step.
 */
int chgb_device_rho(chgb_handle *h, double **d_rho);

/* Number of kernels this handle has launched since creation. */
int64_t chgb_launch_count(const chgb_handle *h);

/* Bounds-check build only (libchgb_bc.so, compiled with -DCHGB_BOUNDS_CHECK):
 * the first out-of-range index the explicit kernels or the transforms met
 * since the last call, as (site << 48) | index, 0 if none; the record is
 * cleared.  The access itself was skipped.  In the normal build it sets
 * *first = 0 and returns CHGB_ERR_UNSUPPORTED.  No counterpart in the
 * reference: a debugging aid, standing in for compute-sanitizer. */
int chgb_bounds_report(unsigned long long *first);

/* Kernel variant the handle runs: 1 fused, 2 split, 3 two steps per launch, 4 cluster-resident,
 * 5 split in block fixed point (see kernel_variant);
 * 1 for the pseudospectral integrators. */
int chgb_kernel_variant(const chgb_handle *h);

/*
 * Message of the last failure on `h` (or of the last failed chgb_create /
 * free-function call when h is NULL).  Never NULL.
 */
const char *chgb_last_error(const chgb_handle *h);

/*
 * Device hook of the free-energy model: rho_der = f'(rho) for `bins` cells
 * of every species, FP64 in and out, device pointers, async on `stream`.
 * Replaces FreeEnergyModel::der_bulk_free_energy(field_type*, float*, int)
 * (src/models/FreeEnergyModel.h:29), whose float* output cannot hold FP64.
 */
int chgb_der_bulk_free_energy(const chgb_model_params *model, const double *d_rho,
                              double *d_rho_der, int64_t bins, void *stream);

/*
 * Device hook of the free-energy mobility: mobility = M0 * rho * X(rho)^valence
 * for `bins` cells (simple_wertheim only).  Replaces
 * FreeEnergyModel::set_mobility(field_type*, double, field_type*, int)
 * (src/models/FreeEnergyModel.h:48; src/models/SimpleWertheim.cpp:104-111).
 */
int chgb_set_mobility(const chgb_model_params *model, const double *d_rho, double M0,
                      double *d_mobility, int64_t bins, void *stream);

/*
 * Radially averaged structure factor of a 2D box, the definition of the
 * reference's analysis script utils/sq_from_traj.py:72-103 (radial_average_Sq
 * with subtract_mean): S(k) = |FFT2(rho_s - mean)|^2 / N^2, shells
 * rint(|k| / dq), dq = 2 pi / (N dx), S(q_b) = shell mean, q_b = b dq.
 * Computed on the device from the current state of species `species`;
 * `sq` (host) receives chgb_structure_factor_bins(N) values.
 */
int chgb_structure_factor_bins(int32_t N);
int chgb_structure_factor(chgb_handle *h, int32_t species, double *sq, int32_t nbins);

/*
 * Adjoint (no counterpart in the reference): gradients of a loss on the state
 * after `nsteps` steps with respect to the initial field and to
 * (epsilon, k, M) in internal units, for 2D Landau boxes with constant
 * mobility, `euler` (N >= 32, multiple of 32) or `pseudospectral`
 * (8 <= N <= 1024).  The forward pass stores a checkpoint every
 * `checkpoint_every` steps (<= 0: ceil(sqrt(nsteps))); the backward pass
 * recomputes one segment at a time and runs the hand-written adjoint steps.
 * The pseudospectral trajectory here starts from the transformed initial
 * field (the round trip FFT -> inverse FFT), which differs from chgb_step's
 * first step at the level of rounding.
 *   forward : rho0 (host, N^2) -> optional S(q) (chgb_structure_factor_bins(N)
 *             values) and final field rho_T of the trajectory.
 *   backward: the loss gradient given as dL/dS(q) (nbins, may be NULL) and/or
 *             dL/drho_T (N^2, may be NULL) -> dL/drho0 (N^2) and
 *             grad_params[3] = dL/d{epsilon, k, M}.  Either output may be NULL.
 * Bit-for-bit reproducible (fixed-order reductions).
 * `euler`: params->kernel_variant sets how many steps one launch of the
 * checkpointed passes takes -- 3 two, 1 or 2 one, 0 or 4 two for N <= 256 and one
 * above.  The fields are the same bits either way; the parameter gradients
 * differ at the level of rounding (another summation order).
 */
typedef struct chgb_adjoint chgb_adjoint;
int chgb_adjoint_create(const chgb_params *params, int64_t nsteps, int32_t checkpoint_every, chgb_adjoint **out);
int chgb_adjoint_destroy(chgb_adjoint *a);
int chgb_adjoint_forward(chgb_adjoint *a, const double *rho0, double *sq, double *rho_T);
int chgb_adjoint_backward(chgb_adjoint *a, const double *dl_dsq, const double *dl_drho_T, double *grad_rho0,
                          double *grad_params);
int64_t chgb_adjoint_launch_count(const chgb_adjoint *a);

/*
 * Batches of independent boxes (no counterpart in the reference, whose
 * integrators keep `static` scratch in evolve() and therefore run one box per
 * process: src/integrators/EulerCPU.cpp:19, PseudospectralCPU.cpp:113).
 * Each replica has its own chgb_params (N, integrator, model, parameters may
 * all differ).  2D `euler` and 2D `pseudospectral` replicas are stepped by
 * shared work-list kernels (one launch per phase for the whole group, replayed
 * from a CUDA graph); any other replica runs on its own stream alongside.
 * A replica gives the same bits stepped in a batch as stepped alone.
 */
typedef struct chgb_batch chgb_batch;

int chgb_batch_create(const chgb_params *params, int32_t n, chgb_batch **out);
int chgb_batch_destroy(chgb_batch *b);
/* Number of replicas. */
int chgb_batch_size(const chgb_batch *b);
/* chgb_upload of replica i (synchronous). */
int chgb_batch_upload(chgb_batch *b, int32_t i, const double *rho);
/* Advance every replica by nsteps (asynchronous). */
int chgb_batch_step(chgb_batch *b, int64_t nsteps);
int chgb_batch_synchronize(chgb_batch *b);
/* chgb_download of replica i's density (synchronous). */
int chgb_batch_download(chgb_batch *b, int32_t i, double *rho);
/* The handle of replica i, for chgb_observables / chgb_device_rho; owned by the batch. */
chgb_handle *chgb_batch_replica(chgb_batch *b, int32_t i);
/* Kernels launched by the batch since creation (loose replicas included). */
int64_t chgb_batch_launch_count(const chgb_batch *b);
/* Euler tile the autotuner picked (16, 32 or 64 for 64x16), 0 without euler replicas. */
int chgb_batch_euler_tile(const chgb_batch *b);

/*
 * No counterpart in the reference.  Mass and free energy of a device field,
 * for callers that cannot allocate device memory when they need them: a host
 * application whose memory pool already owns all of HBM, or a time-stepping
 * loop that cannot pay for cudaMalloc/cudaFree, which may synchronise the
 * device.  Nothing is allocated: the caller passes the field `d_rho`
 * (n_species * N^dims doubles, layout as above) and `d_out`, two device
 * doubles that receive average_mass and average_free_energy (equal to
 * chgb_observables' within round-off: the partial sums are grouped by other
 * blocks; a NaN shows up in them, no flag is returned).  The work is
 * queued on `stream` (NULL = default stream).  The scratch is a fixed array
 * inside the library, held on every device that loads it until the process
 * exits: one (mass, free energy) pair per CHGB_NOALLOC_CELLS_PER_PARTIAL
 * cells, at most CHGB_NOALLOC_MAX_PARTIALS pairs (128 KiB), so fields above
 * 16,777,216 cells are rejected with CHGB_ERR_INVALID, and so is any N above
 * chgb_create's bound for the dimensionality.  The first call on each
 * device looks up that array's device address and should come before any
 * stream capture.  All calls share the array: calls whose kernels overlap on
 * the GPU race on it.  Errors: chgb_last_error(NULL).
 */
#define CHGB_NOALLOC_MAX_PARTIALS 8192
#define CHGB_NOALLOC_CELLS_PER_PARTIAL 2048
int chgb_observables_noalloc(const chgb_params *params, const double *d_rho, double *d_out, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* CHGB_H */
