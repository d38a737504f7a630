// fields.cu — elementwise model hooks and the observable reductions.
//
// * der_bulk: rho_der = f'(rho), the FP64 replacement of the reference's
//   FreeEnergyModel::der_bulk_free_energy(field_type*, float*, int) device
//   hook (src/models/FreeEnergyModel.h:29).
// * set_mobility: M0 rho X^v (src/models/SimpleWertheim.cpp:104-111).
// * observables: average_mass / average_free_energy of
//   src/CahnHilliard.cpp:285-319 as a two-level deterministic reduction
//   (warp shuffles, then one block over the per-block partials).
// * pressure: the Landau pressure field and average_pressure of
//   src/CahnHilliard.cpp:321-356, one pass that writes the field and the
//   same two-level reduction.
#include "common.cuh"
#include "kernels.h"

namespace chgb {

template <int KIND>
__global__ void der_bulk_kernel(ModelDev m, const double *__restrict__ rho, double *__restrict__ der, long long bins) {
    constexpr int S = NSpecies<KIND>::value;
    for(long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < bins;
        i += (long long) gridDim.x * blockDim.x) {
        double r[S], d[S];
#pragma unroll
        for(int s = 0; s < S; s++) r[s] = rho[s * bins + i];
        der_bulk<KIND>(m, r, d);
#pragma unroll
        for(int s = 0; s < S; s++) der[s * bins + i] = d[s];
    }
}

__global__ void set_mobility_kernel(ModelDev m, const double *__restrict__ rho, double M0, double *__restrict__ mob,
                                    long long n) {
    for(long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
        mob[i] = sw_mobility(m, M0, rho[i]);
    }
}

__global__ void fill_kernel(double *p, double v, long long n) {
    for(long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
        p[i] = v;
    }
}

// p[i] = mean + amp * (a hash of i in [-1/2, 1/2)): a varied field of normal
// numbers, for timing kernels whose cost depends on the values they meet.
__global__ void fill_noise_kernel(double *p, double mean, double amp, long long n) {
    for(long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < n; i += (long long) gridDim.x * blockDim.x) {
        unsigned h = (unsigned) i * 2654435761u;
        h ^= h >> 15;
        h *= 2246822519u;
        h ^= h >> 13;
        p[i] = mean + amp * ((double) (h >> 8) * (1.0 / 16777216.0) - 0.5);
    }
}

static int grid_for(long long n) {
    long long b = (n + 255) / 256;
    return (int) (b < 152 * 16 ? (b < 1 ? 1 : b) : 152 * 16);
}

cudaError_t launch_der_bulk(const ModelDev &m, const double *rho, double *der, long long bins, cudaStream_t st) {
    int grid = grid_for(bins);
    switch(m.kind) {
        case CHGB_MODEL_LANDAU: der_bulk_kernel<CHGB_MODEL_LANDAU><<<grid, 256, 0, st>>>(m, rho, der, bins); break;
        case CHGB_MODEL_SIMPLE_WERTHEIM:
            der_bulk_kernel<CHGB_MODEL_SIMPLE_WERTHEIM><<<grid, 256, 0, st>>>(m, rho, der, bins);
            break;
        default: der_bulk_kernel<CHGB_MODEL_SALEH><<<grid, 256, 0, st>>>(m, rho, der, bins); break;
    }
    return cudaGetLastError();
}

namespace {

// src/mobility/RegularisedMobility.h:26-33 and src/mobility/GelMobility.h:41-58.
__global__ void mobility_update_kernel(MobilityDev md, const double *__restrict__ rho, double *__restrict__ gel,
                                       double *__restrict__ mob, int S, long long bins) {
    for(long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < bins; i += (long long) gridDim.x * blockDim.x) {
        if(md.type == CHGB_MOBILITY_REGULARISED) {
            for(int s = 0; s < S; s++) {
                double r = rho[s * bins + i];
                mob[s * bins + i] = md.M * r / (r + md.rho_min);
            }
        }
        else {
            double rho_tot = 0.0;
            for(int s = 0; s < S; s++) rho_tot += rho[s * bins + i];
            double c = gel[i];
            double phi = (rho_tot + 1.0) / 2.0;
            // the two divisions by constants and the exponential take their
            // table-driven / corrected forms (common.cuh): about 28 FP64
            // instructions a cell instead of about 60
            double g = div_known(md.p_gel * phi - md.phi_critical, md.one_m_phic, md.inv_one_m_phic);
            double c_der = md.M_c * (g * c - c * c);
            c += c_der * md.dt;
            gel[i] = c;
            double M = tab_exp(-div_known(c, md.c0, md.inv_c0), md.exptab);
            for(int s = 0; s < S; s++) mob[s * bins + i] = M;
        }
    }
}

}  // namespace

cudaError_t launch_mobility_update(const MobilityDev &md, const double *rho, double *gel, double *mob, int S,
                                   long long bins, cudaStream_t st) {
    mobility_update_kernel<<<grid_for(bins), 256, 0, st>>>(md, rho, gel, mob, S, bins);
    return cudaGetLastError();
}

cudaError_t launch_set_mobility(const ModelDev &m, const double *rho, double M0, double *mob, long long n,
                                cudaStream_t st) {
    set_mobility_kernel<<<grid_for(n), 256, 0, st>>>(m, rho, M0, mob, n);
    return cudaGetLastError();
}

cudaError_t launch_fill(double *p, double v, long long n, cudaStream_t st) {
    fill_kernel<<<grid_for(n), 256, 0, st>>>(p, v, n);
    return cudaGetLastError();
}

cudaError_t launch_fill_noise(double *p, double mean, double amp, long long n, cudaStream_t st) {
    fill_noise_kernel<<<grid_for(n), 256, 0, st>>>(p, mean, amp, n);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// observables
// ---------------------------------------------------------------------------
constexpr int RED_THREADS = 256;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for(int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

template <int KIND, int DIMS>
__global__ void __launch_bounds__(RED_THREADS) observables_partial_kernel(Geom g, ModelDev m, KArr k, double dx,
                                                                         const double *__restrict__ rho,
                                                                         double *__restrict__ partials) {
    constexpr int S = NSpecies<KIND>::value;
    const long long bins = g.bins;
    double mass = 0., fe = 0.;
    for(long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < bins;
        i += (long long) gridDim.x * blockDim.x) {
        int x = (int) (i & g.mask);
        int y = (DIMS >= 2) ? (int) ((i >> g.log2N) & g.mask) : 0;
        int z = (DIMS >= 3) ? (int) ((i >> (2 * g.log2N)) & g.mask) : 0;
        long long nb[3];
        nb[0] = (i - x) + ((x + 1) & g.mask);
        if(DIMS >= 2) nb[1] = i + ((long long) ((((y + 1) & g.mask) - y)) << g.log2N);
        if(DIMS >= 3) nb[2] = i + ((long long) ((((z + 1) & g.mask) - z)) << (2 * g.log2N));
        double r[S];
        double tot = 0.;
        double interfacial = 0.;
#pragma unroll
        for(int s = 0; s < S; s++) {
            r[s] = rho[s * bins + i];
            tot += r[s];
#pragma unroll
            for(int d = 0; d < DIMS; d++) {
                double gr = (rho[s * bins + nb[d]] - r[s]) / dx;
                interfacial += k.v[s] * gr * gr;
            }
        }
        mass += tot;
        fe += bulk_fe<KIND>(m, r) + interfacial;
    }
    __shared__ double sm[2][RED_THREADS / 32];
    mass = warp_sum(mass);
    fe = warp_sum(fe);
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if(lane == 0) {
        sm[0][w] = mass;
        sm[1][w] = fe;
    }
    __syncthreads();
    if(w == 0) {
        mass = (lane < RED_THREADS / 32) ? sm[0][lane] : 0.;
        fe = (lane < RED_THREADS / 32) ? sm[1][lane] : 0.;
        mass = warp_sum(mass);
        fe = warp_sum(fe);
        if(lane == 0) {
            partials[2 * blockIdx.x] = mass;
            partials[2 * blockIdx.x + 1] = fe;
        }
    }
}

__global__ void __launch_bounds__(RED_THREADS) observables_final_kernel(const double *__restrict__ partials,
                                                                       int nblocks, long long nbins_total, double V_bin,
                                                                       double *__restrict__ out) {
    double mass = 0., fe = 0.;
    for(int i = threadIdx.x; i < nblocks; i += blockDim.x) {
        mass += partials[2 * i];
        fe += partials[2 * i + 1];
    }
    __shared__ double sm[2][RED_THREADS / 32];
    mass = warp_sum(mass);
    fe = warp_sum(fe);
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if(lane == 0) {
        sm[0][w] = mass;
        sm[1][w] = fe;
    }
    __syncthreads();
    if(w == 0) {
        mass = (lane < RED_THREADS / 32) ? sm[0][lane] : 0.;
        fe = (lane < RED_THREADS / 32) ? sm[1][lane] : 0.;
        mass = warp_sum(mass);
        fe = warp_sum(fe);
        if(lane == 0) {
            out[0] = mass * V_bin / (double) nbins_total;
            out[1] = fe * V_bin / (double) nbins_total;
        }
    }
}

// Landau pressure of one species, src/models/Landau.cpp:66-71: op mu - f with
// mu = f'(op) and f the bulk free energy, each in the model's own operation
// order (the library is built without FMA contraction).
__device__ __forceinline__ double landau_pressure(double eps, double op) {
    const double mu = -eps * op + op * op * op;
    const double sq = op * op;
    const double f = -0.5 * eps * sq + 0.25 * (sq * sq);
    return op * mu - f;
}

// Per cell and species: p_s(rho) - sum_d 0.5 k_s (grad_d rho_s)^2 with the
// forward difference of src/CahnHilliard.cpp:255-276, written to `field` when
// it is not null, and per-block partial sums of the cells' species sums
// (partials[2b]; partials[2b + 1] = 0 so the observables' final kernel folds them).
template <int DIMS>
__global__ void __launch_bounds__(RED_THREADS) pressure_partial_kernel(Geom g, double eps, KArr k, double dx,
                                                                      const double *__restrict__ rho,
                                                                      double *__restrict__ field,
                                                                      double *__restrict__ partials) {
    const long long bins = g.bins;
    double acc = 0.;
    for(long long i = blockIdx.x * (long long) blockDim.x + threadIdx.x; i < bins;
        i += (long long) gridDim.x * blockDim.x) {
        int x = (int) (i & g.mask);
        int y = (DIMS >= 2) ? (int) ((i >> g.log2N) & g.mask) : 0;
        int z = (DIMS >= 3) ? (int) ((i >> (2 * g.log2N)) & g.mask) : 0;
        long long nb[3];
        nb[0] = (i - x) + ((x + 1) & g.mask);
        if(DIMS >= 2) nb[1] = i + ((long long) ((((y + 1) & g.mask) - y)) << g.log2N);
        if(DIMS >= 3) nb[2] = i + ((long long) ((((z + 1) & g.mask) - z)) << (2 * g.log2N));
        double cell = 0.;
        for(int s = 0; s < g.S; s++) {
            const double r = rho[s * bins + i];
            double v = landau_pressure(eps, r);
#pragma unroll
            for(int d = 0; d < DIMS; d++) {
                const double gr = (rho[s * bins + nb[d]] - r) / dx;
                v -= 0.5 * k.v[s] * gr * gr;
            }
            if(field) field[s * bins + i] = v;
            cell += v;
        }
        acc += cell;
    }
    __shared__ double sm[RED_THREADS / 32];
    acc = warp_sum(acc);
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if(lane == 0) sm[w] = acc;
    __syncthreads();
    if(w == 0) {
        acc = (lane < RED_THREADS / 32) ? sm[lane] : 0.;
        acc = warp_sum(acc);
        if(lane == 0) {
            partials[2 * blockIdx.x] = acc;
            partials[2 * blockIdx.x + 1] = 0.;
        }
    }
}

int observables_blocks(const Geom &g) {
    long long b = ((long long) g.bins + RED_THREADS - 1) / RED_THREADS;
    return (int) (b < 152 * 8 ? b : 152 * 8);
}

template <int KIND>
static void launch_obs_kind(const Geom &g, const ModelDev &m, const KArr &k, double dx, const double *rho,
                            double *partials, int nblocks, cudaStream_t st) {
    switch(g.dims) {
        case 1:
            observables_partial_kernel<KIND, 1><<<nblocks, RED_THREADS, 0, st>>>(g, m, k, dx, rho, partials);
            break;
        case 2:
            observables_partial_kernel<KIND, 2><<<nblocks, RED_THREADS, 0, st>>>(g, m, k, dx, rho, partials);
            break;
        default:
            observables_partial_kernel<KIND, 3><<<nblocks, RED_THREADS, 0, st>>>(g, m, k, dx, rho, partials);
            break;
    }
}

cudaError_t launch_observables(const Geom &g, const ModelDev &m, const double *k, double dx, const double *rho,
                               double *partials, int nblocks, double *out, cudaStream_t st) {
    KArr ka;
    for(int s = 0; s < CHGB_MAX_SPECIES; s++) ka.v[s] = k[s];
    switch(m.kind) {
        case CHGB_MODEL_LANDAU: launch_obs_kind<CHGB_MODEL_LANDAU>(g, m, ka, dx, rho, partials, nblocks, st); break;
        case CHGB_MODEL_SIMPLE_WERTHEIM:
            launch_obs_kind<CHGB_MODEL_SIMPLE_WERTHEIM>(g, m, ka, dx, rho, partials, nblocks, st);
            break;
        default: launch_obs_kind<CHGB_MODEL_SALEH>(g, m, ka, dx, rho, partials, nblocks, st); break;
    }
    cudaError_t e = cudaGetLastError();
    if(e != cudaSuccess) return e;
    double V_bin = dx * dx * dx;
    observables_final_kernel<<<1, RED_THREADS, 0, st>>>(partials, nblocks, (long long) g.bins, V_bin, out);
    return cudaGetLastError();
}

cudaError_t launch_pressure(const Geom &g, double epsilon, const double *k, double dx, const double *rho,
                            double *field, double *partials, int nblocks, double *out, cudaStream_t st) {
    KArr ka;
    for(int s = 0; s < CHGB_MAX_SPECIES; s++) ka.v[s] = k[s];
    switch(g.dims) {
        case 1:
            pressure_partial_kernel<1><<<nblocks, RED_THREADS, 0, st>>>(g, epsilon, ka, dx, rho, field, partials);
            break;
        case 2:
            pressure_partial_kernel<2><<<nblocks, RED_THREADS, 0, st>>>(g, epsilon, ka, dx, rho, field, partials);
            break;
        default:
            pressure_partial_kernel<3><<<nblocks, RED_THREADS, 0, st>>>(g, epsilon, ka, dx, rho, field, partials);
            break;
    }
    cudaError_t e = cudaGetLastError();
    if(e != cudaSuccess) return e;
    // the reference's average_pressure() has no V_bin factor: fold with V_bin = 1
    observables_final_kernel<<<1, RED_THREADS, 0, st>>>(partials, nblocks, (long long) g.bins, 1.0, out);
    return cudaGetLastError();
}

}  // namespace chgb
