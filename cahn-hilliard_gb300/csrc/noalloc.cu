// noalloc.cu — observables of a device field without any allocation.
//
// Some callers of this library cannot call cudaMalloc at the moment they need
// the mass and free energy of a field: a host application that has handed the
// whole of HBM to its own pool (a framework's caching allocator, or a solver
// that sizes its fields to fill the device) has nothing left to give, and a
// time-stepping loop with a latency budget cannot afford cudaMalloc/cudaFree,
// which may synchronise the device.  chgb_observables_noalloc serves them: it
// reduces a field the caller owns into two doubles the caller owns, and keeps
// its only scratch -- one partial (mass, free energy) pair per block of
// CHGB_NOALLOC_CELLS_PER_PARTIAL cells -- in the fixed array below, allocated
// when the library is loaded and held on every device that loads it until the
// process exits (CHGB_NOALLOC_MAX_PARTIALS * 16 bytes = 128 KiB).
//
// In host code `g_noalloc_partials` names a host-side stand-in, not device
// memory, so its device address is looked up once per device with
// cudaGetSymbolAddress, with that device current, by the first call made on
// that device; that first call should therefore come before any stream
// capture.  Every call shares the array: each call rewrites the partials it
// reads (nothing has to start at zero), and two calls whose kernels overlap
// on the GPU race on it.
#include <mutex>
#include <string>

#include "common.cuh"
#include "kernels.h"

static __device__ __align__(256) double g_noalloc_partials[2 * CHGB_NOALLOC_MAX_PARTIALS];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double *g_partials_addr[kMaxDevices] = {nullptr};

// Failures are reported through chgb_last_error(NULL), like chgb_create's.
int noalloc_fail(int code, const std::string &msg) {
    chgb::record_error(msg);
    return code;
}

// Device address of the scratch array on the current device (set-up once per device).
int scratch_address(double **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if(e != cudaSuccess) return noalloc_fail(CHGB_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if(dev < 0 || dev >= kMaxDevices) return noalloc_fail(CHGB_ERR_INVALID, "device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_setup_mutex);
    if(!g_partials_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_partials);
        if(e != cudaSuccess || !p) {
            return noalloc_fail(CHGB_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        }
        g_partials_addr[dev] = static_cast<double *>(p);
    }
    *out = g_partials_addr[dev];
    return CHGB_OK;
}

}  // namespace

extern "C" {

int chgb_observables_noalloc(const chgb_params *params, const double *d_rho, double *d_out, void *stream) {
    if(!params || !d_rho || !d_out) return noalloc_fail(CHGB_ERR_INVALID, "NULL argument");
    const chgb_params &p = *params;
    if(p.dims < 1 || p.dims > 3 || p.N < 4 || (p.N & (p.N - 1)) != 0) {
        return noalloc_fail(CHGB_ERR_INVALID, "dims must be 1..3 and N a power of 2 >= 4");
    }
    // The same per-dimension bound as chgb_create, checked before N^dims is formed,
    // so that the cell count below cannot overflow.
    const int maxN = (p.dims == 1) ? (1 << 24) : (p.dims == 2 ? (1 << 14) : 1024);
    if(p.N > maxN) {
        return noalloc_fail(CHGB_ERR_INVALID, "N should be at most " + std::to_string(maxN) +
                                                  " for this dimensionality");
    }
    if(p.model.kind < CHGB_MODEL_LANDAU || p.model.kind > CHGB_MODEL_SALEH ||
       p.model.n_species != (p.model.kind == CHGB_MODEL_SALEH ? 3 : 1)) {
        return noalloc_fail(CHGB_ERR_INVALID, "unsupported free energy model or species count");
    }
    if(!(p.dx > 0.0)) return noalloc_fail(CHGB_ERR_INVALID, "dx must be positive");
    long long bins = 1;
    for(int d = 0; d < p.dims; d++) bins *= p.N;
    long long nblocks = (bins + CHGB_NOALLOC_CELLS_PER_PARTIAL - 1) / CHGB_NOALLOC_CELLS_PER_PARTIAL;
    if(nblocks > CHGB_NOALLOC_MAX_PARTIALS) {
        return noalloc_fail(CHGB_ERR_INVALID,
                            "field of " + std::to_string(bins) + " cells exceeds the no-allocation scratch (at most " +
                                std::to_string((long long) CHGB_NOALLOC_MAX_PARTIALS * CHGB_NOALLOC_CELLS_PER_PARTIAL) +
                                " cells); use chgb_observables");
    }
    double *partials = nullptr;
    int r = scratch_address(&partials);
    if(r != CHGB_OK) return r;

    chgb::Geom g;
    g.dims = p.dims;
    g.N = p.N;
    g.log2N = 0;
    while((1 << g.log2N) < g.N) g.log2N++;
    g.mask = g.N - 1;
    g.bins = (int) bins;
    g.S = p.model.n_species;
    chgb::ModelDev m = chgb::make_model_dev(p.model, false);
    cudaError_t e = chgb::launch_observables(g, m, p.k, p.dx, d_rho, partials, (int) nblocks, d_out,
                                             (cudaStream_t) stream);
    if(e != cudaSuccess) return noalloc_fail(CHGB_ERR_CUDA, std::string("observables: ") + cudaGetErrorString(e));
    return CHGB_OK;
}

}  // extern "C"
