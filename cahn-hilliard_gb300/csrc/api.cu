// api.cu — the C ABI of include/chgb.h.
//
// A handle is one simulation box on the current device: two FP64 density
// buffers (psi_in / psi_out, swapped every step), a mobility buffer used only
// to answer chgb_download, the pseudospectral state when that integrator is
// selected, and a private stream.  chgb_step queues kernels only, replayed
// from cached CUDA graphs of 64, 32, ..., 1 time steps so that small grids are
// not bound by launch overhead.  Errors never exit the process: each
// entry point returns a CHGB_* status and records a message.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <random>
#include <vector>
#include <string>

#include "trace.h"
#include "common.cuh"
#include "kernels.h"
#include "handle.h"
#include "spectral.h"

using namespace chgb;

namespace {

constexpr int GRAPH_LOG2 = 6;   // the largest cached graph holds 2^6 = 64 time steps
constexpr int CLUSTER_STEPS_PER_LAUNCH = 1024;   // kernel_variant 4: time steps of one launch (about 1 ms)

std::mutex g_err_mutex;
std::string g_last_error = "";

void set_global_error(const std::string &msg) {
    std::lock_guard<std::mutex> lk(g_err_mutex);
    g_last_error = msg;
}

}  // namespace


namespace chgb {

// True while `st` is being captured into a graph: no allocation then.
static bool stream_is_capturing(cudaStream_t st) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if(cudaStreamIsCapturing(st, &cs) != cudaSuccess) {
        cudaGetLastError();
        return true;
    }
    return cs != cudaStreamCaptureStatusNone;
}

// The table of tab_log (common.cuh) on each device, made once per process and
// kept for its lifetime (LOGTAB_N + 1 entries, 2 KB).  Entries are (1/c_j,
// ln c_j) for c_j = 1 + (j + 1/2)/LOGTAB_N, rounded from long double, then
// ln 2 split into a high part with eleven trailing zero bits (so that k times
// it is exact for any double exponent k) and the rest.
static std::mutex g_logtab_mutex;
static std::map<int, double2 *> g_logtab;

static const double2 *device_log_table(bool alloc) {
    int dev = 0;
    if(cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    std::lock_guard<std::mutex> lock(g_logtab_mutex);
    auto it = g_logtab.find(dev);
    if(it != g_logtab.end()) return it->second;
    if(!alloc) return nullptr;
    std::vector<double2> t(LOGTAB_N + 1);
    for(int j = 0; j < LOGTAB_N; j++) {
        const double c = 1.0 + (j + 0.5) / LOGTAB_N;   // exact
        t[j] = make_double2(1.0 / c, (double) std::log((long double) c));
    }
    const long double ln2 = std::log(2.0L);
    double hi = (double) ln2;
    uint64_t bits;
    std::memcpy(&bits, &hi, sizeof bits);
    bits &= ~((uint64_t) 0x7FF);
    std::memcpy(&hi, &bits, sizeof bits);
    t[LOGTAB_N] = make_double2(hi, (double) (ln2 - (long double) hi));
    double2 *d = nullptr;
    if(cudaMalloc(&d, sizeof(double2) * t.size()) != cudaSuccess ||
       cudaMemcpy(d, t.data(), sizeof(double2) * t.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaGetLastError();
        if(d) cudaFree(d);
        return nullptr;
    }
    g_logtab.emplace(dev, d);
    return d;
}

// The table of tab_exp (common.cuh) on each device, made once per process
// and kept for its lifetime (EXPTAB_N + 2 entries, 1 KB): (lead, trail) of
// 2^(j/64) rounded from long double, then ln2/64 split into L1 (37
// significant bits) and L2, then 64/ln2.
static std::mutex g_exptab_mutex;
static std::map<int, double2 *> g_exptab;

static const double2 *device_exp_table() {
    int dev = 0;
    if(cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    std::lock_guard<std::mutex> lock(g_exptab_mutex);
    auto it = g_exptab.find(dev);
    if(it != g_exptab.end()) return it->second;
    std::vector<double2> t(EXPTAB_N + 2);
    for(int j = 0; j < EXPTAB_N; j++) {
        const long double v = std::exp2((long double) j / EXPTAB_N);
        const double lead = (double) v;
        t[j] = make_double2(lead, (double) (v - (long double) lead));
    }
    const long double L = std::log(2.0L) / EXPTAB_N;              // in [2^-7, 2^-6)
    const long double L1 = std::floor(std::ldexp(L, 43)) / std::ldexp(1.0L, 43);   // 37 significant bits
    t[EXPTAB_N] = make_double2((double) L1, (double) (L - L1));
    t[EXPTAB_N + 1] = make_double2((double) (EXPTAB_N / std::log(2.0L)), 0.0);
    double2 *d = nullptr;
    if(cudaMalloc(&d, sizeof(double2) * t.size()) != cudaSuccess ||
       cudaMemcpy(d, t.data(), sizeof(double2) * t.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaGetLastError();
        if(d) cudaFree(d);
        return nullptr;
    }
    g_exptab.emplace(dev, d);
    return d;
}

ModelDev make_model_dev(const chgb_model_params &mp, bool with_log_table) {
    ModelDev m;
    std::memset(&m, 0, sizeof(m));
    m.kind = mp.kind;
    m.S = mp.n_species;
    m.epsilon = mp.epsilon;
    m.valence = (double) mp.valence;
    m.ivalence = mp.valence;
    m.B2 = mp.B2;
    m.B3 = mp.B3;
    m.two_valence_delta = 2.0 * mp.valence * mp.delta;     // src/models/SimpleWertheim.cpp:33
    m.four_valence_delta = 2.0 * m.two_valence_delta;
    m.two_B2 = 2.0 * mp.B2;
    m.reg_delta = mp.regularisation_delta;
    m.log_delta = std::log(mp.regularisation_delta);        // src/models/SimpleWertheim.cpp:32
    m.sv0 = (double) mp.saleh_valence[0];
    m.sv1 = (double) mp.saleh_valence[1];
    m.half = (double) (mp.saleh_valence[2] / 2);            // src/models/SalehWertheim.cpp:28
    m.dAA = mp.delta_AA;
    m.dBB = mp.delta_BB;
    m.dcf = mp.density_conversion_factor;
    m.logtab = mp.kind == CHGB_MODEL_LANDAU ? nullptr : device_log_table(with_log_table);
    return m;
}

void record_error(const std::string &msg) { set_global_error(msg); }

}  // namespace chgb

static int fail(chgb_handle *h, int code, const std::string &msg) {
    if(h) h->err = msg;
    set_global_error(msg);
    return code;
}

static int cuda_fail(chgb_handle *h, cudaError_t e, const char *what) {
    std::string msg = std::string(what) + ": " + cudaGetErrorString(e);
    return fail(h, CHGB_ERR_CUDA, msg);
}

#define CK(h, call, what)                                   \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if(e_ != cudaSuccess) return cuda_fail(h, e_, what); \
    } while(0)

static int validate(const chgb_params *p, std::string &why) {
    if(!p) {
        why = "params is NULL";
        return CHGB_ERR_INVALID;
    }
    if(p->dims < 1 || p->dims > 3) {
        why = "dims must be 1, 2 or 3";
        return CHGB_ERR_INVALID;
    }
    int maxN = (p->dims == 1) ? (1 << 24) : (p->dims == 2 ? (1 << 14) : 1024);
    if(p->N < 4 || p->N > maxN || (p->N & (p->N - 1)) != 0) {
        why = "N should be a power of 2 (4 <= N <= " + std::to_string(maxN) + " for this dimensionality)";
        return CHGB_ERR_INVALID;
    }
    const chgb_model_params &m = p->model;
    if(m.kind < CHGB_MODEL_LANDAU || m.kind > CHGB_MODEL_SALEH) {
        why = "unsupported free energy model";
        return CHGB_ERR_INVALID;
    }
    int want_species = (m.kind == CHGB_MODEL_SALEH) ? 3 : 1;
    if(m.n_species != want_species) {
        why = "n_species does not match the model";
        return CHGB_ERR_INVALID;
    }
    if(p->integrator < CHGB_INTEGRATOR_EULER || p->integrator > CHGB_INTEGRATOR_PSEUDOSPECTRAL_MOBILITY) {
        why = "unsupported integrator";
        return CHGB_ERR_INVALID;
    }
    if(p->mobility_type < CHGB_MOBILITY_CONSTANT || p->mobility_type > CHGB_MOBILITY_GEL) {
        why = "unknown mobility type";
        return CHGB_ERR_INVALID;
    }
    if(p->mobility_type == CHGB_MOBILITY_GEL && (!(p->gel_c0 != 0.0) || !(p->gel_phi_critical != 1.0))) {
        why = "the gel mobility needs c_0 != 0 and phi_critical != 1";
        return CHGB_ERR_INVALID;
    }
    // src/integrators/Integrator.cpp:38-42 (only euler_mobility and pseudospectral_mobility
    // override _supports_nonconstant_mobility)
    if(p->mobility_type != CHGB_MOBILITY_CONSTANT && p->integrator != CHGB_INTEGRATOR_EULER_MOBILITY &&
       p->integrator != CHGB_INTEGRATOR_PSEUDOSPECTRAL_MOBILITY) {
        why = "The selected integrator only supports constant mobility";
        return CHGB_ERR_UNSUPPORTED;
    }
    // src/models/FreeEnergyModel.h:48-53: only simple_wertheim implements set_mobility
    if(p->mobility_type == CHGB_MOBILITY_FREE_ENERGY && m.kind != CHGB_MODEL_SIMPLE_WERTHEIM) {
        why = "this model does not support mobility coupling";
        return CHGB_ERR_UNSUPPORTED;
    }
    if(p->integrator == CHGB_INTEGRATOR_PSEUDOSPECTRAL_MOBILITY && p->use_gmres &&
       (p->gmres_max_iter < 0 || !(p->gmres_tol >= 0.0) || p->gmres_restart > 4096)) {
        why = "gmres_max_iter and gmres_tol must be non-negative and gmres_restart at most 4096";
        return CHGB_ERR_INVALID;
    }
    if(p->kernel_variant < 0 || p->kernel_variant > 5 ||
       (p->kernel_variant == 3 &&
        (p->integrator != CHGB_INTEGRATOR_EULER || p->dims != 2 || p->N < 32 || p->N > 512)) ||
       (p->kernel_variant == 4 &&
        (p->integrator != CHGB_INTEGRATOR_EULER || p->dims != 2 || (p->N != 32 && p->N != 64))) ||
       (p->kernel_variant == 5 &&
        (p->integrator != CHGB_INTEGRATOR_EULER || p->model.kind != CHGB_MODEL_LANDAU || p->dims < 2 || p->N < 32))) {
        why = "kernel_variant must be 0..5; 3 needs a 2D `euler` box with 32 <= N <= 512, 4 one with N = 32 or 64, "
              "5 a 2D or 3D Landau `euler` box with N >= 32";
        return CHGB_ERR_INVALID;
    }
    if(!(p->dt > 0.0) || !(p->dx > 0.0)) {
        why = "dt and dx must be positive";
        return CHGB_ERR_INVALID;
    }
    return CHGB_OK;
}

extern "C" {
static float time_variant(chgb_handle *h, int nsteps);
}

// A typical density for the model: Landau fields hover around 0, the
// Wertheim models' number densities are of order 1e-5 in internal units.
static double m_kind_density_scale(const ModelDev &m) { return m.kind == CHGB_MODEL_LANDAU ? 0.0 : 1e-5; }

static void release(chgb_handle *h) {
    if(!h) return;
    for(int i = 0; i < 2; i++) {
        for(auto &gl : h->graph)
            if(gl[i]) cudaGraphExecDestroy(gl[i]);
        if(h->d_rho[i]) cudaFree(h->d_rho[i]);
    }
    if(h->d_mob) cudaFree(h->d_mob);
    if(h->d_gel) cudaFree(h->d_gel);
    if(h->d_mu) cudaFree(h->d_mu);
    if(h->d_mobk) cudaFree(h->d_mobk);
    if(h->d_bfp) cudaFree(h->d_bfp);
    if(h->d_partials) cudaFree(h->d_partials);
    if(h->d_obs) cudaFree(h->d_obs);
    if(h->d_pressure) cudaFree(h->d_pressure);
    if(h->ps) spectral_destroy(h->ps);
    if(h->psm) psmob_destroy(h->psm);
    if(h->fft) spectral_destroy(h->fft);
    if(h->sq) sq_plan_destroy(h->sq);
    if(h->own_stream && h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

extern "C" {

int chgb_abi_version(void) { return CHGB_ABI_VERSION; }

int chgb_create(const chgb_params *params, chgb_handle **out) {
    CHGB_TRACE("chgb_create");
    if(!out) return fail(nullptr, CHGB_ERR_INVALID, "out is NULL");
    *out = nullptr;
    std::string why;
    int v = validate(params, why);
    if(v != CHGB_OK) return fail(nullptr, v, why);

    chgb_handle *h = new chgb_handle();
    h->p = *params;
    Geom &g = h->g;
    g.dims = params->dims;
    g.N = params->N;
    g.log2N = 0;
    while((1 << g.log2N) < g.N) g.log2N++;
    g.mask = g.N - 1;
    g.bins = 1;
    for(int d = 0; d < g.dims; d++) g.bins *= g.N;
    g.S = params->model.n_species;
    h->n = (size_t) g.bins * g.S;
    h->m = make_model_dev(params->model);
    double dx2 = params->dx * params->dx;
    for(int s = 0; s < CHGB_MAX_SPECIES; s++) h->ec.c2[s] = 2.0 * params->k[s] / dx2;
    h->ec.c1 = params->dt * params->M / dx2;
    h->ec.dt = params->dt;
    h->ec.half_inv_dx2 = 0.5 / dx2;
    h->ec.M = params->M;
    for(int d = 1; d <= 3; d++) h->ec.lshift[d - 1] = 2.0 * d * h->ec.c2[0] - params->model.epsilon;
    h->ec.mobility_type = params->mobility_type;
    h->ec.mobf = nullptr;
    h->md.type = params->mobility_type;
    h->md.M = params->M;
    h->md.rho_min = params->rho_min;
    {
        // src/mobility/GelMobility.h:20-27
        const double e = std::exp(params->gel_beta_delta_F);
        h->md.p_gel = e / (1.0 + e);
    }
    h->md.phi_critical = params->gel_phi_critical;
    h->md.c0 = params->gel_c0;
    h->md.M_c = params->gel_M_c;
    h->md.dt = params->dt;
    h->md.one_m_phic = 1.0 - params->gel_phi_critical;
    h->md.inv_one_m_phic = 1.0 / h->md.one_m_phic;
    h->md.inv_c0 = 1.0 / params->gel_c0;
    h->md.exptab = params->mobility_type == CHGB_MOBILITY_GEL ? device_exp_table() : nullptr;

    cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if(e != cudaSuccess) {
        int r = cuda_fail(nullptr, e, "cudaStreamCreate");
        release(h);
        return r;
    }
    h->own_stream = true;
    size_t bytes = h->n * sizeof(double);
    bool ok = true;
    if(params->integrator == CHGB_INTEGRATOR_PSEUDOSPECTRAL) {
        ok = cudaMalloc(&h->d_rho[0], bytes) == cudaSuccess;
        int r = ok ? spectral_create(h->p, h->g, h->m, &h->ps, why) : CHGB_ERR_ALLOC;
        if(r != CHGB_OK) {
            release(h);
            return fail(nullptr, r == CHGB_ERR_ALLOC ? CHGB_ERR_ALLOC : r, ok ? why : "cudaMalloc failed");
        }
    }
    else if(params->integrator == CHGB_INTEGRATOR_PSEUDOSPECTRAL_MOBILITY) {
        ok = cudaMalloc(&h->d_rho[0], bytes) == cudaSuccess;
        int r = ok ? psmob_create(h->p, h->g, h->m, &h->psm, why) : CHGB_ERR_ALLOC;
        if(r != CHGB_OK) {
            release(h);
            return fail(nullptr, r, ok ? why : "cudaMalloc failed");
        }
    }
    else {
        ok = cudaMalloc(&h->d_rho[0], bytes) == cudaSuccess && cudaMalloc(&h->d_rho[1], bytes) == cudaSuccess;
        e = launch_euler_step(h->p.integrator, h->g, h->m, h->ec, nullptr, nullptr, h->stream, true);
        if(ok && e != cudaSuccess) {
            int r = cuda_fail(nullptr, e, "kernel configuration");
            release(h);
            return r;
        }
    }
    h->obs_blocks = observables_blocks(h->g);
    const bool field_mob = (params->integrator == CHGB_INTEGRATOR_EULER_MOBILITY &&
                            mobility_kind(params->mobility_type) == 3) ||
                           (params->integrator == CHGB_INTEGRATOR_PSEUDOSPECTRAL_MOBILITY &&
                            params->mobility_type != CHGB_MOBILITY_CONSTANT);
    ok = ok && cudaMalloc(&h->d_mob, bytes) == cudaSuccess &&
         (params->mobility_type != CHGB_MOBILITY_GEL ||
          cudaMalloc(&h->d_gel, sizeof(double) * (size_t) h->g.bins) == cudaSuccess) &&
         cudaMalloc(&h->d_partials, sizeof(double) * 2 * h->obs_blocks) == cudaSuccess &&
         cudaMalloc(&h->d_obs, sizeof(double) * 2) == cudaSuccess;
    if(!ok) {
        cudaGetLastError();
        release(h);
        return fail(nullptr, CHGB_ERR_ALLOC, "device allocation failed");
    }
    cudaMemsetAsync(h->d_rho[0], 0, bytes, h->stream);
    if(h->d_rho[1]) cudaMemsetAsync(h->d_rho[1], 0, bytes, h->stream);
    if(field_mob && !h->psm) h->ec.mobf = h->d_mob;
    if(h->psm && params->mobility_type == CHGB_MOBILITY_CONSTANT) {
        // src/mobility/ConstantMobility.h:18-22 fills the field once
        e = launch_fill(h->d_mob, params->M, (long long) h->n, h->stream);
        if(e != cudaSuccess) {
            int r = cuda_fail(nullptr, e, "mobility");
            release(h);
            return r;
        }
    }

    // Explicit integrators: fused kernel, the split pair (no halo
    // recomputation), two fused steps per launch (small 2D boxes), or the box
    // resident in one cluster's shared memory (N = 32, 64).  All give
    // bit-identical fields; with kernel_variant = 0 each candidate is timed
    // once on the zeroed buffers and the fastest is kept.
    h->variant = 1;
    int want = params->kernel_variant;
    const bool two_ok = !h->ps && !h->psm && euler_two_supported(params->integrator, h->g);
    const bool cluster_ok = !h->ps && !h->psm && euler_cluster_supported(params->integrator, h->g) &&
                            launch_euler_cluster(h->g, h->m, h->ec, nullptr, nullptr, 0, h->stream, true) == cudaSuccess;
    cudaGetLastError();
    if(want == 4 && !cluster_ok) {
        release(h);
        return fail(nullptr, CHGB_ERR_UNSUPPORTED, "kernel_variant 4: this GPU cannot hold a 16-CTA cluster");
    }
    if(two_ok) {
        e = launch_euler_two(h->g, h->m, h->ec, nullptr, nullptr, h->stream, true);
        if(e != cudaSuccess) {
            int r = cuda_fail(nullptr, e, "kernel configuration");
            release(h);
            return r;
        }
    }
    if(!h->ps && !h->psm && euler_split_supported(h->g) && want != 1) {
        bool mob = params->integrator == CHGB_INTEGRATOR_EULER_MOBILITY &&
                   params->mobility_type == CHGB_MOBILITY_FREE_ENERGY;
        const bool bfp_ok = (want == 0 || want == 5) &&
                            euler_bfp_supported(params->integrator, params->model.kind, h->g);
        ok = cudaMalloc(&h->d_mu, bytes) == cudaSuccess && (!mob || cudaMalloc(&h->d_mobk, bytes) == cudaSuccess) &&
             (!bfp_ok || cudaMalloc(&h->d_bfp, sizeof(BfpState)) == cudaSuccess);
        if(!ok) {
            cudaGetLastError();
            if(want == 2 || want == 5) {
                release(h);
                return fail(nullptr, CHGB_ERR_ALLOC, "device allocation failed");
            }
        }
        else if(want >= 2) {
            h->variant = want;
        }
        else if(bfp_ok && ((h->g.dims == 2 && h->g.N >= 512) || (h->g.dims == 3 && h->g.N >= 64))) {
            // block fixed point where it was measured fastest on GB300, by a fixed
            // rule rather than by timing: a configuration always runs the same
            // arithmetic (variant 5 agrees with 1-4 to round-off, not bit for bit)
            h->variant = 5;
        }
        else {
            // The variants are timed on a varied field of the model's scale: on
            // zeros the neighbour sums take their all-zero fallback, whose cost
            // is not that of a real run.
            const double mean = m_kind_density_scale(h->m), amp = mean != 0.0 ? 1e-2 * mean : 1e-2;
            for(int b = 0; b < 2; b++) launch_fill_noise(h->d_rho[b], mean, amp, (long long) h->n, h->stream);
            if(h->d_gel) cudaMemsetAsync(h->d_gel, 0, sizeof(double) * (size_t) h->g.bins, h->stream);
            // a few ms of work per timed replay (an even count, for the two-step kernel)
            int steps = (int) std::min<size_t>(256, std::max<size_t>(4, ((size_t) 1 << 26) / h->n)) & ~1;
            float best = -1.f;
            int pick = 1;
            for(int v = 1; v <= (cluster_ok ? 4 : two_ok ? 3 : 2); v++) {
                h->variant = v;
                float t = time_variant(h, steps);
                if(t > 0.f && (best < 0.f || t < best)) {
                    best = t;
                    pick = v;
                }
            }
            h->variant = pick;
            cudaGetLastError();
        }
        if(h->variant != 2 && !(h->variant == 5 && h->g.dims == 3)) {   // mu is stored by the split pairs only
            if(h->d_mu) cudaFree(h->d_mu);
            if(h->d_mobk) cudaFree(h->d_mobk);
            h->d_mu = h->d_mobk = nullptr;
        }
        if(h->variant != 5 && h->d_bfp) {
            cudaFree(h->d_bfp);
            h->d_bfp = nullptr;
        }
        h->launches = 0;
        h->cur = 0;
        cudaMemsetAsync(h->d_rho[0], 0, bytes, h->stream);
        cudaMemsetAsync(h->d_rho[1], 0, bytes, h->stream);
    }
    else if(want == 2 && !h->ps && !h->psm) {
        release(h);
        return fail(nullptr, CHGB_ERR_INVALID, "kernel_variant 2 needs dims >= 2 and N >= 32");
    }
    else if(want == 5) {
        release(h);
        return fail(nullptr, CHGB_ERR_INVALID, "kernel_variant 5 needs a 2D or 3D Landau `euler` box with N >= 32");
    }
    if(field_mob) {
        // the timing above stepped the mobility too: start it (and the gel
        // order parameter) afresh.  The reference holds zeros until the first
        // update_mobility(); the gel parameter starts from GelMobility's
        // default-seeded std::mt19937 draws (src/mobility/GelMobility.h:28-33).
        cudaMemsetAsync(h->d_mob, 0, bytes, h->stream);
        if(h->d_gel) {
            std::vector<double> op((size_t) h->g.bins);
            std::mt19937 generator;
            std::uniform_real_distribution<double> dist(0.0, 1.0);
            for(auto &v : op) v = dist(generator) * 1e-4;
            if(cudaMemcpyAsync(h->d_gel, op.data(), sizeof(double) * op.size(), cudaMemcpyHostToDevice, h->stream) !=
                   cudaSuccess ||
               cudaStreamSynchronize(h->stream) != cudaSuccess) {
                int r = cuda_fail(nullptr, cudaGetLastError(), "gel order parameter");
                release(h);
                return r;
            }
        }
    }
    if(cudaStreamSynchronize(h->stream) != cudaSuccess) {
        int r = cuda_fail(nullptr, cudaGetLastError(), "create");
        release(h);
        return r;
    }
    *out = h;
    return CHGB_OK;
}

int chgb_kernel_variant(const chgb_handle *h) { return h ? h->variant : 0; }

int chgb_destroy(chgb_handle *h) {
    if(!h) return CHGB_OK;
    if(h->stream) cudaStreamSynchronize(h->stream);
    release(h);
    return CHGB_OK;
}

int chgb_upload(chgb_handle *h, const double *rho, const double *mobility) {
    CHGB_TRACE("chgb_upload");
    if(!h || !rho) return fail(h, CHGB_ERR_INVALID, "NULL argument");
    if(mobility && h->p.mobility_type == CHGB_MOBILITY_CONSTANT) {
        const double M = h->p.M, tol = 1e-12 * std::fabs(M);
        for(size_t i = 0; i < h->n; i++) {
            if(!(std::fabs(mobility[i] - M) <= tol)) {
                char msg[160];
                std::snprintf(msg, sizeof msg, "mobility[%zu] = %.17g differs from the constant mobility M = %.17g",
                              i, mobility[i], M);
                return fail(h, CHGB_ERR_UNSUPPORTED, msg);
            }
        }
    }
    CK(h, cudaMemcpyAsync(h->d_rho[0], rho, h->n * sizeof(double), cudaMemcpyHostToDevice, h->stream),
       "upload rho");
    h->cur = 0;
    h->steps_done = 0;
    if(h->ps) {
        int r = spectral_set_rho(h->ps, h->d_rho[0], h->stream, &h->launches, h->err);
        if(r != CHGB_OK) return fail(h, r, h->err);
    }
    if(h->psm) CK(h, psmob_set_rho(h->psm, h->d_rho[0], h->stream, &h->launches), "pseudospectral_mobility init");
    CK(h, cudaStreamSynchronize(h->stream), "upload sync");
    return CHGB_OK;
}

static bool field_mobility(const chgb_handle *h) { return h->ec.mobf != nullptr; }

static int launches_per_step(const chgb_handle *h) {
    if(h->psm) return psmob_launches_per_step(h->psm) + (h->p.mobility_type != CHGB_MOBILITY_CONSTANT ? 1 : 0);
    const bool pair = h->variant == 2 || (h->variant == 5 && h->g.dims == 3);   // 2D variant 5: one kernel
    return (pair ? 2 : 1) + (field_mobility(h) ? 1 : 0);
}

// pseudospectral_mobility: update_mobility() from the current field, then the step in place.
static cudaError_t one_step_psm(chgb_handle *h) {
    double *rho = h->d_rho[0];
    cudaError_t e = cudaSuccess;
    if(h->p.mobility_type == CHGB_MOBILITY_FREE_ENERGY)
        e = launch_set_mobility(h->m, rho, h->p.M, h->d_mob, (long long) h->n, h->stream);
    else if(h->p.mobility_type != CHGB_MOBILITY_CONSTANT)
        e = launch_mobility_update(h->md, rho, h->d_gel, h->d_mob, h->g.S, (long long) h->g.bins, h->stream);
    int64_t n = 0;
    if(e == cudaSuccess) e = psmob_step(h->psm, h->d_mob, rho, h->stream, &n);
    // the GMRES path launches as many kernels as its iterations need; the
    // M0-splitting path always launches launches_per_step()
    h->launches += h->p.use_gmres ? n + (h->p.mobility_type != CHGB_MOBILITY_CONSTANT ? 1 : 0) : launches_per_step(h);
    return e;
}

static cudaError_t one_step(chgb_handle *h) {
    if(h->psm) return one_step_psm(h);
    const double *in = h->d_rho[h->cur];
    double *outp = h->d_rho[h->cur ^ 1];
    cudaError_t e = cudaSuccess;
    // CahnHilliard::evolve: update_mobility() from this step's input, then the step
    if(field_mobility(h)) {
        e = launch_mobility_update(h->md, in, h->d_gel, h->d_mob, h->g.S, (long long) h->g.bins, h->stream);
        if(e != cudaSuccess) return e;
    }
    if(h->variant == 2) e = launch_euler_split(h->p.integrator, h->g, h->m, h->ec, in, outp, h->d_mu, h->d_mobk, h->stream);
    else if(h->variant == 5) e = launch_euler_bfp(h->g, h->ec, in, outp, h->d_mu, h->d_bfp, h->cur, h->stream);
    else e = launch_euler_step(h->p.integrator, h->g, h->m, h->ec, in, outp, h->stream);
    h->cur ^= 1;
    h->launches += launches_per_step(h);
    return e;
}

// Variant 5: set the block-fixed-point key from the current field, before the
// first step of a sequence (the steps keep it up to date from then on).
static cudaError_t bfp_refresh(chgb_handle *h) {
    if(h->variant != 5) return cudaSuccess;
    h->launches += 1;
    return launch_bfp_refresh(h->d_rho[h->cur], (long long) h->n, h->d_bfp, bfp_key_bank(h->g, h->cur), h->stream);
}

// Queue `steps` time steps as chgb_step's graphs hold them (the timing at
// create records the same): with the two-step kernel, pairs of steps per
// launch and a single fused step for an odd count.
static cudaError_t record_steps(chgb_handle *h, int steps) {
    cudaError_t e = cudaSuccess;
    int i = 0;
    if(h->variant == 4) {
        for(; i < steps && e == cudaSuccess; i += CLUSTER_STEPS_PER_LAUNCH) {
            const int n = std::min(steps - i, CLUSTER_STEPS_PER_LAUNCH);
            e = launch_euler_cluster(h->g, h->m, h->ec, h->d_rho[h->cur], h->d_rho[h->cur ^ 1], n, h->stream);
            h->cur ^= 1;
            h->launches += 1;
        }
        return e;
    }
    if(h->variant == 3) {
        for(; i + 1 < steps && e == cudaSuccess; i += 2) {
            e = launch_euler_two(h->g, h->m, h->ec, h->d_rho[h->cur], h->d_rho[h->cur ^ 1], h->stream);
            h->cur ^= 1;
            h->launches += 1;
        }
    }
    for(; i < steps && e == cudaSuccess; i++) e = one_step(h);
    return e;
}

// Time `nsteps` steps of the current variant on the handle's (zeroed) buffers,
// captured in a CUDA graph as chgb_step runs them, so that a variant with more
// launches per step is not charged host launch overhead it never pays.
// Returns the faster of two replays in ms, or -1 on any failure.
static float time_variant(chgb_handle *h, int nsteps) {
    const int start = h->cur;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool ok = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if(ok) {
        cudaError_t le = record_steps(h, nsteps);
        cudaError_t ee = cudaStreamEndCapture(h->stream, &graph);
        ok = le == cudaSuccess && ee == cudaSuccess;
    }
    h->cur = start;
    ok = ok && cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess;
    if(graph) cudaGraphDestroy(graph);
    cudaEvent_t a = nullptr, b = nullptr;
    ok = ok && cudaEventCreate(&a) == cudaSuccess && cudaEventCreate(&b) == cudaSuccess;
    ok = ok && bfp_refresh(h) == cudaSuccess;
    ok = ok && cudaGraphLaunch(exec, h->stream) == cudaSuccess;   // warm-up
    float best = -1.f;
    for(int rep = 0; rep < 2 && ok; rep++) {
        float ms = -1.f;
        ok = cudaEventRecord(a, h->stream) == cudaSuccess && cudaGraphLaunch(exec, h->stream) == cudaSuccess &&
             cudaEventRecord(b, h->stream) == cudaSuccess && cudaEventSynchronize(b) == cudaSuccess &&
             cudaEventElapsedTime(&ms, a, b) == cudaSuccess;
        if(ok && (best < 0.f || ms < best)) best = ms;
    }
    if(a) cudaEventDestroy(a);
    if(b) cudaEventDestroy(b);
    if(exec) cudaGraphExecDestroy(exec);
    return ok ? best : -1.f;
}

// Kernel launches of one pseudospectral time step (spectral_step).
static int ps_launches_per_step(const chgb_handle *h) { return h->g.dims == 3 ? 4 : 2; }

// Capture 2^lg time steps from the current state into h->graph[lg][parity].
static int build_graph(chgb_handle *h, int lg) {
    const int start = (h->ps || h->psm) ? 0 : h->cur;
    const int steps = 1 << lg;
    int64_t launches0 = h->launches;
    cudaGraph_t graph;
    CK(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    cudaError_t le = cudaSuccess;
    if(h->ps) {
        int64_t dummy = 0;
        std::string e2;
        if(spectral_step(h->ps, steps, h->stream, &dummy, e2) != CHGB_OK) le = cudaErrorUnknown;
    }
    else {
        le = record_steps(h, steps);
        h->graph_flip[lg][start] = h->cur != start;
        if(!h->psm) h->cur = start;
    }
    // counted on every replay instead
    h->graph_launches[lg][start] = h->ps ? (int64_t) steps * ps_launches_per_step(h) : h->launches - launches0;
    h->launches = launches0;
    cudaError_t ee = cudaStreamEndCapture(h->stream, &graph);
    if(le != cudaSuccess) return cuda_fail(h, le, "launch during capture");
    if(ee != cudaSuccess) return cuda_fail(h, ee, "end capture");
    cudaError_t ie = cudaGraphInstantiate(&h->graph[lg][start], graph, 0);
    cudaGraphDestroy(graph);
    if(ie != cudaSuccess) return cuda_fail(h, ie, "graph instantiate");
    return CHGB_OK;
}

// Steps are replayed from cached graphs of 64, 32, ..., 1 steps: nsteps = 64 q
// + r costs q + popcount(r) graph launches and no per-kernel host launches.
int chgb_step(chgb_handle *h, int64_t nsteps) {
    CHGB_TRACE("chgb_step");
    if(!h || nsteps < 0) return fail(h, CHGB_ERR_INVALID, "invalid argument");
    if(nsteps == 0) return CHGB_OK;
    int64_t left = nsteps;
    if(h->ps && !spectral_hat_valid(h->ps)) {
        // first step after an upload reads the real field: not the graphs' form
        int r = spectral_step(h->ps, 1, h->stream, &h->launches, h->err);
        if(r != CHGB_OK) return fail(h, r, h->err);
        left--;
    }
    if(h->psm && h->p.use_gmres) {
        // one graph launch per step, whose restart and Arnoldi loops run on the
        // device (psmob_gmres.cu); such graphs cannot be nested in the step graphs
        for(; left > 0; left--) {
            cudaError_t e = one_step(h);
            if(e != cudaSuccess) return cuda_fail(h, e, "pseudospectral_mobility (GMRES) step");
        }
        h->steps_done += nsteps;
        return CHGB_OK;
    }
    if(h->variant == 4) {
        // the box lives in one cluster's shared memory: a launch runs up to
        // CLUSTER_STEPS_PER_LAUNCH steps, no graphs needed
        cudaError_t e = cudaSuccess;
        while(left > 0 && e == cudaSuccess) {
            const int n = (int) std::min<int64_t>(left, CLUSTER_STEPS_PER_LAUNCH);
            e = record_steps(h, n);
            left -= n;
        }
        if(e != cudaSuccess) return cuda_fail(h, e, "cluster step");
        h->steps_done += nsteps;
        return CHGB_OK;
    }
    const bool no_parity = h->ps || h->psm;
    CK(h, bfp_refresh(h), "block fixed point key");
    while(left > 0) {
        int lg = GRAPH_LOG2;
        while(((int64_t) 1 << lg) > left) lg--;
        const int parity = no_parity ? 0 : h->cur;
        if(!h->graph[lg][parity]) {
            int r = build_graph(h, lg);
            if(r != CHGB_OK) return r;
        }
        CK(h, cudaGraphLaunch(h->graph[lg][parity], h->stream), "graph launch");
        h->launches += h->graph_launches[lg][parity];
        left -= (int64_t) 1 << lg;
        if(h->ps) spectral_mark_stepped(h->ps);
        else if(h->graph_flip[lg][parity]) h->cur ^= 1;
    }
    h->steps_done += nsteps;
    return CHGB_OK;
}

static double *current_rho(chgb_handle *h, int *status) {
    *status = CHGB_OK;
    if(h->ps) {
        *status = spectral_real(h->ps, h->d_rho[0], h->stream, &h->launches, h->err);
        return h->d_rho[0];
    }
    return h->d_rho[h->cur];
}

int chgb_download(chgb_handle *h, double *rho, double *mobility) {
    CHGB_TRACE("chgb_download");
    if(!h) return fail(h, CHGB_ERR_INVALID, "NULL handle");
    int st;
    double *cur = current_rho(h, &st);
    if(st != CHGB_OK) return fail(h, st, h->err);
    if(rho) CK(h, cudaMemcpyAsync(rho, cur, h->n * sizeof(double), cudaMemcpyDeviceToHost, h->stream), "download rho");
    if(mobility) {
        if(field_mobility(h) || h->psm) {
            // the field the last step's update_mobility() computed (zeros before the
            // first step; M everywhere for a constant mobility)
        }
        else if(h->p.mobility_type == CHGB_MOBILITY_FREE_ENERGY) {
            if(h->steps_done > 0) {
                // the mobility of the last step was computed from that step's input,
                // which is the other ping-pong buffer (src/CahnHilliard.cpp:278-282)
                CK(h, launch_set_mobility(h->m, h->d_rho[h->cur ^ 1], h->p.M, h->d_mob, (long long) h->n, h->stream),
                   "mobility");
                h->launches++;
            }
            else {
                CK(h, cudaMemsetAsync(h->d_mob, 0, h->n * sizeof(double), h->stream), "mobility");
            }
        }
        else {
            CK(h, launch_fill(h->d_mob, h->p.M, (long long) h->n, h->stream), "mobility");
            h->launches++;
        }
        CK(h, cudaMemcpyAsync(mobility, h->d_mob, h->n * sizeof(double), cudaMemcpyDeviceToHost, h->stream),
           "download mobility");
    }
    CK(h, cudaStreamSynchronize(h->stream), "download sync");
    return CHGB_OK;
}

int chgb_observables(chgb_handle *h, double *mass, double *free_energy, int32_t *nan_flag) {
    CHGB_TRACE("chgb_observables");
    if(!h) return fail(h, CHGB_ERR_INVALID, "NULL handle");
    int st;
    double *cur = current_rho(h, &st);
    if(st != CHGB_OK) return fail(h, st, h->err);
    CK(h, launch_observables(h->g, h->m, h->p.k, h->p.dx, cur, h->d_partials, h->obs_blocks, h->d_obs, h->stream),
       "observables");
    h->launches += 2;
    double res[2];
    CK(h, cudaMemcpyAsync(res, h->d_obs, sizeof(res), cudaMemcpyDeviceToHost, h->stream), "observables copy");
    CK(h, cudaStreamSynchronize(h->stream), "observables sync");
    bool nan = std::isnan(res[0]) || std::isnan(res[1]);
    if(mass) *mass = res[0];
    if(free_energy) *free_energy = res[1];
    if(nan_flag) *nan_flag = nan ? 1 : 0;
    if(nan) return fail(h, CHGB_ERR_NAN, "Encountered a nan while computing the total mass or free energy");
    return CHGB_OK;
}

int chgb_pressure(chgb_handle *h, double *field, double *average) {
    CHGB_TRACE("chgb_pressure");
    if(!h) return fail(h, CHGB_ERR_INVALID, "NULL handle");
    // FreeEnergyModel::pressure() is critical() for every model but Landau (src/models/FreeEnergyModel.h:43-44)
    if(h->p.model.kind != CHGB_MODEL_LANDAU)
        return fail(h, CHGB_ERR_UNSUPPORTED, "this model does not support the pressure coupling");
    int st;
    double *cur = current_rho(h, &st);
    if(st != CHGB_OK) return fail(h, st, h->err);
    if(field && !h->d_pressure) {
        cudaError_t e = cudaMalloc(&h->d_pressure, h->n * sizeof(double));
        if(e != cudaSuccess) {
            h->d_pressure = nullptr;
            cudaGetLastError();
            return fail(h, CHGB_ERR_ALLOC, std::string("pressure field: ") + cudaGetErrorString(e));
        }
    }
    CK(h, launch_pressure(h->g, h->p.model.epsilon, h->p.k, h->p.dx, cur, field ? h->d_pressure : nullptr,
                          h->d_partials, h->obs_blocks, h->d_obs, h->stream),
       "pressure");
    h->launches += 2;
    double res[2];
    CK(h, cudaMemcpyAsync(res, h->d_obs, sizeof(res), cudaMemcpyDeviceToHost, h->stream), "pressure copy");
    if(field)
        CK(h, cudaMemcpyAsync(field, h->d_pressure, h->n * sizeof(double), cudaMemcpyDeviceToHost, h->stream),
           "pressure field copy");
    CK(h, cudaStreamSynchronize(h->stream), "pressure sync");
    if(average) *average = res[0];
    return CHGB_OK;
}

int chgb_set_stream(chgb_handle *h, void *stream) {
    if(!h) return fail(h, CHGB_ERR_INVALID, "NULL handle");
    CK(h, cudaStreamSynchronize(h->stream), "stream sync");
    if(h->own_stream) cudaStreamDestroy(h->stream);
    for(auto &gl : h->graph) {
        for(auto &ge : gl) {
            if(ge) cudaGraphExecDestroy(ge);
            ge = nullptr;
        }
    }
    if(stream) {
        h->stream = (cudaStream_t) stream;
        h->own_stream = false;
    }
    else {
        CK(h, cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking), "cudaStreamCreate");
        h->own_stream = true;
    }
    return CHGB_OK;
}

int chgb_synchronize(chgb_handle *h) {
    if(!h) return fail(h, CHGB_ERR_INVALID, "NULL handle");
    CK(h, cudaStreamSynchronize(h->stream), "synchronize");
    return CHGB_OK;
}

int chgb_device_rho(chgb_handle *h, double **d_rho) {
    if(!h || !d_rho) return fail(h, CHGB_ERR_INVALID, "NULL argument");
    int st;
    *d_rho = current_rho(h, &st);
    if(st != CHGB_OK) return fail(h, st, h->err);
    return CHGB_OK;
}

int64_t chgb_launch_count(const chgb_handle *h) {
    if(!h) return 0;
    // the GMRES path runs its restart cycles and Arnoldi steps in device-side
    // loops: their kernels are counted on the device
    if(h->psm && h->p.use_gmres) return h->launches + psmob_gmres_loop_launches(h->psm, h->stream);
    return h->launches;
}

int chgb_structure_factor_bins(int32_t N) {
    if(N < 4 || (N & (N - 1)) != 0) return 0;
    return sq_nbins(N);
}

int chgb_structure_factor(chgb_handle *h, int32_t species, double *sq, int32_t nbins) {
    CHGB_TRACE("chgb_structure_factor");
    if(!h || !sq) return fail(h, CHGB_ERR_INVALID, "NULL argument");
    if(h->g.dims != 2) return fail(h, CHGB_ERR_UNSUPPORTED, "S(q) is defined for 2D boxes");
    if(species < 0 || species >= h->g.S) return fail(h, CHGB_ERR_INVALID, "species out of range");
    if(nbins != sq_nbins(h->g.N)) return fail(h, CHGB_ERR_INVALID, "nbins must be chgb_structure_factor_bins(N)");
    std::string err;
    if(!h->sq) {
        h->sq = sq_plan_create(h->g.N, err);
        if(!h->sq) return fail(h, CHGB_ERR_ALLOC, err);
    }
    const double2 *hat;
    if(h->ps) {
        hat = spectral_psi_hat(h->ps, species);
    }
    else {
        if(!h->fft) {
            chgb_params q = h->p;
            q.integrator = CHGB_INTEGRATOR_PSEUDOSPECTRAL;
            q.mobility_type = CHGB_MOBILITY_CONSTANT;
            int r = spectral_create(q, h->g, h->m, &h->fft, err);
            if(r != CHGB_OK) return fail(h, r, err);
        }
        int r = spectral_set_rho(h->fft, h->d_rho[h->cur], h->stream, &h->launches, err);
        if(r != CHGB_OK) return fail(h, r, err);
        hat = spectral_psi_hat(h->fft, species);
    }
    CK(h, sq_compute(h->sq, hat, (double) h->g.bins, h->stream), "S(q)");
    h->launches++;
    CK(h, cudaMemcpyAsync(sq, h->sq->d_sq, sizeof(double) * nbins, cudaMemcpyDeviceToHost, h->stream), "S(q) copy");
    CK(h, cudaStreamSynchronize(h->stream), "S(q) sync");
    return CHGB_OK;
}

const char *chgb_last_error(const chgb_handle *h) {
    if(h) return h->err.c_str();
    std::lock_guard<std::mutex> lk(g_err_mutex);
    return g_last_error.c_str();
}

int chgb_der_bulk_free_energy(const chgb_model_params *model, const double *d_rho, double *d_rho_der, int64_t bins,
                              void *stream) {
    if(!model || !d_rho || !d_rho_der || bins < 0) return fail(nullptr, CHGB_ERR_INVALID, "invalid argument");
    if(model->kind < CHGB_MODEL_LANDAU || model->kind > CHGB_MODEL_SALEH)
        return fail(nullptr, CHGB_ERR_INVALID, "unsupported model");
    if(bins == 0) return CHGB_OK;
    ModelDev m = make_model_dev(*model, !stream_is_capturing((cudaStream_t) stream));
    cudaError_t e = launch_der_bulk(m, d_rho, d_rho_der, bins, (cudaStream_t) stream);
    if(e != cudaSuccess) return cuda_fail(nullptr, e, "der_bulk_free_energy");
    return CHGB_OK;
}

int chgb_set_mobility(const chgb_model_params *model, const double *d_rho, double M0, double *d_mobility,
                      int64_t bins, void *stream) {
    if(!model || !d_rho || !d_mobility || bins < 0) return fail(nullptr, CHGB_ERR_INVALID, "invalid argument");
    if(model->kind != CHGB_MODEL_SIMPLE_WERTHEIM)
        return fail(nullptr, CHGB_ERR_UNSUPPORTED, "this model does not support mobility coupling");
    if(bins == 0) return CHGB_OK;
    ModelDev m = make_model_dev(*model, !stream_is_capturing((cudaStream_t) stream));
    cudaError_t e = launch_set_mobility(m, d_rho, M0, d_mobility, bins, (cudaStream_t) stream);
    if(e != cudaSuccess) return cuda_fail(nullptr, e, "set_mobility");
    return CHGB_OK;
}

}  // extern "C"
