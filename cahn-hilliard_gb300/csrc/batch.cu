// batch.cu — many independent boxes stepped together (chgb_batch_*).
//
// The reference runs one box per process: its integrators keep `static`
// scratch inside evolve() (src/integrators/EulerCPU.cpp:19,
// PseudospectralCPU.cpp:113), so replicas cannot share a process.  Here each
// replica is an ordinary handle (chgb_create), and the batch steps them
// together:
//
// * 2D `euler` replicas of one model form a group stepped by ONE kernel per
//   time step whose CTAs walk a work list of (replica, tile) items.  All tiles
//   have the same shape, so every CTA carries the same work whatever the
//   replicas' N and the SMs stay balanced.  The tile shape (16x16, 32x32 or
//   64x16) is picked at creation by timing each candidate (autotune).
// * 2D `pseudospectral` replicas of one model form a group stepped by two
//   kernels per time step: a row pass over (replica, rows) items and a column
//   pass (forward FFT, update, inverse FFT) over (replica, species, columns)
//   items, longest items first.
// * Everything else runs on its own handle and stream, concurrently.
// Consecutive steps are replayed from one CUDA graph of GRAPH_STEPS steps of
// all groups.  The per-replica arithmetic is the single-box kernels', so a
// replica stepped in a batch gives the same bits as stepped alone.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "trace.h"
#include "handle.h"
#include "kernels.h"
#include "spectral.h"

using namespace chgb;

namespace {

constexpr int GRAPH_STEPS = 32;   // even: the ping-pong parity returns to its start

struct EulerGroup {
    int kind = 0;
    int tile = 32;
    std::vector<int> members;
    EulerBatchRep *d_reps = nullptr;
    int2 *d_items = nullptr;
    int nitems = 0;
};

struct PsGroup {
    int kind = 0;
    std::vector<int> members;
    PsBatchRep *d_reps = nullptr;
    int2 *d_rows = nullptr;
    int4 *d_cols = nullptr;
    int nrows = 0, ncols = 0;
    size_t row_smem = 0, col_smem = 0;
};

}  // namespace

struct chgb_batch {
    std::vector<chgb_handle *> h;
    cudaStream_t stream = nullptr;
    std::vector<EulerGroup> eg;
    std::vector<PsGroup> pg;
    std::vector<int> loose;
    cudaGraphExec_t graph = nullptr;
    int parity = 0;            // every euler-group replica is at cur == parity
    int64_t launches = 0;
    std::string err;
};

static int bfail(chgb_batch *b, int code, const std::string &msg) {
    if(b) b->err = msg;
    record_error(msg);
    return code;
}

static void batch_release(chgb_batch *b) {
    if(!b) return;
    if(b->stream) cudaStreamSynchronize(b->stream);
    if(b->graph) cudaGraphExecDestroy(b->graph);
    for(auto &g : b->eg) {
        if(g.d_reps) cudaFree(g.d_reps);
        if(g.d_items) cudaFree(g.d_items);
    }
    for(auto &g : b->pg) {
        if(g.d_reps) cudaFree(g.d_reps);
        if(g.d_rows) cudaFree(g.d_rows);
        if(g.d_cols) cudaFree(g.d_cols);
    }
    for(auto *h : b->h) chgb_destroy(h);
    if(b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

// Device arrays of one euler group for a tile size; parity-agnostic (a/b are
// the replicas' buffers 0 and 1).
static cudaError_t euler_group_upload(chgb_batch *b, EulerGroup &g, int tile) {
    int TX = (tile == 64) ? 64 : tile, TY = (tile == 64) ? 16 : tile;
    std::vector<EulerBatchRep> reps;
    std::vector<int2> items;
    for(size_t r = 0; r < g.members.size(); r++) {
        chgb_handle *h = b->h[g.members[r]];
        EulerBatchRep e;
        e.a = h->d_rho[0];
        e.b = h->d_rho[1];
        e.g = h->g;
        e.m = h->m;
        e.c = h->ec;
        reps.push_back(e);
        int nt = (h->g.N / TX) * (h->g.N / TY);
        for(int t = 0; t < nt; t++) items.push_back(make_int2((int) r, t));
    }
    if(g.d_reps) cudaFree(g.d_reps);
    if(g.d_items) cudaFree(g.d_items);
    g.d_reps = nullptr;
    g.d_items = nullptr;
    cudaError_t e = cudaMalloc(&g.d_reps, sizeof(EulerBatchRep) * reps.size());
    if(e == cudaSuccess) e = cudaMalloc(&g.d_items, sizeof(int2) * items.size());
    if(e == cudaSuccess) e = cudaMemcpy(g.d_reps, reps.data(), sizeof(EulerBatchRep) * reps.size(), cudaMemcpyHostToDevice);
    if(e == cudaSuccess) e = cudaMemcpy(g.d_items, items.data(), sizeof(int2) * items.size(), cudaMemcpyHostToDevice);
    g.nitems = (int) items.size();
    g.tile = tile;
    if(e == cudaSuccess) e = launch_euler2d_batch(g.kind, tile, nullptr, nullptr, 0, 0, true, b->stream);
    return e;
}

static cudaError_t ps_group_upload(chgb_batch *b, PsGroup &g) {
    std::vector<PsBatchRep> reps(g.members.size());
    struct Work {
        long long cost;
        int4 v;
    };
    std::vector<Work> rows, cols;
    for(size_t r = 0; r < g.members.size(); r++) {
        chgb_handle *h = b->h[g.members[r]];
        size_t rs, cs;
        spectral_batch_rep(h->ps, &reps[r], &rs, &cs);
        g.row_smem = std::max(g.row_smem, rs);
        g.col_smem = std::max(g.col_smem, cs);
        const PsBatchRep &p = reps[r];
        long long lg = p.log2N;
        for(int row0 = 0; row0 < p.N; row0 += p.row_rpc)
            rows.push_back({(long long) p.row_rpc * p.N * lg * h->g.S, make_int4((int) r, row0, 0, 0)});
        for(int s = 0; s < h->g.S; s++)
            for(int kx0 = 0; kx0 < p.H; kx0 += p.col_C)
                cols.push_back({(long long) std::min(p.col_C, p.H - kx0) * p.N * lg, make_int4((int) r, s, kx0, 0)});
    }
    // longest items first, so the last wave is made of the short ones
    auto by_cost = [](const Work &a, const Work &c) { return a.cost > c.cost; };
    std::stable_sort(rows.begin(), rows.end(), by_cost);
    std::stable_sort(cols.begin(), cols.end(), by_cost);
    std::vector<int2> r2;
    for(auto &w : rows) r2.push_back(make_int2(w.v.x, w.v.y));
    std::vector<int4> c4;
    for(auto &w : cols) c4.push_back(w.v);
    g.nrows = (int) r2.size();
    g.ncols = (int) c4.size();
    cudaError_t e = cudaMalloc(&g.d_reps, sizeof(PsBatchRep) * reps.size());
    if(e == cudaSuccess) e = cudaMalloc(&g.d_rows, sizeof(int2) * r2.size());
    if(e == cudaSuccess) e = cudaMalloc(&g.d_cols, sizeof(int4) * c4.size());
    if(e == cudaSuccess) e = cudaMemcpy(g.d_reps, reps.data(), sizeof(PsBatchRep) * reps.size(), cudaMemcpyHostToDevice);
    if(e == cudaSuccess) e = cudaMemcpy(g.d_rows, r2.data(), sizeof(int2) * r2.size(), cudaMemcpyHostToDevice);
    if(e == cudaSuccess) e = cudaMemcpy(g.d_cols, c4.data(), sizeof(int4) * c4.size(), cudaMemcpyHostToDevice);
    if(e == cudaSuccess) e = configure_ps2d_batch(g.kind, g.row_smem, g.col_smem);
    return e;
}

// One time step of every group on the batch stream.
static cudaError_t batched_step(chgb_batch *b, int parity, bool ps_batched) {
    for(auto &g : b->eg) {
        cudaError_t e = launch_euler2d_batch(g.kind, g.tile, g.d_reps, g.d_items, g.nitems, parity, false, b->stream);
        if(e != cudaSuccess) return e;
    }
    if(ps_batched) {
        for(auto &g : b->pg) {
            cudaError_t e = launch_ps2d_batch(g.kind, g.d_reps, g.d_rows, g.nrows, g.d_cols, g.ncols, g.row_smem,
                                              g.col_smem, b->stream);
            if(e != cudaSuccess) return e;
        }
    }
    return cudaSuccess;
}

static int launches_per_batched_step(const chgb_batch *b) {
    int n = 0;
    for(auto &g : b->eg) n += g.nitems > 0 ? 1 : 0;
    for(auto &g : b->pg) n += (g.nrows > 0 ? 1 : 0) + (g.ncols > 0 ? 1 : 0);
    return n;
}

// Pick the euler tile of each group by timing a few batched steps of each candidate.
static cudaError_t autotune(chgb_batch *b) {
    for(auto &g : b->eg) {
        int minN = 1 << 30;
        for(int i : g.members) minN = std::min(minN, b->h[i]->g.N);
        std::vector<int> cands;
        if(minN >= 32) cands.push_back(32);
        if(minN >= 64) cands.push_back(64);
        cands.push_back(16);
        float best = -1.f;
        int best_tile = cands.front();
        for(int tile : cands) {
            cudaError_t e = euler_group_upload(b, g, tile);
            if(e != cudaSuccess) return e;
            if(cands.size() == 1) break;
            cudaEvent_t t0, t1;
            cudaEventCreate(&t0);
            cudaEventCreate(&t1);
            launch_euler2d_batch(g.kind, tile, g.d_reps, g.d_items, g.nitems, 0, false, b->stream);
            cudaEventRecord(t0, b->stream);
            for(int s = 0; s < 4; s++)
                launch_euler2d_batch(g.kind, tile, g.d_reps, g.d_items, g.nitems, (s + 1) & 1, false, b->stream);
            cudaEventRecord(t1, b->stream);
            e = cudaEventSynchronize(t1);
            float ms = -1.f;
            if(e == cudaSuccess) cudaEventElapsedTime(&ms, t0, t1);
            cudaEventDestroy(t0);
            cudaEventDestroy(t1);
            if(e != cudaSuccess) return e;
            if(ms > 0.f && (best < 0.f || ms < best)) {
                best = ms;
                best_tile = tile;
            }
        }
        if(g.tile != best_tile) {
            cudaError_t e = euler_group_upload(b, g, best_tile);
            if(e != cudaSuccess) return e;
        }
        // timing runs wrote the zeroed buffers; clear them again
        for(int i : g.members) {
            chgb_handle *h = b->h[i];
            cudaMemsetAsync(h->d_rho[0], 0, h->n * sizeof(double), b->stream);
            cudaMemsetAsync(h->d_rho[1], 0, h->n * sizeof(double), b->stream);
        }
    }
    return cudaStreamSynchronize(b->stream);
}

extern "C" {

int chgb_batch_create(const chgb_params *params, int32_t n, chgb_batch **out) {
    CHGB_TRACE("chgb_batch_create");
    if(!params || !out || n <= 0) return bfail(nullptr, CHGB_ERR_INVALID, "invalid argument");
    *out = nullptr;
    chgb_batch *b = new chgb_batch();
    if(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
        batch_release(b);
        return bfail(nullptr, CHGB_ERR_CUDA, "cudaStreamCreate failed");
    }
    for(int i = 0; i < n; i++) {
        chgb_params p = params[i];
        bool batchable_euler = p.integrator == CHGB_INTEGRATOR_EULER && p.dims == 2 && p.N >= 16;
        if(batchable_euler) p.kernel_variant = 1;   // the batch runs its own kernels: skip the per-handle autotune
        chgb_handle *h = nullptr;
        int r = chgb_create(&p, &h);
        if(r != CHGB_OK) {
            std::string msg = "replica " + std::to_string(i) + ": " + chgb_last_error(nullptr);
            batch_release(b);
            return bfail(nullptr, r, msg);
        }
        b->h.push_back(h);
        int kind = p.model.kind;
        if(batchable_euler) {
            auto it = std::find_if(b->eg.begin(), b->eg.end(), [&](const EulerGroup &g) { return g.kind == kind; });
            if(it == b->eg.end()) {
                b->eg.push_back(EulerGroup());
                b->eg.back().kind = kind;
                it = b->eg.end() - 1;
            }
            it->members.push_back(i);
            h->in_batch = true;
        }
        else if(h->ps && spectral_batchable(h->ps)) {
            auto it = std::find_if(b->pg.begin(), b->pg.end(), [&](const PsGroup &g) { return g.kind == kind; });
            if(it == b->pg.end()) {
                b->pg.push_back(PsGroup());
                b->pg.back().kind = kind;
                it = b->pg.end() - 1;
            }
            it->members.push_back(i);
            h->in_batch = true;
        }
        else {
            b->loose.push_back(i);
        }
    }
    cudaError_t e = cudaSuccess;
    for(auto &g : b->pg)
        if(e == cudaSuccess) e = ps_group_upload(b, g);
    if(e == cudaSuccess) e = autotune(b);
    if(e != cudaSuccess) {
        std::string msg = std::string("batch set-up: ") + cudaGetErrorString(e);
        batch_release(b);
        return bfail(nullptr, CHGB_ERR_CUDA, msg);
    }
    *out = b;
    return CHGB_OK;
}

int chgb_batch_destroy(chgb_batch *b) {
    batch_release(b);
    return CHGB_OK;
}

int chgb_batch_size(const chgb_batch *b) { return b ? (int) b->h.size() : 0; }

int chgb_batch_upload(chgb_batch *b, int32_t i, const double *rho) {
    if(!b || i < 0 || i >= (int) b->h.size()) return bfail(b, CHGB_ERR_INVALID, "replica index out of range");
    if(cudaStreamSynchronize(b->stream) != cudaSuccess) return bfail(b, CHGB_ERR_CUDA, "batch synchronize failed");
    chgb_handle *h = b->h[i];
    int r = chgb_upload(h, rho, nullptr);
    if(r != CHGB_OK) return bfail(b, r, chgb_last_error(h));
    return CHGB_OK;
}

int chgb_batch_step(chgb_batch *b, int64_t nsteps) {
    CHGB_TRACE("chgb_batch_step");
    if(!b || nsteps < 0) return bfail(b, CHGB_ERR_INVALID, "invalid argument");
    if(nsteps == 0) return CHGB_OK;
    // euler groups: bring every replica to the same parity
    for(auto &g : b->eg) {
        for(int i : g.members) {
            chgb_handle *h = b->h[i];
            if(h->cur != b->parity) {
                cudaMemcpyAsync(h->d_rho[b->parity], h->d_rho[h->cur], h->n * sizeof(double), cudaMemcpyDeviceToDevice,
                                b->stream);
                h->cur = b->parity;
            }
        }
    }
    int64_t done = 0;
    // pseudospectral groups: a replica just uploaded takes its first step from
    // the real field, alone; the group then continues batched
    bool fresh = false;
    for(auto &g : b->pg)
        for(int i : g.members) fresh = fresh || !spectral_hat_valid(b->h[i]->ps);
    if(fresh) {
        cudaError_t e = batched_step(b, b->parity, false);
        if(e != cudaSuccess) return bfail(b, CHGB_ERR_CUDA, std::string("batched step: ") + cudaGetErrorString(e));
        b->launches += (int64_t) b->eg.size();
        for(auto &g : b->pg) {
            for(int i : g.members) {
                chgb_handle *h = b->h[i];
                std::string err;
                int r = spectral_step(h->ps, 1, b->stream, &b->launches, err);
                if(r != CHGB_OK) return bfail(b, r, err);
            }
        }
        b->parity ^= 1;
        done = 1;
    }
    // loose replicas run on their own streams, concurrently with the batched groups
    for(int i : b->loose) {
        int r = chgb_step(b->h[i], nsteps);
        if(r != CHGB_OK) return bfail(b, r, chgb_last_error(b->h[i]));
    }
    const int per_step = launches_per_batched_step(b);
    while(nsteps - done >= GRAPH_STEPS && per_step > 0) {
        if(!b->graph || b->parity != 0) {
            if(b->parity != 0) {   // a graph is recorded from parity 0 only
                cudaError_t e = batched_step(b, b->parity, true);
                if(e != cudaSuccess) return bfail(b, CHGB_ERR_CUDA, std::string("batched step: ") + cudaGetErrorString(e));
                b->launches += per_step;
                b->parity ^= 1;
                done++;
                continue;
            }
            cudaGraph_t graph;
            if(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
                return bfail(b, CHGB_ERR_CUDA, "begin capture failed");
            cudaError_t le = cudaSuccess;
            for(int s = 0; s < GRAPH_STEPS && le == cudaSuccess; s++) le = batched_step(b, s & 1, true);
            cudaError_t ee = cudaStreamEndCapture(b->stream, &graph);
            if(le != cudaSuccess || ee != cudaSuccess)
                return bfail(b, CHGB_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(le != cudaSuccess ? le : ee));
            cudaError_t ie = cudaGraphInstantiate(&b->graph, graph, 0);
            cudaGraphDestroy(graph);
            if(ie != cudaSuccess) return bfail(b, CHGB_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(ie));
        }
        if(cudaGraphLaunch(b->graph, b->stream) != cudaSuccess) return bfail(b, CHGB_ERR_CUDA, "graph launch failed");
        b->launches += (int64_t) GRAPH_STEPS * per_step;
        done += GRAPH_STEPS;
    }
    for(; done < nsteps; done++) {
        cudaError_t e = batched_step(b, b->parity, true);
        if(e != cudaSuccess) return bfail(b, CHGB_ERR_CUDA, std::string("batched step: ") + cudaGetErrorString(e));
        b->launches += per_step;
        b->parity ^= 1;
    }
    for(auto &g : b->eg) {
        for(int i : g.members) {
            b->h[i]->cur = b->parity;
            b->h[i]->steps_done += nsteps;
        }
    }
    for(auto &g : b->pg) {
        for(int i : g.members) {
            spectral_mark_stepped(b->h[i]->ps);
            b->h[i]->steps_done += nsteps;
        }
    }
    return CHGB_OK;
}

int chgb_batch_synchronize(chgb_batch *b) {
    if(!b) return bfail(b, CHGB_ERR_INVALID, "NULL batch");
    if(cudaStreamSynchronize(b->stream) != cudaSuccess) return bfail(b, CHGB_ERR_CUDA, "batch synchronize failed");
    for(int i : b->loose) {
        int r = chgb_synchronize(b->h[i]);
        if(r != CHGB_OK) return bfail(b, r, chgb_last_error(b->h[i]));
    }
    return CHGB_OK;
}

int chgb_batch_download(chgb_batch *b, int32_t i, double *rho) {
    CHGB_TRACE("chgb_batch_download");
    if(!b || i < 0 || i >= (int) b->h.size()) return bfail(b, CHGB_ERR_INVALID, "replica index out of range");
    if(cudaStreamSynchronize(b->stream) != cudaSuccess) return bfail(b, CHGB_ERR_CUDA, "batch synchronize failed");
    int r = chgb_download(b->h[i], rho, nullptr);
    if(r != CHGB_OK) return bfail(b, r, chgb_last_error(b->h[i]));
    return CHGB_OK;
}

chgb_handle *chgb_batch_replica(chgb_batch *b, int32_t i) {
    if(!b || i < 0 || i >= (int) b->h.size()) return nullptr;
    cudaStreamSynchronize(b->stream);
    return b->h[i];
}

int64_t chgb_batch_launch_count(const chgb_batch *b) {
    if(!b) return 0;
    int64_t n = b->launches;
    for(int i : b->loose) n += chgb_launch_count(b->h[i]);
    return n;
}

int chgb_batch_euler_tile(const chgb_batch *b) { return (b && !b->eg.empty()) ? b->eg.front().tile : 0; }

}  // extern "C"
