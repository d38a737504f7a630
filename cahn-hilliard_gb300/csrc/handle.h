// handle.h — the state behind a chgb_handle (api.cu, batch.cu).
#pragma once

#include <stdint.h>

#include <string>

#include "common.cuh"
#include "psmob.h"
#include "spectral.h"
#include "sq.h"

namespace chgb {
struct BfpState;   // kernels.h
}

// One simulation box on the current device: two FP64 density buffers
// (psi_in / psi_out, swapped every step), a mobility buffer used only to answer
// chgb_download, the pseudospectral state when that integrator is selected,
// and a private stream.
struct chgb_handle {
    chgb_params p;
    chgb::Geom g;
    chgb::ModelDev m;
    chgb::EulerConsts ec;
    size_t n = 0;                  // S * bins
    double *d_rho[2] = {nullptr, nullptr};
    int cur = 0;
    double *d_mob = nullptr;       // regularised / gel: the mobility field of the last step (a kernel input)
    double *d_gel = nullptr;       // gel: the order parameter, one value per cell
    chgb::MobilityDev md{};        // regularised / gel: the per-step update's constants
    double *d_partials = nullptr;  // 2 * obs_blocks
    double *d_obs = nullptr;       // 2 doubles
    double *d_pressure = nullptr;  // Landau pressure field (S * bins), made on the first chgb_pressure that asks for it
    int obs_blocks = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int64_t steps_done = 0;
    int64_t launches = 0;
    // graph[lg][parity]: 2^lg time steps captured from ping-pong parity `cur`
    // (pseudospectral states have no ping-pong: parity 0 only)
    cudaGraphExec_t graph[7][2] = {};
    int64_t graph_launches[7][2] = {};   // kernels one replay launches
    bool graph_flip[7][2] = {};          // whether a replay swaps the ping-pong buffers
    bool in_batch = false;         // stepped by a chgb_batch only
    chgb::SpectralState *ps = nullptr;
    chgb::PsMob *psm = nullptr;            // pseudospectral_mobility state
    int variant = 1;               // 1 = fused kernel, 2 = split (mu stored once per cell), 3 = two steps per launch,
                                   // 4 = the box resident in one cluster's shared memory, 5 = split in block fixed point
    double *d_mu = nullptr;        // split variant: mu of every cell
    double *d_mobk = nullptr;      // split variant with the free-energy mobility: M of every cell
    chgb::BfpState *d_bfp = nullptr;   // variant 5: the block-fixed-point key and this step's mu scale
    chgb::SqPlan *sq = nullptr;            // S(q) shells, built on first use
    chgb::SpectralState *fft = nullptr;    // forward transform of euler boxes for S(q)
    std::string err;
};
