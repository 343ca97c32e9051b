// wf_kernels.h -- launchers of the step kernels (one set per arithmetic form).
#pragma once

#include <cuda_runtime.h>

#include "wf_fields.cuh"

struct WfLaunchCfg {
    cudaStream_t stream;
    int num_sms;
    int vertical_block;   // threads per block of per-cell kernels
    int walk_warps;       // warps per block of wavefront kernels
    int walk_blocks;      // blocks of the persistent wavefront grid (0 = occupancy)
    int sub_lanes;        // cap of the sub-step lanes of the diagonal schedule (0 = default)
    int vertical_blocks_per_sm;  // grid of the split vertical kernel (0 = 16 per SM)
    int walk_inputs;      // bit k: node-major sweep k (0 subsurface, 1 overland, 2 river) holds its inputs
                          // in registers instead of staging them in shared memory
};

// FP64 plain form (kernels_fp64.cu)
cudaError_t wf_fp64_vertical(const WfDevFields& F, const WfLaunchCfg& c);
cudaError_t wf_fp64_ssf(const WfDevFields& F, const WfDevGraph& g, const WfSweep& sw, const WfLaunchCfg& c);
cudaError_t wf_fp64_overland(const WfDevFields& F, const WfDevGraph& g, const WfSweep& sw, const WfLaunchCfg& c);
cudaError_t wf_fp64_river(const WfDevFields& F, const WfDevGraph& g, const WfSweep& sw, const WfLaunchCfg& c);
cudaError_t wf_fp64_balance(const WfDevFields& F, const WfLaunchCfg& c);
cudaError_t wf_fp64_vwc(const WfDevFields& F, int layer, double* out, const WfLaunchCfg& c);
// the per-cell update split at the gravitational snow transport: interception and snow, then
// glacier, open water and soil
cudaError_t wf_fp64_vertical_snow(const WfDevFields& F, const WfLaunchCfg& c);
cudaError_t wf_fp64_vertical_soil(const WfDevFields& F, const WfLaunchCfg& c);

// Gravitational snow transport, both forms (kernels_fp64.cu): one material's sweep over the land
// graph (0 snow storage, 1 snow water; one sub-step of the model step) and the inflow per cell.
cudaError_t wf_snow_transport_sweep(const WfDevFields& F, const WfDevGraph& g, const WfSweep& sw, int material,
                                    const WfLaunchCfg& c);
cudaError_t wf_snow_in(const WfDevFields& F, const WfDevGraph& g, const WfLaunchCfg& c);

// Local-inertial land and river routing in the step (wf_li_couple.cuh; FP64 form, one member):
// the scheme's inputs before its step, its results and (balance != 0) the overland balance after it.
struct WfLiCoupleView;
cudaError_t wf_fp64_li_couple_in(const WfDevFields& F, const WfLiCoupleView& v, const WfLaunchCfg& c);
cudaError_t wf_fp64_li_couple_out(const WfDevFields& F, const WfLiCoupleView& v, int balance, const WfLaunchCfg& c);

// FP32/FP64 split form (kernels_split.cu)
cudaError_t wf_split_vertical(const WfDevFields& F, const WfLaunchCfg& c);
cudaError_t wf_split_vertical_snow(const WfDevFields& F, const WfLaunchCfg& c);
cudaError_t wf_split_vertical_soil(const WfDevFields& F, const WfLaunchCfg& c);
cudaError_t wf_split_ssf(const WfDevFields& F, const WfDevGraph& g, const WfSweep& sw, const WfLaunchCfg& c);
cudaError_t wf_split_balance(const WfDevFields& F, const WfLaunchCfg& c);
// slim wavefronts of the split form (wf_wave.cuh) and their per-cell completion kernels
cudaError_t wf_split_ssf_wave(const WfDevFields& F, const WfDevGraph& g, const WfSweep& sw, const WfLaunchCfg& c);
cudaError_t wf_split_overland_wave(const WfDevFields& F, const WfDevGraph& g, const WfSweep& sw,
                                   const WfLaunchCfg& c);
cudaError_t wf_split_river_wave(const WfDevFields& F, const WfDevGraph& g, const WfSweep& sw, const WfLaunchCfg& c);
// The overland sweep (all its sub-steps, swl) and the river's first sub-step group (swr) in one
// persistent launch; the land graph's ticket counter serves both (overland tickets first).
cudaError_t wf_split_overland_river_wave(const WfDevFields& F, const WfDevGraph& gl, const WfSweep& swl,
                                         const WfDevGraph& gr, const WfSweep& swr, const WfLaunchCfg& c);
cudaError_t wf_split_ssf_post(const WfDevFields& F, const WfDevGraph& g, const WfLaunchCfg& c);
cudaError_t wf_split_overland_post(const WfDevFields& F, const WfDevGraph& g, const WfLaunchCfg& c);
cudaError_t wf_split_river_post(const WfDevFields& F, const WfDevGraph& g, const WfLaunchCfg& c);
cudaError_t wf_split_sync_u(const WfDevFields& F, const WfLaunchCfg& c);
cudaError_t wf_split_vwc(const WfDevFields& F, int layer, double* out, const WfLaunchCfg& c);

// Reservoirs, both forms (kernels_fp64.cu): before the river sweep (start-of-step storage,
// inflow from the outlet cell's land routing, reset of the step's cumulatives) and after it
// (averages and water balance). No launch without reservoirs.
cudaError_t wf_reservoir_prep(const WfDevFields& F, const WfLaunchCfg& c);
cudaError_t wf_reservoir_post(const WfDevFields& F, const WfLaunchCfg& c);

// Adaptive sub-stepping (kernels_adaptive.cu): size and flags of every member's next sub-step
// of the sweep A.kind, from the current state; sets *A.more when a further sub-step follows.
cudaError_t wf_adaptive_substep(const WfDevFields& F, const WfAdaptive& A, const WfLaunchCfg& c);

// gather/scatter between the external (land/river) order and the slot order
cudaError_t wf_gather_ext(const double* src_ext, double* dst_slots, const int64_t* node_of_slot, int64_t slots,
                          int M, int64_t n_ext, cudaStream_t s);
cudaError_t wf_scatter_ext(const double* src_slots, double* dst_ext, const int64_t* node_of_slot, int64_t slots,
                           int M, int64_t n_ext, cudaStream_t s);
