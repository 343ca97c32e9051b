// wf_launch.cuh -- grid of the persistent wavefront kernels.
#pragma once

#include <algorithm>
#include <cstdint>

#include <cuda_runtime.h>

#include "wf_fields.cuh"
#include "wf_kernels.h"

// Blocks of a persistent wavefront launch and the number of work items dispatched first.
//
// The grid is every block that fits on the device at once (occupancy), capped by the work.
// The longest chains (the plan's trailing long chunks) carry the critical path, so up to half
// of the resident warps take them first; the remaining warps take the other chunks in chain
// length order. Progress is guaranteed: a chunk only waits for shorter chains; shorter chains
// are either long chunks already resident or ordinary chunks, which at least half of the
// resident warps keep dispatching in dependency order.
template <class Kernel>
cudaError_t wave_grid(Kernel kernel, int threads, size_t smem, const WfLaunchCfg& c, const WfDevGraph& g, int& blocks,
                      int64_t& prio_items, int64_t items_per_chunk = 0) {
    int per_sm = 0;
    const cudaError_t err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
    if (err != cudaSuccess) return err;
    if (per_sm < 1) per_sm = 1;
    blocks = c.walk_blocks > 0 ? c.walk_blocks : c.num_sms * per_sm;
    const int wpb = threads / 32;
    const int64_t ipc = items_per_chunk > 0 ? items_per_chunk : (g.M > 32 ? g.M / 32 : 1);
    const int64_t items = g.n_chunks * ipc;
    const int64_t need = (items + wpb - 1) / wpb;
    if (blocks > need) blocks = (int)(need < 1 ? 1 : need);
    const int64_t resident = (int64_t)std::min(blocks, c.num_sms * per_sm) * wpb;
    prio_items = std::min<int64_t>(g.n_long_chunks * ipc, resident / 2);
    return cudaSuccess;
}

// Sub-step lanes of a diagonal-schedule launch of S sub-steps: the smallest power of two that
// covers S, at most the cap (tuning; 8 by default) and at most 32.
inline int wave_sub_lanes(int S, const WfLaunchCfg& c) {
    const int cap = c.sub_lanes > 0 ? std::min(c.sub_lanes, 32) : 8;
    int sl = 1;
    while (sl < S && sl < cap) sl <<= 1;
    return sl;
}
