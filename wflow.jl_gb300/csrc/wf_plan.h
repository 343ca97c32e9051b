// wf_plan.h -- wavefront schedule of a drainage graph for the routing kernels.
//
// Wflow sweeps the kinematic wave over the D8 graph in topological order, each cell using the
// new discharge of its upstream cells (Wflow/src/routing/surface/surface_kinwave.jl:293-341,
// routing/subsurface/lateral_subsurface_flow.jl:198-273). The GPU schedule decomposes the
// forest into chains by a long-path decomposition: every node continues the chain of its
// highest upstream child (the "heavy" child), so a chain is walked leaf-to-outlet by one warp
// lane with the heavy inflow carried in registers, and the other (light) upstream children are
// ends of strictly shorter chains. A node at position k of its chain has height k, so chains
// sorted by length form a valid dependency order: a lane only ever waits for chains dispatched
// before its own, which guarantees forward progress of the persistent kernels.
//
// A first group of chains is placed at the end, one chain per chunk: the longest chains (which
// carry the critical path) and the most urgent tributaries (smallest latest start;
// wf_build_plan), in an order that is itself a dependency order; the sweeps dispatch them first
// and all at once. The other chains keep the length order and are packed G per chunk (G = 32 /
// members for <= 32 members, else 1); chunks are laid out
// node-position-major: slot(c, k, g) = chunk_base[c] + k * G_c + g. With M members per
// node the element index is slot * M + m, so one warp touches 32 consecutive elements at
// every step of the walk. Every kernel of the step uses this slot layout.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

struct WfRoutingPlan {
    int64_t n = 0;          // graph nodes
    int32_t M = 1;          // members per node
    int32_t G = 32;         // chains per chunk
    int64_t n_chains = 0;   // padded to a multiple of G
    int64_t n_chunks = 0;
    int64_t n_slots = 0;    // node slots including padding
    int32_t max_len = 0;    // longest chain = graph height + 1
    int64_t n_long_chunks = 0;  // trailing chunks of the first-dispatched group (one chain each)
    bool hinted = false;        // built with heavy-child hints (chains ordered by end height, not length)
    std::vector<int64_t> chunk_base;    // [n_chunks + 1]
    std::vector<int32_t> chunk_len;     // [n_chunks]
    std::vector<int32_t> chunk_g;       // [n_chunks] chains in the chunk (G, or 1 for a long chain)
    std::vector<int64_t> chunk_chain0;  // [n_chunks] index of the chunk's first chain
    std::vector<int32_t> chain_len;     // [n_chains] (0 for padding chains)
    std::vector<int64_t> slot_of_node;  // [n]
    std::vector<int64_t> node_of_slot;  // [n_slots], -1 for padding
    std::vector<int32_t> chain_of_node; // [n]
    std::vector<int64_t> ds_slot;       // [n_slots] downstream slot, -1 for a pit or padding
    std::vector<int32_t> up_ptr;        // [n_slots + 1] CSR of upstream nodes per slot
    std::vector<int64_t> up_slot;       // upstream slot, ascending original node index
    std::vector<int32_t> up_chain;      // chain of a light upstream node (its chain end), -1 = heavy
    std::vector<uint8_t> is_chain_end;  // [n_slots]
};

// Build the plan; returns 0 or -3 (cycle) / -1 (bad input); err receives a message.
// heavy_hint (optional, [n]): a child of node v that must continue v's chain (-1: the planner's
// choice, the highest child); it keeps a given river path on one chain.
int wf_build_plan(int64_t n, const int32_t* downstream, int32_t members, WfRoutingPlan& plan, std::string& err,
                  const int64_t* heavy_hint = nullptr);

// Host check of the schedule invariants (tests): every light upstream chain precedes the
// chain that consumes it, and positions equal heights.
bool wf_check_plan(const WfRoutingPlan& plan, const int32_t* downstream, std::string& err);
