// wf_walker.cuh -- persistent wavefront kernel over a chain-decomposed drainage graph.
//
// Work items are (chunk, group of chain-member pairs) in dependency order, taken from a global
// ticket counter: a bounded number of the longest chains first (see wave_grid in wf_launch.cuh
// for why that keeps progress guaranteed), then the others in chain-length order, so an ordinary
// item only waits for chain ends of items dispatched earlier. A node at chain position k depends
// on its heavy child (position k - 1 of the same chain) and on light children (ends of shorter
// chains). Its sub-step s depends on (k - 1, s) and (k, s - 1) only, so a launch of S sub-steps
// runs on a diagonal schedule: SL lanes per chain-member pair (a power of two), lane l takes
// sub-step r * SL + l of round r, and at time t works on position t - l. A chain of length L takes
// ceil(S / SL) * (L + SL - 1) time steps instead of L * S. Lane l reads the node state that lane
// l - 1 wrote one time step earlier (the same warp, after __syncwarp), and the heavy child's
// discharge of its own sub-step, which it computed itself one time step earlier, from a register.
// Chain ends publish their discharge of every sub-step into a per-sub-step buffer and then
// release an epoch flag; consumers acquire the flag and read the buffer, so no producer can
// overwrite a value a consumer still needs.
//
// Every wait is bounded by a wall-clock budget (globaltimer); a wait that runs out sets
// WF_DEV_SPIN_TIMEOUT in the device status word, and all lanes that see the status abort, so
// the kernel always terminates and the host reports WF_ERR_SPIN.
#pragma once

#include <cstdint>

#include "wf_fields.cuh"

namespace wfw {

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(uint32_t* p, uint32_t v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint64_t now_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ int32_t status_ld(const int32_t* s) {
    return *reinterpret_cast<const volatile int32_t*>(s);
}

// Wait until *flag >= want (wrap-safe); false when the budget ran out or another lane aborted.
__device__ __forceinline__ bool wait_epoch(const uint32_t* flag, uint32_t want, const WfSweep& sw,
                                           int32_t* status) {
    if ((int32_t)(ld_acquire(flag) - want) >= 0) return true;
    const uint64_t t0 = now_ns();
    while (true) {
        __nanosleep(40);
        if ((int32_t)(ld_acquire(flag) - want) >= 0) return true;
        if (status_ld(status) & WF_DEV_SPIN_TIMEOUT) return false;
        if (now_ns() - t0 > sw.wait_ns) {
            atomicOr(status, WF_DEV_SPIN_TIMEOUT);
            return false;
        }
    }
}

// q of upstream entry `o` for member m at sub-step s: the heavy child's (`hq`, computed by this
// lane one time step earlier) or a published light child's chain end.
__device__ __forceinline__ bool upstream_q(const WfDevGraph& g, const WfSweep& sw, double hq, int32_t o, int m,
                                           int s, uint32_t ep, int32_t* status, double& out) {
    const int32_t uc = g.up_chain[o];
    if (uc < 0) {
        out = hq;
        return true;
    }
    const int64_t fe = (int64_t)uc * g.M + m;
    if (!wait_epoch(&g.flags[fe], ep + sw.wait_offset, sw, status)) return false;
    out = __ldcg(&g.end_q[fe * g.s_cap + s]);
    return true;
}

__device__ __forceinline__ void publish(const WfDevGraph& g, int64_t chain, int m, int s, uint32_t ep, double q) {
    const int64_t fe = chain * g.M + m;
    g.end_q[fe * g.s_cap + s] = q;
    st_release(&g.flags[fe], ep);
}

// Phys::node(slot, e, m, s, ep, chain, is_end, hq) -> false to abort; hq holds the heavy child's
// discharge of sub-step s on entry (unused at chain position 0) and the value this node hands
// downstream on return.
template <class Phys>
__device__ __forceinline__ void walk(const WfDevGraph& g, const WfSweep& sw, Phys& phys, int32_t* status) {
    const unsigned lane = threadIdx.x & 31u;
    const int M = g.M;
    const int SL = sw.SL > 1 ? sw.SL : 1;
    const int J = 32 / SL;
    const int sl = (int)lane % SL;  // sub-step lane
    const int j = (int)lane / SL;   // chain-member pair of the item
    const int64_t ipc = wf_items_per_chunk(g.G, M, SL);
    const uint64_t n_items = (uint64_t)g.n_chunks * ipc;
    const uint64_t prio = (uint64_t)sw.prio_items;
    const int rounds = (sw.S + SL - 1) / SL;
    while (true) {
        unsigned long long t = 0;
        if (lane == 0) t = atomicAdd(g.ticket, 1ULL);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= n_items) return;
        // the first prio_items tickets take the longest chains, longest first; the rest take
        // the other items in dependency (chain length) order
        const unsigned long long item = t < prio ? n_items - 1 - t : t - prio;
        if (status_ld(status) & WF_DEV_SPIN_TIMEOUT) return;
        const int64_t chunk = (int64_t)(item / ipc);
        const int64_t p = (int64_t)(item % ipc) * J + j;
        const int Gc = g.chunk_g[chunk];
        int gi, m;
        bool valid;
        if (M <= 32) {
            gi = (int)(p / M);
            m = (int)(p % M);
            valid = gi < Gc;
        } else {
            gi = 0;
            m = (int)p;
            valid = p < M;
        }
        const int64_t chain = g.chunk_chain0[chunk] + (valid ? gi : 0);
        const int len = valid ? g.chain_len[chain] : 0;
        if (!__any_sync(0xffffffffu, len > 0)) continue;  // an item past the chunk's pairs
        const int L = g.chunk_len[chunk];
        const int64_t base = g.chunk_base[chunk];
        for (int r = 0; r < rounds; ++r) {
            const int s = r * SL + sl;
            const uint32_t ep = sw.epoch0 + (uint32_t)s;
            double hq = 0.0;
            for (int tt = 0; tt < L + SL - 1; ++tt) {
                const int k = tt - sl;
                bool ok = true;
                if (s < sw.S && k >= 0 && k < len) {
                    const int64_t slot = base + (int64_t)k * Gc + gi;
                    ok = phys.node(slot, slot * M + m, m, s, ep, chain, k == len - 1, hq);
                }
                if (__any_sync(0xffffffffu, !ok)) return;
                __syncwarp();
            }
        }
    }
}

}  // namespace wfw
