// wf_walker.cuh -- persistent wavefront kernel over a chain-decomposed drainage graph.
//
// One warp owns one chunk (G chains x M members, or one chain x 32 members) at a time and
// walks it in lockstep from the leaves to the chain ends, sub-step by sub-step. Chunks are
// taken from a global ticket counter: a bounded number of the longest chains first (see
// wave_grid in wf_launch.cuh for why that keeps progress guaranteed), then the others in
// chain-length order, so an ordinary chunk only waits for chain ends of chunks dispatched
// earlier (or of shorter chains of its own chunk, which the lockstep walk has already
// finished). Chain ends publish their discharge of every sub-step into a
// per-sub-step buffer and then release an epoch flag; consumers acquire the flag and read the
// buffer, so no producer can overwrite a value a consumer still needs.
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

// q of upstream entry `o` for member m at sub-step s: the heavy child was written by this
// lane at the previous chain position; a light child is a published chain end.
__device__ __forceinline__ bool upstream_q(const WfDevGraph& g, const WfSweep& sw, const double* q, int32_t o,
                                           int m, int s, uint32_t ep, int32_t* status, double& out) {
    const int32_t uc = g.up_chain[o];
    if (uc < 0) {
        out = q[g.up_slot[o] * g.M + m];
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

// Phys::node(slot, e, m, s, ep, chain, is_end) -> false to abort.
template <class Phys>
__device__ __forceinline__ void walk(const WfDevGraph& g, const WfSweep& sw, Phys& phys, int32_t* status) {
    const unsigned lane = threadIdx.x & 31u;
    const int M = g.M;
    const int gpc = M > 32 ? M / 32 : 1;
    const uint64_t n_items = (uint64_t)g.n_chunks * gpc;
    const uint64_t prio = (uint64_t)sw.prio_items;
    while (true) {
        unsigned long long t = 0;
        if (lane == 0) t = atomicAdd(g.ticket, 1ULL);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= n_items) return;
        // the first prio_items tickets take the longest chains, longest first; the rest take
        // the other items in dependency (chain length) order
        const unsigned long long item = t < prio ? n_items - 1 - t : t - prio;
        if (status_ld(status) & WF_DEV_SPIN_TIMEOUT) return;
        const int64_t chunk = (int64_t)(item / gpc);
        int gi, m;
        if (M <= 32) {
            gi = (int)lane / M;
            m = (int)lane % M;
        } else {
            gi = 0;
            m = (int)(item % gpc) * 32 + (int)lane;
        }
        const int Gc = g.chunk_g[chunk];
        const int64_t chain = g.chunk_chain0[chunk] + (gi < Gc ? gi : 0);
        const int len = gi < Gc ? g.chain_len[chain] : 0;
        const int L = g.chunk_len[chunk];
        const int64_t base = g.chunk_base[chunk];
        for (int s = 0; s < sw.S; ++s) {
            const uint32_t ep = sw.epoch0 + (uint32_t)s;
            for (int k = 0; k < L; ++k) {
                bool ok = true;
                if (k < len) {
                    const int64_t slot = base + (int64_t)k * Gc + gi;
                    ok = phys.node(slot, slot * M + m, m, s, ep, chain, k == len - 1);
                }
                if (__any_sync(0xffffffffu, !ok)) return;
                __syncwarp();
            }
        }
    }
}

}  // namespace wfw
