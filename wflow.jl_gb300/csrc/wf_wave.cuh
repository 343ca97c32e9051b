// wf_wave.cuh -- slim persistent wavefront walker (node-major sub-steps, sentinel hand-off).
//
// Only the discharge propagates downstream in a kinematic-wave sweep, so the walker carries
// nothing but the solve: per-node terms that do not depend on the upstream discharge are
// prepared by the per-cell kernels before the sweep, and every output that nothing downstream
// reads (water depths, storages, averages, soil-column updates) is finished by per-cell
// kernels after it. What remains on the critical path of a chain position is the gather of
// the upstream discharges and the solve.
//
// A warp owns one chunk (G chains x M members, or one chain x 32 members) taken from a global
// ticket counter (a bounded number of the longest chains first, then the others in chain-length
// order; wave_grid in wf_launch.cuh) and walks it leaf -> chain end. Each node is advanced
// through all sub-steps of the launch before the walker moves downstream (node-major order):
// the node's own state stays in registers across sub-steps and the heavy child's discharge
// of every sub-step is handed over in a per-thread shared-memory row. Chain ends publish the
// discharge of each sub-step into end_q, which is filled with a sentinel bit pattern before
// the launch; a consumer reads the slot with a relaxed 64-bit load until the sentinel is gone
// (one round trip instead of flag-then-value). No value other than the published discharge
// itself crosses warps, so no acquire/release pairing is needed: 64-bit aligned stores and
// loads are single-copy atomic.
//
// Every wait is bounded by a wall-clock budget (globaltimer); a wait that runs out sets
// WF_DEV_SPIN_TIMEOUT in the device status word and all lanes abort.
#pragma once

#include <cstdint>

#include "wf_ff.cuh"
#include "wf_fields.cuh"

namespace wfv {

constexpr unsigned long long SENTINEL = 0xFFFFFFFFFFFFFFFFULL;   // end_q fill (a NaN pair no arithmetic yields here)
constexpr unsigned long long QUIET_NAN = 0x7FC000007FC00000ULL;  // published in place of the sentinel pattern
constexpr int MAX_GROUP = 16;                                    // sub-steps per launch of the slim walker
constexpr int PREFETCH_SUBSTEPS = 4;                             // light-child values prefetched per node

__device__ __forceinline__ unsigned long long ld_relaxed(const void* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(void* p, unsigned long long v) {
    if (v == SENTINEL) v = QUIET_NAN;
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint64_t now_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ int32_t status_ld(const int32_t* s) {
    return *reinterpret_cast<const volatile int32_t*>(s);
}

// end_q index of chain `chain`, member m, sub-step s of the launch (members innermost, so a
// warp of 32 members reads 256 contiguous bytes). Each slot holds one packed double-FP32
// discharge (wf_ff.cuh).
__device__ __forceinline__ int64_t end_index(const WfDevGraph& g, int64_t chain, int m, int s) {
    return (chain * g.s_cap + s) * g.M + m;
}

// Discharge word published at end_q[idx]; `first` is a value already loaded from that slot (or
// the sentinel). False when the budget ran out or another lane aborted. A non-zero
// sw.wait_offset (test hook, 0 in production) makes every wait run out.
__device__ __forceinline__ bool await_end(const WfDevGraph& g, const WfSweep& sw, int64_t idx,
                                          unsigned long long first, int32_t* status, unsigned long long& out) {
    unsigned long long b = first;
    if (b != SENTINEL && sw.wait_offset == 0) {
        out = b;
        return true;
    }
    const uint64_t t0 = now_ns();
    while (true) {
        __nanosleep(32);
        b = ld_relaxed(&g.end_q[idx]);
        if (b != SENTINEL && sw.wait_offset == 0) {
            out = b;
            return true;
        }
        if (status_ld(status) & WF_DEV_SPIN_TIMEOUT) return false;
        if (now_ns() - t0 > sw.wait_ns) {
            atomicOr(status, WF_DEV_SPIN_TIMEOUT);
            return false;
        }
    }
}

__device__ __forceinline__ void publish(const WfDevGraph& g, int64_t chain, int m, int s, wff::ff q) {
    st_relaxed(&g.end_q[end_index(g, chain, m, s)], wff::pack(q));
}

// Upstream list of one node with the first light entry's words of the first sub-steps
// prefetched (loaded together, so they cost one round trip).
struct UpList {
    int32_t o0, o1;
    int32_t lo;                                  // up entry of the prefetched light child (-1: none)
    int64_t lbase;                               // its end_q index at sub-step 0
    unsigned long long lq[PREFETCH_SUBSTEPS];    // its end_q words at prefetch time (may be sentinels)
};

__device__ __forceinline__ void load_up(const WfDevGraph& g, const WfSweep& sw, int64_t slot, int m, UpList& u) {
    u.o0 = g.up_ptr[slot];
    u.o1 = g.up_ptr[slot + 1];
    u.lo = -1;
    u.lbase = 0;
#pragma unroll
    for (int s = 0; s < PREFETCH_SUBSTEPS; ++s) u.lq[s] = SENTINEL;
    for (int32_t o = u.o0; o < u.o1; ++o) {
        const int32_t uc = g.up_chain[o];
        if (uc >= 0) {
            u.lo = o;
            u.lbase = end_index(g, uc, m, 0);
#pragma unroll
            for (int s = 0; s < PREFETCH_SUBSTEPS; ++s)
                if (s < sw.S) u.lq[s] = ld_relaxed(&g.end_q[u.lbase + (int64_t)s * g.M]);
            break;
        }
    }
}

// Weighted upstream sum at sub-step s in up-list order: qin = sum w*q (w = 1 - fraction to
// river on land, 1 on rivers), in double-FP32. `qh` is the heavy child's word of this sub-step.
template <bool WEIGHTED>
__device__ __forceinline__ bool gather(const WfDevGraph& g, const WfSweep& sw, const UpList& u, int m, int s,
                                       unsigned long long qh, int32_t* status, wff::ff& qin) {
    wff::ff acc = {0.0f, 0.0f};
    for (int32_t o = u.o0; o < u.o1; ++o) {
        const int32_t uc = g.up_chain[o];
        unsigned long long w;
        if (uc < 0) {
            w = qh;
        } else {
            const int64_t idx = end_index(g, uc, m, s);
            unsigned long long first = SENTINEL;
            if (o == u.lo) {
#pragma unroll
                for (int j = 0; j < PREFETCH_SUBSTEPS; ++j)
                    if (j == s) first = u.lq[j];
            }
            if (first == SENTINEL) first = ld_relaxed(&g.end_q[idx]);
            if (!await_end(g, sw, idx, first, status, w)) return false;
        }
        const wff::ff q = wff::unpack(w);
        acc = WEIGHTED ? wff::add(acc, wff::mul(q, g.up_wf[o])) : wff::add(acc, q);
    }
    qin = acc;
    return true;
}

// Phys interface:
//   struct In;                                               per-node inputs (prefetched)
//   void load(int64_t slot, int64_t e, int m, In&)           independent of upstream discharge
//   bool node(const In&, int64_t slot, int64_t e, int m, int64_t chain, bool is_end,
//             unsigned long long* qh)
//     advances the node through sw.S sub-steps; qh[s * stride] holds the heavy child's packed
//     discharge of sub-step s on entry and this node's on exit. Returns false to abort.
template <class Phys>
__device__ __forceinline__ void walk(const WfDevGraph& g, const WfSweep& sw, Phys& phys, int32_t* status) {
    extern __shared__ unsigned long long wave_smem[];
    const unsigned lane = threadIdx.x & 31u;
    unsigned long long* qh = wave_smem + threadIdx.x;  // row of this thread: qh[s * blockDim.x]
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
        typename Phys::In cur, nxt;
        if (len > 0) phys.load(base + gi, (base + gi) * M + m, m, cur);
        for (int k = 0; k < L; ++k) {
            const int64_t slot = base + (int64_t)k * Gc + gi;
            if (k + 1 < len) {
                const int64_t ns = slot + Gc;
                phys.load(ns, ns * M + m, m, nxt);
            }
            bool ok = true;
            if (k < len) ok = phys.node(cur, slot, slot * M + m, m, chain, k == len - 1, qh);
            if (__any_sync(0xffffffffu, !ok)) return;
            __syncwarp();
            cur = nxt;
        }
    }
}

}  // namespace wfv
