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
// ticket counter (a bounded number of the longest chains first, then the others in the plan's
// dependency order, chain length for plans without heavy-child hints; wave_grid in
// wf_launch.cuh) and walks it leaf -> chain end. Two sweeps can share one launch (walk_pair). Each node is advanced
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
#include <cstring>

#include "wf_ff.cuh"
#include "wf_fields.cuh"

namespace wfv {

constexpr unsigned long long SENTINEL = 0xFFFFFFFFFFFFFFFFULL;   // end_q fill (a NaN pair no arithmetic yields here)
constexpr unsigned long long QUIET_NAN = 0x7FC000007FC00000ULL;  // published in place of the sentinel pattern
constexpr int MAX_GROUP = 16;                                    // sub-steps per launch of the slim walker
constexpr int PREFETCH_SUBSTEPS = 4;                             // light-child values prefetched per node

// The relaxed loads and stores of published discharges carry no ordering duty (a consumer uses
// only the value it reads), so they have no compiler memory clobber: a clobber would make the
// compiler reload every shared-memory value it holds in registers after each of them.
__device__ __forceinline__ unsigned long long ld_relaxed(const void* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ void st_relaxed(void* p, unsigned long long v) {
    if (v == SENTINEL) v = QUIET_NAN;
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v));
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

// A published word at `p` other than an end_q slot (same sentinel and budget as await_end).
__device__ __forceinline__ bool await_word(const WfSweep& sw, const unsigned long long* p, int32_t* status,
                                           unsigned long long& out) {
    unsigned long long b = ld_relaxed(p);
    if (b != SENTINEL && sw.wait_offset == 0) {
        out = b;
        return true;
    }
    const uint64_t t0 = now_ns();
    while (true) {
        __nanosleep(32);
        b = ld_relaxed(p);
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

// Upstream inflow record of one node. A node at chain position k > 0 has its heavy child at
// position k - 1 (its discharge is handed over in shared memory); its light children are chain
// ends of shorter chains. The first two light children come from the per-slot record (one
// 16-byte load, no dependent index loads), the rare further ones from the CSR list; the
// end_q words of light child 0 for the first sub-steps and of light child 1 for sub-step 0 are
// prefetched (load_ends), so a producer that finished earlier costs no round trip in gather.
struct UpRec {
    int32_t lt0, lt1;     // chains of light children 0 and 1 (-1: none)
    float w_lt0, w_lt1;   // their weights
    float w_hv;           // weight of the heavy child
    int32_t n_lt;         // light children in all
};
// The prefetched end_q words of one node (kept apart from UpRec so that only the positions
// whose words are in flight hold them).
struct Ends {
    unsigned long long lq0[PREFETCH_SUBSTEPS];  // light child 0, first sub-steps (may be sentinels)
    unsigned long long lq1;                     // light child 1, sub-step 0
};

// Level-1 loads of the record (WEIGHTED: the land graph's weights, else all weights are 1).
template <bool WEIGHTED>
__device__ __forceinline__ void load_rec(const WfDevGraph& g, int64_t slot, UpRec& r) {
    const int4 v = g.up_rec[slot];
    r.lt0 = v.x;
    r.lt1 = v.y;
    r.w_lt0 = WEIGHTED ? __int_as_float(v.z) : 1.0f;
    r.w_lt1 = WEIGHTED ? __int_as_float(v.w) : 1.0f;
    r.w_hv = WEIGHTED ? g.up_whv[slot] : 1.0f;
    r.n_lt = g.up_nlt[slot];
}

// Level-2 loads: the light children's end_q words of the first sub-steps.
__device__ __forceinline__ void load_ends(const WfDevGraph& g, const WfSweep& sw, int m, const UpRec& r, Ends& x) {
#pragma unroll
    for (int s = 0; s < PREFETCH_SUBSTEPS; ++s) x.lq0[s] = SENTINEL;
    x.lq1 = SENTINEL;
    if (r.lt0 >= 0) {
        const int64_t b = end_index(g, r.lt0, m, 0);
#pragma unroll
        for (int s = 0; s < PREFETCH_SUBSTEPS; ++s)
            if (s < sw.S) x.lq0[s] = ld_relaxed(&g.end_q[b + (int64_t)s * g.M]);
    }
    if (r.lt1 >= 0) x.lq1 = ld_relaxed(&g.end_q[end_index(g, r.lt1, m, 0)]);
}

// Weighted upstream sum at sub-step s: qin = sum w*q (w = 1 - fraction to river on land, 1 on
// rivers) in double-FP32, heavy child first, then the light children. `qh` is the heavy child's
// word of this sub-step, `heavy` whether the node has one (chain position > 0); w0 / w1 are the
// end_q words of light children 0 / 1 at sub-step s loaded earlier (SENTINEL when not loaded or
// not yet published).
template <bool WEIGHTED>
__device__ __forceinline__ bool gather_w(const WfDevGraph& g, const WfSweep& sw, const UpRec& r, unsigned long long w0,
                                         unsigned long long w1, int64_t slot, int m, int s, bool heavy,
                                         unsigned long long qh, int32_t* status, wff::ff& qin) {
    wff::ff acc = {0.0f, 0.0f};
    if (heavy) {
        const wff::ff q = wff::unpack(qh);
        acc = WEIGHTED ? wff::mul(q, r.w_hv) : q;
    }
    if (r.lt0 >= 0) {
        const int64_t idx = end_index(g, r.lt0, m, s);
        unsigned long long first = w0;
        if (first == SENTINEL) first = ld_relaxed(&g.end_q[idx]);
        unsigned long long w;
        if (!await_end(g, sw, idx, first, status, w)) return false;
        const wff::ff q = wff::unpack(w);
        acc = WEIGHTED ? wff::add(acc, wff::mul(q, r.w_lt0)) : wff::add(acc, q);
    }
    if (r.lt1 >= 0) {
        const int64_t idx = end_index(g, r.lt1, m, s);
        unsigned long long first = w1;
        if (first == SENTINEL) first = ld_relaxed(&g.end_q[idx]);
        unsigned long long w;
        if (!await_end(g, sw, idx, first, status, w)) return false;
        const wff::ff q = wff::unpack(w);
        acc = WEIGHTED ? wff::add(acc, wff::mul(q, r.w_lt1)) : wff::add(acc, q);
    }
    if (r.n_lt > 2) {  // further light children, in up-list order after the first two
        int seen = 0;
        for (int32_t o = g.up_ptr[slot]; o < g.up_ptr[slot + 1]; ++o) {
            const int32_t uc = g.up_chain[o];
            if (uc < 0 || ++seen <= 2) continue;
            const int64_t idx = end_index(g, uc, m, s);
            unsigned long long w;
            if (!await_end(g, sw, idx, ld_relaxed(&g.end_q[idx]), status, w)) return false;
            const wff::ff q = wff::unpack(w);
            acc = WEIGHTED ? wff::add(acc, wff::mul(q, g.up_wf[o])) : wff::add(acc, q);
        }
    }
    qin = acc;
    return true;
}

// The prefetched word of light child 0 at sub-step s (SENTINEL beyond the prefetched ones).
__device__ __forceinline__ unsigned long long end_word0(const Ends& x, int s) {
    unsigned long long w = SENTINEL;
#pragma unroll
    for (int j = 0; j < PREFETCH_SUBSTEPS; ++j)
        if (j == s) w = x.lq0[j];
    return w;
}

// gather_w with the words of a node-major walk (light child 0 prefetched for the first
// sub-steps, light child 1 for sub-step 0).
template <bool WEIGHTED>
__device__ __forceinline__ bool gather(const WfDevGraph& g, const WfSweep& sw, const UpRec& r, const Ends& x,
                                       int64_t slot, int m, int s, bool heavy, unsigned long long qh, int32_t* status,
                                       wff::ff& qin) {
    return gather_w<WEIGHTED>(g, sw, r, end_word0(x, s), s == 0 ? x.lq1 : SENTINEL, slot, m, s, heavy, qh, status,
                              qin);
}

// The end_q words of light children 0 and 1 of record r at sub-step s (SENTINEL for a missing
// child); a load that finds the producer not yet done also returns the sentinel.
__device__ __forceinline__ void load_words(const WfDevGraph& g, int m, const UpRec& r, int s, unsigned long long& w0,
                                           unsigned long long& w1) {
    w0 = r.lt0 >= 0 ? ld_relaxed(&g.end_q[end_index(g, r.lt0, m, s)]) : SENTINEL;
    w1 = r.lt1 >= 0 ? ld_relaxed(&g.end_q[end_index(g, r.lt1, m, s)]) : SENTINEL;
}

// Work items are (chunk, member group) pairs in dependency (chain length) order. One ticket takes
// a batch of up to BATCH consecutive short items (chunk length <= SHORT_LEN: the bulk of a
// drainage forest is short tributary chains, and a ticket per chain would pay the ticket, the
// descriptor loads and the prefetch start-up per chain), or a single longer item. The items of
// a batch are walked as one sequence of positions, so the prefetch runs on across item
// boundaries. Order and progress are unchanged: a batch holds consecutive items and a chain
// waits only for strictly shorter chains, which come earlier in the batch or in the order.
constexpr int BATCH = 8;
constexpr int SHORT_LEN = 8;

struct WarpBatch {  // per-warp shared descriptors of the items of the current ticket
    long long base[BATCH];
    long long chain0[BATCH];
    int L[BATCH];
    int Gc[BATCH];
    int mbase[BATCH];     // first member of the item (more than 32 members)
    int len[BATCH][32];   // length of each lane's chain (0: the lane idles in that item)
};

__host__ __device__ constexpr size_t walk_smem(int threads, int substeps) {
    return (size_t)threads * substeps * sizeof(unsigned long long) + (size_t)(threads / 32) * sizeof(WarpBatch);
}

// Phys interface:
//   struct In;                                   per-node inputs, including an UpRec `up`
//   static constexpr int kDepth;                 1: prefetch one position ahead; 2: two (the
//                                                inputs two ahead, their end_q words one ahead)
//   void load(int64_t slot, int64_t e, int m, In&)   level-1 loads (state, statics, load_rec)
//   bool node(const In&, const Ends&, int64_t slot, int64_t e, int m, int64_t chain, bool is_end,
//             bool heavy, unsigned long long* qh)
//     advances the node through sw.S sub-steps; qh[s * stride] holds the heavy child's packed
//     discharge of sub-step s on entry and this node's on exit. Returns false to abort.
// Tickets of a node-major sweep: the first prio_items take the longest items, longest first; the
// rest take the others in dependency order, short ones in batches of BATCH.
__device__ __forceinline__ uint64_t walk_tickets(const WfDevGraph& g, const WfSweep& sw) {
    const int gpc = g.M > 32 ? g.M / 32 : 1;
    const int64_t n_items = g.n_chunks * gpc;
    const int64_t n_norm = n_items - sw.prio_items;
    const int64_t n_short = min(g.n_short_chunks * gpc, n_norm);
    const int64_t n_sb = (n_short + BATCH - 1) / BATCH;
    return (uint64_t)(sw.prio_items + n_sb + (n_norm - n_short));
}

// One ticket t of a node-major sweep (walk_tickets). `wb` is the warp's batch descriptor, qh the
// thread's hand-off row (qh[s * blockDim.x]). False when the sweep aborts (a wait ran out).
template <class Phys>
__device__ __forceinline__ bool walk_ticket(const WfDevGraph& g, const WfSweep& sw, Phys& phys, int32_t* status,
                                            uint64_t t, WarpBatch* wb, unsigned long long* qh) {
    constexpr int DEPTH = Phys::kDepth;
    const unsigned lane = threadIdx.x & 31u;
    const int M = g.M;
    const int gpc = M > 32 ? M / 32 : 1;
    const int gi = M <= 32 ? (int)lane / M : 0;
    const int64_t n_items = g.n_chunks * gpc;
    const int64_t prio = sw.prio_items;
    const int64_t n_norm = n_items - prio;
    const int64_t n_short = min(g.n_short_chunks * gpc, n_norm);
    const int64_t n_sb = (n_short + BATCH - 1) / BATCH;
    int64_t first;
    int count = 1;
    if ((int64_t)t < prio) {
        first = n_items - 1 - (int64_t)t;
    } else {
        const int64_t u = (int64_t)t - prio;
        if (u < n_sb) {
            first = u * BATCH;
            count = (int)min((int64_t)BATCH, n_short - first);
        } else {
            first = n_short + (u - n_sb);
        }
    }
    if (status_ld(status) & WF_DEV_SPIN_TIMEOUT) return false;
    if ((int)lane < count) {
        const int64_t item = first + lane;
        const int64_t chunk = item / gpc;
        wb->base[lane] = g.chunk_base[chunk];
        wb->chain0[lane] = g.chunk_chain0[chunk];
        wb->L[lane] = g.chunk_len[chunk];
        wb->Gc[lane] = g.chunk_g[chunk];
        wb->mbase[lane] = (int)(item % gpc) * 32;
    }
    __syncwarp();
    for (int j = 0; j < count; ++j) {
        const int Gc = wb->Gc[j];
        wb->len[j][lane] = gi < Gc ? g.chain_len[wb->chain0[j] + gi] : 0;
    }
    __syncwarp();
    const int m_fixed = (int)lane % (M <= 32 ? M : 32);
    // the walk over the positions (item it, chain position k) of the batch
    auto valid = [&](int it, int k) { return it < count && k < wb->len[it][lane]; };
    auto slot_of = [&](int it, int k) { return wb->base[it] + (int64_t)k * wb->Gc[it] + gi; };
    auto member = [&](int it) { return M > 32 ? wb->mbase[it] + (int)lane : m_fixed; };
    auto advance = [&](int& it, int& k) {
        if (k + 1 < wb->L[it]) {
            ++k;
        } else {
            ++it;
            k = 0;
        }
    };
    typename Phys::In cur, nxt;
    Ends ecur, enxt;
    int cit = 0, ck = 0;
    if (valid(cit, ck)) {
        const int64_t sl = slot_of(cit, ck);
        const int mm = member(cit);
        phys.load(sl, sl * M + mm, mm, cur);
        load_ends(g, sw, mm, cur.up, ecur);
    }
    int nit = cit, nk = ck;
    advance(nit, nk);
    if (DEPTH > 1 && valid(nit, nk)) {
        const int64_t sl = slot_of(nit, nk);
        const int mm = member(nit);
        phys.load(sl, sl * M + mm, mm, nxt);
    }
    while (cit < count) {
        int nnit = nit, nnk = nk;
        if (nnit < count) advance(nnit, nnk);
        typename Phys::In nn;
        if (DEPTH > 1) {
            if (valid(nit, nk)) load_ends(g, sw, member(nit), nxt.up, enxt);
            if (valid(nnit, nnk)) {
                const int64_t sl = slot_of(nnit, nnk);
                const int mm = member(nnit);
                phys.load(sl, sl * M + mm, mm, nn);
            }
        } else if (valid(nit, nk)) {
            const int64_t sl = slot_of(nit, nk);
            const int mm = member(nit);
            phys.load(sl, sl * M + mm, mm, nxt);
            load_ends(g, sw, mm, nxt.up, enxt);
        }
        bool ok = true;
        if (valid(cit, ck)) {
            const int64_t sl = slot_of(cit, ck);
            const int mm = member(cit);
            ok = phys.node(cur, ecur, sl, sl * M + mm, mm, wb->chain0[cit] + gi, ck == wb->len[cit][lane] - 1, ck > 0,
                           qh);
        }
        if (__any_sync(0xffffffffu, !ok)) return false;
        __syncwarp();
        cur = nxt;
        ecur = enxt;
        if (DEPTH > 1) nxt = nn;
        cit = nit;
        ck = nk;
        nit = nnit;
        nk = nnk;
    }
    __syncwarp();
    return true;
}

template <class Phys>
__device__ __forceinline__ void walk(const WfDevGraph& g, const WfSweep& sw, Phys& phys, int32_t* status) {
    extern __shared__ unsigned long long wave_smem[];
    const unsigned lane = threadIdx.x & 31u;
    unsigned long long* qh = wave_smem + threadIdx.x;  // row of this thread: qh[s * blockDim.x]
    WarpBatch* wb = reinterpret_cast<WarpBatch*>(wave_smem + (size_t)blockDim.x * sw.S) + (threadIdx.x >> 5);
    const uint64_t n_tickets = walk_tickets(g, sw);
    while (true) {
        unsigned long long t = 0;
        if (lane == 0) t = atomicAdd(g.ticket, 1ULL);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= n_tickets) return;
        if (!walk_ticket(g, sw, phys, status, t, wb, qh)) return;
    }
}

// Two node-major sweeps in one persistent launch: the tickets of sweep A (ga's counter) come
// first, then those of sweep B, so every wait of a B node is on A work or on earlier B tickets,
// all of them already dispatched to resident warps (A never waits on B). The hand-off rows are
// sized for the larger sub-step count S_alloc of the two.
template <class PhysA, class PhysB>
__device__ __forceinline__ void walk_pair(PhysA& pa, PhysB& pb, int S_alloc, int32_t* status) {
    extern __shared__ unsigned long long wave_smem[];
    const unsigned lane = threadIdx.x & 31u;
    unsigned long long* qh = wave_smem + threadIdx.x;
    WarpBatch* wb = reinterpret_cast<WarpBatch*>(wave_smem + (size_t)blockDim.x * S_alloc) + (threadIdx.x >> 5);
    const uint64_t na = walk_tickets(pa.g, pa.sw), nb = walk_tickets(pb.g, pb.sw);
    while (true) {
        unsigned long long t = 0;
        if (lane == 0) t = atomicAdd(pa.g.ticket, 1ULL);
        t = __shfl_sync(0xffffffffu, t, 0);
        bool ok;
        if (t < na) ok = walk_ticket(pa.g, pa.sw, pa, status, t, wb, qh);
        else if (t < na + nb) ok = walk_ticket(pb.g, pb.sw, pb, status, t - na, wb, qh);
        else return;
        if (!ok) return;
    }
}

// ------------------------------------------------------------- staged walk ---------------
//
// The walk above keeps the next positions' inputs in registers, one or two positions ahead, and a
// position whose loads have not landed waits for them: on a long chain every position then costs
// a memory round trip. The staged walk copies the inputs of the next RING_D positions of every
// lane into a per-warp ring in shared memory with asynchronous copies (cp.async, one commit group
// per position, issued whether or not the lane has work there), so a position's inputs have had
// RING_D positions to arrive; the light children's end_q words are loaded two positions ahead from
// the staged records. Each lane reads back only what it copied itself, so the waits are per thread
// (cp.async.wait_group) and no barrier is involved. The computation is the node-major walk's.
//
// Phys staged interface:
//   static constexpr int kWords;                          32-bit input words per position
//   void sources(int64_t slot, int64_t e, const void** src)   their global addresses
//   void from_words(const uint32_t* w, int stride, In&)   the inputs from the staged words (and
//                                                         the record, set by the walk)
//   static constexpr bool kWeighted;                      the land graph's weights (load_rec)
// The copies and their commit carry no compiler memory clobber (it would force every shared
// value held in registers to be reloaded after each copy); cp.async.wait_group has one, so the
// reads of a slot stay after the wait that covers it, and a slot's earlier reads stay before the
// next wait, which precedes its refill.
constexpr int RING_D = 6;           // positions staged ahead
constexpr int RING_R = RING_D + 1;  // ring slots (the slot refilled is the one read a position ago)

__device__ __forceinline__ void cpa4(void* smem, const void* gmem) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(a), "l"(gmem));
}
__device__ __forceinline__ void cpa16(void* smem, const void* gmem) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(a), "l"(gmem));
}
__device__ __forceinline__ void cpa_commit() { asm volatile("cp.async.commit_group;"); }
template <int N>
__device__ __forceinline__ void cpa_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ void cpa_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Bytes of one warp's ring: per slot, kWords words of 32 lanes, then 32 records (16 B each).
__host__ __device__ constexpr size_t ring_slot_bytes(int words) { return (size_t)words * 128 + 512; }
__host__ __device__ constexpr size_t ring_smem(int threads, int substeps, int words) {
    return (walk_smem(threads, substeps) + 15) / 16 * 16 + (size_t)(threads / 32) * RING_R * ring_slot_bytes(words);
}

template <class Phys>
__device__ __forceinline__ void walk_ring(const WfDevGraph& g, const WfSweep& sw, Phys& phys, int32_t* status) {
    extern __shared__ unsigned long long wave_smem[];
    constexpr int KW = Phys::kWords;
    using In = typename Phys::In;
    const unsigned lane = threadIdx.x & 31u;
    unsigned long long* qh = wave_smem + threadIdx.x;
    WarpBatch* wb = reinterpret_cast<WarpBatch*>(wave_smem + (size_t)blockDim.x * sw.S) + (threadIdx.x >> 5);
    unsigned char* const ring =
        reinterpret_cast<unsigned char*>(wave_smem) + (walk_smem(blockDim.x, sw.S) + 15) / 16 * 16 +
        (size_t)(threadIdx.x >> 5) * RING_R * ring_slot_bytes(KW);
    auto words_of = [&](int r) { return reinterpret_cast<uint32_t*>(ring + (size_t)r * ring_slot_bytes(KW)); };
    auto rec_of = [&](int r) {
        return reinterpret_cast<int4*>(ring + (size_t)r * ring_slot_bytes(KW) + (size_t)KW * 128) + lane;
    };
    const int M = g.M;
    const int gpc = M > 32 ? M / 32 : 1;
    const int gi = M <= 32 ? (int)lane / M : 0;
    const int64_t n_items = g.n_chunks * gpc;
    const int64_t prio = sw.prio_items;
    const int64_t n_norm = n_items - prio;
    const int64_t n_short = min(g.n_short_chunks * gpc, n_norm);
    const int64_t n_sb = (n_short + BATCH - 1) / BATCH;
    const uint64_t n_tickets = (uint64_t)(prio + n_sb + (n_norm - n_short));
    const int m_fixed = (int)lane % (M <= 32 ? M : 32);
    while (true) {
        unsigned long long t = 0;
        if (lane == 0) t = atomicAdd(g.ticket, 1ULL);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= n_tickets) return;
        int64_t first;
        int count = 1;
        if ((int64_t)t < prio) {
            first = n_items - 1 - (int64_t)t;
        } else {
            const int64_t u = (int64_t)t - prio;
            if (u < n_sb) {
                first = u * BATCH;
                count = (int)min((int64_t)BATCH, n_short - first);
            } else {
                first = n_short + (u - n_sb);
            }
        }
        if (status_ld(status) & WF_DEV_SPIN_TIMEOUT) return;
        if ((int)lane < count) {
            const int64_t item = first + lane;
            const int64_t chunk = item / gpc;
            wb->base[lane] = g.chunk_base[chunk];
            wb->chain0[lane] = g.chunk_chain0[chunk];
            wb->L[lane] = g.chunk_len[chunk];
            wb->Gc[lane] = g.chunk_g[chunk];
            wb->mbase[lane] = (int)(item % gpc) * 32;
        }
        __syncwarp();
        int npos = 0;
        for (int j = 0; j < count; ++j) {
            const int Gc = wb->Gc[j];
            wb->len[j][lane] = gi < Gc ? g.chain_len[wb->chain0[j] + gi] : 0;
            npos += wb->L[j];
        }
        __syncwarp();
        auto valid = [&](int it, int k) { return it < count && k < wb->len[it][lane]; };
        auto slot_of = [&](int it, int k) { return wb->base[it] + (int64_t)k * wb->Gc[it] + gi; };
        auto member = [&](int it) { return M > 32 ? wb->mbase[it] + (int)lane : m_fixed; };
        auto advance = [&](int& it, int& k) {
            if (k + 1 < wb->L[it]) {
                ++k;
            } else {
                ++it;
                k = 0;
            }
        };
        // stage position (it, k) into ring slot r (one commit group, possibly empty)
        auto stage = [&](int it, int k, int r) {
            if (valid(it, k)) {
                const int64_t sl = slot_of(it, k);
                const void* src[KW];
                phys.sources(sl, sl * M + member(it), src);
                uint32_t* w = words_of(r) + lane;
#pragma unroll
                for (int i = 0; i < KW; ++i) cpa4(w + i * 32, src[i]);
                cpa16(rec_of(r), &g.up_rec[sl]);
            }
            cpa_commit();
        };
        // the record of a staged position and its light children's words (issued, not awaited)
        auto ends_of = [&](int it, int k, int r, UpRec& up, Ends& ex) {
            if (valid(it, k)) {
                const int64_t sl = slot_of(it, k);
                const int4 v = *rec_of(r);
                up.lt0 = v.x;
                up.lt1 = v.y;
                up.w_lt0 = Phys::kWeighted ? __int_as_float(v.z) : 1.0f;
                up.w_lt1 = Phys::kWeighted ? __int_as_float(v.w) : 1.0f;
                up.w_hv = Phys::kWeighted ? g.up_whv[sl] : 1.0f;
                up.n_lt = g.up_nlt[sl];
                load_ends(g, sw, member(it), up, ex);
            }
        };
        int sit = 0, sk = 0;  // staging cursor, RING_D positions ahead of the walk
        for (int d = 0; d < RING_D; ++d) {
            stage(sit, sk, d);
            if (sit < count) advance(sit, sk);
        }
        // the records and end words of positions 0 and 1 (groups 0 and 1 complete)
        cpa_wait<RING_D - 2>();
        UpRec u0, u1, u2;
        Ends e0, e1, e2;
        int it1 = 0, k1 = 0;
        ends_of(0, 0, 0, u0, e0);
        advance(it1, k1);
        ends_of(it1, k1, 1, u1, e1);
        int cit = 0, ck = 0, nit = it1, nk = k1;  // positions t and t + 1
        int t2it = it1, t2k = k1;
        if (t2it < count) advance(t2it, t2k);    // position t + 2
        bool ok = true;
        int tpos = 0;
        // One position: uc / ec hold its record and end words (issued two positions ago), u2 / e2
        // receive those of position t + 2. The three register sets rotate by unrolling (below)
        // rather than by copies: a copy of a register whose load is in flight would wait for it.
        auto step = [&](UpRec& uc, Ends& ec, UpRec& u2, Ends& e2) -> bool {
            if (tpos >= npos || cit >= count) return false;
            // groups up to position t + 2 complete: read its record and issue its end words
            cpa_wait<RING_D - 3>();
            ends_of(t2it, t2k, (tpos + 2) % RING_R, u2, e2);
            // position t's inputs from its slot, then refill the slot read a position ago
            In x;
            if (valid(cit, ck)) {
                phys.from_words(words_of(tpos % RING_R) + lane, 32, x);
                x.up = uc;
            }
            stage(sit, sk, (tpos + RING_D) % RING_R);
            if (sit < count) advance(sit, sk);
            if (valid(cit, ck)) {
                const int64_t sl = slot_of(cit, ck);
                const int mm = member(cit);
                ok = phys.node(x, ec, sl, sl * M + mm, mm, wb->chain0[cit] + gi, ck == wb->len[cit][lane] - 1,
                               ck > 0, qh);
            }
            if (__any_sync(0xffffffffu, !ok)) {
                ok = false;
                return false;
            }
            __syncwarp();
            cit = nit;
            ck = nk;
            nit = t2it;
            nk = t2k;
            if (t2it < count) advance(t2it, t2k);
            ++tpos;
            return true;
        };
        while (step(u0, e0, u2, e2) && step(u1, e1, u0, e0) && step(u2, e2, u1, e1)) {
        }
        cpa_wait_all();  // the ring is refilled by the next ticket
        __syncwarp();
        if (!ok) return;
    }
}

// ------------------------------------------------------------- diagonal schedule ---------
//
// A launch of S > 1 fixed sub-steps: sub-step s of the node at chain position k depends only on
// (k - 1, s) (the heavy child) and (k, s - 1) (the node's own previous state), so the walker
// gives every chain-member pair SL lanes (a power of two, sw.SL) and runs the sub-steps on a
// diagonal: in round r lane l takes sub-step r * SL + l, and at time step t it works on the
// position t - l of the item sequence. A chain of L positions takes ceil(S / SL) rounds of
// L + SL - 1 time steps instead of the node-major L * S. Lane 0 loads the node inputs (its
// prefetch pipeline as in walk); at the end of each time step every lane hands the node's
// inputs, its state after its sub-step and the end_q words of the node's light children for the
// next sub-step (loaded during the step) to the next lane with one warp shuffle. The heavy
// child's discharge of a lane's sub-step is the value the lane itself computed one time step
// earlier. The lane of the last sub-step of a round stores the node state; the next round's lane
// 0 loads it again.
//
// Phys interface beyond walk():
//   struct St;                                   state carried from sub-step to sub-step
//   void start(const In&, St&)                   state at the start of a round (from In)
//   bool sub(const In&, St&, w0, w1, slot, e, m, s, chain, is_end, heavy, qh_in, qh_out)
//     one sub-step: w0 / w1 the light children's end_q words of sub-step s (or SENTINEL),
//     qh_in the heavy child's packed discharge of sub-step s, qh_out this node's. False to abort.
//   void finish(const St&, e, add_stored)        stores after the last sub-step of a round
//                                                (add_stored: add the stored cumulative sums)

template <class T>
__device__ __forceinline__ void shfl_up_pod(T& v, int width) {
    static_assert(sizeof(T) % 4 == 0, "shuffled structs are whole 32-bit words");
    uint32_t w[sizeof(T) / 4];
    memcpy(w, &v, sizeof(T));
#pragma unroll
    for (int i = 0; i < (int)(sizeof(T) / 4); ++i) w[i] = __shfl_up_sync(0xffffffffu, w[i], 1, width);
    memcpy(&v, w, sizeof(T));
}

struct DiagBatch {  // per-warp shared descriptors of the items of the current ticket
    long long base[BATCH];
    long long chain0[BATCH];
    int L[BATCH];
    int Gc[BATCH];
    int p0[BATCH];        // first chain-member pair of the item
    int len[BATCH][32];   // length of each lane's chain (0: the lane idles in that item)
};

__host__ __device__ constexpr size_t diag_smem(int threads) { return (size_t)(threads / 32) * sizeof(DiagBatch); }

// One ticket of a diagonal-schedule sweep: `count` consecutive items from `first` (wb: the warp's
// descriptors). False when the sweep aborts.
template <class Phys>
__device__ __forceinline__ bool diag_ticket(const WfDevGraph& g, const WfSweep& sw, Phys& phys, int32_t* status,
                                            int64_t first, int count, DiagBatch* wb) {
    constexpr int DEPTH = Phys::kDepth;
    using In = typename Phys::In;
    using St = typename Phys::St;
    const unsigned lane = threadIdx.x & 31u;
    const int M = g.M;
    const int SL = sw.SL;
    const int J = 32 / SL;
    const int sl = (int)lane % SL;
    const int j = (int)lane / SL;
    const int64_t ipc = wf_items_per_chunk(g.G, M, SL);
    const int rounds = (sw.S + SL - 1) / SL;
    const bool launch_first = sw.first == 0;
    if (status_ld(status) & WF_DEV_SPIN_TIMEOUT) return false;
    if ((int)lane < count) {
        const int64_t item = first + lane;
        const int64_t chunk = item / ipc;
        wb->base[lane] = g.chunk_base[chunk];
        wb->chain0[lane] = g.chunk_chain0[chunk];
        wb->L[lane] = g.chunk_len[chunk];
        wb->Gc[lane] = g.chunk_g[chunk];
        wb->p0[lane] = (int)(item % ipc) * J;
    }
    __syncwarp();
    int npos = 0, work = 0;
    for (int it = 0; it < count; ++it) {
        const int p = wb->p0[it] + j;
        const int gi = M <= 32 ? p / M : 0;
        const bool ok = M <= 32 ? gi < wb->Gc[it] : p < M;
        const int len = ok ? g.chain_len[wb->chain0[it] + gi] : 0;
        wb->len[it][lane] = len;
        work |= len;
        npos += wb->L[it];
    }
    __syncwarp();
    if (!__any_sync(0xffffffffu, work > 0)) return true;  // items past their chunks' pairs
    auto gi_of = [&](int it) { return M <= 32 ? (wb->p0[it] + j) / M : 0; };
    auto m_of = [&](int it) { return M <= 32 ? (wb->p0[it] + j) % M : wb->p0[it] + j; };
    auto slot_of = [&](int it, int k) { return wb->base[it] + (int64_t)k * wb->Gc[it] + gi_of(it); };
    auto valid = [&](int it, int k) { return it < count && k < wb->len[it][lane]; };
    auto advance = [&](int& it, int& k) {
        if (k + 1 < wb->L[it]) {
            ++k;
        } else {
            ++it;
            k = 0;
        }
    };
    for (int r = 0; r < rounds; ++r) {
        const int s = r * SL + sl;
        const int s0 = r * SL;  // lane 0's sub-step
        const bool last_lane = (s == sw.S - 1) || (sl == SL - 1);
        // lane 0's pipeline over the sequence positions: cur (this time step), nxt, nn
        In cur, nxt;
        unsigned long long c0 = SENTINEL, c1 = SENTINEL, n0 = SENTINEL, n1 = SENTINEL;
        int cit = 0, ck = 0;
        if (sl == 0 && valid(cit, ck)) {
            const int64_t sl0 = slot_of(cit, ck);
            const int mm = m_of(cit);
            phys.load(sl0, sl0 * M + mm, mm, cur);
            load_words(g, mm, cur.up, s0, c0, c1);
        }
        int nit = cit, nk = ck;
        advance(nit, nk);
        if (DEPTH > 1 && sl == 0 && valid(nit, nk)) {
            const int64_t sl1 = slot_of(nit, nk);
            const int mm = m_of(nit);
            phys.load(sl1, sl1 * M + mm, mm, nxt);
        }
        // what this lane works on at the current time step
        In x;
        St st;
        unsigned long long w0 = SENTINEL, w1 = SENTINEL;
        int pit = count, pk = 0;
        unsigned long long hq = 0ull;
        bool entered = true;  // lane 0: the node's entry hook succeeded (Phys::enter)
        for (int tt = 0; tt < npos + SL - 1; ++tt) {
            if (sl == 0) {
                x = cur;
                w0 = c0;
                w1 = c1;
                pit = cit;
                pk = ck;
                phys.start(x, st);
                entered = !valid(pit, pk) || phys.enter(st, slot_of(pit, pk) * M + m_of(pit));
                // advance the pipeline: the words of nxt, the inputs of the position after it
                int nnit = nit, nnk = nk;
                if (nnit < count) advance(nnit, nnk);
                In nn;
                if (DEPTH > 1) {
                    if (valid(nit, nk)) load_words(g, m_of(nit), nxt.up, s0, n0, n1);
                    if (valid(nnit, nnk)) {
                        const int64_t sl2 = slot_of(nnit, nnk);
                        const int mm = m_of(nnit);
                        phys.load(sl2, sl2 * M + mm, mm, nn);
                    }
                } else if (valid(nit, nk)) {
                    const int64_t sl1 = slot_of(nit, nk);
                    const int mm = m_of(nit);
                    phys.load(sl1, sl1 * M + mm, mm, nxt);
                    load_words(g, mm, nxt.up, s0, n0, n1);
                }
                cur = nxt;
                c0 = n0;
                c1 = n1;
                n0 = n1 = SENTINEL;
                if (DEPTH > 1) nxt = nn;
                cit = nit;
                ck = nk;
                nit = nnit;
                nk = nnk;
            }
            bool ok = entered;
            unsigned long long v0 = SENTINEL, v1 = SENTINEL;  // words of sub-step s + 1 for the next lane
            if (pit < count && pk < wb->len[pit][lane] && s < sw.S) {
                const int64_t slot = slot_of(pit, pk);
                const int mm = m_of(pit);
                const int64_t e = slot * M + mm;
                if (sl + 1 < SL && s + 1 < sw.S) load_words(g, mm, x.up, s + 1, v0, v1);
                unsigned long long out = 0ull;
                ok = phys.sub(x, st, w0, w1, slot, e, mm, s, wb->chain0[pit] + gi_of(pit),
                              pk == wb->len[pit][lane] - 1, pk > 0, hq, out);
                hq = out;
                if (ok && last_lane) phys.finish(st, e, r > 0 || !launch_first);
            }
            if (__any_sync(0xffffffffu, !ok)) return false;
            // hand the node to the next lane
            shfl_up_pod(x, SL);
            shfl_up_pod(st, SL);
            const int pit_up = __shfl_up_sync(0xffffffffu, pit, 1, SL);
            const int pk_up = __shfl_up_sync(0xffffffffu, pk, 1, SL);
            const unsigned long long v0_up = __shfl_up_sync(0xffffffffu, v0, 1, SL);
            const unsigned long long v1_up = __shfl_up_sync(0xffffffffu, v1, 1, SL);
            if (sl > 0) {
                pit = pit_up;
                pk = pk_up;
                w0 = v0_up;
                w1 = v1_up;
            }
            __syncwarp();
        }
    }
    __syncwarp();
    return true;
}

template <class Phys>
__device__ __forceinline__ void walk_diag(const WfDevGraph& g, const WfSweep& sw, Phys& phys, int32_t* status) {
    extern __shared__ unsigned long long wave_smem[];
    const unsigned lane = threadIdx.x & 31u;
    DiagBatch* wb = reinterpret_cast<DiagBatch*>(wave_smem) + (threadIdx.x >> 5);
    const int64_t ipc = wf_items_per_chunk(g.G, g.M, sw.SL);
    const int64_t n_items = g.n_chunks * ipc;
    const int64_t prio = sw.prio_items;
    const int64_t n_norm = n_items - prio;
    const int64_t n_short = min(g.n_short_chunks * ipc, n_norm);
    const int64_t n_sb = (n_short + BATCH - 1) / BATCH;
    const uint64_t n_tickets = (uint64_t)(prio + n_sb + (n_norm - n_short));
    while (true) {
        unsigned long long t = 0;
        if (lane == 0) t = atomicAdd(g.ticket, 1ULL);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= n_tickets) return;
        int64_t first;
        int count = 1;
        if ((int64_t)t < prio) {
            first = n_items - 1 - (int64_t)t;
        } else {
            const int64_t u = (int64_t)t - prio;
            if (u < n_sb) {
                first = u * BATCH;
                count = (int)min((int64_t)BATCH, n_short - first);
            } else {
                first = n_short + (u - n_sb);
            }
        }
        if (!diag_ticket(g, sw, phys, status, first, count, wb)) return;
    }
}

// The overland sweep A (node-major) and the river sweep B in one launch, B's first-dispatched
// chunks on the diagonal schedule (their long chains are the critical path; sw.SL lanes per
// chain-member pair) and its other chunks node-major. Tickets: A's, then B's p_chunks last chunks
// as diagonal items (longest first), then B's remaining chunks node-major (pb.sw.prio_items of
// them dispatched first). Each warp has a node-major batch descriptor after the hand-off rows
// and a diagonal one after those.
template <class PhysA, class PhysB>
__device__ __forceinline__ void walk_pair_diag(PhysA& pa, PhysB& pb, int S_alloc, int64_t p_chunks, int SL,
                                               int32_t* status) {
    extern __shared__ unsigned long long wave_smem[];
    const unsigned lane = threadIdx.x & 31u;
    unsigned long long* qh = wave_smem + threadIdx.x;
    const int warps = blockDim.x >> 5;
    WarpBatch* wbn = reinterpret_cast<WarpBatch*>(wave_smem + (size_t)blockDim.x * S_alloc) + (threadIdx.x >> 5);
    DiagBatch* wbd = reinterpret_cast<DiagBatch*>(reinterpret_cast<WarpBatch*>(wave_smem + (size_t)blockDim.x * S_alloc) +
                                                  warps) + (threadIdx.x >> 5);
    WfSweep swd = pb.sw;
    swd.SL = SL;
    WfDevGraph gn = pb.g;  // the node-major part: every chunk but the last p_chunks
    gn.n_chunks = pb.g.n_chunks - p_chunks;
    const int64_t ipc = wf_items_per_chunk(pb.g.G, pb.g.M, SL);
    const uint64_t na = walk_tickets(pa.g, pa.sw);
    const uint64_t nd = (uint64_t)(p_chunks * ipc);
    const uint64_t nn = walk_tickets(gn, pb.sw);
    const int64_t n_items_d = pb.g.n_chunks * ipc;
    while (true) {
        unsigned long long t = 0;
        if (lane == 0) t = atomicAdd(pa.g.ticket, 1ULL);
        t = __shfl_sync(0xffffffffu, t, 0);
        bool ok;
        if (t < na) {
            ok = walk_ticket(pa.g, pa.sw, pa, status, t, wbn, qh);
        } else if (t < na + nd) {
            swd.SL = SL;
            ok = diag_ticket(pb.g, swd, pb, status, n_items_d - 1 - (int64_t)(t - na), 1, wbd);
        } else if (t < na + nd + nn) {
            ok = walk_ticket(gn, pb.sw, pb, status, t - na - nd, wbn, qh);
        } else {
            return;
        }
        if (!ok) return;
    }
}

__host__ __device__ constexpr size_t pair_diag_smem(int threads, int substeps) {
    return walk_smem(threads, substeps) + (size_t)(threads / 32) * sizeof(DiagBatch);
}

}  // namespace wfv
