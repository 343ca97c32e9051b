// wf_api.cu -- C ABI of the step library (include/wflow_gb300.h).
//
// wf_create restates the reference's model initialisation for the hot-path state:
// derived soil parameters (Wflow/src/soil/soil.jl:319-617), vegetation clip
// (sbm.jl:57-58), cold state (soil.jl:152-200), lateral subsurface initial q / q_max
// (utils.jl:916-937) and storage (lateral_subsurface_flow.jl:134-141), Manning alpha of the
// overland and river kinematic waves (surface_kinwave.jl:32-44, 67-86). It then plans the
// wavefront schedule of both drainage graphs (wf_plan.cpp), permutes every array into the
// slot layout and uploads it. wf_step runs one update_model! + compute_mass_balance! on the
// handle's stream; the fixed-sub-step sequence is captured once in a CUDA graph and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "wf_fields.cuh"
#include "wf_kernels.h"
#include "wf_li_couple.cuh"
#include "wf_wave.cuh"
#include "wf_math.cuh"
#include "wf_plan.h"
#include "wflow_gb300.h"

namespace {

thread_local std::string g_create_error;

struct DevGraphAlloc {
    WfRoutingPlan plan;
    int64_t *chunk_base = nullptr, *up_slot = nullptr, *node_of_slot = nullptr;
    int32_t *chunk_len = nullptr, *chain_len = nullptr, *up_ptr = nullptr, *up_chain = nullptr, *chunk_g = nullptr;
    int64_t* chunk_chain0 = nullptr;
    uint8_t* is_chain_end = nullptr;
    double *up_w = nullptr, *up_fr = nullptr;
    float *up_wf = nullptr, *up_frf = nullptr;
    int4* up_rec = nullptr;
    float* up_whv = nullptr;
    uint8_t* up_nlt = nullptr;
    float4* up_frec = nullptr;
    uint32_t* flags = nullptr;
    double* end_q = nullptr;
    unsigned long long* ticket = nullptr;
    int32_t s_cap = 1;
    int32_t* snow_up = nullptr;  // land graph with snow transport: up entries in topological-sort order
};

}  // namespace

struct WfHandle {
    WfConfig cfg{};
    std::string err;
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    int64_t n = 0, nr = 0;
    int M = 1, N = 4;
    DevGraphAlloc land, river;
    WfDevFields F{};
    std::vector<void*> allocs;
    int32_t* status = nullptr;  // device status word
    double* staging = nullptr;  // [max(n, nr) * M] external-order staging
    double* host_pinned = nullptr;
    size_t host_pinned_bytes = 0;
    double* dts_land = nullptr;
    double* dts_river = nullptr;
    double* dts_ssf = nullptr;
    std::vector<double> h_dts_land, h_dts_river, h_dts_ssf;
    std::vector<int64_t> outlet_slots;
    int64_t* d_outlet_slots = nullptr;  // river slots of river pits
    int64_t* d_land_node_of_slot = nullptr;
    int64_t* d_land_slot_of_node = nullptr;  // [n] land slot of each external cell (forcing tiles)
    WfTuning tuning{};
    WfMetrics metrics{};
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    bool graph_valid = false;
    bool u_dirty = false;  // split form: discharges were set from outside, u = Q^0.2 is stale
    // per-wait budget of the wavefront spin waits: a safety net against a wait that cannot end
    // (a legitimate wait lasts at most about one sweep launch, seconds for the largest FP64
    // sweeps); a wait that runs out ends the launch with WF_ERR_SPIN
    uint64_t wait_ns = 30000000000ull;
    uint32_t wait_offset = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int64_t launches_per_step = 0;
    bool kernel_timing = false;
    cudaEvent_t kev[6] = {};
    double kernel_ms[5] = {0, 0, 0, 0, 0};
    int64_t kernel_calls = 0;
    // adaptive (Courant) sub-stepping
    bool adaptive = false;
    WfAdaptive ad[3] = {};        // WF_ADAPT_SSF, WF_ADAPT_LAND, WF_ADAPT_RIVER
    int32_t* h_more = nullptr;    // pinned host copy of WfAdaptive::more
    int64_t last_substeps[3] = {0, 0, 0};
    // wf_set_forcing_async: host-to-device copies on a stream of their own
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_fcopied = nullptr, ev_fconsumed = nullptr;
    double* fstage = nullptr;     // [3][n_land * M] staged forcing in external order
    double* outlets_buf = nullptr;  // [outlets * M] outlet discharge for wf_get_outlets
    int64_t nres = 0;               // reservoirs
    std::vector<int32_t> river_land;  // [nr] land cell of each river cell
    // local-inertial land and river routing in place of the kinematic waves
    // (wf_attach_local_inertial; the domain stays the caller's)
    WfLiDomain* li = nullptr;
    WfLiCoupleView liv{};
    int64_t li_substeps = 0;
};

namespace {

int set_err(WfHandle* h, int code, const std::string& msg) {
    if (h) h->err = msg;
    else g_create_error = msg;
    return code;
}

int static_scratch(WfHandle* h, unsigned char** out);  // wf_step_static's scratch (below)

#define CK(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return set_err(h, WF_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));   \
    } while (0)

template <class T>
int dalloc(WfHandle* h, T** p, size_t count) {
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
    if (e != cudaSuccess) return set_err(h, WF_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    h->allocs.push_back(*p);
    return WF_OK;
}

template <class T>
int upload(WfHandle* h, T** p, const std::vector<T>& v) {
    int rc = dalloc(h, p, v.size());
    if (rc) return rc;
    if (!v.empty()) CK(cudaMemcpy(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return WF_OK;
}

// Upload an external-order array of n_ext*M (member-major) values into slot layout.
int upload_slots(WfHandle* h, double** dst, const std::vector<double>& ext, const WfRoutingPlan& P, int M,
                 int64_t n_ext, bool per_member) {
    std::vector<double> v((size_t)P.n_slots * (per_member ? M : 1), 0.0);
    for (int64_t s = 0; s < P.n_slots; ++s) {
        int64_t node = P.node_of_slot[s];
        if (node < 0) continue;
        if (per_member) {
            for (int m = 0; m < M; ++m) v[s * M + m] = ext[(size_t)m * n_ext + node];
        } else {
            v[s] = ext[node];
        }
    }
    return upload(h, dst, v);
}

// FP32 copy of an external-order array in slot layout (split form).
int upload_slots_f32(WfHandle* h, float** dst, const std::vector<double>& ext, const WfRoutingPlan& P, int M,
                     int64_t n_ext, bool per_member) {
    std::vector<float> v((size_t)P.n_slots * (per_member ? M : 1), 0.0f);
    for (int64_t s = 0; s < P.n_slots; ++s) {
        int64_t node = P.node_of_slot[s];
        if (node < 0) continue;
        if (per_member) {
            for (int m = 0; m < M; ++m) v[s * M + m] = (float)ext[(size_t)m * n_ext + node];
        } else {
            v[s] = (float)ext[node];
        }
    }
    return upload(h, dst, v);
}

// Double-FP32 pair (high part, low part) of an external-order array in slot layout (split form).
int upload_slots_ff(WfHandle* h, float** hi, float** lo, const std::vector<double>& ext, const WfRoutingPlan& P,
                    int M, int64_t n_ext, bool per_member) {
    std::vector<float> vh((size_t)P.n_slots * (per_member ? M : 1), 0.0f), vl(vh.size(), 0.0f);
    auto put = [&](size_t i, double x) {
        const float a = (float)x;
        vh[i] = a;
        vl[i] = (float)(x - (double)a);
    };
    for (int64_t s = 0; s < P.n_slots; ++s) {
        int64_t node = P.node_of_slot[s];
        if (node < 0) continue;
        if (per_member) {
            for (int m = 0; m < M; ++m) put(s * M + m, ext[(size_t)m * n_ext + node]);
        } else {
            put(s, ext[node]);
        }
    }
    int rc = upload(h, hi, vh);
    return rc ? rc : upload(h, lo, vl);
}

int plan_graph(WfHandle* h, DevGraphAlloc& G, int64_t n, const int32_t* ds, int M, int32_t s_cap,
               const int64_t* heavy_hint = nullptr) {
    std::string err;
    int rc = wf_build_plan(n, ds, M, G.plan, err, heavy_hint);
    if (rc) return set_err(h, rc == WF_ERR_CYCLE ? WF_ERR_CYCLE : WF_ERR_INVALID, err);
    const WfRoutingPlan& P = G.plan;
    if ((rc = upload(h, &G.chunk_base, P.chunk_base))) return rc;
    if ((rc = upload(h, &G.chunk_len, P.chunk_len))) return rc;
    if ((rc = upload(h, &G.chunk_g, P.chunk_g))) return rc;
    if ((rc = upload(h, &G.chunk_chain0, P.chunk_chain0))) return rc;
    if ((rc = upload(h, &G.chain_len, P.chain_len))) return rc;
    if ((rc = upload(h, &G.up_ptr, P.up_ptr))) return rc;
    if ((rc = upload(h, &G.up_slot, P.up_slot))) return rc;
    if ((rc = upload(h, &G.up_chain, P.up_chain))) return rc;
    if ((rc = upload(h, &G.is_chain_end, P.is_chain_end))) return rc;
    if ((rc = upload(h, &G.node_of_slot, P.node_of_slot))) return rc;
    G.s_cap = s_cap;
    if ((rc = dalloc(h, &G.flags, (size_t)P.n_chains * M))) return rc;
    if ((rc = dalloc(h, &G.end_q, (size_t)P.n_chains * M * s_cap))) return rc;
    if ((rc = dalloc(h, &G.ticket, 1))) return rc;
    return WF_OK;
}

WfDevGraph dev_graph(const DevGraphAlloc& G, int M) {
    WfDevGraph g{};
    g.n_slots = G.plan.n_slots;
    g.n_chunks = G.plan.n_chunks;
    g.n_chains = G.plan.n_chains;
    g.n_long_chunks = G.plan.n_long_chunks;
    {
        int64_t ns = 0;
        while (ns < G.plan.n_chunks && G.plan.chunk_len[ns] <= wfv::SHORT_LEN) ++ns;
        g.n_short_chunks = ns;
    }
    g.G = G.plan.G;
    g.M = M;
    g.chunk_base = G.chunk_base;
    g.chunk_len = G.chunk_len;
    g.chunk_g = G.chunk_g;
    g.chunk_chain0 = G.chunk_chain0;
    g.chain_len = G.chain_len;
    g.up_ptr = G.up_ptr;
    g.up_slot = G.up_slot;
    g.up_chain = G.up_chain;
    g.is_chain_end = G.is_chain_end;
    g.up_w = G.up_w;
    g.up_fr = G.up_fr;
    g.up_wf = G.up_wf;
    g.up_frf = G.up_frf;
    g.up_rec = G.up_rec;
    g.up_whv = G.up_whv;
    g.up_nlt = G.up_nlt;
    g.up_frec = G.up_frec;
    g.flags = G.flags;
    g.end_q = G.end_q;
    g.ticket = G.ticket;
    g.s_cap = G.s_cap;
    g.snow_up = G.snow_up;
    return g;
}

// Graphs.jl v1.14 topological_sort_by_dfs (Wflow's network.order, network.jl:99) of a graph of
// out-degree <= 1: vertices in index order; from an unvisited vertex follow the downstream links
// to unvisited vertices, finish the path from its downstream end back; the order is the reverse
// of the finishing order. Empty on a cycle.
std::vector<int64_t> topo_order_dfs(int64_t n, const int32_t* ds) {
    std::vector<uint8_t> color((size_t)n, 0);
    std::vector<int64_t> verts, stack;
    verts.reserve((size_t)n);
    for (int64_t v = 0; v < n; ++v) {
        if (color[v]) continue;
        stack.assign(1, v);
        color[v] = 1;
        while (!stack.empty()) {
            const int64_t u = stack.back();
            const int32_t w = ds[u];
            if (w >= 0 && color[w] == 1) return {};
            if (w >= 0 && color[w] == 0) {
                color[w] = 1;
                stack.push_back(w);
            } else {
                color[u] = 2;
                verts.push_back(u);
                stack.pop_back();
            }
        }
    }
    return std::vector<int64_t>(verts.rbegin(), verts.rend());
}

// fixed sub-steps of a sweep (routing/timestepping.jl:11-16 with the while loop of the
// update_*_flow_model! drivers)
std::vector<double> fixed_substeps(double dt_fixed, double dt) {
    std::vector<double> v;
    double t = 0.0;
    while (t < dt) {
        double ts = dt_fixed;
        if (t + ts > dt) ts = dt - t;
        v.push_back(ts);
        t += ts;
        if (v.size() > 1000000) break;
    }
    return v;
}

// Device state of the adaptive sub-step selection (one per sweep kind); the Courant-time keys
// are shared, the sweeps run one after the other.
int alloc_adaptive(WfHandle* h) {
    const WfRoutingPlan& PL = h->land.plan;
    const WfRoutingPlan& PR = h->river.plan;
    const int M = h->M;
    int rc;
    unsigned long long* keys = nullptr;
    if ((rc = dalloc(h, &keys, (size_t)std::max(PL.n_slots, PR.n_slots) * M))) return rc;
    for (int k = 0; k < 3; ++k) {
        WfAdaptive& A = h->ad[k];
        A.kind = k;
        A.M = M;
        A.fp32_keys = h->F.split;
        A.kv_profile = h->cfg.kv_profile;
        A.p = k == WF_ADAPT_LAND ? 0.02 : 0.05;  // surface_kinwave.jl:374 (land), :638 (river)
        A.dt = h->cfg.dt;
        A.alpha = h->cfg.subsurface_alpha;
        A.n_slots = k == WF_ADAPT_RIVER ? PR.n_slots : PL.n_slots;
        A.keys = keys;
        if ((rc = dalloc(h, &A.hist, (size_t)2 * M * 256))) return rc;
        if ((rc = dalloc(h, &A.prefix, (size_t)2 * M))) return rc;
        if ((rc = dalloc(h, &A.rank, (size_t)2 * M))) return rc;
        if ((rc = dalloc(h, &A.count, (size_t)M))) return rc;
        if ((rc = dalloc(h, &A.minkey, (size_t)M))) return rc;
        if ((rc = dalloc(h, &A.done, 1))) return rc;
        if ((rc = dalloc(h, &A.t, (size_t)M))) return rc;
        if ((rc = dalloc(h, &A.dt_s, (size_t)M))) return rc;
        if ((rc = dalloc(h, &A.dt_hi, (size_t)M))) return rc;
        if ((rc = dalloc(h, &A.dt_lo, (size_t)M))) return rc;
        if ((rc = dalloc(h, &A.flags, (size_t)M))) return rc;
        if ((rc = dalloc(h, &A.nsub, (size_t)M))) return rc;
        if ((rc = dalloc(h, &A.sig, (size_t)M))) return rc;
        if ((rc = dalloc(h, &A.more, 1))) return rc;
        CK(cudaMemset(A.hist, 0, (size_t)2 * M * 256 * sizeof(uint32_t)));
        CK(cudaMemset(A.count, 0, (size_t)M * sizeof(long long)));
        CK(cudaMemset(A.minkey, 0xFF, (size_t)M * sizeof(unsigned long long)));
        CK(cudaMemset(A.done, 0, sizeof(uint32_t)));
    }
    CK(cudaHostAlloc((void**)&h->h_more, sizeof(int32_t), cudaHostAllocDefault));
    return WF_OK;
}

WfLaunchCfg launch_cfg(const WfHandle* h) {
    WfLaunchCfg c{};
    c.stream = h->stream;
    c.num_sms = h->num_sms;
    c.vertical_block = h->tuning.vertical_block;
    c.walk_warps = h->tuning.routing_warps;
    c.walk_blocks = h->tuning.routing_blocks_per_sm > 0 ? h->tuning.routing_blocks_per_sm * h->num_sms : 0;
    c.sub_lanes = h->tuning.reserved[3];
    c.walk_inputs = h->tuning.reserved[4];
    c.vertical_blocks_per_sm = h->tuning.reserved[5];
    return c;
}

// ------------------------------------------------------------------ gather/scatter kernels
__global__ void gather_kernel(const double* src, double* dst, const int64_t* node_of_slot, int64_t slots, int M,
                              int64_t n_ext) {
    const int64_t E = slots * M;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = e / M;
        const int m = (int)(e - s * M);
        const int64_t node = node_of_slot[s];
        if (node >= 0) dst[e] = src[(int64_t)m * n_ext + node];
    }
}
__global__ void scatter_kernel(const double* src, double* dst, const int64_t* node_of_slot, int64_t slots, int M,
                               int64_t n_ext) {
    const int64_t E = slots * M;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = e / M;
        const int m = (int)(e - s * M);
        const int64_t node = node_of_slot[s];
        if (node >= 0) dst[(int64_t)m * n_ext + node] = src[e];
    }
}
// FP64 external order -> FP32 (or a double-FP32 pair when lo is given) in slot order
__global__ void gather_f32_kernel(const double* src, float* dst, const int64_t* node_of_slot, int64_t slots, int M,
                                  int64_t n_ext, float* lo = nullptr) {
    const int64_t E = slots * M;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = e / M;
        const int m = (int)(e - s * M);
        const int64_t node = node_of_slot[s];
        if (node < 0) continue;
        const double x = src[(int64_t)m * n_ext + node];
        const float a = (float)x;
        dst[e] = a;
        if (lo) lo[e] = (float)(x - (double)a);
    }
}
// FP32 (or double-FP32 pair) in slot order -> FP64 external order
__global__ void scatter_f32_kernel(const float* src, double* dst, const int64_t* node_of_slot, int64_t slots, int M,
                                   int64_t n_ext, const float* lo = nullptr) {
    const int64_t E = slots * M;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = e / M;
        const int m = (int)(e - s * M);
        const int64_t node = node_of_slot[s];
        if (node >= 0) dst[(int64_t)m * n_ext + node] = (double)src[e] + (lo ? (double)lo[e] : 0.0);
    }
}
// Discharge at the outlets from double-FP32 pairs, member-major (split form).
__global__ void outlets_ff_kernel(const float* hi, const float* lo, const int64_t* slots, int64_t n_out, int M,
                                  double* dst) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n_out * M) return;
    const int m = (int)(i / n_out);
    const int64_t e = slots[i - (int64_t)m * n_out] * M + m;
    dst[i] = (double)hi[e] + (double)lo[e];
}
__global__ void to_f32_kernel(const double* src, float* dst, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = (float)src[i];
}
// Member-major forcing (external cell order) into the slot order, through a shared-memory tile
// of 32 cells x 32 members: a warp reads 32 consecutive cells of one member (coalesced) and
// writes the 32 members of one cell (one contiguous run of the slot-order array), where an
// element-wise gather would read one isolated word per member. FP32 destination (split form) or
// FP64. Grid: (ceil(n / 32), ceil(M / 32)); block 32 x 8.
template <typename S>
__global__ void __launch_bounds__(256) forcing_tile_kernel(const S* src, float* dst32, double* dst64,
                                                           const int64_t* slot_of_node, int64_t n, int M) {
    __shared__ S tile[32][33];
    const int64_t node0 = (int64_t)blockIdx.x * 32;
    const int m0 = blockIdx.y * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
    for (int j = ty; j < 32; j += 8) {
        const int m = m0 + j;
        const int64_t node = node0 + tx;
        if (m < M && node < n) tile[j][tx] = src[(int64_t)m * n + node];
    }
    __syncthreads();
    for (int k = ty; k < 32; k += 8) {
        const int64_t node = node0 + k;
        const int m = m0 + tx;
        if (node >= n || m >= M) continue;
        const int64_t e = slot_of_node[node] * M + m;
        if (dst32) dst32[e] = (float)tile[tx][k];
        else dst64[e] = (double)tile[tx][k];
    }
}
// The same for fewer than 32 members: one thread per (member, cell) in external order (coalesced
// reads; the writes follow the slot permutation).
template <typename S>
__global__ void forcing_scatter_small_kernel(const S* src, float* dst32, double* dst64, const int64_t* slot_of_node,
                                             int64_t n, int M) {
    const int64_t E = n * M;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < E; i += (int64_t)gridDim.x * blockDim.x) {
        const int m = (int)(i / n);
        const int64_t node = i - (int64_t)m * n;
        const int64_t e = slot_of_node[node] * M + m;
        if (dst32) dst32[e] = (float)src[i];
        else dst64[e] = (double)src[i];
    }
}
int grid_of(int64_t n, int block);
template <typename S>
void launch_forcing_full(const WfHandle* h, const S* src, float* dst32, double* dst64) {
    if (h->M >= 32) {
        const dim3 grid((unsigned)((h->n + 31) / 32), (unsigned)((h->M + 31) / 32));
        forcing_tile_kernel<S><<<grid, dim3(32, 8), 0, h->stream>>>(src, dst32, dst64, h->d_land_slot_of_node, h->n,
                                                                     h->M);
    } else {
        forcing_scatter_small_kernel<S><<<grid_of(h->n * h->M, 256), 256, 0, h->stream>>>(
            src, dst32, dst64, h->d_land_slot_of_node, h->n, h->M);
    }
}

// FP32 forcing of n_ext cells per member (member-major, or one set for every member when
// `broadcast`) into the slot order: FP32 destination (split form) or FP64 (FP64 form).
__global__ void gather_from_f32_kernel(const float* src, float* dst32, double* dst64, const int64_t* node_of_slot,
                                       int64_t slots, int M, int64_t n_ext, int broadcast) {
    const int64_t E = slots * M;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = e / M;
        const int m = (int)(e - s * M);
        const int64_t node = node_of_slot[s];
        if (node < 0) continue;
        const float x = src[(broadcast ? 0 : (int64_t)m * n_ext) + node];
        if (dst32) dst32[e] = x;
        else dst64[e] = (double)x;
    }
}
__global__ void broadcast_member_f32_kernel(const double* src, float* dst, const int64_t* node_of_slot, int64_t slots,
                                            int M) {
    const int64_t E = slots * M;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = e / M;
        const int64_t node = node_of_slot[s];
        if (node >= 0) dst[e] = (float)src[node];
    }
}
__global__ void broadcast_member_kernel(const double* src, double* dst, const int64_t* node_of_slot, int64_t slots,
                                        int M, const double* scale) {
    const int64_t E = slots * M;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = e / M;
        const int64_t node = node_of_slot[s];
        if (node >= 0) dst[e] = scale ? src[node] * scale[e - s * M] : src[node];
    }
}

int grid_of(int64_t n, int block) {
    int64_t b = (n + block - 1) / block;
    if (b > 65535LL * 16) b = 65535LL * 16;
    return (int)(b < 1 ? 1 : b);
}

// Field table: WfField -> device array
struct FieldRef {
    double* p = nullptr;      // FP64 array (FP64 form)
    float* p32 = nullptr;     // FP32 array, or the high part of a double-FP32 pair (split form)
    float* p32lo = nullptr;   // low part of a double-FP32 pair (split form)
    int idx = -1;             // member / river-member field index
    bool usld = false;        // unsaturated layer store of layer `layer`
    bool river = false;
    bool member = true;
    bool derived_vwc = false;
    bool settable = false;
};

FieldRef field_ref(WfHandle* h, int field, int layer) {
    FieldRef r;
    auto& Mf = h->F.Mf;
    auto& RM = h->F.RM;
    switch (field) {
        case WF_F_CANOPY_STORAGE: r.idx = CANOPY; r.settable = true; break;
        case WF_F_SNOW_STORAGE: r.idx = SNOW; r.settable = true; break;
        case WF_F_SNOW_WATER: r.idx = SNOW_WATER; r.settable = true; break;
        case WF_F_SOIL_SURFACE_TEMPERATURE: r.idx = TSOIL; r.settable = true; break;
        case WF_F_SATURATED_WATER_DEPTH: r.idx = SAT; r.settable = true; break;
        case WF_F_UNSATURATED_LAYER_DEPTH:
            r.usld = layer >= 0 && layer < h->N;
            r.settable = true;
            break;
        case WF_F_SSF_Q: r.idx = SSF_Q; r.settable = true; break;
        case WF_F_LAND_Q: r.idx = OL_Q; r.settable = true; break;
        case WF_F_LAND_H: r.idx = OL_H; r.settable = true; break;
        case WF_F_WATER_TABLE_DEPTH: r.idx = ZI; break;
        case WF_F_UNSATURATED_STORE_DEPTH: r.idx = USTOREDEPTH; break;
        case WF_F_TOTAL_SOIL_WATER_STORAGE: r.idx = TSWS; r.settable = true; break;
        case WF_F_RECHARGE: r.idx = RECHARGE; break;
        case WF_F_NET_RUNOFF: r.idx = NET_RUNOFF; break;
        case WF_F_RUNOFF: r.idx = RUNOFF; break;
        case WF_F_ACTUAL_EVAPOTRANSPIRATION: r.idx = AET; break;
        case WF_F_ACTUAL_LEAKAGE: r.idx = LEAKAGE; break;
        case WF_F_TRANSPIRATION: r.idx = TRANSPIRATION; break;
        case WF_F_SOIL_EVAPORATION: r.idx = SOIL_EVAP; break;
        case WF_F_ACTUAL_INFILTRATION: r.idx = ACT_INFILT; break;
        case WF_F_EXFILTRATION_SATURATED_WATER: r.idx = EXFILT; break;
        case WF_F_INTERCEPTION_RATE: r.idx = INTERCEPTION; break;
        case WF_F_SNOW_WATER_EQUIVALENT: r.idx = SWE; break;
        case WF_F_NET_RUNOFF_RIVER: r.idx = NET_RUNOFF_RIVER; break;
        case WF_F_SSF_Q_AVERAGE: r.idx = SSF_Q_AVG; break;
        case WF_F_SSF_WATER_TABLE_DEPTH: r.idx = SSF_ZI; break;
        case WF_F_SSF_STORAGE: r.idx = SSF_STORAGE; break;
        case WF_F_SSF_TO_RIVER_AVERAGE: r.idx = SSF_TR_AVG; break;
        case WF_F_LAND_Q_AVERAGE: r.idx = OL_Q_AVG; break;
        case WF_F_LAND_QIN_AVERAGE: r.idx = OL_QIN_AVG; break;
        case WF_F_LAND_STORAGE: r.idx = OL_STORAGE; r.settable = true; break;
        case WF_F_LAND_TO_RIVER_AVERAGE: r.idx = OL_TR_AVG; break;
        case WF_F_LAND_INWATER: r.idx = OL_INWATER; break;
        case WF_F_TOTAL_STORAGE: r.idx = TOTAL_STORAGE; break;
        case WF_F_BALANCE_LAND_ERROR: r.idx = BL_ERR; break;
        case WF_F_BALANCE_LAND_RELATIVE_ERROR: r.idx = BL_REL; break;
        case WF_F_BALANCE_OVERLAND_ERROR: r.idx = BO_ERR; break;
        case WF_F_BALANCE_OVERLAND_RELATIVE_ERROR: r.idx = BO_REL; break;
        case WF_F_BALANCE_SUBSURFACE_ERROR: r.idx = BS_ERR; break;
        case WF_F_BALANCE_SUBSURFACE_RELATIVE_ERROR: r.idx = BS_REL; break;
        case WF_F_VOLUMETRIC_WATER_CONTENT:
            r.derived_vwc = (layer >= 0 && layer < h->N);
            break;
        case WF_F_GLACIER_STORE:
            r.p = h->F.glacier ? h->F.GM[GM_STORE] : nullptr;
            r.settable = true;
            break;
        case WF_F_GLACIER_MELT: r.p = h->F.glacier ? h->F.GM[GM_MELT] : nullptr; break;
        case WF_F_SNOW_IN: r.p = h->F.snow_transport ? h->F.GM[GM_SNOW_IN] : nullptr; break;
        case WF_F_SNOW_OUT: r.p = h->F.snow_transport ? h->F.GM[GM_SNOW_OUT] : nullptr; break;
        case WF_F_RIVER_Q: r.idx = RV_Q; r.river = true; r.settable = true; break;
        case WF_F_RIVER_H: r.idx = RV_H; r.river = true; r.settable = true; break;
        case WF_F_RIVER_STORAGE: r.idx = RV_STORAGE; r.river = true; r.settable = true; break;
        case WF_F_RIVER_Q_AVERAGE: r.idx = RV_Q_AVG; r.river = true; break;
        case WF_F_RIVER_QIN_AVERAGE: r.idx = RV_QIN_AVG; r.river = true; break;
        case WF_F_RIVER_INWATER: r.idx = RV_INWATER; r.river = true; break;
        case WF_F_BALANCE_RIVER_ERROR: r.idx = BR_ERR; r.river = true; break;
        case WF_F_BALANCE_RIVER_RELATIVE_ERROR: r.idx = BR_REL; r.river = true; break;
        default: break;
    }
    const WfDevFields& F = h->F;
    if (r.usld) {
        if (!F.split) {
            r.p = F.LY[LY_USLD][layer];
        } else {
            r.p32 = F.LYf[LY_USLD][layer];
            r.p32lo = F.LYl[layer];
        }
    } else if (r.idx >= 0) {
        if (!F.split) {
            r.p = r.river ? RM[r.idx] : Mf[r.idx];
        } else if (r.river) {
            r.p32 = F.RMh[r.idx];
            r.p32lo = F.RMl[r.idx];
        } else if (wf_split_fp64_member(r.idx)) {
            r.p = Mf[r.idx];
        } else {
            r.p32 = F.Mh[r.idx];
            if (!wf_split_f32_member(r.idx)) r.p32lo = F.Ml[r.idx];
        }
    }
    return r;
}

// State carried from one step to the next (checkpoint content), in this order.
struct StateItem {
    int field;
    int layer;
};
std::vector<StateItem> state_items(const WfHandle* h) {
    std::vector<StateItem> v;
    for (int f : {WF_F_CANOPY_STORAGE, WF_F_SNOW_STORAGE, WF_F_SNOW_WATER, WF_F_SOIL_SURFACE_TEMPERATURE,
                  WF_F_SATURATED_WATER_DEPTH, WF_F_TOTAL_SOIL_WATER_STORAGE, WF_F_SSF_Q, WF_F_LAND_Q, WF_F_LAND_H,
                  WF_F_LAND_STORAGE, WF_F_RIVER_Q, WF_F_RIVER_H, WF_F_RIVER_STORAGE})
        v.push_back({f, 0});
    for (int k = 0; k < h->N; ++k) v.push_back({WF_F_UNSATURATED_LAYER_DEPTH, k});
    if (h->F.glacier) v.push_back({WF_F_GLACIER_STORE, 0});
    if (h->nres > 0) {  // reservoir states (water level; storage kept alongside for exact restarts)
        v.push_back({WF_F_RESERVOIR_STORAGE, 0});
        v.push_back({WF_F_RESERVOIR_WATERLEVEL, 0});
    }
    return v;
}

// Values per member of a field: reservoirs, river cells or land cells.
int64_t field_extent(const WfHandle* h, int field) {
    if (field >= WF_F_RESERVOIR_STORAGE) return h->nres;
    return field >= WF_F_RIVER_Q ? h->nr : h->n;
}

// Reservoir fields: device arrays of element r * M + m to and from the member-major external
// order. Exactly one of dst (get) and src (set) is non-null.
int reservoir_io(WfHandle* h, int32_t field, double* dst, const double* src, int64_t offset, int64_t count) {
    if (field < WF_F_RESERVOIR_STORAGE || field >= WF_F_RESERVOIR_END_ || h->nres <= 0)
        return set_err(h, WF_ERR_INVALID, "unknown field or model without reservoirs");
    const bool settable = field == WF_F_RESERVOIR_STORAGE || field == WF_F_RESERVOIR_WATERLEVEL ||
                          field == WF_F_RESERVOIR_PRECIPITATION || field == WF_F_RESERVOIR_EVAPORATION ||
                          field == WF_F_RESERVOIR_EXTERNAL_INFLOW || field == WF_F_RESERVOIR_OUTFLOW_OBS;
    if (src && !settable) return set_err(h, WF_ERR_INVALID, "field is not settable");
    const int64_t nres = h->nres, M = h->M, total = nres * M;
    if (offset < 0 || count < 0 || offset + count > total) return set_err(h, WF_ERR_INVALID, "range out of bounds");
    double* dev_p = h->F.RS[field - WF_F_RESERVOIR_STORAGE];
    std::vector<double> dev((size_t)total), ext((size_t)total);
    CK(cudaMemcpyAsync(dev.data(), dev_p, total * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (int64_t r = 0; r < nres; ++r)
        for (int64_t m = 0; m < M; ++m) ext[m * nres + r] = dev[r * M + m];
    if (dst) {
        if (count) std::memcpy(dst, ext.data() + offset, count * sizeof(double));
        return WF_OK;
    }
    if (count) std::memcpy(ext.data() + offset, src, count * sizeof(double));
    for (int64_t r = 0; r < nres; ++r)
        for (int64_t m = 0; m < M; ++m) dev[r * M + m] = ext[m * nres + r];
    CK(cudaMemcpyAsync(dev_p, dev.data(), total * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return WF_OK;
}

struct StateHeader {
    char magic[8];
    int32_t version;
    int32_t n_members;
    int64_t n_land;
    int64_t n_river;
    int32_t n_layers;
    int32_t n_items;
};

int run_step(WfHandle* h);

__global__ void set_day_kernel(int32_t* day, int32_t v) { *day = v; }

// reservoir.jl:363-375 on n rows at xp[i] and fp[i * fs], xp strictly increasing (the host copy of
// wfr::interpolate_linear, for the initial and maximum storages)
double interpolate_linear_host(double x, const double* xp, const double* fp, int64_t fs, int64_t n) {
    double fmin = fp[0], fmax = fp[0];
    for (int64_t i = 1; i < n; ++i) {
        fmin = wfm::jmin(fmin, fp[i * fs]);
        fmax = wfm::jmax(fmax, fp[i * fs]);
    }
    if (x <= xp[0]) return fmin;
    if (x >= xp[n - 1]) return fmax;
    int64_t i1 = 0;
    while (i1 + 1 < n && xp[i1 + 1] <= x) ++i1;
    const int64_t i2 = i1 + 1;
    const double f1 = fp[i1 * fs], f2 = fp[i2 * fs];
    return f1 * (1.0 - (x - xp[i1]) / (xp[i2] - xp[i1])) + f2 * (x - xp[i1]) / (xp[i2] - xp[i1]);
}

// The reservoirs' tables and links, checked and laid out for the device (ReservoirParameters,
// reservoir.jl:5-44, 152-192), with each reservoir's initial storage (initialize_storage,
// :343-360), a rating curve's maximum storage (get_maximum_storage, :322-340) and, for linked
// reservoirs, the river planner's hints that keep each upper-to-lower path on one chain.
struct ResTables {
    bool any = false, linked = false;
    std::vector<int32_t> profile, lower;
    std::vector<int64_t> meta;  // [4 n]: S-H start, rows, H-Q start, rows (into tab)
    std::vector<double> tab, initial_storage, maximum_storage;
    std::vector<int64_t> heavy_hint;  // [n_river]
};

int res_tables(const WfReservoirs* rs, const WfReservoirTables* tb, int64_t nr, const int32_t* rds, ResTables& rt) {
    const int64_t n = rs->n;
    const double NaN = wfm::from_bits(0x7ff8000000000000ULL);
    rt.profile.assign(n, WF_RES_PROFILE_LINEAR);
    rt.lower.assign(n, -1);
    rt.meta.assign(4 * n, 0);
    rt.initial_storage.assign(n, 0.0);
    rt.maximum_storage.assign(n, NaN);
    auto bad = [](int rc, const char* msg) { return set_err(nullptr, rc, msg); };
    auto increasing = [](const double* v, int64_t a, int64_t b) {
        for (int64_t i = a; i < b; ++i)
            if (!std::isfinite(v[i]) || (i > a && !(v[i] > v[i - 1]))) return false;
        return true;
    };
    for (int64_t k = 0; k < n; ++k) {
        const int32_t prof = tb && tb->storage_curve_type ? tb->storage_curve_type[k] : WF_RES_PROFILE_LINEAR;
        if (prof != WF_RES_PROFILE_LINEAR && prof != WF_RES_PROFILE_INTERPOLATION)
            return bad(WF_ERR_INVALID, "unknown reservoir storage curve type");
        rt.profile[k] = prof;
        if (prof == WF_RES_PROFILE_INTERPOLATION) {
            if (!tb->sh_offset || !tb->sh_h || !tb->sh_s) return bad(WF_ERR_INVALID, "reservoir S-H tables missing");
            const int64_t a = tb->sh_offset[k], b = tb->sh_offset[k + 1];
            if (a < 0 || b <= a) return bad(WF_ERR_INVALID, "empty reservoir S-H table");
            if (!increasing(tb->sh_h, a, b) || !increasing(tb->sh_s, a, b))
                return bad(WF_ERR_INVALID, "reservoir S-H table not strictly increasing");
            rt.meta[4 * k] = (int64_t)rt.tab.size();
            rt.meta[4 * k + 1] = b - a;
            rt.tab.insert(rt.tab.end(), tb->sh_h + a, tb->sh_h + b);
            rt.tab.insert(rt.tab.end(), tb->sh_s + a, tb->sh_s + b);
            rt.any = true;
        }
        if (rs->outflow_curve_type[k] == WF_RES_RATING_CURVE) {
            if (!tb || !tb->hq_offset || !tb->hq_h || !tb->hq_q)
                return bad(WF_ERR_INVALID, "reservoir H-Q tables missing for a rating curve");
            const int64_t a = tb->hq_offset[k], b = tb->hq_offset[k + 1];
            if (a < 0 || b <= a) return bad(WF_ERR_INVALID, "empty reservoir H-Q table");
            if (!increasing(tb->hq_h, a, b)) return bad(WF_ERR_INVALID, "reservoir H-Q table not strictly increasing");
            for (int64_t i = a * 365; i < b * 365; ++i)
                if (!std::isfinite(tb->hq_q[i])) return bad(WF_ERR_INVALID, "reservoir H-Q table not finite");
            rt.meta[4 * k + 2] = (int64_t)rt.tab.size();
            rt.meta[4 * k + 3] = b - a;
            rt.tab.insert(rt.tab.end(), tb->hq_h + a, tb->hq_h + b);
            rt.tab.insert(rt.tab.end(), tb->hq_q + a * 365, tb->hq_q + b * 365);
            rt.any = true;
        }
        if (tb && tb->lower_reservoir) {
            const int32_t lo = tb->lower_reservoir[k];
            if (lo < -1 || lo >= n || lo == k) return bad(WF_ERR_INVALID, "linked lower reservoir out of range");
            rt.lower[k] = lo;
            if (lo >= 0) rt.any = rt.linked = true;
        }
    }
    for (int64_t k = 0; k < n; ++k) {
        const double* sh = rt.tab.data() + rt.meta[4 * k];
        const int64_t nsh = rt.meta[4 * k + 1];
        const double wl = rs->waterlevel[k];
        rt.initial_storage[k] = rt.profile[k] == WF_RES_PROFILE_INTERPOLATION
                                    ? interpolate_linear_host(wl, sh, sh + nsh, 1, nsh)
                                    : rs->area[k] * wl;
        if (rs->outflow_curve_type[k] == WF_RES_RATING_CURVE) {
            const double* hq = rt.tab.data() + rt.meta[4 * k + 2];
            double hmax = hq[0];
            for (int64_t i = 1; i < rt.meta[4 * k + 3]; ++i) hmax = wfm::jmax(hmax, hq[i]);
            rt.maximum_storage[k] = rt.profile[k] == WF_RES_PROFILE_INTERPOLATION
                                        ? interpolate_linear_host(hmax, sh, sh + nsh, 1, nsh)
                                        : rs->area[k] * hmax;
        }
    }
    if (rt.linked) {
        rt.heavy_hint.assign(nr, -1);
        for (int64_t k = 0; k < n; ++k) {
            if (rt.lower[k] < 0) continue;
            const int64_t target = rs->river_index[rt.lower[k]];
            int64_t prev = rs->river_index[k], x = rds[prev], steps = 0;
            while (x >= 0 && steps++ <= nr) {
                if (x >= nr) return bad(WF_ERR_INVALID, "river_downstream out of range");
                if (rt.heavy_hint[x] >= 0 && rt.heavy_hint[x] != prev)
                    return bad(WF_ERR_UNSUPPORTED, "the river paths of two linked reservoir pairs join");
                rt.heavy_hint[x] = prev;
                if (x == target) break;
                prev = x;
                x = rds[x];
            }
            if (x != target)
                return bad(WF_ERR_UNSUPPORTED,
                           "a linked lower reservoir must lie downstream of its upper reservoir on the river");
        }
    }
    return WF_OK;
}

}  // namespace

// ============================================================================ C ABI =======
extern "C" {

int32_t wf_abi_version(void) { return WF_ABI_VERSION; }

int32_t wf_struct_size(int32_t which) {
    switch (which) {
        case 0: return (int32_t)sizeof(WfConfig);
        case 1: return (int32_t)sizeof(WfDomain);
        case 2: return (int32_t)sizeof(WfParams);
        case 3: return (int32_t)sizeof(WfMetrics);
        case 4: return (int32_t)sizeof(WfTuning);
        case 5: return (int32_t)sizeof(WfReservoirs);
        case 6: return (int32_t)sizeof(WfReservoirTables);
        default: return -1;
    }
}

const char* wf_last_error(const WfHandle* h) { return h ? h->err.c_str() : g_create_error.c_str(); }

int32_t wf_create(const WfConfig* c, const WfDomain* d, const WfParams* p, int32_t device, WfHandle** out) {
    return wf_create_with_reservoirs(c, d, p, nullptr, device, out);
}

int32_t wf_create_with_reservoirs(const WfConfig* c, const WfDomain* d, const WfParams* p, const WfReservoirs* rs,
                                  int32_t device, WfHandle** out) {
    return wf_create_with_reservoir_tables(c, d, p, rs, nullptr, device, out);
}

int32_t wf_create_with_reservoir_tables(const WfConfig* c, const WfDomain* d, const WfParams* p,
                                        const WfReservoirs* rs, const WfReservoirTables* tb, int32_t device,
                                        WfHandle** out) {
    WfHandle* h = nullptr;
    if (!out) return set_err(nullptr, WF_ERR_INVALID, "null output handle");
    *out = nullptr;
    if (!c || !d || !p) return set_err(nullptr, WF_ERR_INVALID, "null argument");
    const int N = c->n_soil_layer_thickness + 1;
    if (N < 2 || N > WF_MAX_LAYERS) return set_err(nullptr, WF_ERR_INVALID, "soil_layer__thickness length out of range");
    if (d->n_land <= 0 || d->n_river < 0) return set_err(nullptr, WF_ERR_INVALID, "empty domain");
    if (c->dt <= 0.0) return set_err(nullptr, WF_ERR_INVALID, "dt must be positive");
    if (c->form != WF_FORM_FP64 && c->form != WF_FORM_SPLIT) return set_err(nullptr, WF_ERR_INVALID, "unknown form");
    if (c->kv_profile != WF_KV_EXPONENTIAL && c->kv_profile != WF_KV_EXPONENTIAL_CONSTANT)
        return set_err(nullptr, WF_ERR_UNSUPPORTED, "only the exponential and exponential_constant Kv profiles");
    const int M = c->n_members > 0 ? c->n_members : 1;
    if (!((M <= 32 && (M & (M - 1)) == 0) || (M > 32 && M % 32 == 0)))
        return set_err(nullptr, WF_ERR_INVALID, "n_members must be a power of two up to 32 or a multiple of 32");
    const double* req[] = {d->area, d->flow_width, d->flow_length, d->surface_flow_width, d->slope,
                           d->flow_fraction_to_river, d->river_fraction, d->water_fraction, d->elevation,
                           d->land_manning_n, p->canopy_gap_fraction, p->maximum_canopy_storage, p->crop_coefficient,
                           p->rooting_depth, p->theta_s, p->theta_r, p->kv_0, p->f, p->soil_thickness,
                           p->air_entry_pressure, p->h1, p->h2, p->h3_high, p->h3_low, p->h4, p->alpha_h1,
                           p->infiltration_capacity_compacted_soil, p->compacted_soil_area_fraction,
                           p->wet_root_distribution_parameter, p->cap_hmax, p->cap_n, p->maximum_leakage, p->w_soil,
                           p->cf_soil, p->brooks_corey_exponent, p->kv_factor, p->horizontal_to_vertical_ratio};
    for (const double* a : req)
        if (!a) return set_err(nullptr, WF_ERR_INVALID, "missing required input array");
    if (c->snow && (!p->degree_day_factor || !p->temperature_threshold_snowfall || !p->temperature_interval_snowfall ||
                    !p->temperature_threshold_melt || !p->water_holding_capacity))
        return set_err(nullptr, WF_ERR_INVALID, "snow parameters missing");
    if ((c->snow_gravitational_transport || c->glacier) && !c->snow)
        return set_err(nullptr, WF_ERR_INVALID,
                       "gravitational snow transport and glaciers need the snow model (snow__flag, sbm.jl:45-49)");
    if (c->snow_gravitational_transport && rs && rs->n > 0)
        return set_err(nullptr, WF_ERR_UNSUPPORTED, "gravitational snow transport with reservoirs is not supported");
    if (d->n_river > 0 && (!d->river_land_index || !d->river_downstream || !d->river_width || !d->river_length ||
                           !d->river_slope || !d->river_manning_n || !d->river_bankfull_depth))
        return set_err(nullptr, WF_ERR_INVALID, "river arrays missing");
    if (!d->land_downstream) return set_err(nullptr, WF_ERR_INVALID, "land_downstream missing");
    // reservoirs: outlets at river cells with a downstream river cell, at most one reservoir
    // draining into a river cell (ReservoirModel, reservoir.jl; surface_kinwave.jl:473-485)
    const int64_t nres = rs ? rs->n : 0;
    std::vector<int32_t> land_ds(d->land_downstream, d->land_downstream + d->n_land);
    std::vector<int32_t> res_of_river;
    if (nres < 0) return set_err(nullptr, WF_ERR_INVALID, "negative reservoir count");
    if (nres > 0) {
        if (!rs->river_index || !rs->outflow_curve_type || !rs->area || !rs->waterlevel)
            return set_err(nullptr, WF_ERR_INVALID, "reservoir arrays missing");
        res_of_river.assign(d->n_river, -1);
        std::vector<uint8_t> fed(d->n_river, 0);
        for (int64_t k = 0; k < nres; ++k) {
            const int32_t v = rs->river_index[k];
            if (v < 0 || v >= d->n_river) return set_err(nullptr, WF_ERR_INVALID, "reservoir river index out of range");
            if (res_of_river[v] >= 0) return set_err(nullptr, WF_ERR_INVALID, "two reservoirs at one river cell");
            const int32_t dv = d->river_downstream[v];
            if (dv < 0 || dv >= d->n_river)
                return set_err(nullptr, WF_ERR_INVALID, "a reservoir without a downstream river node is not supported");
            if (fed[dv]) return set_err(nullptr, WF_ERR_UNSUPPORTED, "two reservoirs drain into one river cell");
            const int32_t t = rs->outflow_curve_type[k];
            if (t != WF_RES_RATING_CURVE && t != WF_RES_FREE_WEIR && t != WF_RES_MODIFIED_PULS && t != WF_RES_SIMPLE)
                return set_err(nullptr, WF_ERR_UNSUPPORTED, "reservoir outflow type must be 1, 2, 3 or 4");
            if (!(rs->area[k] > 0.0)) return set_err(nullptr, WF_ERR_INVALID, "reservoir area must be positive");
            const bool simple_ok = rs->maximum_storage && rs->maximum_release && rs->demand &&
                                   rs->target_minimum_fraction && rs->target_full_fraction;
            const bool weir_ok = rs->threshold && rs->rating_curve_coefficient &&
                                 (t != WF_RES_FREE_WEIR || rs->rating_curve_exponent);
            if (t == WF_RES_SIMPLE ? !simple_ok : t != WF_RES_RATING_CURVE && !weir_ok)
                return set_err(nullptr, WF_ERR_INVALID, "reservoir parameter array missing for its outflow type");
            fed[dv] = 1;
            res_of_river[v] = (int32_t)k;
            const int32_t li = d->river_land_index[v];
            if (li < 0 || li >= d->n_land) return set_err(nullptr, WF_ERR_INVALID, "river_land_index out of range");
            land_ds[li] = -1;  // the outlet cell is a pit of the land upstream lists (domain.jl:95-121)
        }
    }
    ResTables rt;
    if (nres > 0) {
        const int rc = res_tables(rs, tb, d->n_river, d->river_downstream, rt);
        if (rc) return rc;
    }

    h = new WfHandle();
    h->cfg = *c;
    h->cfg.n_members = M;
    h->n = d->n_land;
    h->nr = d->n_river;
    h->M = M;
    h->N = N;
    h->device = device;
    auto fail = [&](int rc) {
        g_create_error = h->err;
        wf_destroy(h);
        return rc;
    };
    if (cudaSetDevice(device) != cudaSuccess) {
        set_err(h, WF_ERR_CUDA, "cudaSetDevice failed");
        return fail(WF_ERR_CUDA);
    }
    {
        cudaDeviceProp prop;
        if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) {
            set_err(h, WF_ERR_CUDA, "cudaGetDeviceProperties failed");
            return fail(WF_ERR_CUDA);
        }
        h->num_sms = prop.multiProcessorCount;
    }
    int rc;
#define CKR(expr)                  \
    do {                           \
        if ((rc = (expr))) return fail(rc); \
    } while (0)
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
        set_err(h, WF_ERR_CUDA, "cudaStreamCreate failed");
        return fail(WF_ERR_CUDA);
    }
    cudaEventCreate(&h->ev0);
    cudaEventCreate(&h->ev1);
    for (auto& e : h->kev) cudaEventCreate(&e);
    const int64_t n = h->n, nr = h->nr;
    // river indices
    for (int64_t r = 0; r < nr; ++r) {
        if (d->river_land_index[r] < 0 || d->river_land_index[r] >= n) {
            set_err(h, WF_ERR_INVALID, "river_land_index out of range");
            return fail(WF_ERR_INVALID);
        }
    }
    // sub-steps: fixed sizes, or adaptive (sizes chosen on the device every sub-step; one
    // sub-step per sweep launch)
    h->adaptive = c->adaptive_timestep != 0;
    if (h->adaptive) {
        if (!(c->subsurface_alpha > 0.0) || !(c->dt > 0.0)) {
            set_err(h, WF_ERR_INVALID, "adaptive time stepping needs a positive subsurface alpha coefficient and dt");
            return fail(WF_ERR_INVALID);
        }
        h->h_dts_land = h->h_dts_river = h->h_dts_ssf = std::vector<double>{c->dt};
    } else {
        h->h_dts_land = fixed_substeps(c->land_dt_fixed, c->dt);
        h->h_dts_river = fixed_substeps(c->river_dt_fixed, c->dt);
        h->h_dts_ssf = fixed_substeps(c->subsurface_dt_fixed, c->dt);
    }
    if (h->h_dts_land.empty() || h->h_dts_river.empty() || h->h_dts_ssf.empty() || h->h_dts_land.size() > 100000 ||
        h->h_dts_river.size() > 100000 || h->h_dts_ssf.size() > 100000) {
        set_err(h, WF_ERR_INVALID, "invalid fixed kinematic-wave time steps");
        return fail(WF_ERR_INVALID);
    }
    CKR(upload(h, &h->dts_land, h->h_dts_land));
    CKR(upload(h, &h->dts_river, h->h_dts_river));
    CKR(upload(h, &h->dts_ssf, h->h_dts_ssf));
    // wavefront schedules
    // sub-steps per sweep launch: the split form's slim wavefronts take at most 16 (a shared-
    // memory row per sub-step), the FP64 walker 32 (which bounds a launch to about a second on
    // the largest domains)
    const size_t cap = c->form == WF_FORM_SPLIT ? (size_t)wfv::MAX_GROUP : (size_t)32;
    const int cap_land = (int)std::min<size_t>(std::max(h->h_dts_land.size(), h->h_dts_ssf.size()), cap);
    // linked reservoirs: the river runs one sub-step per launch and keeps every upper-to-lower
    // path on one chain (wf_reservoir.cuh)
    const int cap_river = rt.linked ? 1 : (int)std::min<size_t>(h->h_dts_river.size(), cap);
    CKR(plan_graph(h, h->land, n, land_ds.data(), M, cap_land));
    CKR(plan_graph(h, h->river, nr, d->river_downstream ? d->river_downstream : nullptr, M, cap_river,
                   rt.linked ? rt.heavy_hint.data() : nullptr));
    for (int64_t k = 0; k < nres && rt.linked; ++k)
        if (rt.lower[k] >= 0 && h->river.plan.chain_of_node[rs->river_index[k]] !=
                                    h->river.plan.chain_of_node[rs->river_index[rt.lower[k]]]) {
            set_err(h, WF_ERR_INVALID, "linked reservoirs not on one routing chain");
            return fail(WF_ERR_INVALID);
        }
    const WfRoutingPlan& PL = h->land.plan;
    const WfRoutingPlan& PR = h->river.plan;

    // ---- derived parameters and cold state in external order (reference initialisation)
    const int per_member = c->per_member_soil != 0;
    std::vector<double> theta_fc(n), swc(n), rdclip(n), sy(n), ol_alpha(n);
    std::vector<int8_t> nlayers(n);
    std::vector<double> act((size_t)N * n), rootfrac((size_t)N * n);
    double cfg_thick[WF_MAX_LAYERS], cfg_cum[WF_MAX_LAYERS + 1];
    for (int k = 0; k < N - 1; ++k) cfg_thick[k] = c->soil_layer_thickness[k];
    cfg_thick[N - 1] = wfm::from_bits(0x7ff8000000000000ULL);
    cfg_cum[0] = 0.0;
    for (int k = 0; k < N; ++k) cfg_cum[k + 1] = cfg_cum[k] + cfg_thick[k];
    const double NaN = wfm::from_bits(0x7ff8000000000000ULL);
    for (int64_t i = 0; i < n; ++i) {
        const double dsoil = p->soil_thickness[i];
        double a[WF_MAX_LAYERS], cum[WF_MAX_LAYERS + 1];
        int nl = N;
        for (int k = 0; k < N; ++k) {  // set_layerthickness (utils.jl:390-404)
            double t = cfg_thick[k] * NaN;
            if (dsoil > cfg_cum[k + 1]) t = cfg_thick[k];
            else if (dsoil - cfg_cum[k] > 0.0) t = dsoil - cfg_cum[k];
            a[k] = t;
            if (t != t) nl -= 1;
        }
        cum[0] = 0.0;
        for (int k = 0; k < N; ++k) cum[k + 1] = cum[k] + a[k];
        nlayers[i] = (int8_t)nl;
        const double ts = p->theta_s[i], tr = p->theta_r[i], psi = p->air_entry_pressure[i];
        // field_capacity (soil_process.jl:137-159) at h = -1 m
        double tfc = 0.0, tot = 0.0;
        for (int k = 0; k < nl; ++k) {
            const double cexp = p->brooks_corey_exponent[i * N + k];
            double v = ts;
            if (-1.0 < psi) {
                const double lam = 2.0 / (cexp - 3.0);
                v = (ts - tr) * wfm::pow(psi / -1.0, lam) + tr;
            }
            tfc += v * a[k];
            tot += a[k];
        }
        theta_fc[i] = tfc / tot;
        swc[i] = dsoil * (ts - tr);
        rdclip[i] = wfm::jmin(dsoil * 0.99, p->rooting_depth[i]);
        const double rd0 = p->rooting_depth[i];
        for (int k = 0; k < N; ++k) {  // default root fraction (soil.jl:543-563)
            double rf = 0.0;
            if (rd0 > 0.0) {
                if ((rd0 - cum[k]) >= a[k]) rf = a[k] / rd0;
                else rf = wfm::jmax((rd0 - cum[k]) / rd0, 0.0);
            }
            rootfrac[(size_t)k * n + i] = rf;
            act[(size_t)k * n + i] = a[k];
        }
        sy[i] = wfm::jmax(ts - theta_fc[i], 0.02);
        ol_alpha[i] = wfm::pow(d->land_manning_n[i] / wfm::sqrt_(d->slope[i]), 0.6) *
                      wfm::pow(d->surface_flow_width[i], (2.0 / 3.0) * 0.6);
    }
    // per-member parameters and cold state
    std::vector<double> kv0((size_t)n * M), fsc((size_t)n * M), qmax((size_t)n * M), sat((size_t)n * M),
        zi((size_t)n * M), ssf_q((size_t)n * M), ssf_st((size_t)n * M), tsoil((size_t)n * M, 10.0 + 273.15);
    for (int m = 0; m < M; ++m) {
        for (int64_t i = 0; i < n; ++i) {
            const size_t j = (size_t)m * n + i;
            const int64_t ip = per_member ? (int64_t)j : i;
            kv0[j] = p->kv_0[ip];
            fsc[j] = p->f[ip];
            const double ts = p->theta_s[i], tr = p->theta_r[i], dsoil = p->soil_thickness[i];
            sat[j] = 0.85 * swc[i];
            zi[j] = wfm::jmax(0.0, dsoil - sat[j] / (ts - tr));
            const double kh0 = p->horizontal_to_vertical_ratio[i] * kv0[j];
            const double f = fsc[j], slope = d->slope[i];
            if (c->kv_profile == WF_KV_EXPONENTIAL) {
                qmax[j] = ((kh0 * slope) / f) * (1.0 - wfm::exp(-f * dsoil));
                ssf_q[j] = ((kh0 * slope) / f) * (wfm::exp(-f * zi[j]) - wfm::exp(-f * dsoil)) * d->flow_width[i];
            } else {
                const double zx = p->z_exp ? p->z_exp[i] : 0.0;
                const double qc = kh0 * wfm::exp(-f * zx) * slope * (dsoil - zx);
                qmax[j] = ((kh0 * slope) / f) * (1.0 - wfm::exp(-f * zx)) + qc;
                if (zi[j] < zx)
                    ssf_q[j] = (((kh0 * slope) / f) * (wfm::exp(-f * zi[j]) - wfm::exp(-f * zx)) + qc) * d->flow_width[i];
                else
                    ssf_q[j] = kh0 * wfm::exp(-f * zi[j]) * slope * (dsoil - zi[j]) * d->flow_width[i];
            }
            ssf_st[j] = sy[i] * (dsoil - zi[j]) * d->area[i];
        }
    }
    // ---- land static fields (slot layout)
    WfDevFields& F = h->F;
    F.split = c->form == WF_FORM_SPLIT;
    auto ext_vec = [&](const double* src, double dflt) {
        std::vector<double> v(n);
        for (int64_t i = 0; i < n; ++i) v[i] = src ? src[i] : dflt;
        return v;
    };
    struct LS {
        int idx;
        std::vector<double> v;
    };
    std::vector<LS> ls = {
        {AREA, ext_vec(d->area, 0)}, {FLOW_WIDTH, ext_vec(d->flow_width, 0)}, {FLOW_LENGTH, ext_vec(d->flow_length, 0)},
        {SFW, ext_vec(d->surface_flow_width, 0)}, {SLOPE, ext_vec(d->slope, 0)},
        {FRAC_TO_RIVER, ext_vec(d->flow_fraction_to_river, 0)}, {RIVER_FRACTION, ext_vec(d->river_fraction, 0)},
        {WATER_FRACTION, ext_vec(d->water_fraction, 0)}, {TOP, ext_vec(d->elevation, 0)}, {OL_ALPHA, ol_alpha},
        {SY, sy}, {GAP, ext_vec(p->canopy_gap_fraction, 0)}, {CMAX, ext_vec(p->maximum_canopy_storage, 0)},
        {KC, ext_vec(p->crop_coefficient, 0)}, {E_R, ext_vec(p->evaporation_to_precipitation_ratio, 0.1)},
        {DDF, ext_vec(p->degree_day_factor, 0)}, {TT, ext_vec(p->temperature_threshold_snowfall, 273.15)},
        {TTI, ext_vec(p->temperature_interval_snowfall, 1.0)}, {TTM, ext_vec(p->temperature_threshold_melt, 273.15)},
        {WHC, ext_vec(p->water_holding_capacity, 0.1)}, {THETA_S, ext_vec(p->theta_s, 0)},
        {THETA_R, ext_vec(p->theta_r, 0)}, {THETA_FC, theta_fc}, {SWC, swc},
        {SOIL_THICKNESS, ext_vec(p->soil_thickness, 0)}, {PSI_B, ext_vec(p->air_entry_pressure, 0)},
        {H1, ext_vec(p->h1, 0)}, {H2, ext_vec(p->h2, 0)}, {H3_HIGH, ext_vec(p->h3_high, 0)},
        {H3_LOW, ext_vec(p->h3_low, 0)}, {H4, ext_vec(p->h4, 0)}, {ALPHA_H1, ext_vec(p->alpha_h1, 0)},
        {CAP_COMP, ext_vec(p->infiltration_capacity_compacted_soil, 0)},
        {COMPACT_FRAC, ext_vec(p->compacted_soil_area_fraction, 0)},
        {ROOTDISTPAR, ext_vec(p->wet_root_distribution_parameter, 0)}, {CAP_HMAX, ext_vec(p->cap_hmax, 0)},
        {CAP_N, ext_vec(p->cap_n, 0)}, {MAX_LEAKAGE, ext_vec(p->maximum_leakage, 0)}, {W_SOIL, ext_vec(p->w_soil, 0)},
        {CF_SOIL, ext_vec(p->cf_soil, 0)}, {ROOTING_DEPTH, rdclip}, {Z_EXP, ext_vec(p->z_exp, 0)},
        {KH_RATIO, ext_vec(p->horizontal_to_vertical_ratio, 0)}};
    {
        // per-cell constants of the slim wavefronts (split form): 1/dx and the subsurface terms
        // of a single sub-step dt_s
        const double dts = h->h_dts_ssf[0];
        std::vector<double> inv_dx(n), dtdx(n), idwdx(n), dtsy(n), k2(n), inv_te(n), inv_area(n), inv_sfw(n), inv_dx_lo(n);
        for (int64_t i = 0; i < n; ++i) {
            const double dx = d->flow_length[i], dw = d->flow_width[i];
            inv_area[i] = 1.0 / d->area[i];
            inv_sfw[i] = d->surface_flow_width[i] > 0.0 ? 1.0 / d->surface_flow_width[i] : 0.0;
            inv_te[i] = 1.0 / (p->theta_s[i] - p->theta_r[i]);
            inv_dx[i] = 1.0 / dx;
            inv_dx_lo[i] = inv_dx[i] - (double)(float)inv_dx[i];
            dtdx[i] = dts / dx;
            idwdx[i] = 1.0 / (dw * dx);
            dtsy[i] = dts / sy[i];
            k2[i] = (dw * dx) * sy[i] / dts;
        }
        ls.push_back({INV_FLOW_LENGTH, inv_dx});
        ls.push_back({SSF_DTDX, dtdx});
        ls.push_back({SSF_IDWDX, idwdx});
        ls.push_back({SSF_DTSY, dtsy});
        ls.push_back({SSF_K2, k2});
        ls.push_back({INV_TE, inv_te});
        ls.push_back({INV_AREA, inv_area});
        ls.push_back({INV_SFW, inv_sfw});
        ls.push_back({INV_DX_LO, inv_dx_lo});
    }
    for (auto& x : ls) CKR(upload_slots(h, &F.L[x.idx], x.v, PL, M, n, false));
    for (int k = 0; k < N; ++k) {
        std::vector<double> va(act.begin() + (size_t)k * n, act.begin() + (size_t)(k + 1) * n);
        std::vector<double> vr(rootfrac.begin() + (size_t)k * n, rootfrac.begin() + (size_t)(k + 1) * n);
        std::vector<double> vc(n), vk(n);
        for (int64_t i = 0; i < n; ++i) {
            vc[i] = p->brooks_corey_exponent[i * N + k];
            vk[i] = p->kv_factor[i * N + k];
        }
        CKR(upload_slots(h, &F.LY[LY_ACT_THICK][k], va, PL, M, n, false));
        CKR(upload_slots(h, &F.LY[LY_ROOTFRAC][k], vr, PL, M, n, false));
        CKR(upload_slots(h, &F.LY[LY_C][k], vc, PL, M, n, false));
        CKR(upload_slots(h, &F.LY[LY_KVFRAC][k], vk, PL, M, n, false));
        std::vector<double> vcum(n);
        for (int64_t i = 0; i < n; ++i) {
            double c = 0.0;
            for (int j = 0; j <= k; ++j) c += act[(size_t)j * n + i];
            vcum[i] = c;
        }
        CKR(upload_slots(h, &F.LY[LY_CUM][k], vcum, PL, M, n, false));
        std::vector<double> zeros((size_t)n * M, 0.0);
        if (F.split) CKR(upload_slots_ff(h, &F.LYf[LY_USLD][k], &F.LYl[k], zeros, PL, M, n, true));
        else CKR(upload_slots(h, &F.LY[LY_USLD][k], zeros, PL, M, n, true));
    }
    {
        std::vector<int8_t> nl_slots(PL.n_slots, 0);
        for (int64_t s = 0; s < PL.n_slots; ++s)
            if (PL.node_of_slot[s] >= 0) nl_slots[s] = nlayers[PL.node_of_slot[s]];
        int8_t* dnl;
        CKR(upload(h, &dnl, nl_slots));
        F.nlayers = dnl;
    }
    // ---- land member fields
    std::vector<double> zeros_m((size_t)n * M, 0.0);
    for (int f = 0; f < M_COUNT; ++f) {
        if (!F.split && wf_split_only_member(f)) continue;
        if (F.split && !wf_split_ff_member(f) && !wf_split_fp64_member(f)) continue;  // FP32 arrays only (below)
        const std::vector<double>* src = &zeros_m;
        switch (f) {
            case KV0: src = &kv0; break;
            case FSCALE: src = &fsc; break;
            case Q_MAX: src = &qmax; break;
            case TSOIL: src = &tsoil; break;
            case SAT: src = &sat; break;
            case TSWS: src = &sat; break;
            case ZI: src = &zi; break;
            case SSF_ZI: src = &zi; break;
            case SSF_Q: src = &ssf_q; break;
            case SSF_STORAGE: src = &ssf_st; break;
            default: break;
        }
        if (F.split && wf_split_ff_member(f)) CKR(upload_slots_ff(h, &F.Mh[f], &F.Ml[f], *src, PL, M, n, true));
        else CKR(upload_slots(h, &F.Mf[f], *src, PL, M, n, true));
    }
    // ---- gravitational snow transport and glacier (FP64 in both forms)
    F.snow_transport = c->snow_gravitational_transport != 0;
    F.glacier = c->glacier != 0;
    F.g_max_rate = 8.0 * ((1.0 / 86400.0) * 1e-3);  // to_SI(8.0, MM_PER_DAY) (glacier.jl:90)
    if (F.glacier) {  // defaults: standard_name_sbm.jl:70-108, in SI
        CKR(upload_slots(h, &F.G[G_FRAC], ext_vec(p->glacier_fraction, 0.0), PL, M, n, false));
        CKR(upload_slots(h, &F.G[G_TTM], ext_vec(p->glacier_temperature_threshold_melt, 0.0 + 273.15), PL, M, n,
                         false));
        CKR(upload_slots(h, &F.G[G_DDF], ext_vec(p->glacier_degree_day_factor, 3.0 * ((1.0 / 86400.0) * 1e-3)), PL,
                         M, n, false));
        CKR(upload_slots(h, &F.G[G_SIFRAC], ext_vec(p->glacier_snow_to_ice_fraction, 0.001 * (1.0 / 86400.0)), PL,
                         M, n, false));
    }
    if (F.glacier || F.snow_transport) {
        for (int f = 0; f < GM_COUNT; ++f) {
            std::vector<double> v((size_t)n * M, 0.0);
            if (f == GM_STORE && F.glacier)
                for (int m = 0; m < M; ++m)
                    for (int64_t i = 0; i < n; ++i)
                        v[(size_t)m * n + i] = p->glacier_initial_store ? p->glacier_initial_store[i] : 5.5;
            CKR(upload_slots(h, &F.GM[f], v, PL, M, n, true));
        }
    }
    if (F.snow_transport) {
        // each slot's upstream entries in the order of the land graph's topological sort
        const std::vector<int64_t> order = topo_order_dfs(n, d->land_downstream);
        if ((int64_t)order.size() != n) {
            set_err(h, WF_ERR_CYCLE, "the land drainage graph has a cycle (routing/utils.jl:26-31)");
            return fail(WF_ERR_CYCLE);
        }
        std::vector<int64_t> pos((size_t)n);
        for (int64_t k = 0; k < n; ++k) pos[order[k]] = k;
        std::vector<int32_t> su(std::max<size_t>(PL.up_slot.size(), 1), 0);
        for (int64_t sl = 0; sl < PL.n_slots; ++sl) {
            const int32_t o0 = PL.up_ptr[sl], o1 = PL.up_ptr[sl + 1];
            for (int32_t o = o0; o < o1; ++o) su[o] = o;
            std::sort(su.begin() + o0, su.begin() + o1, [&](int32_t a, int32_t b) {
                return pos[PL.node_of_slot[PL.up_slot[a]]] < pos[PL.node_of_slot[PL.up_slot[b]]];
            });
        }
        CKR(upload(h, &h->land.snow_up, su));
    }
    // ---- river fields
    std::vector<double> r_width(nr), r_length(nr), r_alpha(nr), r_ext(nr), r_area(nr), r_inv_len(nr), r_inv_w(nr), r_inv_len_lo(nr);
    for (int64_t r = 0; r < nr; ++r) {
        r_width[r] = d->river_width[r];
        r_length[r] = d->river_length[r];
        r_inv_len[r] = 1.0 / d->river_length[r];
        r_inv_w[r] = 1.0 / d->river_width[r];
        r_inv_len_lo[r] = r_inv_len[r] - (double)(float)r_inv_len[r];
        r_ext[r] = d->river_external_inflow ? d->river_external_inflow[r] : 0.0;
        r_area[r] = d->area[d->river_land_index[r]];
        h->river_land.push_back(d->river_land_index[r]);
        const double wp = d->river_width[r] + d->river_bankfull_depth[r];
        r_alpha[r] = wfm::pow(d->river_manning_n[r] / wfm::sqrt_(d->river_slope[r]), 0.6) *
                     wfm::pow(wp, (2.0 / 3.0) * 0.6);
    }
    CKR(upload_slots(h, &F.R[R_WIDTH], r_width, PR, M, nr, false));
    CKR(upload_slots(h, &F.R[R_LENGTH], r_length, PR, M, nr, false));
    CKR(upload_slots(h, &F.R[R_ALPHA], r_alpha, PR, M, nr, false));
    CKR(upload_slots(h, &F.R[R_EXT_INFLOW], r_ext, PR, M, nr, false));
    CKR(upload_slots(h, &F.R[R_AREA], r_area, PR, M, nr, false));
    CKR(upload_slots(h, &F.R[R_INV_LENGTH], r_inv_len, PR, M, nr, false));
    CKR(upload_slots(h, &F.R[R_INV_WIDTH], r_inv_w, PR, M, nr, false));
    CKR(upload_slots(h, &F.R[R_INV_LEN_LO], r_inv_len_lo, PR, M, nr, false));
    std::vector<double> zeros_r((size_t)std::max<int64_t>(nr, 1) * M, 0.0);
    for (int f = 0; f < RM_COUNT; ++f) {
        if (wf_split_only_river_member(f)) {
            if (F.split) CKR(upload_slots_f32(h, &F.RMh[f], zeros_r, PR, M, nr, true));
            continue;
        }
        if (F.split) CKR(upload_slots_ff(h, &F.RMh[f], &F.RMl[f], zeros_r, PR, M, nr, true));
        else CKR(upload_slots(h, &F.RM[f], zeros_r, PR, M, nr, true));
    }
    // ---- upstream weights of the wavefront gathers: land discharge splits into the part that
    // goes to the river (flow_fraction_to_river) and the rest that flows downstream
    for (int g = 0; g < 2; ++g) {
        DevGraphAlloc& G = g == 0 ? h->land : h->river;
        const WfRoutingPlan& P = G.plan;
        const size_t ne = P.up_slot.size();
        std::vector<double> w(std::max<size_t>(ne, 1), 1.0), fr(std::max<size_t>(ne, 1), 0.0);
        for (size_t o = 0; o < ne; ++o) {
            if (g != 0) continue;
            const int64_t node = P.node_of_slot[P.up_slot[o]];
            const double f = d->flow_fraction_to_river ? d->flow_fraction_to_river[node] : 0.0;
            w[o] = 1.0 - f;
            fr[o] = f;
        }
        CKR(upload(h, &G.up_w, w));
        CKR(upload(h, &G.up_fr, fr));
        std::vector<float> wf(w.begin(), w.end()), frf(fr.begin(), fr.end());
        CKR(upload(h, &G.up_wf, wf));
        CKR(upload(h, &G.up_frf, frf));
        // per-slot records of the slim wavefronts: the first two light children and the weights
        std::vector<int4> rec(std::max<int64_t>(P.n_slots, 1), int4{-1, -1, 0, 0});
        std::vector<float> whv(rec.size(), 0.0f);
        std::vector<uint8_t> nlt(rec.size(), 0);
        std::vector<float4> frec(rec.size(), float4{0.0f, 0.0f, 0.0f, 0.0f});
        for (int64_t sl = 0; sl < P.n_slots; ++sl) {
            int lights = 0;
            for (int32_t o = P.up_ptr[sl]; o < P.up_ptr[sl + 1]; ++o) {
                if (P.up_chain[o] < 0) {
                    whv[sl] = wf[o];
                    frec[sl].x = frf[o];
                    continue;
                }
                float wo = wf[o];
                int32_t bits;
                std::memcpy(&bits, &wo, sizeof(bits));
                if (lights == 0) {
                    rec[sl].x = P.up_chain[o];
                    rec[sl].z = bits;
                    frec[sl].y = frf[o];
                } else if (lights == 1) {
                    rec[sl].y = P.up_chain[o];
                    rec[sl].w = bits;
                    frec[sl].z = frf[o];
                }
                ++lights;
            }
            nlt[sl] = (uint8_t)std::min(lights, 255);
        }
        CKR(upload(h, &G.up_rec, rec));
        CKR(upload(h, &G.up_whv, whv));
        CKR(upload(h, &G.up_nlt, nlt));
        CKR(upload(h, &G.up_frec, frec));
    }
    // ---- split form: FP32 copies of the static fields and FP32 member fields
    if (F.split) {
        for (auto& x : ls) {
            float* dummy = nullptr;
            CKR(upload_slots_ff(h, &dummy, &F.Ll[x.idx], x.v, PL, M, n, false));
            F.Lf[x.idx] = dummy;
        }
        for (int k = 0; k < N; ++k) {
            std::vector<double> va(act.begin() + (size_t)k * n, act.begin() + (size_t)(k + 1) * n);
            std::vector<double> vr(rootfrac.begin() + (size_t)k * n, rootfrac.begin() + (size_t)(k + 1) * n);
            std::vector<double> vc(n), vk(n);
            for (int64_t i = 0; i < n; ++i) {
                vc[i] = p->brooks_corey_exponent[i * N + k];
                vk[i] = p->kv_factor[i * N + k];
            }
            CKR(upload_slots_ff(h, &F.LYf[LY_ACT_THICK][k], &F.LYsl[LY_ACT_THICK][k], va, PL, M, n, false));
            CKR(upload_slots_f32(h, &F.LYf[LY_ROOTFRAC][k], vr, PL, M, n, false));
            CKR(upload_slots_f32(h, &F.LYf[LY_C][k], vc, PL, M, n, false));
            CKR(upload_slots_f32(h, &F.LYf[LY_KVFRAC][k], vk, PL, M, n, false));
            std::vector<double> vcum(n);
            for (int64_t i = 0; i < n; ++i) {
                double cc = 0.0;
                for (int j = 0; j <= k; ++j) cc += act[(size_t)j * n + i];
                vcum[i] = cc;
            }
            CKR(upload_slots_ff(h, &F.LYf[LY_CUM][k], &F.LYsl[LY_CUM][k], vcum, PL, M, n, false));
        }
        for (int f = 0; f < M_COUNT; ++f) {
            if (!wf_split_f32_member(f) && !wf_split_f32_only(f)) continue;
            const std::vector<double>* src = &zeros_m;
            if (f == KV0) src = &kv0;
            if (f == FSCALE) src = &fsc;
            if (f == Q_MAX) src = &qmax;
            if (f == TSOIL) src = &tsoil;
            CKR(upload_slots_f32(h, &F.Mh[f], *src, PL, M, n, true));
        }
        CKR(upload_slots_ff(h, &F.Rf[R_WIDTH], &F.Rl[R_WIDTH], r_width, PR, M, nr, false));
        CKR(upload_slots_ff(h, &F.Rf[R_LENGTH], &F.Rl[R_LENGTH], r_length, PR, M, nr, false));
        CKR(upload_slots_ff(h, &F.Rf[R_ALPHA], &F.Rl[R_ALPHA], r_alpha, PR, M, nr, false));
        CKR(upload_slots_ff(h, &F.Rf[R_EXT_INFLOW], &F.Rl[R_EXT_INFLOW], r_ext, PR, M, nr, false));
        CKR(upload_slots_ff(h, &F.Rf[R_AREA], &F.Rl[R_AREA], r_area, PR, M, nr, false));
        CKR(upload_slots_ff(h, &F.Rf[R_INV_LENGTH], &F.Rl[R_INV_LENGTH], r_inv_len, PR, M, nr, false));
        CKR(upload_slots_ff(h, &F.Rf[R_INV_LEN_LO], &F.Rl[R_INV_LEN_LO], r_inv_len_lo, PR, M, nr, false));
        CKR(upload_slots_ff(h, &F.Rf[R_INV_WIDTH], &F.Rl[R_INV_WIDTH], r_inv_w, PR, M, nr, false));
    }
    // ---- maps
    {
        std::vector<int64_t> land_river_slot(PL.n_slots, -1), river_land_slot(std::max<int64_t>(PR.n_slots, 1), -1);
        for (int64_t r = 0; r < nr; ++r) {
            const int64_t ls_ = PL.slot_of_node[d->river_land_index[r]];
            const int64_t rs_ = PR.slot_of_node[r];
            land_river_slot[ls_] = rs_;
            river_land_slot[rs_] = ls_;
        }
        int64_t *a, *b;
        CKR(upload(h, &a, land_river_slot));
        CKR(upload(h, &b, river_land_slot));
        F.land_river_slot = a;
        F.river_land_slot = b;
        F.land_node_of_slot = h->land.node_of_slot;
        F.river_node_of_slot = h->river.node_of_slot;
        for (int64_t r = 0; r < nr; ++r)
            if (d->river_downstream[r] < 0) h->outlet_slots.push_back(PR.slot_of_node[r]);
        if (!h->outlet_slots.empty()) CKR(upload(h, &h->d_outlet_slots, h->outlet_slots));
        CKR(upload(h, &h->d_land_slot_of_node, PL.slot_of_node));
    }
    // ---- reservoirs: parameters per reservoir, state per reservoir and member (r * M + m)
    h->nres = nres;
    F.n_res = nres;
    if (nres > 0) {
        std::vector<int32_t> rtype(nres), rofs(PR.n_slots, -1);
        std::vector<int64_t> rls(nres);
        for (int64_t k = 0; k < nres; ++k) {
            const int32_t v = rs->river_index[k];
            rtype[k] = rs->outflow_curve_type[k];
            rofs[PR.slot_of_node[v]] = (int32_t)k;
            rls[k] = PL.slot_of_node[d->river_land_index[v]];
        }
        int32_t *a32, *b32;
        int64_t* c64;
        CKR(upload(h, &a32, rtype));
        CKR(upload(h, &b32, rofs));
        CKR(upload(h, &c64, rls));
        F.res_type = a32;
        F.res_of_rslot = b32;
        F.res_land_slot = c64;
        const double* src[RP_COUNT] = {rs->area, rs->maximum_storage, rs->threshold, rs->rating_curve_coefficient,
                                       rs->rating_curve_exponent, rs->maximum_release, rs->demand,
                                       rs->target_minimum_fraction, rs->target_full_fraction};
        for (int f = 0; f < RP_COUNT; ++f) {
            std::vector<double> v(nres, NaN);
            if (src[f]) v.assign(src[f], src[f] + nres);
            if (f == RP_MAXSTOR)  // a rating curve's maximum storage follows from its tables
                for (int64_t k = 0; k < nres; ++k)
                    if (rs->outflow_curve_type[k] == WF_RES_RATING_CURVE) v[k] = rt.maximum_storage[k];
            CKR(upload(h, &F.RP[f], v));
        }
        for (int f = 0; f < RS_COUNT; ++f) {
            std::vector<double> v((size_t)nres * M, 0.0);
            for (int64_t k = 0; k < nres; ++k)
                for (int m = 0; m < M; ++m) {
                    double x = 0.0;
                    if (f == RS_WATERLEVEL) x = rs->waterlevel[k];
                    if (f == RS_STORAGE) x = rt.initial_storage[k];  // initialize_storage (reservoir.jl:343-360)
                    if (f == RS_OUTFLOW || f == RS_OBS) x = NaN;
                    v[(size_t)k * M + m] = x;
                }
            CKR(upload(h, &F.RS[f], v));
        }
        if (rt.any) {
            int32_t *prof, *lower, *day;
            int64_t* meta;
            double* tab;
            CKR(upload(h, &prof, rt.profile));
            CKR(upload(h, &lower, rt.lower));
            CKR(upload(h, &meta, rt.meta));
            CKR(upload(h, &tab, rt.tab.empty() ? std::vector<double>{0.0} : rt.tab));
            CKR(upload(h, &day, std::vector<int32_t>{1}));
            F.res_profile = prof;
            F.res_lower = lower;
            F.res_tab_meta = meta;
            F.res_tab = tab;
            F.res_hq_day = day;
        }
    }
    F.land_slots = PL.n_slots;
    F.river_slots = PR.n_slots;
    F.N = N;
    F.M = M;
    F.snow = c->snow;
    F.infilt_reduction = c->soil_infiltration_reduction;
    F.gash = c->dt >= 23.0 * 3600.0;
    F.kv_profile = c->kv_profile;
    F.mass_balance = c->water_mass_balance;
    F.dt = c->dt;
    F.inv_dt = 1.0 / c->dt;
    // split form: the vertical kernel prepares the terms of a single subsurface sub-step; with
    // adaptive sub-steps that sub-step is the whole model step (used when every member's first
    // Courant sub-step reaches the end of the step, the usual case)
    F.ssf_single = F.split && h->h_dts_ssf.size() == 1;
    if (F.split && PR.n_slots > 0) CKR(dalloc(h, &F.rv_lat_pub, (size_t)PR.n_slots * M));
    F.dt_ssf = h->h_dts_ssf[0];
    F.inv_dt_ssf = 1.0 / h->h_dts_ssf[0];
    F.inv_dt_hi = (float)F.inv_dt;
    F.inv_dt_lo = (float)(F.inv_dt - (double)F.inv_dt_hi);
    F.inv_dts_hi = (float)F.inv_dt_ssf;
    F.inv_dts_lo = (float)(F.inv_dt_ssf - (double)F.inv_dts_hi);
    F.r_s = (float)(F.dt_ssf / F.dt);
    CKR(dalloc(h, &h->status, 1));
    CK(cudaMemset(h->status, 0, sizeof(int32_t)));
    F.status = h->status;
    CKR(dalloc(h, &h->staging, (size_t)std::max<int64_t>(std::max(n, nr), 1) * M * 3));
    h->tuning.use_graph = 1;
    h->u_dirty = F.split != 0;  // double-FP32 routing state from the FP64 discharges on the first step
    h->metrics.n_chains_land = (int32_t)PL.n_chains;
    h->metrics.n_chains_river = (int32_t)PR.n_chains;
    h->metrics.max_chain_land = PL.max_len;
    h->metrics.max_chain_river = PR.max_len;
    h->metrics.padding_slots_land = (int32_t)(PL.n_slots - n);
    if (h->adaptive) CKR(alloc_adaptive(h));
    CK(cudaDeviceSynchronize());
    {
        // the static scratch of wf_step_static is looked up (and its module loaded) now, at set-up,
        // so that its first call allocates nothing even under lazy module loading
        unsigned char* scratch = nullptr;
        CKR(static_scratch(h, &scratch));
    }
#undef CKR
    *out = h;
    return WF_OK;
}

void wf_destroy(WfHandle* h) {
    if (!h) return;
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
    if (h->graph) cudaGraphDestroy(h->graph);
    for (void* p : h->allocs) cudaFree(p);
    if (h->host_pinned) cudaFreeHost(h->host_pinned);
    if (h->h_more) cudaFreeHost(h->h_more);
    if (h->copy_stream) {
        cudaStreamSynchronize(h->copy_stream);
        cudaStreamDestroy(h->copy_stream);
    }
    if (h->ev_fcopied) cudaEventDestroy(h->ev_fcopied);
    if (h->ev_fconsumed) cudaEventDestroy(h->ev_fconsumed);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    for (auto& e : h->kev)
        if (e) cudaEventDestroy(e);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

}  // extern "C"

namespace {

// Forcing arrays staged on the device in external order (stg[k], k = P, PET, T) into the slot
// order (and FP32 for the split form), on the handle's stream.
int enqueue_forcing_gathers(WfHandle* h, double* const stg_of[3], int64_t count) {
    const int64_t full = h->n * h->M;
    const int dst[3] = {PRECIP, POTEVAP, TEMP};
    const int block = 256;
    for (int k = 0; k < 3; ++k) {
        double* stg = stg_of[k];
        const int g = grid_of(h->F.land_slots * h->M, block);
        if (count == full) {
            launch_forcing_full<double>(h, stg, h->F.split ? h->F.Mh[dst[k]] : nullptr,
                                        h->F.split ? nullptr : h->F.Mf[dst[k]]);
        } else if (h->F.split) {
            broadcast_member_f32_kernel<<<g, block, 0, h->stream>>>(stg, h->F.Mh[dst[k]], h->F.land_node_of_slot,
                                                                    h->F.land_slots, h->M);
        } else {
            broadcast_member_kernel<<<g, block, 0, h->stream>>>(stg, h->F.Mf[dst[k]], h->F.land_node_of_slot,
                                                                h->F.land_slots, h->M, nullptr);
        }
        CK(cudaGetLastError());
    }
    return WF_OK;
}

// The gathers of FP32 forcing staged at stg[k] (count values each).
int enqueue_forcing_gathers_f32(WfHandle* h, float* const stg[3], const int64_t count[3]) {
    const int dst[3] = {PRECIP, POTEVAP, TEMP};
    const int g = grid_of(h->F.land_slots * h->M, 256);
    for (int k = 0; k < 3; ++k) {
        float* d32 = h->F.split ? h->F.Mh[dst[k]] : nullptr;
        double* d64 = h->F.split ? nullptr : h->F.Mf[dst[k]];
        if (count[k] != h->n * h->M)
            gather_from_f32_kernel<<<g, 256, 0, h->stream>>>(stg[k], d32, d64, h->F.land_node_of_slot,
                                                             h->F.land_slots, h->M, h->n, 1);
        else
            launch_forcing_full<float>(h, stg[k], d32, d64);
        CK(cudaGetLastError());
    }
    return WF_OK;
}

}  // namespace

extern "C" {

int32_t wf_set_forcing_counts_f32(WfHandle* h, const float* P, int64_t count_p, const float* PET, int64_t count_pet,
                                  const float* T, int64_t count_t) {
    if (!h || !P || !PET || !T) return set_err(h, WF_ERR_INVALID, "null forcing");
    const int64_t full = h->n * h->M;
    const float* src[3] = {P, PET, T};
    const int64_t cnt[3] = {count_p, count_pet, count_t};
    float* stg[3];
    for (int k = 0; k < 3; ++k) {
        if (cnt[k] != full && cnt[k] != h->n)
            return set_err(h, WF_ERR_INVALID, "forcing count must be n_land*n_members or n_land");
        stg[k] = reinterpret_cast<float*>(h->staging + (size_t)k * std::max(h->n, h->nr) * h->M);
        CK(cudaMemcpyAsync(stg[k], src[k], cnt[k] * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    }
    return enqueue_forcing_gathers_f32(h, stg, cnt);
}

int32_t wf_set_forcing_counts_async_f32(WfHandle* h, const float* P, int64_t count_p, const float* PET,
                                        int64_t count_pet, const float* T, int64_t count_t) {
    if (!h || !P || !PET || !T) return set_err(h, WF_ERR_INVALID, "null forcing");
    const int64_t full = h->n * h->M;
    const int64_t cnt[3] = {count_p, count_pet, count_t};
    for (int k = 0; k < 3; ++k)
        if (cnt[k] != full && cnt[k] != h->n)
            return set_err(h, WF_ERR_INVALID, "forcing count must be n_land*n_members or n_land");
    if (!h->copy_stream) {  // first call: copy stream, events and a staging buffer of its own
        CK(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&h->ev_fcopied, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&h->ev_fconsumed, cudaEventDisableTiming));
        int rc = dalloc(h, &h->fstage, (size_t)3 * full);
        if (rc) return rc;
    }
    CK(cudaStreamWaitEvent(h->copy_stream, h->ev_fconsumed, 0));
    const float* src[3] = {P, PET, T};
    float* stg[3];
    for (int k = 0; k < 3; ++k) {
        stg[k] = reinterpret_cast<float*>(h->fstage + (size_t)k * full);
        CK(cudaMemcpyAsync(stg[k], src[k], cnt[k] * sizeof(float), cudaMemcpyHostToDevice, h->copy_stream));
    }
    CK(cudaEventRecord(h->ev_fcopied, h->copy_stream));
    CK(cudaStreamWaitEvent(h->stream, h->ev_fcopied, 0));
    int rc = enqueue_forcing_gathers_f32(h, stg, cnt);
    if (rc) return rc;
    CK(cudaEventRecord(h->ev_fconsumed, h->stream));
    return WF_OK;
}

int32_t wf_set_forcing_f32(WfHandle* h, const float* P, const float* PET, const float* T, int64_t count) {
    return wf_set_forcing_counts_f32(h, P, count, PET, count, T, count);
}

int32_t wf_set_forcing_async_f32(WfHandle* h, const float* P, const float* PET, const float* T, int64_t count) {
    return wf_set_forcing_counts_async_f32(h, P, count, PET, count, T, count);
}

int32_t wf_set_forcing(WfHandle* h, const double* P, const double* PET, const double* T, int64_t count) {
    if (!h || !P || !PET || !T) return set_err(h, WF_ERR_INVALID, "null forcing");
    const int64_t full = h->n * h->M;
    if (count != full && count != h->n) return set_err(h, WF_ERR_INVALID, "forcing count must be n_land*n_members or n_land");
    const double* src[3] = {P, PET, T};
    double* stg[3];
    for (int k = 0; k < 3; ++k) {
        stg[k] = h->staging + (size_t)k * std::max(h->n, h->nr) * h->M;
        CK(cudaMemcpyAsync(stg[k], src[k], count * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    }
    return enqueue_forcing_gathers(h, stg, count);
}

int32_t wf_set_forcing_async(WfHandle* h, const double* P, const double* PET, const double* T, int64_t count) {
    if (!h || !P || !PET || !T) return set_err(h, WF_ERR_INVALID, "null forcing");
    const int64_t full = h->n * h->M;
    if (count != full && count != h->n) return set_err(h, WF_ERR_INVALID, "forcing count must be n_land*n_members or n_land");
    if (!h->copy_stream) {  // first call: copy stream, events and a staging buffer of its own
        CK(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&h->ev_fcopied, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&h->ev_fconsumed, cudaEventDisableTiming));
        int rc = dalloc(h, &h->fstage, (size_t)3 * full);
        if (rc) return rc;
    }
    // the staging buffer is free once the gathers of the previous call ran
    CK(cudaStreamWaitEvent(h->copy_stream, h->ev_fconsumed, 0));
    const double* src[3] = {P, PET, T};
    double* stg[3];
    for (int k = 0; k < 3; ++k) {
        stg[k] = h->fstage + (size_t)k * full;
        CK(cudaMemcpyAsync(stg[k], src[k], count * sizeof(double), cudaMemcpyHostToDevice, h->copy_stream));
    }
    CK(cudaEventRecord(h->ev_fcopied, h->copy_stream));
    CK(cudaStreamWaitEvent(h->stream, h->ev_fcopied, 0));
    int rc = enqueue_forcing_gathers(h, stg, count);
    if (rc) return rc;
    CK(cudaEventRecord(h->ev_fconsumed, h->stream));
    return WF_OK;
}

int32_t wf_set_forcing_device_slots(WfHandle* h, const void* P, const void* PET, const void* T) {
    if (!h || !P || !PET || !T) return set_err(h, WF_ERR_INVALID, "null forcing");
    const int64_t cnt = h->F.land_slots * h->M;
    if (h->F.split) {
        const int g = grid_of(cnt, 256);
        to_f32_kernel<<<g, 256, 0, h->stream>>>((const double*)P, h->F.Mh[PRECIP], cnt);
        to_f32_kernel<<<g, 256, 0, h->stream>>>((const double*)PET, h->F.Mh[POTEVAP], cnt);
        to_f32_kernel<<<g, 256, 0, h->stream>>>((const double*)T, h->F.Mh[TEMP], cnt);
        CK(cudaGetLastError());
        return WF_OK;
    }
    const size_t bytes = (size_t)cnt * sizeof(double);
    CK(cudaMemcpyAsync(h->F.Mf[PRECIP], P, bytes, cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaMemcpyAsync(h->F.Mf[POTEVAP], PET, bytes, cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaMemcpyAsync(h->F.Mf[TEMP], T, bytes, cudaMemcpyDeviceToDevice, h->stream));
    return WF_OK;
}

int32_t wf_step_async(WfHandle* h) {
    if (!h) return WF_ERR_INVALID;
    return run_step(h);
}

int32_t wf_synchronize(WfHandle* h) {
    if (!h) return WF_ERR_INVALID;
    CK(cudaStreamSynchronize(h->stream));
    int32_t st = 0;
    CK(cudaMemcpy(&st, h->status, sizeof(int32_t), cudaMemcpyDeviceToHost));
    h->metrics.device_status = st;
    if (st & WF_DEV_SPIN_TIMEOUT) {
        cudaMemset(h->status, 0, sizeof(int32_t));
        return set_err(h, WF_ERR_SPIN, "a routing wavefront wait ran out of its time budget");
    }
    return WF_OK;
}

int32_t wf_step(WfHandle* h) {
    if (!h) return WF_ERR_INVALID;
    CK(cudaEventRecord(h->ev0, h->stream));
    int rc = run_step(h);
    if (rc) return rc;
    CK(cudaEventRecord(h->ev1, h->stream));
    rc = wf_synchronize(h);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    h->metrics.step_ms_total += ms;
    return rc;
}

int32_t wf_get_field(WfHandle* h, int32_t field, int32_t layer, double* dst, int64_t offset, int64_t count) {
    if (!h || !dst) return set_err(h, WF_ERR_INVALID, "null argument");
    if (field >= WF_F_RESERVOIR_STORAGE) return reservoir_io(h, field, dst, nullptr, offset, count);
    FieldRef r = field_ref(h, field, layer);
    if (!r.p && !r.p32 && !r.derived_vwc) return set_err(h, WF_ERR_INVALID, "unknown field or layer");
    const int64_t n_ext = r.river ? h->nr : h->n;
    const int64_t total = n_ext * h->M;
    if (offset < 0 || count < 0 || offset + count > total) return set_err(h, WF_ERR_INVALID, "range out of bounds");
    WfLaunchCfg lc = launch_cfg(h);
    double* src = r.p;
    double* tmp = h->staging + (size_t)std::max(h->n, h->nr) * h->M;  // second staging third
    if (r.derived_vwc) {
        CK(h->F.split ? wf_split_vwc(h->F, layer, tmp, lc) : wf_fp64_vwc(h->F, layer, tmp, lc));
        src = tmp;
    }
    const int block = 256;
    const int64_t slots = r.river ? h->F.river_slots : h->F.land_slots;
    const int64_t* nos = r.river ? h->F.river_node_of_slot : h->F.land_node_of_slot;
    if (r.p32)
        scatter_f32_kernel<<<grid_of(slots * h->M, block), block, 0, h->stream>>>(r.p32, h->staging, nos, slots, h->M,
                                                                                  n_ext, r.p32lo);
    else
        scatter_kernel<<<grid_of(slots * h->M, block), block, 0, h->stream>>>(src, h->staging, nos, slots, h->M, n_ext);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(dst, h->staging + offset, count * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return WF_OK;
}

int32_t wf_set_field(WfHandle* h, int32_t field, int32_t layer, const double* src, int64_t offset, int64_t count) {
    if (!h || !src) return set_err(h, WF_ERR_INVALID, "null argument");
    if (field >= WF_F_RESERVOIR_STORAGE) return reservoir_io(h, field, nullptr, src, offset, count);
    FieldRef r = field_ref(h, field, layer);
    if ((!r.p && !r.p32) || !r.settable) return set_err(h, WF_ERR_INVALID, "field is not settable");
    const int64_t n_ext = r.river ? h->nr : h->n;
    const int64_t total = n_ext * h->M;
    if (offset < 0 || count < 0 || offset + count > total) return set_err(h, WF_ERR_INVALID, "range out of bounds");
    const int block = 256;
    const int64_t slots = r.river ? h->F.river_slots : h->F.land_slots;
    const int64_t* nos = r.river ? h->F.river_node_of_slot : h->F.land_node_of_slot;
    if (r.p32)
        scatter_f32_kernel<<<grid_of(slots * h->M, block), block, 0, h->stream>>>(r.p32, h->staging, nos, slots, h->M,
                                                                                  n_ext, r.p32lo);
    else
        scatter_kernel<<<grid_of(slots * h->M, block), block, 0, h->stream>>>(r.p, h->staging, nos, slots, h->M,
                                                                              n_ext);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(h->staging + offset, src, count * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    if (r.p32)
        gather_f32_kernel<<<grid_of(slots * h->M, block), block, 0, h->stream>>>(h->staging, r.p32, nos, slots, h->M,
                                                                                 n_ext, r.p32lo);
    else
        gather_kernel<<<grid_of(slots * h->M, block), block, 0, h->stream>>>(h->staging, r.p, nos, slots, h->M,
                                                                             n_ext);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(h->stream));
    if (field == WF_F_LAND_Q || field == WF_F_RIVER_Q) h->u_dirty = true;
    return WF_OK;
}

int32_t wf_get_outlets(WfHandle* h, int32_t which, double* dst, int64_t capacity, int64_t* n_written) {
    if (!h || !dst || !n_written) return set_err(h, WF_ERR_INVALID, "null argument");
    const int64_t need = (int64_t)h->outlet_slots.size() * h->M;
    *n_written = 0;
    if (capacity < need) return set_err(h, WF_ERR_INVALID, "capacity too small");
    if (h->F.split) {  // double-FP32 pairs: convert on the device, one copy out
        if (need > 0) {
            const int f = which == 0 ? RV_Q_AVG : RV_Q;
            if (!h->outlets_buf) {
                int rc = dalloc(h, &h->outlets_buf, (size_t)need);
                if (rc) return rc;
            }
            outlets_ff_kernel<<<(unsigned)((need + 255) / 256), 256, 0, h->stream>>>(
                h->F.RMh[f], h->F.RMl[f], h->d_outlet_slots, (int64_t)h->outlet_slots.size(), h->M, h->outlets_buf);
            CK(cudaGetLastError());
            CK(cudaMemcpyAsync(dst, h->outlets_buf, need * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        }
        CK(cudaStreamSynchronize(h->stream));
        *n_written = need;
        return WF_OK;
    }
    double* src = which == 0 ? h->F.RM[RV_Q_AVG] : h->F.RM[RV_Q];
    int64_t k = 0;
    for (int m = 0; m < h->M; ++m)
        for (int64_t s : h->outlet_slots) {
            CK(cudaMemcpyAsync(dst + k, src + s * h->M + m, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
            ++k;
        }
    CK(cudaStreamSynchronize(h->stream));
    *n_written = k;
    return WF_OK;
}

int32_t wf_get_state(WfHandle* h, void* dst, size_t* size) {
    if (!h || !size) return set_err(h, WF_ERR_INVALID, "null argument");
    auto items = state_items(h);
    size_t bytes = sizeof(StateHeader);
    for (auto& it : items) bytes += (size_t)field_extent(h, it.field) * h->M * sizeof(double);
    if (!dst) {
        *size = bytes;
        return WF_OK;
    }
    if (*size < bytes) return set_err(h, WF_ERR_STATE, "state buffer too small");
    StateHeader hd{};
    std::memcpy(hd.magic, "WFGB300S", 8);
    hd.version = 1;
    hd.n_members = h->M;
    hd.n_land = h->n;
    hd.n_river = h->nr;
    hd.n_layers = h->N;
    hd.n_items = (int32_t)items.size();
    std::memcpy(dst, &hd, sizeof(hd));
    char* p = (char*)dst + sizeof(hd);
    for (auto& it : items) {
        const int64_t cnt = field_extent(h, it.field) * h->M;
        int rc = wf_get_field(h, it.field, it.layer, (double*)p, 0, cnt);
        if (rc) return rc;
        p += cnt * sizeof(double);
    }
    *size = bytes;
    return WF_OK;
}

int32_t wf_set_state(WfHandle* h, const void* src, size_t size) {
    if (!h || !src) return set_err(h, WF_ERR_INVALID, "null argument");
    if (size < sizeof(StateHeader)) return set_err(h, WF_ERR_STATE, "state blob too small");
    StateHeader hd;
    std::memcpy(&hd, src, sizeof(hd));
    auto items = state_items(h);
    if (std::memcmp(hd.magic, "WFGB300S", 8) != 0 || hd.version != 1 || hd.n_members != h->M || hd.n_land != h->n ||
        hd.n_river != h->nr || hd.n_layers != h->N || hd.n_items != (int32_t)items.size())
        return set_err(h, WF_ERR_STATE, "state blob does not match this model");
    const char* p = (const char*)src + sizeof(hd);
    size_t used = sizeof(hd);
    for (auto& it : items) {
        const int64_t cnt = field_extent(h, it.field) * h->M;
        used += cnt * sizeof(double);
        if (used > size) return set_err(h, WF_ERR_STATE, "state blob truncated");
        int rc = wf_set_field(h, it.field, it.layer, (const double*)p, 0, cnt);
        if (rc) return rc;
        p += cnt * sizeof(double);
    }
    return WF_OK;
}

int32_t wf_get_metrics(WfHandle* h, WfMetrics* out) {
    if (!h || !out) return WF_ERR_INVALID;
    *out = h->metrics;
    return WF_OK;
}

int32_t wf_reset_metrics(WfHandle* h) {
    if (!h) return WF_ERR_INVALID;
    WfMetrics keep = h->metrics;
    h->metrics = WfMetrics{};
    h->metrics.n_chains_land = keep.n_chains_land;
    h->metrics.n_chains_river = keep.n_chains_river;
    h->metrics.max_chain_land = keep.max_chain_land;
    h->metrics.max_chain_river = keep.max_chain_river;
    h->metrics.padding_slots_land = keep.padding_slots_land;
    return WF_OK;
}

int32_t wf_set_tuning(WfHandle* h, const WfTuning* t) {
    if (!h || !t) return WF_ERR_INVALID;
    if (t->vertical_block < 0 || t->vertical_block > 1024 || (t->vertical_block % 32) != 0 || t->routing_warps < 0 ||
        t->routing_warps > 32 || t->routing_blocks_per_sm < 0 || t->routing_blocks_per_sm > 64)
        return set_err(h, WF_ERR_INVALID, "tuning out of range");
    if (t->reserved[3] < 0 || t->reserved[3] > 32) return set_err(h, WF_ERR_INVALID, "sub-step lanes out of range");
    if (t->reserved[4] < 0 || t->reserved[4] > 7) return set_err(h, WF_ERR_INVALID, "sweep input mask out of range");
    if (t->reserved[5] < 0 || t->reserved[5] > 64)
        return set_err(h, WF_ERR_INVALID, "vertical blocks per SM out of range");
    if (t->reserved[6] < 0 || t->reserved[6] > 1)
        return set_err(h, WF_ERR_INVALID, "overland-river launch switch must be 0 or 1");
    if (t->reserved[7] != 0) return set_err(h, WF_ERR_INVALID, "reserved tuning fields must be 0");
    h->tuning = *t;
    h->graph_valid = false;
    // reserved[]: [0] = wait budget in microseconds, [1] = awaited-epoch offset (test hooks),
    // [2] = per-kernel event timing, [3] = cap of the routing sweeps' sub-step lanes (0 = default),
    // [4] = bit k: node-major sweep k (0 subsurface, 1 overland, 2 river) keeps its inputs in
    // registers instead of staging them in shared memory, [5] = blocks per SM of the split
    // vertical kernel's grid-stride loop (0 = 16), [6] = 1: the split form's overland and river
    // sweeps in separate launches (0: one launch where the model allows it)
    if (t->reserved[0] > 0) h->wait_ns = (uint64_t)t->reserved[0] * 1000ull;
    h->wait_offset = (uint32_t)t->reserved[1];
    h->kernel_timing = t->reserved[2] != 0;
    return WF_OK;
}

int32_t wf_get_slot_order(WfHandle* h, int64_t* ext_of_slot, int64_t capacity, int64_t* n_slots) {
    if (!h || !n_slots) return WF_ERR_INVALID;
    *n_slots = h->land.plan.n_slots;
    if (ext_of_slot) {
        if (capacity < *n_slots) return set_err(h, WF_ERR_INVALID, "capacity too small");
        for (int64_t s = 0; s < *n_slots; ++s) ext_of_slot[s] = h->land.plan.node_of_slot[s];
    }
    return WF_OK;
}

int32_t wf_get_stream(WfHandle* h, void** stream) {
    if (!h || !stream) return WF_ERR_INVALID;
    *stream = (void*)h->stream;
    return WF_OK;
}

int32_t wf_get_kernel_times(WfHandle* h, double* ms5, int64_t* calls) {
    if (!h || !ms5) return WF_ERR_INVALID;
    CK(cudaStreamSynchronize(h->stream));
    for (int k = 0; k < 5; ++k) ms5[k] = h->kernel_ms[k];
    if (calls) *calls = h->kernel_calls;
    return WF_OK;
}

int32_t wf_get_sizes(WfHandle* h, int64_t* n_land, int64_t* n_river, int64_t* n_outlets, int32_t* n_layers,
                     int32_t* n_members) {
    if (!h) return WF_ERR_INVALID;
    if (n_land) *n_land = h->n;
    if (n_river) *n_river = h->nr;
    if (n_outlets) *n_outlets = (int64_t)h->outlet_slots.size();
    if (n_layers) *n_layers = h->N;
    if (n_members) *n_members = h->M;
    return WF_OK;
}

int32_t wf_get_substep_signature(WfHandle* h, int32_t kind, double* sig, int32_t n_members) {
    if (!h || !sig || kind < 0 || kind > 2 || n_members != h->M) return set_err(h, WF_ERR_INVALID, "invalid argument");
    if (!h->adaptive) return set_err(h, WF_ERR_INVALID, "the model takes fixed sub-steps");
    CK(cudaMemcpyAsync(sig, h->ad[kind].sig, (size_t)h->M * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return WF_OK;
}

int32_t wf_set_rating_curve_day(WfHandle* h, int32_t day_of_year) {
    if (!h) return WF_ERR_INVALID;
    if (day_of_year < 1 || day_of_year > 365) return set_err(h, WF_ERR_INVALID, "day of the year must be 1..365");
    if (!h->F.res_hq_day) return WF_OK;  // no reservoir tables: nothing reads the day
    set_day_kernel<<<1, 1, 0, h->stream>>>(const_cast<int32_t*>(h->F.res_hq_day), day_of_year);
    if (cudaGetLastError() != cudaSuccess) return set_err(h, WF_ERR_CUDA, "setting the rating-curve day failed");
    return WF_OK;
}

int32_t wf_get_reservoir_count(WfHandle* h, int64_t* n_reservoirs) {
    if (!h || !n_reservoirs) return WF_ERR_INVALID;
    *n_reservoirs = h->nres;
    return WF_OK;
}

int32_t wf_attach_local_inertial(WfHandle* h, WfLiDomain* d) {
    if (!h || !d) return set_err(h, WF_ERR_INVALID, "null argument");
    if (h->cfg.form != WF_FORM_FP64 || h->M != 1 || h->nres > 0 || h->adaptive)
        return set_err(h, WF_ERR_UNSUPPORTED,
                       "local-inertial routing in the step needs the FP64 form, one member, no reservoirs and "
                       "fixed kinematic-wave sub-steps");
    WfLiCoupleView v{};
    const int64_t* ri = nullptr;
    if (wf_li_domain_couple_view(d, &v, &ri) != WF_OK) return set_err(h, WF_ERR_INVALID, "invalid domain");
    if (v.n != h->n || v.n_active != h->nr)
        return set_err(h, WF_ERR_INVALID, "the grid's land and active river cells must be the model's");
    for (int64_t r = 0; r < h->nr; ++r)
        if (ri[h->river_land[r]] != r)
            return set_err(h, WF_ERR_INVALID, "river_index must map the land cell of river cell r to r");
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaDeviceSynchronize());  // the domain's own stream may still be setting its state
    h->li = d;
    h->liv = v;
    h->F.li_coupled = 1;
    h->graph_valid = false;
    CK(wf_fp64_li_couple_out(h->F, v, 0, launch_cfg(h)));  // the model starts from the scheme's depths
    CK(cudaStreamSynchronize(h->stream));
    return WF_OK;
}

}  // extern "C"

namespace {

constexpr int64_t kMaxAdaptiveSubsteps = 100000;

// The per-cell update of the step. With gravitational snow transport its snow part, the two
// material sweeps over the land graph (one sub-step of the model step each, in the land graph's
// wavefront scratch) and the inflow kernel run before its soil part (sbm.jl:92-131).
int enqueue_vertical(WfHandle* h, const WfLaunchCfg& lc, const WfDevGraph& gl, int64_t& nl) {
    const bool split = h->cfg.form == WF_FORM_SPLIT;
    if (!h->F.snow_transport) {
        CK(split ? wf_split_vertical(h->F, lc) : wf_fp64_vertical(h->F, lc));
        ++nl;
        return WF_OK;
    }
    CK(split ? wf_split_vertical_snow(h->F, lc) : wf_fp64_vertical_snow(h->F, lc));
    ++nl;
    for (int material = 0; material < 2; ++material) {
        WfSweep sw{};
        sw.S = 1;
        sw.first = 0;
        sw.last_of_step = 1;
        sw.total = 1;
        sw.epoch0 = 1;
        sw.dt = h->cfg.dt;
        sw.dts = h->dts_ssf;
        sw.wait_ns = h->wait_ns;
        sw.wait_offset = h->wait_offset;
        CK(cudaMemsetAsync(gl.flags, 0, (size_t)h->land.plan.n_chains * h->M * sizeof(uint32_t), h->stream));
        CK(cudaMemsetAsync(gl.ticket, 0, sizeof(unsigned long long), h->stream));
        CK(wf_snow_transport_sweep(h->F, gl, sw, material, lc));
        ++nl;
    }
    CK(wf_snow_in(h->F, gl, lc));
    ++nl;
    CK(split ? wf_split_vertical_soil(h->F, lc) : wf_fp64_vertical_soil(h->F, lc));
    ++nl;
    return WF_OK;
}

// Enqueue one model step on the handle's stream (with adaptive sub-steps the host waits for
// the device after every sub-step, see below).
int enqueue_step(WfHandle* h, int64_t* launches) {
    const WfLaunchCfg lc = launch_cfg(h);
    const bool split = h->cfg.form == WF_FORM_SPLIT;
    int64_t nl = 0;
    WfDevGraph gl = dev_graph(h->land, h->M), gr = dev_graph(h->river, h->M);
    const bool timing = h->kernel_timing && !h->tuning.use_graph;
    auto mark = [&](int i) {
        if (timing) cudaEventRecord(h->kev[i], h->stream);
    };
    mark(0);
    int rcv = enqueue_vertical(h, lc, gl, nl);
    if (rcv) return rcv;
    mark(1);
    auto sweep = [&](DevGraphAlloc& G, const WfDevGraph& g, const std::vector<double>& dts, double* d_dts,
                     int which) -> int {
        const int total = (int)dts.size();
        for (int first = 0; first < total; first += G.s_cap) {
            WfSweep sw{};
            sw.S = std::min(G.s_cap, total - first);
            sw.first = first;
            sw.last_of_step = (first + sw.S == total);
            sw.total = total;
            sw.epoch0 = 1;
            sw.dt = h->cfg.dt;
            sw.dts = d_dts + first;
            sw.wait_ns = h->wait_ns;
            sw.wait_offset = h->wait_offset;
            CK(cudaMemsetAsync(G.flags, 0, (size_t)G.plan.n_chains * h->M * sizeof(uint32_t), h->stream));
            CK(cudaMemsetAsync(G.ticket, 0, sizeof(unsigned long long), h->stream));
            cudaError_t e;
            if (which == 0) e = split ? wf_split_ssf(h->F, g, sw, lc) : wf_fp64_ssf(h->F, g, sw, lc);
            else if (which == 1) e = wf_fp64_overland(h->F, g, sw, lc);
            else e = wf_fp64_river(h->F, g, sw, lc);
            CK(e);
            ++nl;
        }
        return WF_OK;
    };
    // split form: slim wavefronts (end_q sentinel hand-off, node-major sub-step groups)
    // followed by their per-cell completion kernels
    auto wave_sw = [&](const DevGraphAlloc& G, const std::vector<double>& dts, double* d_dts, int first) {
        const int total = (int)dts.size();
        const int group = std::min<int>(G.s_cap, wfv::MAX_GROUP);
        WfSweep sw{};
        sw.S = std::min(group, total - first);
        sw.first = first;
        sw.last_of_step = (first + sw.S == total);
        sw.total = total;
        sw.epoch0 = 1;
        sw.dt = h->cfg.dt;
        sw.dts = d_dts + first;
        for (int j = 0; j < sw.S && j < 16; ++j) sw.dts_f[j] = (float)dts[first + j];
        sw.wait_ns = h->wait_ns;
        sw.wait_offset = h->wait_offset;
        return sw;
    };
    auto wave = [&](DevGraphAlloc& G, const WfDevGraph& g, const std::vector<double>& dts, double* d_dts, int which,
                    int first0 = 0) -> int {
        const int total = (int)dts.size();
        const int group = std::min<int>(G.s_cap, wfv::MAX_GROUP);
        for (int first = first0; first < total; first += group) {
            const WfSweep sw = wave_sw(G, dts, d_dts, first);
            CK(cudaMemsetAsync(G.end_q, 0xFF, (size_t)G.plan.n_chains * h->M * G.s_cap * sizeof(double), h->stream));
            CK(cudaMemsetAsync(G.ticket, 0, sizeof(unsigned long long), h->stream));
            cudaError_t e;
            if (which == 0) e = wf_split_ssf_wave(h->F, g, sw, lc);
            else if (which == 1) e = wf_split_overland_wave(h->F, g, sw, lc);
            else e = wf_split_river_wave(h->F, g, sw, lc);
            CK(e);
            ++nl;
        }
        if (which == 0) CK(wf_split_ssf_post(h->F, g, lc));
        else if (which == 1) CK(wf_split_overland_post(h->F, g, lc));
        else CK(wf_split_river_post(h->F, g, lc));
        ++nl;
        return WF_OK;
    };
    // adaptive sub-steps: the size of a sub-step follows from the state the previous one left
    // (a quantile or minimum over the whole graph), so every sub-step is its own launch, preceded
    // by the selection kernels and followed by a host read of whether a member needs another
    auto adaptive = [&](DevGraphAlloc& G, const WfDevGraph& g, int kind) -> int {
        WfAdaptive& A = h->ad[kind];
        CK(cudaMemsetAsync(A.t, 0, (size_t)h->M * sizeof(double), h->stream));
        CK(cudaMemsetAsync(A.nsub, 0, (size_t)h->M * sizeof(int32_t), h->stream));
        CK(cudaMemsetAsync(A.sig, 0, (size_t)h->M * sizeof(double), h->stream));
        const bool slim = split && kind != WF_ADAPT_SSF;
        int64_t it = 0;
        while (true) {
            if (it >= kMaxAdaptiveSubsteps)
                return set_err(h, WF_ERR_INVALID, "adaptive sub-stepping needed more than 100000 sub-steps in one step");
            CK(wf_adaptive_substep(h->F, A, lc));
            nl += (kind == WF_ADAPT_SSF ? 1 : (A.fp32_keys ? 4 : 8)) + 1;
            if (split && kind == WF_ADAPT_SSF && it == 0) {
                // every member's first sub-step spans the model step: the slim subsurface
                // wavefront with the terms the vertical kernel prepared for a sub-step of dt
                CK(cudaMemcpyAsync(h->h_more, A.more, sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
                CK(cudaStreamSynchronize(h->stream));
                if (!*h->h_more) {
                    h->last_substeps[kind] = 1;
                    return wave(G, g, h->h_dts_ssf, h->dts_ssf, 0);
                }
            }
            WfSweep sw{};
            sw.S = 1;
            sw.epoch0 = 1;
            sw.dt = h->cfg.dt;
            sw.dts = A.dt_s;
            sw.adt = A.dt_s;
            sw.adt_hi = A.dt_hi;
            sw.adt_lo = A.dt_lo;
            sw.aflag = A.flags;
            sw.wait_ns = h->wait_ns;
            sw.wait_offset = h->wait_offset;
            CK(cudaMemsetAsync(G.ticket, 0, sizeof(unsigned long long), h->stream));
            cudaError_t e;
            if (slim) {
                CK(cudaMemsetAsync(G.end_q, 0xFF, (size_t)G.plan.n_chains * h->M * G.s_cap * sizeof(double),
                                   h->stream));
                e = kind == WF_ADAPT_LAND ? wf_split_overland_wave(h->F, g, sw, lc) : wf_split_river_wave(h->F, g, sw, lc);
            } else {
                CK(cudaMemsetAsync(G.flags, 0, (size_t)G.plan.n_chains * h->M * sizeof(uint32_t), h->stream));
                if (kind == WF_ADAPT_SSF) e = split ? wf_split_ssf(h->F, g, sw, lc) : wf_fp64_ssf(h->F, g, sw, lc);
                else if (kind == WF_ADAPT_LAND) e = wf_fp64_overland(h->F, g, sw, lc);
                else e = wf_fp64_river(h->F, g, sw, lc);
            }
            CK(e);
            ++nl;
            ++it;
            CK(cudaMemcpyAsync(h->h_more, A.more, sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
            CK(cudaStreamSynchronize(h->stream));
            if (!*h->h_more) break;
        }
        h->last_substeps[kind] = it;
        if (slim) {
            CK(kind == WF_ADAPT_LAND ? wf_split_overland_post(h->F, g, lc) : wf_split_river_post(h->F, g, lc));
            ++nl;
        }
        return WF_OK;
    };
    // reservoirs: inflow from the land routing before the river sweep, averages and balance after
    auto res_prep = [&]() -> int {
        if (h->nres <= 0) return WF_OK;
        CK(wf_reservoir_prep(h->F, lc));
        ++nl;
        return WF_OK;
    };
    auto res_post = [&]() -> int {
        if (h->nres <= 0) return WF_OK;
        CK(wf_reservoir_post(h->F, lc));
        ++nl;
        return WF_OK;
    };
    int rc;
    if (h->adaptive) {
        if ((rc = adaptive(h->land, gl, WF_ADAPT_SSF))) return rc;
        mark(2);
        if ((rc = adaptive(h->land, gl, WF_ADAPT_LAND))) return rc;
        mark(3);
        if ((rc = res_prep())) return rc;
        if (h->nr > 0 && (rc = adaptive(h->river, gr, WF_ADAPT_RIVER))) return rc;
        if ((rc = res_post())) return rc;
        mark(4);
    } else if (split) {
        if (h->F.ssf_single) rc = wave(h->land, gl, h->h_dts_ssf, h->dts_ssf, 0);
        else rc = sweep(h->land, gl, h->h_dts_ssf, h->dts_ssf, 0);
        if (rc) return rc;
        mark(2);
        // the overland sweep and the river's first sub-step group in one launch (the river cells
        // take their lateral inflow from the overland walker as it passes them), unless the
        // tuning asks for separate launches; models with reservoirs (whose inflow is the
        // overland step average) and steps of more overland sub-steps than one launch holds
        // keep them apart
        const bool fuse = h->tuning.reserved[6] == 0 && h->nres == 0 && h->nr > 0 &&
                          (int)h->h_dts_land.size() <= std::min<int>(h->land.s_cap, wfv::MAX_GROUP);
        if (fuse) {
            const WfSweep swl = wave_sw(h->land, h->h_dts_land, h->dts_land, 0);
            const WfSweep swr = wave_sw(h->river, h->h_dts_river, h->dts_river, 0);
            CK(cudaMemsetAsync(h->land.end_q, 0xFF,
                               (size_t)h->land.plan.n_chains * h->M * h->land.s_cap * sizeof(double), h->stream));
            CK(cudaMemsetAsync(h->river.end_q, 0xFF,
                               (size_t)h->river.plan.n_chains * h->M * h->river.s_cap * sizeof(double), h->stream));
            CK(cudaMemsetAsync(h->F.rv_lat_pub, 0xFF, (size_t)h->river.plan.n_slots * h->M * sizeof(double),
                               h->stream));
            CK(cudaMemsetAsync(h->land.ticket, 0, sizeof(unsigned long long), h->stream));
            CK(wf_split_overland_river_wave(h->F, gl, swl, gr, swr, lc));
            CK(wf_split_overland_post(h->F, gl, lc));
            nl += 2;
            mark(3);
            if ((rc = wave(h->river, gr, h->h_dts_river, h->dts_river, 2, swr.S))) return rc;
            mark(4);
        } else {
            if ((rc = wave(h->land, gl, h->h_dts_land, h->dts_land, 1))) return rc;
            mark(3);
            if ((rc = res_prep())) return rc;
            if (h->nr > 0 && (rc = wave(h->river, gr, h->h_dts_river, h->dts_river, 2))) return rc;
            if ((rc = res_post())) return rc;
            mark(4);
        }
    } else if (h->li) {
        // local-inertial land and river routing (surface_routing.jl:62-89) after the subsurface
        if ((rc = sweep(h->land, gl, h->h_dts_ssf, h->dts_ssf, 0))) return rc;
        mark(2);
        CK(wf_fp64_li_couple_in(h->F, h->liv, lc));
        ++nl;
        if ((rc = wf_li_domain_enqueue_step(h->li, h->cfg.dt, h->stream)))
            return set_err(h, rc, "local-inertial step could not be enqueued");
        nl += 4;
        mark(3);
        CK(wf_fp64_li_couple_out(h->F, h->liv, 1, lc));
        ++nl;
        mark(4);
    } else {
        if ((rc = sweep(h->land, gl, h->h_dts_ssf, h->dts_ssf, 0))) return rc;
        mark(2);
        if ((rc = sweep(h->land, gl, h->h_dts_land, h->dts_land, 1))) return rc;
        mark(3);
        if ((rc = res_prep())) return rc;
        if (h->nr > 0 && (rc = sweep(h->river, gr, h->h_dts_river, h->dts_river, 2))) return rc;
        if ((rc = res_post())) return rc;
        mark(4);
    }
    CK(split ? wf_split_balance(h->F, lc) : wf_fp64_balance(h->F, lc));
    ++nl;
    mark(5);
    if (timing) {
        CK(cudaEventSynchronize(h->kev[5]));
        for (int k = 0; k < 5; ++k) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, h->kev[k], h->kev[k + 1]);
            h->kernel_ms[k] += ms;
        }
        h->kernel_calls += 1;
    }
    if (launches) *launches = nl;
    return WF_OK;
}

int run_step(WfHandle* h) {
    int64_t launches = 0;
    if (h->u_dirty) {
        if (h->cfg.form == WF_FORM_SPLIT) CK(wf_split_sync_u(h->F, launch_cfg(h)));
        h->u_dirty = false;
    }
    if (h->tuning.use_graph && !h->adaptive && !h->li) {
        if (!h->graph_valid) {
            if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
            if (h->graph) cudaGraphDestroy(h->graph);
            h->graph_exec = nullptr;
            h->graph = nullptr;
            CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
            int rc = enqueue_step(h, &launches);
            cudaGraph_t g = nullptr;
            cudaError_t ee = cudaStreamEndCapture(h->stream, &g);
            if (rc) {
                if (g) cudaGraphDestroy(g);
                return rc;
            }
            CK(ee);
            h->graph = g;
            CK(cudaGraphInstantiate(&h->graph_exec, h->graph, 0));
            h->graph_valid = true;
            h->launches_per_step = launches;
        }
        CK(cudaGraphLaunch(h->graph_exec, h->stream));
        launches = h->launches_per_step;
    } else {
        int rc = enqueue_step(h, &launches);
        if (rc) return rc;
    }
    h->metrics.steps += 1;
    h->metrics.cell_steps += h->n * h->M;
    h->metrics.kernel_launches += launches;
    if (h->li) {  // the scheme's loop status and sub-step count (one read per step)
        CK(cudaStreamSynchronize(h->stream));
        const char* msg = nullptr;
        int64_t k = 0;
        const int rc = wf_li_domain_complete_step(h->li, &k, &msg);
        if (rc) return set_err(h, rc, msg ? msg : "local-inertial step failed");
        h->li_substeps = k;
        h->metrics.substeps_subsurface += (int64_t)h->h_dts_ssf.size();
        h->metrics.substeps_land += k;
        h->metrics.substeps_river += k;
        return WF_OK;
    }
    if (h->adaptive) {
        h->metrics.substeps_subsurface += h->last_substeps[WF_ADAPT_SSF];
        h->metrics.substeps_land += h->last_substeps[WF_ADAPT_LAND];
        h->metrics.substeps_river += h->nr > 0 ? h->last_substeps[WF_ADAPT_RIVER] : 0;
        return WF_OK;
    }
    h->metrics.substeps_land += (int64_t)h->h_dts_land.size();
    h->metrics.substeps_river += (int64_t)h->h_dts_river.size();
    h->metrics.substeps_subsurface += (int64_t)h->h_dts_ssf.size();
    return WF_OK;
}

}  // namespace

cudaError_t wf_gather_ext(const double* src_ext, double* dst_slots, const int64_t* node_of_slot, int64_t slots, int M,
                          int64_t n_ext, cudaStream_t s) {
    gather_kernel<<<grid_of(slots * M, 256), 256, 0, s>>>(src_ext, dst_slots, node_of_slot, slots, M, n_ext);
    return cudaGetLastError();
}

cudaError_t wf_scatter_ext(const double* src_slots, double* dst_ext, const int64_t* node_of_slot, int64_t slots, int M,
                           int64_t n_ext, cudaStream_t s) {
    scatter_kernel<<<grid_of(slots * M, 256), 256, 0, s>>>(src_slots, dst_ext, node_of_slot, slots, M, n_ext);
    return cudaGetLastError();
}

// ===================================================================== static scratch ====
//
// wf_step_static: the model step without any allocation. The routing wavefronts take their
// scratch (work ticket, chain-end flags, published chain-end discharges) from one file-scope
// device array instead of the handle's buffers, and the step's launches are issued directly
// (no CUDA graph is built or instantiated). The array is shared by every handle and every call
// on a device and keeps the last call's contents; each sweep launch clears what must start at
// zero (ticket, flags) or at the sentinel (published discharges) before it runs.

static __device__ __align__(256) unsigned char wf_static_scratch[WF_STATIC_SCRATCH_BYTES];

namespace {

constexpr int kStaticMaxDevices = 64;
std::mutex g_static_mu;
unsigned char* g_static_ptr[kStaticMaxDevices] = {};

// Device address of the static scratch on the handle's device, looked up once per device with
// that device current (wf_create does this, so that wf_step_static itself allocates nothing).
int static_scratch(WfHandle* h, unsigned char** out) {
    std::lock_guard<std::mutex> lock(g_static_mu);
    if (h->device < 0 || h->device >= kStaticMaxDevices)
        return set_err(h, WF_ERR_INVALID, "wf_step_static: device index out of range");
    if (!g_static_ptr[h->device]) {
        int prev = -1;
        CK(cudaGetDevice(&prev));
        CK(cudaSetDevice(h->device));
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, wf_static_scratch);
        const cudaError_t e2 = cudaSetDevice(prev);
        if (e != cudaSuccess)
            return set_err(h, WF_ERR_CUDA,
                           std::string("wf_step_static: cudaGetSymbolAddress of the static scratch failed: ") +
                               cudaGetErrorString(e));
        if (e2 != cudaSuccess) return set_err(h, WF_ERR_CUDA, "wf_step_static: restoring the current device failed");
        g_static_ptr[h->device] = (unsigned char*)p;
    }
    *out = g_static_ptr[h->device];
    return WF_OK;
}

// Scratch bytes one sweep launch of graph G needs: ticket, flags, published discharges.
size_t static_need(const DevGraphAlloc& G, int M) {
    const size_t slots = (size_t)G.plan.n_chains * M;
    const size_t flags = (slots * sizeof(uint32_t) + 255) / 256 * 256;
    return 256 + flags + slots * G.s_cap * sizeof(double);
}

// Graph view whose scratch points into the static array.
WfDevGraph static_graph(const DevGraphAlloc& G, int M, unsigned char* base) {
    WfDevGraph g = dev_graph(G, M);
    const size_t slots = (size_t)G.plan.n_chains * M;
    g.ticket = (unsigned long long*)base;
    g.flags = (uint32_t*)(base + 256);
    g.end_q = (double*)(base + 256 + (slots * sizeof(uint32_t) + 255) / 256 * 256);
    return g;
}

// The launches of enqueue_step with the wavefront scratch of the static array.
int enqueue_step_static(WfHandle* h, unsigned char* base, int64_t* launches) {
    const WfLaunchCfg lc = launch_cfg(h);
    const bool split = h->cfg.form == WF_FORM_SPLIT;
    int64_t nl = 0;
    const WfDevGraph gl = static_graph(h->land, h->M, base), gr = static_graph(h->river, h->M, base);
    int rcv = enqueue_vertical(h, lc, gl, nl);
    if (rcv) return rcv;
    auto clear = [&](const DevGraphAlloc& G, const WfDevGraph& g, bool sentinel) -> int {
        const size_t slots = (size_t)G.plan.n_chains * h->M;
        CK(cudaMemsetAsync(g.ticket, 0, sizeof(unsigned long long), h->stream));
        if (sentinel) CK(cudaMemsetAsync(g.end_q, 0xFF, slots * G.s_cap * sizeof(double), h->stream));
        else CK(cudaMemsetAsync(g.flags, 0, slots * sizeof(uint32_t), h->stream));
        return WF_OK;
    };
    auto sweep = [&](const DevGraphAlloc& G, const WfDevGraph& g, const std::vector<double>& dts, double* d_dts,
                     int which, bool wave) -> int {
        const int total = (int)dts.size();
        const int group = wave ? std::min<int>(G.s_cap, wfv::MAX_GROUP) : G.s_cap;
        for (int first = 0; first < total; first += group) {
            WfSweep sw{};
            sw.S = std::min(group, total - first);
            sw.first = first;
            sw.last_of_step = (first + sw.S == total);
            sw.total = total;
            sw.epoch0 = 1;
            sw.dt = h->cfg.dt;
            sw.dts = d_dts + first;
            for (int j = 0; j < sw.S && j < 16; ++j) sw.dts_f[j] = (float)dts[first + j];
            sw.wait_ns = h->wait_ns;
            sw.wait_offset = h->wait_offset;
            int rc = clear(G, g, wave);
            if (rc) return rc;
            cudaError_t e;
            if (wave) {
                if (which == 0) e = wf_split_ssf_wave(h->F, g, sw, lc);
                else if (which == 1) e = wf_split_overland_wave(h->F, g, sw, lc);
                else e = wf_split_river_wave(h->F, g, sw, lc);
            } else if (which == 0) {
                e = split ? wf_split_ssf(h->F, g, sw, lc) : wf_fp64_ssf(h->F, g, sw, lc);
            } else if (which == 1) {
                e = wf_fp64_overland(h->F, g, sw, lc);
            } else {
                e = wf_fp64_river(h->F, g, sw, lc);
            }
            CK(e);
            ++nl;
        }
        if (wave) {
            if (which == 0) CK(wf_split_ssf_post(h->F, g, lc));
            else if (which == 1) CK(wf_split_overland_post(h->F, g, lc));
            else CK(wf_split_river_post(h->F, g, lc));
            ++nl;
        }
        return WF_OK;
    };
    int rc;
    if ((rc = sweep(h->land, gl, h->h_dts_ssf, h->dts_ssf, 0, split && h->F.ssf_single))) return rc;
    if ((rc = sweep(h->land, gl, h->h_dts_land, h->dts_land, 1, split))) return rc;
    if (h->nres > 0) {
        CK(wf_reservoir_prep(h->F, lc));
        ++nl;
    }
    if (h->nr > 0 && (rc = sweep(h->river, gr, h->h_dts_river, h->dts_river, 2, split))) return rc;
    if (h->nres > 0) {
        CK(wf_reservoir_post(h->F, lc));
        ++nl;
    }
    CK(split ? wf_split_balance(h->F, lc) : wf_fp64_balance(h->F, lc));
    ++nl;
    if (launches) *launches = nl;
    return WF_OK;
}

}  // namespace

extern "C" int32_t wf_step_static(WfHandle* h) {
    if (!h) return WF_ERR_INVALID;
    if (h->adaptive)
        return set_err(h, WF_ERR_UNSUPPORTED,
                       "wf_step_static: adaptive sub-stepping synchronises with the host every sub-step; use wf_step");
    if (h->li)
        return set_err(h, WF_ERR_UNSUPPORTED,
                       "wf_step_static: the local-inertial routing reads its loop status back every step; use wf_step");
    const size_t need = std::max(static_need(h->land, h->M), h->nr > 0 ? static_need(h->river, h->M) : (size_t)0);
    if (need > (size_t)WF_STATIC_SCRATCH_BYTES) {
        char msg[256];
        std::snprintf(msg, sizeof(msg),
                      "wf_step_static: the routing wavefronts of this model need %zu bytes of scratch, more than "
                      "the %zu-byte static scratch; use wf_step",
                      need, (size_t)WF_STATIC_SCRATCH_BYTES);
        return set_err(h, WF_ERR_UNSUPPORTED, msg);
    }
    unsigned char* base = nullptr;
    int rc = static_scratch(h, &base);
    if (rc) return rc;
    if (h->u_dirty) {
        if (h->cfg.form == WF_FORM_SPLIT) CK(wf_split_sync_u(h->F, launch_cfg(h)));
        h->u_dirty = false;
    }
    int64_t launches = 0;
    if ((rc = enqueue_step_static(h, base, &launches))) return rc;
    h->metrics.steps += 1;
    h->metrics.cell_steps += h->n * h->M;
    h->metrics.kernel_launches += launches;
    h->metrics.substeps_land += (int64_t)h->h_dts_land.size();
    h->metrics.substeps_river += (int64_t)h->h_dts_river.size();
    h->metrics.substeps_subsurface += (int64_t)h->h_dts_ssf.size();
    return wf_synchronize(h);
}
