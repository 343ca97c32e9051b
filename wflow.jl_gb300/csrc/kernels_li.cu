// kernels_li.cu -- local-inertial routing on a staggered grid (include/wflow_gb300_li.h).
//
// River alone (WfLiRiver). Per sub-step: one thread per edge computes the edge discharge from the
// previous discharge and the water-surface slope (local_inertial_flow, Wflow/src/routing/surface/
// surface_process.jl:88-115; the edge update of update_river_channel_flow!,
// surface_staggered_scheme.jl:326-385); then one thread per active cell sums the discharge of
// its incoming and outgoing edges (CSR lists in ascending edge order, the order of sum_at) and
// updates storage and depth (update_water_depth_and_storage!, :723-760). The stable sub-step is
// a min-reduction over the cells (:1004-1020).
//
// Land grid with the river (WfLiDomain, update_overland_flow_model!, :1153-1193). Per sub-step:
// one thread per land cell computes its x and y edge discharges from the previous sub-step's
// (two buffers per direction, swapped each sub-step, so no copy pass); the river edge kernel as
// above; then one thread per land cell updates its storage and depths, a river cell together
// with its river cell (the land-to-river map is one-to-one, so no two threads write one river
// cell). The stable sub-step reduces the river and the land minima in one block.
//
// Every operation is FP64 in the reference's order; the translation unit is compiled without
// FMA contraction, and cbrt and sqrt are the library's own (wf_math.cuh), so the results equal
// the CPU oracle's. The per-edge and per-cell arithmetic lives in li_scheme.cuh.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "li_scheme.cuh"
#include "wf_li_couple.cuh"
#include "wflow_gb300.h"
#include "wflow_gb300_li.h"

namespace {

using LiDev = wfli::LiNet;

__global__ void li_edge_kernel(LiDev d, double dt) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < d.n_edges;
         k += (int64_t)gridDim.x * blockDim.x) {
        if (d.manning) wfli::update_edge_manning(d, k, dt);
        else wfli::update_edge(d, k, dt);
    }
}

__global__ void li_cell_kernel(LiDev d, double dt) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < d.n_active;
         i += (int64_t)gridDim.x * blockDim.x)
        wfli::update_cell(d, i, dt);
}

// the reductions run in one block of LI_DT_THREADS threads (the launches use exactly that many;
// the shared arrays are sized for it)
constexpr int LI_DT_THREADS = 256;
constexpr uint64_t INF_BITS = 0x7ff0000000000000ULL;

__device__ double block_min(double m, double* red) {
    red[threadIdx.x] = m;
    __syncthreads();
    for (int w = LI_DT_THREADS / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] = wfm::jmin(red[threadIdx.x + w], red[threadIdx.x]);
        __syncthreads();
    }
    const double v = red[0];
    __syncthreads();
    return v;
}

__global__ void li_dt_kernel(LiDev d) {
    __shared__ double red[LI_DT_THREADS];
    double m = wfm::from_bits(INF_BITS);
    if (d.manning)
        for (int64_t k = threadIdx.x; k < d.n_edges; k += LI_DT_THREADS)
            m = wfm::jmin(wfli::edge_timestep_manning(d, k), m);
    else
        for (int64_t i = threadIdx.x; i < d.n_dt; i += LI_DT_THREADS) m = wfm::jmin(wfli::cell_timestep(d, i), m);
    const double v = block_min(m, red);
    if (threadIdx.x == 0) *d.dt_min = wfli::finish_timestep(v);
}

// q_average = q_cumulative / dt (average_flow_vars!, routing/surface/surface_kinwave.jl:283-290
// for the river, surface_staggered_scheme.jl:1138-1147 for the land)
__global__ void li_average_kernel(const double* q_cum, double* q_avg, int64_t n, double dt) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        q_avg[k] = q_cum[k] / dt;
}

__global__ void li_land_flux_kernel(wfli::LiLand L, double dt) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < L.n; i += (int64_t)gridDim.x * blockDim.x) {
        wfli::land_direction(L, i, dt, true);
        wfli::land_direction(L, i, dt, false);
    }
}

__global__ void li_land_depth_kernel(wfli::LiLand L, LiDev R, wfli::LiRiverBC B, double dt) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < L.n; i += (int64_t)gridDim.x * blockDim.x)
        wfli::land_depth(L, R, B, i, dt);
}

// min(river minimum, land minimum), each 60 s when infinite (surface_staggered_scheme.jl:
// 1171-1173); the river minimum covers its real cells, not the ghost cells (:1004-1020 loops
// over parameters.n, the river cells without the ghosts)
__global__ void li_domain_dt_kernel(wfli::LiLand L, LiDev R) {
    __shared__ double red[LI_DT_THREADS];
    double m = wfm::from_bits(INF_BITS);
    for (int64_t i = threadIdx.x; i < R.n_dt; i += LI_DT_THREADS) m = wfm::jmin(wfli::cell_timestep(R, i), m);
    const double dt_river = wfli::finish_timestep(block_min(m, red));
    m = wfm::from_bits(INF_BITS);
    for (int64_t i = threadIdx.x; i < L.n; i += LI_DT_THREADS) m = wfm::jmin(wfli::land_timestep(L, i), m);
    const double dt_land = wfli::finish_timestep(block_min(m, red));
    if (threadIdx.x == 0) *L.dt_min = wfm::jmin(dt_river, dt_land);
}

int grid_of(int64_t n) {
    const int64_t g = (n + 255) / 256;
    return (int)(g < 1 ? 1 : (g > 65535 ? 65535 : g));
}

// ---- device-side sub-step loops ----------------------------------------------------------------
// One persistent cooperative launch per model step runs the reference's sub-step loop
// (update_river_flow_model!, surface_staggered_scheme.jl:800-826; update_overland_flow_model!,
// :1153-1193) on the device: the stable time step (a grid-wide min-reduction), check_timestepsize
// (routing/timestepping.jl:11-16), the edge and then the cell updates, separated by grid barriers,
// until the step is covered. The host reads the sub-step count and the status once per model
// step instead of the time step every sub-step. Every thread takes the same sub-step sizes (the
// same minimum and the same FP64 operations), so the results equal the host-driven loop's.

struct LiLoop {
    unsigned count, gen;                  // grid barrier: arrivals and generation
    int status;                           // 1: a barrier wait ran out of its budget, 2: too many sub-steps
    int pad;
    unsigned long long minbits[2][2];     // [sub-step parity][river, land] minimum stable sub-step (bits)
    int nanflag[2][2];                    // a NaN among the candidates (Julia's min propagates NaN)
    long long substeps;
    double t;
};

constexpr uint64_t LI_BARRIER_BUDGET_NS = 10ull * 1000 * 1000 * 1000;  // a safety net: a wait lasts one phase
constexpr long long LI_MAX_SUBSTEPS = 10000000;

__device__ __forceinline__ uint64_t li_now_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid barrier of a cooperative launch (all blocks resident), every wait bounded: a wait that runs
// out sets the status and every block returns false.
__device__ bool li_grid_sync(LiLoop* s) {
    __shared__ int ok_s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        volatile unsigned* gen = &s->gen;
        const unsigned g = *gen;
        __threadfence();
        if (atomicAdd(&s->count, 1u) == gridDim.x - 1) {
            atomicExch(&s->count, 0u);
            __threadfence();
            atomicAdd(&s->gen, 1u);
        } else {
            const uint64_t t0 = li_now_ns();
            while (*gen == g) {
                __nanosleep(32);
                if (*(volatile int*)&s->status) {
                    ok = 0;
                    break;
                }
                if (li_now_ns() - t0 > LI_BARRIER_BUDGET_NS) {
                    atomicOr(&s->status, 1);
                    ok = 0;
                    break;
                }
            }
        }
        __threadfence();
        ok_s = ok && !*(volatile int*)&s->status;
    }
    __syncthreads();
    return ok_s != 0;
}

// Block minimum of the non-NaN candidates into minbits[p][w] (the bit patterns of non-negative
// doubles order as the values), and the NaN flag.
__device__ void li_reduce_min(LiLoop* s, int p, int w, double m, bool nan) {
    __shared__ double red[32];
    __shared__ int nan_s;
    if (threadIdx.x == 0) nan_s = 0;
    __syncthreads();
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) m = fmin(m, __shfl_xor_sync(0xffffffffu, m, off));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    if (nan) nan_s = 1;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = red[0];
        for (int k = 1; k < (int)(blockDim.x >> 5); ++k) b = fmin(b, red[k]);
        atomicMin(&s->minbits[p][w], (unsigned long long)__double_as_longlong(b));
        if (nan_s) atomicOr(&s->nanflag[p][w], 1);
    }
}

__device__ __forceinline__ double li_read_min(LiLoop* s, int p, int w) {
    if (*(volatile int*)&s->nanflag[p][w]) return __longlong_as_double(0x7ff8000000000000LL);
    return __longlong_as_double((long long)*(volatile unsigned long long*)&s->minbits[p][w]);
}

__global__ void li_loop_init_kernel(LiLoop* s) {
    s->count = 0;
    s->gen = 0;
    s->status = 0;
    for (int p = 0; p < 2; ++p)
        for (int w = 0; w < 2; ++w) {
            s->minbits[p][w] = INF_BITS;
            s->nanflag[p][w] = 0;
        }
    s->substeps = 0;
    s->t = 0.0;
}

// the river alone (wf_li_river_step)
__global__ void __launch_bounds__(256) li_river_loop_kernel(LiDev d, LiLoop* s, double dt) {
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, nt = (int64_t)gridDim.x * blockDim.x;
    double t = 0.0;
    long long k = 0;
    while (t < dt) {
        const int p = (int)(k & 1);
        double m = wfm::from_bits(INF_BITS);
        bool nan = false;
        const int64_t nv = d.manning ? d.n_edges : d.n_dt;  // Manning: the edges' sub-steps
        for (int64_t i = tid; i < nv; i += nt) {
            const double v = d.manning ? wfli::edge_timestep_manning(d, i) : wfli::cell_timestep(d, i);
            if (v != v) nan = true;
            else m = fmin(m, v);
        }
        li_reduce_min(s, p, 0, m, nan);
        if (!li_grid_sync(s)) return;
        if (tid == 0) {  // the other parity's slot serves the next sub-step
            s->minbits[p ^ 1][0] = INF_BITS;
            s->nanflag[p ^ 1][0] = 0;
        }
        double dt_s = wfli::finish_timestep(li_read_min(s, p, 0));
        if (t + dt_s > dt) dt_s = dt - t;
        for (int64_t e = tid; e < d.n_edges; e += nt) {
            if (d.manning) wfli::update_edge_manning(d, e, dt_s);
            else wfli::update_edge(d, e, dt_s);
        }
        if (!li_grid_sync(s)) return;
        for (int64_t i = tid; i < d.n_active; i += nt) wfli::update_cell(d, i, dt_s);
        t += dt_s;
        ++k;
        if (!li_grid_sync(s)) return;
        if (k >= LI_MAX_SUBSTEPS) {
            if (tid == 0) atomicOr(&s->status, 2);
            return;
        }
    }
    if (tid == 0) {
        s->substeps = k;
        s->t = t;
    }
}

// the land grid with its river (wf_li_domain_step); qx_buf / qy_buf hold the discharges of the
// last two sub-steps, buffer cur0 the latest at the start
__global__ void __launch_bounds__(256) li_domain_loop_kernel(wfli::LiLand L, LiDev R, wfli::LiRiverBC B, LiLoop* s,
                                                             double dt, double* qx0b, double* qx1b, double* qy0b,
                                                             double* qy1b, int cur0) {
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, nt = (int64_t)gridDim.x * blockDim.x;
    double t = 0.0;
    long long k = 0;
    while (t < dt) {
        const int p = (int)(k & 1);
        double mr = wfm::from_bits(INF_BITS), ml = wfm::from_bits(INF_BITS);
        bool nr = false, nl = false;
        for (int64_t i = tid; i < R.n_dt; i += nt) {
            const double v = wfli::cell_timestep(R, i);
            if (v != v) nr = true;
            else mr = fmin(mr, v);
        }
        for (int64_t i = tid; i < L.n; i += nt) {
            const double v = wfli::land_timestep(L, i);
            if (v != v) nl = true;
            else ml = fmin(ml, v);
        }
        li_reduce_min(s, p, 0, mr, nr);
        li_reduce_min(s, p, 1, ml, nl);
        if (!li_grid_sync(s)) return;
        if (tid == 0) {
            s->minbits[p ^ 1][0] = s->minbits[p ^ 1][1] = INF_BITS;
            s->nanflag[p ^ 1][0] = s->nanflag[p ^ 1][1] = 0;
        }
        const double dt_river = wfli::finish_timestep(li_read_min(s, p, 0));
        const double dt_land = wfli::finish_timestep(li_read_min(s, p, 1));
        double dt_s = wfm::jmin(dt_river, dt_land);
        if (t + dt_s > dt) dt_s = dt - t;
        const int prev = (cur0 + (int)(k & 1)) & 1;
        L.qx0 = prev ? qx1b : qx0b;
        L.qy0 = prev ? qy1b : qy0b;
        L.qx = prev ? qx0b : qx1b;
        L.qy = prev ? qy0b : qy1b;
        for (int64_t i = tid; i < L.n; i += nt) {
            wfli::land_direction(L, i, dt_s, true);
            wfli::land_direction(L, i, dt_s, false);
        }
        for (int64_t e = tid; e < R.n_edges; e += nt) wfli::update_edge(R, e, dt_s);
        if (!li_grid_sync(s)) return;
        for (int64_t i = tid; i < L.n; i += nt) wfli::land_depth(L, R, B, i, dt_s);
        t += dt_s;
        ++k;
        if (!li_grid_sync(s)) return;
        if (k >= LI_MAX_SUBSTEPS) {
            if (tid == 0) atomicOr(&s->status, 2);
            return;
        }
    }
    if (tid == 0) {
        s->substeps = k;
        s->t = t;
    }
}

// Blocks of a cooperative loop launch: every block resident (occupancy x SMs), no more than the
// work needs.
template <class Kernel>
int li_loop_blocks(Kernel kernel, int device, int64_t work) {
    int per_sm = 0, sms = 0, coop = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 256, 0) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device) != cudaSuccess || !coop) return 0;
    const int64_t need = (work + 255) / 256;
    int64_t b = (int64_t)per_sm * sms;
    if (b > need) b = need;
    return (int)(b < 1 ? 1 : b);
}

// device memory, stream and error text of a handle
struct LiOwner {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<void*> allocs;
    std::string err;
    LiLoop* loop = nullptr;      // state of the device-side sub-step loop
    LiLoop* loop_host = nullptr; // pinned read-back of it
    bool host_loop = false;      // drive the sub-steps from the host (no cooperative launch)
};

thread_local std::string g_li_error;

int li_fail(LiOwner* o, int code, const std::string& msg) {
    if (o) o->err = msg;
    else g_li_error = msg;
    return code;
}

// device array of count values (at least one allocated), copied from src or zeroed
template <class T>
int li_upload(LiOwner* o, T** p, const T* src, size_t count) {
    const size_t bytes = (count ? count : 1) * sizeof(T);
    if (cudaMalloc((void**)p, bytes) != cudaSuccess) return li_fail(o, WF_ERR_NOMEM, "cudaMalloc failed");
    o->allocs.push_back(*p);
    if (cudaMemset(*p, 0, bytes) != cudaSuccess) return li_fail(o, WF_ERR_CUDA, "cudaMemset failed");
    if (src && count && cudaMemcpy(*p, src, count * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
        return li_fail(o, WF_ERR_CUDA, "cudaMemcpy failed");
    return WF_OK;
}

int li_check(LiOwner* o, const char* what) {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return li_fail(o, WF_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    return WF_OK;
}

int li_sync(LiOwner* o, const char* what) {
    int rc = li_check(o, what);
    if (rc) return rc;
    if (cudaStreamSynchronize(o->stream) != cudaSuccess) return li_fail(o, WF_ERR_CUDA, std::string(what) + " failed");
    return WF_OK;
}

void li_release(LiOwner* o) {
    if (o->stream) cudaStreamSynchronize(o->stream);
    for (void* p : o->allocs) cudaFree(p);
    if (o->loop_host) cudaFreeHost(o->loop_host);
    if (o->stream) cudaStreamDestroy(o->stream);
}

// Device-side loop state of a handle (at create).
int li_alloc_loop(LiOwner* o) {
    if (cudaMalloc((void**)&o->loop, sizeof(LiLoop)) != cudaSuccess) return li_fail(o, WF_ERR_NOMEM, "cudaMalloc failed");
    o->allocs.push_back(o->loop);
    if (cudaHostAlloc((void**)&o->loop_host, sizeof(LiLoop), cudaHostAllocDefault) != cudaSuccess)
        return li_fail(o, WF_ERR_NOMEM, "cudaHostAlloc failed");
    return WF_OK;
}

// After a loop launch: the sub-step count (and the status) back to the host, one read per step.
int li_finish_loop(LiOwner* o, int64_t* substeps) {
    if (cudaMemcpyAsync(o->loop_host, o->loop, sizeof(LiLoop), cudaMemcpyDeviceToHost, o->stream) != cudaSuccess)
        return li_fail(o, WF_ERR_CUDA, "read-back of the sub-step loop failed");
    int rc = li_sync(o, "sub-step loop");
    if (rc) return rc;
    if (o->loop_host->status & 1)
        return li_fail(o, WF_ERR_SPIN, "a grid barrier of the sub-step loop ran out of its wait budget");
    if (o->loop_host->status & 2) return li_fail(o, WF_ERR_INVALID, "more than 1e7 sub-steps in one step");
    if (substeps) *substeps = o->loop_host->substeps;
    return WF_OK;
}

int li_open(LiOwner* o, int device) {
    o->device = device;
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&o->stream, cudaStreamNonBlocking) != cudaSuccess)
        return li_fail(o, WF_ERR_CUDA, "no CUDA device or stream");
    return WF_OK;
}

// the uploads ran on the legacy stream, which the non-blocking stream does not wait for
int li_finish_uploads(LiOwner* o) {
    if (cudaDeviceSynchronize() != cudaSuccess) return li_fail(o, WF_ERR_CUDA, "upload of the network failed");
    return WF_OK;
}

// Checks of a river network (host arrays); 0 or WF_ERR_INVALID with the message in g_li_error.
int li_check_river(int64_t n, int64_t n_active, int64_t n_edges, const int64_t* src, const int64_t* dst,
                   const double* zb, const double* flow_length, const double* flow_width, const double* zb_edge,
                   const double* width_edge, const double* length_edge, const double* mannings_n_sq_edge,
                   double alpha) {
    if (n <= 0 || n_active < 0 || n_active > n || n_edges < 0)
        return li_fail(nullptr, WF_ERR_INVALID, "sizes out of range");
    if (!src || !dst || !zb || !flow_length || !flow_width || !zb_edge || !width_edge || !length_edge ||
        !mannings_n_sq_edge)
        return li_fail(nullptr, WF_ERR_INVALID, "missing input array");
    if (!(alpha > 0.0)) return li_fail(nullptr, WF_ERR_INVALID, "alpha must be positive");
    for (int64_t k = 0; k < n_edges; ++k)
        if (src[k] < 0 || src[k] >= n || dst[k] < 0 || dst[k] >= n || src[k] == dst[k])
            return li_fail(nullptr, WF_ERR_INVALID, "edge cell index out of range");
    for (int64_t i = 0; i < n_active; ++i)
        if (!(flow_length[i] > 0.0) || !(flow_width[i] > 0.0))
            return li_fail(nullptr, WF_ERR_INVALID, "flow length and width must be positive on active cells");
    return WF_OK;
}

// Uploads a checked river network and its zeroed state; h from h_init (NULL: zero).
int li_upload_river(LiOwner* o, LiDev& d, int64_t n, int64_t n_active, int64_t n_edges, const int64_t* src,
                    const int64_t* dst, const double* zb, const double* flow_length, const double* flow_width,
                    const double* h_init, const double* zb_edge, const double* width_edge, const double* length_edge,
                    const double* mannings_n_sq_edge, double h_thresh, int32_t froude_limit, double alpha) {
    std::vector<int64_t> in_ptr, in_edge, out_ptr, out_edge;
    wfli::build_csr(n, n_edges, src, dst, in_ptr, in_edge, out_ptr, out_edge);
    d.n = n;
    d.n_active = n_active;
    d.n_edges = n_edges;
    d.n_dt = n;
    d.h_thresh = h_thresh;
    d.alpha = alpha;
    d.froude = froude_limit;
    int rc;
    int64_t *p_src, *p_dst, *p_ip, *p_ie, *p_op, *p_oe;
    double *p_zb, *p_fl, *p_fw, *p_zbe, *p_we, *p_le, *p_ne;
    if ((rc = li_upload(o, &p_src, src, n_edges)) || (rc = li_upload(o, &p_dst, dst, n_edges)) ||
        (rc = li_upload(o, &p_ip, (const int64_t*)in_ptr.data(), n + 1)) ||
        (rc = li_upload(o, &p_ie, (const int64_t*)in_edge.data(), n_edges)) ||
        (rc = li_upload(o, &p_op, (const int64_t*)out_ptr.data(), n + 1)) ||
        (rc = li_upload(o, &p_oe, (const int64_t*)out_edge.data(), n_edges)) || (rc = li_upload(o, &p_zb, zb, n)) ||
        (rc = li_upload(o, &p_fl, flow_length, n)) || (rc = li_upload(o, &p_fw, flow_width, n)) ||
        (rc = li_upload(o, &p_zbe, zb_edge, n_edges)) || (rc = li_upload(o, &p_we, width_edge, n_edges)) ||
        (rc = li_upload(o, &p_le, length_edge, n_edges)) || (rc = li_upload(o, &p_ne, mannings_n_sq_edge, n_edges)) ||
        (rc = li_upload(o, &d.h, h_init, n)) || (rc = li_upload<double>(o, &d.storage, nullptr, n)) ||
        (rc = li_upload<double>(o, &d.q, nullptr, n_edges)) || (rc = li_upload<double>(o, &d.q_prev, nullptr, n_edges)) ||
        (rc = li_upload<double>(o, &d.q_cum, nullptr, n_edges)) || (rc = li_upload<double>(o, &d.inwater, nullptr, n)) ||
        (rc = li_upload<double>(o, &d.dt_min, nullptr, 1)) || (rc = li_upload<double>(o, &d.error, nullptr, n)) ||
        (rc = li_upload<double>(o, &d.abstraction_cum, nullptr, n)))
        return rc;
    double *p_abs, *p_ext;
    if ((rc = li_upload<double>(o, &p_abs, nullptr, n)) || (rc = li_upload<double>(o, &p_ext, nullptr, n))) return rc;
    d.abstraction = p_abs;
    d.external_inflow = p_ext;
    d.src = p_src;
    d.dst = p_dst;
    d.in_ptr = p_ip;
    d.in_edge = p_ie;
    d.out_ptr = p_op;
    d.out_edge = p_oe;
    d.zb = p_zb;
    d.flow_length = p_fl;
    d.flow_width = p_fw;
    d.zb_e = p_zbe;
    d.width_e = p_we;
    d.length_e = p_le;
    d.nsq_e = p_ne;
    return WF_OK;
}

int li_copy_out(LiOwner* o, double* dst, const double* src, int64_t count) {
    if (count > 0 && (cudaMemcpyAsync(dst, src, count * sizeof(double), cudaMemcpyDeviceToHost, o->stream) !=
                          cudaSuccess ||
                      cudaStreamSynchronize(o->stream) != cudaSuccess))
        return li_fail(o, WF_ERR_CUDA, "copy failed");
    return WF_OK;
}

int li_copy_in(LiOwner* o, double* dst, const double* src, int64_t count) {
    if (count > 0 && (cudaMemcpyAsync(dst, src, count * sizeof(double), cudaMemcpyHostToDevice, o->stream) !=
                          cudaSuccess ||
                      cudaStreamSynchronize(o->stream) != cudaSuccess))
        return li_fail(o, WF_ERR_CUDA, "copy failed");
    return WF_OK;
}

}  // namespace

struct WfLiRiver : LiOwner {
    LiDev d{};
    double* q_avg = nullptr;            // q_cumulative / dt of the last wf_li_river_step
    std::vector<double> width, length;  // flow_width and flow_length of the active cells
};

struct WfLiDomain : LiOwner {
    wfli::LiLand L{};
    LiDev R{};
    wfli::LiRiverBC B{};
    double* qx_buf[2] = {nullptr, nullptr};  // discharges of this and the previous sub-step [n + 1]
    double* qy_buf[2] = {nullptr, nullptr};
    int cur = 0;                              // qx_buf[cur] / qy_buf[cur] hold the latest discharges
    double *qx_avg = nullptr, *qy_avg = nullptr, *q_avg = nullptr;
    double *runoff = nullptr, *ext = nullptr, *abstraction = nullptr;
    std::vector<int64_t> river_index;
    std::vector<double> xl, yl, r_width, r_length, bankfull_storage;
};

extern "C" {

// ---------------------------------------------------------------- river alone -------------

const char* wf_li_river_last_error(const WfLiRiver* r) { return r ? r->err.c_str() : g_li_error.c_str(); }

int32_t wf_li_river_create(int64_t n, int64_t n_active, int64_t n_edges, const int64_t* src, const int64_t* dst,
                           const double* zb, const double* flow_length, const double* flow_width,
                           const double* h_init, const double* zb_edge, const double* width_edge,
                           const double* length_edge, const double* mannings_n_sq_edge, double h_thresh,
                           int32_t froude_limit, double alpha, int32_t device, WfLiRiver** out) {
    if (!out) return li_fail(nullptr, WF_ERR_INVALID, "null output");
    *out = nullptr;
    if (!h_init) return li_fail(nullptr, WF_ERR_INVALID, "missing input array");
    int rc = li_check_river(n, n_active, n_edges, src, dst, zb, flow_length, flow_width, zb_edge, width_edge,
                            length_edge, mannings_n_sq_edge, alpha);
    if (rc) return rc;
    WfLiRiver* r = new WfLiRiver();
    if ((rc = li_open(r, device)) ||
        (rc = li_upload_river(r, r->d, n, n_active, n_edges, src, dst, zb, flow_length, flow_width, h_init, zb_edge,
                              width_edge, length_edge, mannings_n_sq_edge, h_thresh, froude_limit, alpha)) ||
        (rc = li_upload<double>(r, &r->q_avg, nullptr, n_edges)) || (rc = li_alloc_loop(r)) ||
        (rc = li_finish_uploads(r))) {
        g_li_error = r->err;
        wf_li_river_destroy(r);
        return rc;
    }
    r->width.assign(flow_width, flow_width + n_active);
    r->length.assign(flow_length, flow_length + n_active);
    *out = r;
    return WF_OK;
}

void wf_li_river_destroy(WfLiRiver* r) {
    if (!r) return;
    li_release(r);
    delete r;
}

int32_t wf_li_river_set_timestep_cells(WfLiRiver* r, int64_t n_cells) {
    if (!r || n_cells < 0 || n_cells > r->d.n) return li_fail(r, WF_ERR_INVALID, "cell count out of range");
    r->d.n_dt = n_cells;
    return WF_OK;
}

int32_t wf_li_river_set_manning(WfLiRiver* r, const double* slope_edge, const double* mannings_n_edge) {
    if (!r || !slope_edge || !mannings_n_edge) return li_fail(r, WF_ERR_INVALID, "null argument");
    const int64_t ne = r->d.n_edges;
    for (int64_t k = 0; k < ne; ++k)
        if (!(slope_edge[k] > 0.0) || !(mannings_n_edge[k] > 0.0))
            return li_fail(r, WF_ERR_INVALID, "edge slope and Manning's n must be positive");
    double *ps, *pn, *ph;
    int rc;
    if ((rc = li_upload(r, &ps, slope_edge, ne)) || (rc = li_upload(r, &pn, mannings_n_edge, ne)) ||
        (rc = li_upload<double>(r, &ph, nullptr, ne)) || (rc = li_finish_uploads(r)))
        return rc;
    r->d.slope_e = ps;
    r->d.n_e = pn;
    r->d.hf_e = ph;
    r->d.manning = 1;
    return WF_OK;
}

int32_t wf_li_river_set_inwater(WfLiRiver* r, const double* inwater) {
    if (!r || !inwater) return li_fail(r, WF_ERR_INVALID, "null argument");
    return li_copy_in(r, r->d.inwater, inwater, r->d.n);
}

int32_t wf_li_river_set_boundary(WfLiRiver* r, const double* external_inflow, const double* abstraction) {
    if (!r) return li_fail(r, WF_ERR_INVALID, "null argument");
    const int64_t n = r->d.n;
    std::vector<double> zero;
    if (!external_inflow || !abstraction) zero.assign(n, 0.0);
    int rc;
    if ((rc = li_copy_in(r, const_cast<double*>(r->d.external_inflow), external_inflow ? external_inflow : zero.data(),
                         n)) ||
        (rc = li_copy_in(r, const_cast<double*>(r->d.abstraction), abstraction ? abstraction : zero.data(), n)))
        return rc;
    return WF_OK;
}

int32_t wf_li_river_stable_timestep(WfLiRiver* r, double* dt) {
    if (!r || !dt) return li_fail(r, WF_ERR_INVALID, "null argument");
    li_dt_kernel<<<1, LI_DT_THREADS, 0, r->stream>>>(r->d);
    const int rc = li_check(r, "stable time step");
    if (rc) return rc;
    return li_copy_out(r, dt, r->d.dt_min, 1);
}

int32_t wf_li_river_substep(WfLiRiver* r, double dt_s) {
    if (!r || !(dt_s > 0.0)) return li_fail(r, WF_ERR_INVALID, "sub-step must be positive");
    if (r->d.n_edges > 0) li_edge_kernel<<<grid_of(r->d.n_edges), 256, 0, r->stream>>>(r->d, dt_s);
    if (r->d.n_active > 0) li_cell_kernel<<<grid_of(r->d.n_active), 256, 0, r->stream>>>(r->d, dt_s);
    return li_sync(r, "sub-step");
}

int32_t wf_li_river_step(WfLiRiver* r, double dt, int64_t* substeps) {
    if (!r || !(dt > 0.0)) return li_fail(r, WF_ERR_INVALID, "step must be positive");
    // set_flow_vars!: the cumulative discharge and abstraction restart each model step
    if ((r->d.n_edges > 0 &&
         cudaMemsetAsync(r->d.q_cum, 0, r->d.n_edges * sizeof(double), r->stream) != cudaSuccess) ||
        cudaMemsetAsync(r->d.abstraction_cum, 0, r->d.n * sizeof(double), r->stream) != cudaSuccess)
        return li_fail(r, WF_ERR_CUDA, "reset of the cumulative discharge failed");
    const int blocks = r->host_loop ? 0 : li_loop_blocks(li_river_loop_kernel, r->device,
                                                          std::max(r->d.n, r->d.n_edges));
    if (blocks > 0) {  // the sub-step loop on the device, one launch
        li_loop_init_kernel<<<1, 1, 0, r->stream>>>(r->loop);
        LiDev dd = r->d;
        LiLoop* lp = r->loop;
        double dtv = dt;
        void* args[] = {&dd, &lp, &dtv};
        if (cudaLaunchCooperativeKernel((const void*)li_river_loop_kernel, blocks, 256, args, 0, r->stream) !=
            cudaSuccess)
            return li_fail(r, WF_ERR_CUDA, "cooperative launch of the sub-step loop failed");
        if (r->d.n_edges > 0)
            li_average_kernel<<<grid_of(r->d.n_edges), 256, 0, r->stream>>>(r->d.q_cum, r->q_avg, r->d.n_edges, dt);
        return li_finish_loop(r, substeps);
    }
    double t = 0.0;
    int64_t k = 0;
    while (t < dt) {
        double dt_s;
        int rc = wf_li_river_stable_timestep(r, &dt_s);
        if (rc) return rc;
        if (t + dt_s > dt) dt_s = dt - t;  // check_timestepsize (routing/timestepping.jl:11-16)
        if ((rc = wf_li_river_substep(r, dt_s))) return rc;
        t += dt_s;
        if (++k > 10000000) return li_fail(r, WF_ERR_INVALID, "more than 1e7 sub-steps in one step");
    }
    if (r->d.n_edges > 0) {
        li_average_kernel<<<grid_of(r->d.n_edges), 256, 0, r->stream>>>(r->d.q_cum, r->q_avg, r->d.n_edges, dt);
        const int rc = li_sync(r, "average discharge");
        if (rc) return rc;
    }
    if (substeps) *substeps = k;
    return WF_OK;
}

int32_t wf_li_river_set_host_loop(WfLiRiver* r, int32_t host_loop) {
    if (!r) return WF_ERR_INVALID;
    r->host_loop = host_loop != 0;
    return WF_OK;
}

int32_t wf_li_river_set_state(WfLiRiver* r, const double* h, const double* q) {
    if (!r || !h) return li_fail(r, WF_ERR_INVALID, "null argument");
    std::vector<double> storage(r->d.n, 0.0);
    for (int64_t i = 0; i < r->d.n_active; ++i) storage[i] = h[i] * r->width[i] * r->length[i];
    int rc;
    if ((rc = li_copy_in(r, r->d.h, h, r->d.n)) || (rc = li_copy_in(r, r->d.storage, storage.data(), r->d.n)) ||
        (q && (rc = li_copy_in(r, r->d.q, q, r->d.n_edges))))
        return rc;
    return WF_OK;
}

int32_t wf_li_river_get(WfLiRiver* r, int32_t field, double* dst) {
    if (!r || !dst) return li_fail(r, WF_ERR_INVALID, "null argument");
    const double* src = field == 0   ? r->d.h
                        : field == 1 ? r->d.storage
                        : field == 2 ? r->d.q
                        : field == 3 ? r->d.q_cum
                        : field == 4 ? r->q_avg
                        : field == 5 ? r->d.error
                        : field == 6 ? r->d.abstraction_cum
                                     : nullptr;
    if (!src) return li_fail(r, WF_ERR_INVALID, "unknown field");
    return li_copy_out(r, dst, src, (field <= 1 || field >= 5) ? r->d.n : r->d.n_edges);
}

// ---------------------------------------------------------------- land with river ---------

const char* wf_li_domain_last_error(const WfLiDomain* d) { return d ? d->err.c_str() : g_li_error.c_str(); }

int32_t wf_li_domain_create(const WfLiLandGrid* land, const WfLiRiverNetwork* river, const double* h_river,
                            int32_t device, WfLiDomain** out) {
    if (!out) return li_fail(nullptr, WF_ERR_INVALID, "null output");
    *out = nullptr;
    if (!land || !river || !h_river) return li_fail(nullptr, WF_ERR_INVALID, "null argument");
    const WfLiRiverNetwork& rv = *river;
    int rc = li_check_river(rv.n, rv.n_active, rv.n_edges, rv.src, rv.dst, rv.zb, rv.flow_length, rv.flow_width,
                            rv.zb_edge, rv.width_edge, rv.length_edge, rv.mannings_n_sq_edge, rv.alpha);
    if (rc) return rc;
    if (!rv.bankfull_depth) return li_fail(nullptr, WF_ERR_INVALID, "missing input array");
    const WfLiLandGrid& ld = *land;
    const int64_t n = ld.n;
    if (n <= 0) return li_fail(nullptr, WF_ERR_INVALID, "land cell count must be positive");
    if (!ld.ind_x_up || !ld.ind_x_down || !ld.ind_y_up || !ld.ind_y_down || !ld.river_index || !ld.x_length ||
        !ld.y_length || !ld.elevation || !ld.mannings_n_sq || !ld.xwidth_at_edge || !ld.ywidth_at_edge)
        return li_fail(nullptr, WF_ERR_INVALID, "missing input array");
    if (!(ld.alpha > 0.0)) return li_fail(nullptr, WF_ERR_INVALID, "alpha must be positive");
    std::vector<int32_t> seen(rv.n_active, 0);
    for (int64_t i = 0; i < n; ++i) {
        const int64_t nb[4] = {ld.ind_x_up[i], ld.ind_x_down[i], ld.ind_y_up[i], ld.ind_y_down[i]};
        for (int64_t v : nb)
            if (v < 0 || v > n) return li_fail(nullptr, WF_ERR_INVALID, "land neighbour index out of range");
        if (!(ld.x_length[i] > 0.0) || !(ld.y_length[i] > 0.0))
            return li_fail(nullptr, WF_ERR_INVALID, "land cell lengths must be positive");
        const int64_t r = ld.river_index[i];
        if (r < -1 || r >= rv.n_active)
            return li_fail(nullptr, WF_ERR_INVALID, "river index must be -1 or an active river cell");
        if (r >= 0 && seen[r]++) return li_fail(nullptr, WF_ERR_INVALID, "two land cells hold one river cell");
    }
    for (int64_t r = 0; r < rv.n_active; ++r)
        if (!seen[r]) return li_fail(nullptr, WF_ERR_INVALID, "an active river cell lies in no land cell");
    std::vector<double> zx_max, zy_max, bankfull;
    wfli::land_edge_parameters(n, ld.ind_x_up, ld.ind_y_up, ld.elevation, zx_max, zy_max);
    wfli::bankfull_storage(rv.n, rv.bankfull_depth, rv.flow_width, rv.flow_length, bankfull);

    WfLiDomain* d = new WfLiDomain();
    wfli::LiLand& L = d->L;
    L.n = n;
    L.theta = ld.theta;
    L.h_thresh = ld.h_thresh;
    L.alpha = ld.alpha;
    L.froude = ld.froude_limit;
    int64_t *p_ixu, *p_ixd, *p_iyu, *p_iyd, *p_riv;
    double *p_xl, *p_yl, *p_z, *p_nsq, *p_xw, *p_yw, *p_zx, *p_zy, *p_bd, *p_bs;
    const double *c_zx = zx_max.data(), *c_zy = zy_max.data(), *c_bs = bankfull.data();
    if ((rc = li_open(d, device)) ||
        (rc = li_upload_river(d, d->R, rv.n, rv.n_active, rv.n_edges, rv.src, rv.dst, rv.zb, rv.flow_length,
                              rv.flow_width, h_river, rv.zb_edge, rv.width_edge, rv.length_edge,
                              rv.mannings_n_sq_edge, rv.h_thresh, rv.froude_limit, rv.alpha)) ||
        (rc = li_upload(d, &p_ixu, ld.ind_x_up, n)) || (rc = li_upload(d, &p_ixd, ld.ind_x_down, n)) ||
        (rc = li_upload(d, &p_iyu, ld.ind_y_up, n)) || (rc = li_upload(d, &p_iyd, ld.ind_y_down, n)) ||
        (rc = li_upload(d, &p_riv, ld.river_index, n)) || (rc = li_upload(d, &p_xl, ld.x_length, n)) ||
        (rc = li_upload(d, &p_yl, ld.y_length, n)) || (rc = li_upload(d, &p_z, ld.elevation, n)) ||
        (rc = li_upload(d, &p_nsq, ld.mannings_n_sq, n)) || (rc = li_upload(d, &p_xw, ld.xwidth_at_edge, n)) ||
        (rc = li_upload(d, &p_yw, ld.ywidth_at_edge, n)) || (rc = li_upload(d, &p_zx, c_zx, n)) ||
        (rc = li_upload(d, &p_zy, c_zy, n)) || (rc = li_upload(d, &p_bd, rv.bankfull_depth, rv.n)) ||
        (rc = li_upload(d, &p_bs, c_bs, rv.n)) || (rc = li_upload<double>(d, &d->runoff, nullptr, n)) ||
        (rc = li_upload<double>(d, &d->ext, nullptr, rv.n)) ||
        (rc = li_upload<double>(d, &d->abstraction, nullptr, rv.n)) ||
        (rc = li_upload<double>(d, &d->B.abstraction_cum, nullptr, rv.n)) ||
        (rc = li_upload<double>(d, &L.h, nullptr, n)) || (rc = li_upload<double>(d, &L.storage, nullptr, n)) ||
        (rc = li_upload<double>(d, &L.error, nullptr, n)) ||
        (rc = li_upload<double>(d, &d->qx_buf[0], nullptr, n + 1)) ||
        (rc = li_upload<double>(d, &d->qx_buf[1], nullptr, n + 1)) ||
        (rc = li_upload<double>(d, &d->qy_buf[0], nullptr, n + 1)) ||
        (rc = li_upload<double>(d, &d->qy_buf[1], nullptr, n + 1)) ||
        (rc = li_upload<double>(d, &L.qx_cum, nullptr, n + 1)) ||
        (rc = li_upload<double>(d, &L.qy_cum, nullptr, n + 1)) ||
        (rc = li_upload<double>(d, &d->qx_avg, nullptr, n + 1)) ||
        (rc = li_upload<double>(d, &d->qy_avg, nullptr, n + 1)) ||
        (rc = li_upload<double>(d, &d->q_avg, nullptr, rv.n_edges)) ||
        (rc = li_upload<double>(d, &L.dt_min, nullptr, 1)) || (rc = li_alloc_loop(d)) || (rc = li_finish_uploads(d))) {
        g_li_error = d->err;
        wf_li_domain_destroy(d);
        return rc;
    }
    d->R.n_dt = rv.n_active;  // the river's stable time step over its real cells
    L.ixu = p_ixu;
    L.ixd = p_ixd;
    L.iyu = p_iyu;
    L.iyd = p_iyd;
    L.river = p_riv;
    L.xl = p_xl;
    L.yl = p_yl;
    L.z = p_z;
    L.nsq = p_nsq;
    L.xw = p_xw;
    L.yw = p_yw;
    L.zx_max = p_zx;
    L.zy_max = p_zy;
    L.runoff = d->runoff;
    d->B.bankfull_depth = p_bd;
    d->B.bankfull_storage = p_bs;
    d->B.external_inflow = d->ext;
    d->B.abstraction = d->abstraction;
    d->river_index.assign(ld.river_index, ld.river_index + n);
    d->xl.assign(ld.x_length, ld.x_length + n);
    d->yl.assign(ld.y_length, ld.y_length + n);
    d->r_width.assign(rv.flow_width, rv.flow_width + rv.n);
    d->r_length.assign(rv.flow_length, rv.flow_length + rv.n);
    d->bankfull_storage = bankfull;
    *out = d;
    return WF_OK;
}

void wf_li_domain_destroy(WfLiDomain* d) {
    if (!d) return;
    li_release(d);
    delete d;
}

int32_t wf_li_domain_set_state(WfLiDomain* d, const double* h_land, const double* h_river, const double* qx,
                               const double* qy, const double* q_river) {
    if (!d || !h_land || !h_river) return li_fail(d, WF_ERR_INVALID, "null argument");
    const int64_t n = d->L.n, nr = d->R.n;
    // land storage (sbm_model.jl:135-150) and river storage of the active cells (:168-172)
    std::vector<double> storage(n), storage_river(nr, 0.0);
    for (int64_t i = 0; i < n; ++i) {
        const int64_t r = d->river_index[i];
        if (r >= 0)
            storage[i] = h_land[i] > 0.0 ? h_land[i] * d->xl[i] * d->yl[i] + d->bankfull_storage[r]
                                         : h_river[r] * d->r_width[r] * d->r_length[r];
        else
            storage[i] = h_land[i] * d->xl[i] * d->yl[i];
    }
    for (int64_t r = 0; r < d->R.n_active; ++r) storage_river[r] = h_river[r] * d->r_width[r] * d->r_length[r];
    int rc;
    if ((rc = li_copy_in(d, d->L.h, h_land, n)) || (rc = li_copy_in(d, d->L.storage, storage.data(), n)) ||
        (rc = li_copy_in(d, d->R.h, h_river, nr)) || (rc = li_copy_in(d, d->R.storage, storage_river.data(), nr)) ||
        (qx && (rc = li_copy_in(d, d->qx_buf[d->cur], qx, n))) ||
        (qy && (rc = li_copy_in(d, d->qy_buf[d->cur], qy, n))) ||
        (q_river && (rc = li_copy_in(d, d->R.q, q_river, d->R.n_edges))))
        return rc;
    return WF_OK;
}

int32_t wf_li_domain_set_inputs(WfLiDomain* d, const double* runoff, const double* external_inflow,
                                const double* abstraction) {
    if (!d || !runoff) return li_fail(d, WF_ERR_INVALID, "null argument");
    const int64_t nr = d->R.n;
    std::vector<double> zero;
    if (!external_inflow || !abstraction) zero.assign(nr, 0.0);
    int rc;
    if ((rc = li_copy_in(d, d->runoff, runoff, d->L.n)) ||
        (rc = li_copy_in(d, d->ext, external_inflow ? external_inflow : zero.data(), nr)) ||
        (rc = li_copy_in(d, d->abstraction, abstraction ? abstraction : zero.data(), nr)))
        return rc;
    return WF_OK;
}

int32_t wf_li_domain_stable_timestep(WfLiDomain* d, double* dt) {
    if (!d || !dt) return li_fail(d, WF_ERR_INVALID, "null argument");
    li_domain_dt_kernel<<<1, LI_DT_THREADS, 0, d->stream>>>(d->L, d->R);
    const int rc = li_check(d, "stable time step");
    if (rc) return rc;
    return li_copy_out(d, dt, d->L.dt_min, 1);
}

int32_t wf_li_domain_substep(WfLiDomain* d, double dt_s) {
    if (!d || !(dt_s > 0.0)) return li_fail(d, WF_ERR_INVALID, "sub-step must be positive");
    const int prev = d->cur, next = 1 - d->cur;
    d->L.qx0 = d->qx_buf[prev];
    d->L.qy0 = d->qy_buf[prev];
    d->L.qx = d->qx_buf[next];
    d->L.qy = d->qy_buf[next];
    li_land_flux_kernel<<<grid_of(d->L.n), 256, 0, d->stream>>>(d->L, dt_s);
    if (d->R.n_edges > 0) li_edge_kernel<<<grid_of(d->R.n_edges), 256, 0, d->stream>>>(d->R, dt_s);
    li_land_depth_kernel<<<grid_of(d->L.n), 256, 0, d->stream>>>(d->L, d->R, d->B, dt_s);
    d->cur = next;
    return li_sync(d, "sub-step");
}

namespace {
// set_flow_vars! of the river and the land (:1165-1166), the device sub-step loop (one
// cooperative launch) and the averages, on stream st; 0 blocks when the device cannot run it.
int li_domain_launch(WfLiDomain* d, double dt, cudaStream_t st, int blocks) {
    const int64_t n = d->L.n, ne = d->R.n_edges;
    if ((ne > 0 && cudaMemsetAsync(d->R.q_cum, 0, ne * sizeof(double), st) != cudaSuccess) ||
        cudaMemsetAsync(d->B.abstraction_cum, 0, d->R.n * sizeof(double), st) != cudaSuccess ||
        cudaMemsetAsync(d->L.qx_cum, 0, (n + 1) * sizeof(double), st) != cudaSuccess ||
        cudaMemsetAsync(d->L.qy_cum, 0, (n + 1) * sizeof(double), st) != cudaSuccess)
        return li_fail(d, WF_ERR_CUDA, "reset of the cumulative discharges failed");
    li_loop_init_kernel<<<1, 1, 0, st>>>(d->loop);
    wfli::LiLand LL = d->L;
    LiDev RR = d->R;
    wfli::LiRiverBC BB = d->B;
    LiLoop* lp = d->loop;
    double dtv = dt;
    double *qx0b = d->qx_buf[0], *qx1b = d->qx_buf[1], *qy0b = d->qy_buf[0], *qy1b = d->qy_buf[1];
    int cur0 = d->cur;
    void* args[] = {&LL, &RR, &BB, &lp, &dtv, &qx0b, &qx1b, &qy0b, &qy1b, &cur0};
    if (cudaLaunchCooperativeKernel((const void*)li_domain_loop_kernel, blocks, 256, args, 0, st) != cudaSuccess)
        return li_fail(d, WF_ERR_CUDA, "cooperative launch of the sub-step loop failed");
    if (ne > 0) li_average_kernel<<<grid_of(ne), 256, 0, st>>>(d->R.q_cum, d->q_avg, ne, dt);
    li_average_kernel<<<grid_of(n + 1), 256, 0, st>>>(d->L.qx_cum, d->qx_avg, n + 1, dt);
    li_average_kernel<<<grid_of(n + 1), 256, 0, st>>>(d->L.qy_cum, d->qy_avg, n + 1, dt);
    return li_check(d, "sub-step loop");
}

int li_domain_blocks(WfLiDomain* d) {
    const int64_t n = d->L.n, ne = d->R.n_edges;
    return li_loop_blocks(li_domain_loop_kernel, d->device, std::max(std::max(n + 1, d->R.n), ne));
}
}  // namespace

int32_t wf_li_domain_step(WfLiDomain* d, double dt, int64_t* substeps) {
    if (!d || !(dt > 0.0)) return li_fail(d, WF_ERR_INVALID, "step must be positive");
    const int64_t n = d->L.n, ne = d->R.n_edges;
    const int blocks = d->host_loop ? 0 : li_domain_blocks(d);
    if (blocks > 0) {  // the sub-step loop on the device, one launch
        int rc = li_domain_launch(d, dt, d->stream, blocks);
        if (rc) return rc;
        int64_t k = 0;
        rc = li_finish_loop(d, &k);
        if (rc) return rc;
        d->cur = (int)((d->cur + k) & 1);  // the buffer of the last sub-step's discharges
        if (substeps) *substeps = k;
        return WF_OK;
    }
    // set_flow_vars! of the river and the land (:1165-1166)
    if ((ne > 0 && cudaMemsetAsync(d->R.q_cum, 0, ne * sizeof(double), d->stream) != cudaSuccess) ||
        cudaMemsetAsync(d->B.abstraction_cum, 0, d->R.n * sizeof(double), d->stream) != cudaSuccess ||
        cudaMemsetAsync(d->L.qx_cum, 0, (n + 1) * sizeof(double), d->stream) != cudaSuccess ||
        cudaMemsetAsync(d->L.qy_cum, 0, (n + 1) * sizeof(double), d->stream) != cudaSuccess)
        return li_fail(d, WF_ERR_CUDA, "reset of the cumulative discharges failed");
    double t = 0.0;
    int64_t k = 0;
    while (t < dt) {
        double dt_s;
        int rc = wf_li_domain_stable_timestep(d, &dt_s);
        if (rc) return rc;
        if (t + dt_s > dt) dt_s = dt - t;  // check_timestepsize (routing/timestepping.jl:11-16)
        if ((rc = wf_li_domain_substep(d, dt_s))) return rc;
        t += dt_s;
        if (++k > 10000000) return li_fail(d, WF_ERR_INVALID, "more than 1e7 sub-steps in one step");
    }
    if (ne > 0) li_average_kernel<<<grid_of(ne), 256, 0, d->stream>>>(d->R.q_cum, d->q_avg, ne, dt);
    li_average_kernel<<<grid_of(n + 1), 256, 0, d->stream>>>(d->L.qx_cum, d->qx_avg, n + 1, dt);
    li_average_kernel<<<grid_of(n + 1), 256, 0, d->stream>>>(d->L.qy_cum, d->qy_avg, n + 1, dt);
    const int rc = li_sync(d, "average discharge");
    if (rc) return rc;
    if (substeps) *substeps = k;
    return WF_OK;
}

int32_t wf_li_domain_set_host_loop(WfLiDomain* d, int32_t host_loop) {
    if (!d) return WF_ERR_INVALID;
    d->host_loop = host_loop != 0;
    return WF_OK;
}

int32_t wf_li_domain_get(WfLiDomain* d, int32_t field, double* dst) {
    if (!d || !dst) return li_fail(d, WF_ERR_INVALID, "null argument");
    const int64_t n = d->L.n, nr = d->R.n, ne = d->R.n_edges;
    switch (field) {
        case WF_LI_LAND_H: return li_copy_out(d, dst, d->L.h, n);
        case WF_LI_LAND_STORAGE: return li_copy_out(d, dst, d->L.storage, n);
        case WF_LI_LAND_ERROR: return li_copy_out(d, dst, d->L.error, n);
        case WF_LI_LAND_QX: return li_copy_out(d, dst, d->qx_buf[d->cur], n);
        case WF_LI_LAND_QY: return li_copy_out(d, dst, d->qy_buf[d->cur], n);
        case WF_LI_LAND_QX_AVERAGE: return li_copy_out(d, dst, d->qx_avg, n);
        case WF_LI_LAND_QY_AVERAGE: return li_copy_out(d, dst, d->qy_avg, n);
        case WF_LI_RIVER_H: return li_copy_out(d, dst, d->R.h, nr);
        case WF_LI_RIVER_STORAGE: return li_copy_out(d, dst, d->R.storage, nr);
        case WF_LI_RIVER_Q: return li_copy_out(d, dst, d->R.q, ne);
        case WF_LI_RIVER_Q_AVERAGE: return li_copy_out(d, dst, d->q_avg, ne);
        case WF_LI_RIVER_ABSTRACTION_CUMULATIVE: return li_copy_out(d, dst, d->B.abstraction_cum, nr);
        default: return li_fail(d, WF_ERR_INVALID, "unknown field");
    }
}

}  // extern "C"

// ---------------------------------------------------------------- coupling to the SBM step ---

int wf_li_domain_couple_view(WfLiDomain* d, WfLiCoupleView* v, const int64_t** river_index_host) {
    if (!d || !v) return WF_ERR_INVALID;
    v->n = d->L.n;
    v->nr_total = d->R.n;
    v->n_active = d->R.n_active;
    v->n_edges = d->R.n_edges;
    v->runoff = d->runoff;
    v->ext = d->ext;
    v->abstraction = d->abstraction;
    v->abstraction_cum = d->B.abstraction_cum;
    v->h_land = d->L.h;
    v->storage = d->L.storage;
    v->h_river = d->R.h;
    v->storage_river = d->R.storage;
    v->q = d->R.q;
    v->q_avg = d->q_avg;
    v->qx_avg = d->qx_avg;
    v->qy_avg = d->qy_avg;
    v->ixd = d->L.ixd;
    v->iyd = d->L.iyd;
    v->river_index = d->L.river;
    v->in_ptr = d->R.in_ptr;
    v->in_edge = d->R.in_edge;
    v->out_ptr = d->R.out_ptr;
    v->out_edge = d->R.out_edge;
    if (river_index_host) *river_index_host = d->river_index.data();
    return WF_OK;
}

int wf_li_domain_enqueue_step(WfLiDomain* d, double dt, cudaStream_t stream) {
    if (!d || !(dt > 0.0)) return WF_ERR_INVALID;
    const int blocks = li_domain_blocks(d);
    if (blocks <= 0) return li_fail(d, WF_ERR_UNSUPPORTED, "the device cannot run the cooperative sub-step loop");
    return li_domain_launch(d, dt, stream, blocks);
}

int wf_li_domain_complete_step(WfLiDomain* d, int64_t* substeps, const char** err) {
    if (!d) return WF_ERR_INVALID;
    LiLoop host{};
    if (cudaMemcpy(&host, d->loop, sizeof(LiLoop), cudaMemcpyDeviceToHost) != cudaSuccess) {
        if (err) *err = "read-back of the local-inertial sub-step loop failed";
        return WF_ERR_CUDA;
    }
    if (host.status & 1) {
        if (err) *err = "a grid barrier of the local-inertial sub-step loop ran out of its wait budget";
        return WF_ERR_SPIN;
    }
    if (host.status & 2) {
        if (err) *err = "more than 1e7 local-inertial sub-steps in one step";
        return WF_ERR_INVALID;
    }
    d->cur = (int)((d->cur + host.substeps) & 1);
    if (substeps) *substeps = host.substeps;
    return WF_OK;
}
