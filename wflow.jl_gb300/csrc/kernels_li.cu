// kernels_li.cu -- local-inertial river flow on a staggered grid (include/wflow_gb300_li.h).
//
// Per sub-step: one thread per edge computes the edge discharge from the previous discharge and
// the water-surface slope (local_inertial_flow, Wflow/src/routing/surface/surface_process.jl:
// 88-115; the edge update of update_river_channel_flow!, surface_staggered_scheme.jl:326-385);
// then one thread per active cell sums the discharge of its incoming and outgoing edges (CSR
// lists in ascending edge order, the order of sum_at) and updates storage and depth
// (update_water_depth_and_storage!, :723-760). The stable sub-step is a min-reduction over the
// cells (:1004-1020). Every operation is FP64 in the reference's order; the translation unit is
// compiled without FMA contraction, and cbrt and sqrt are the library's own (wf_math.cuh), so
// the results equal the CPU oracle's. The per-edge and per-cell arithmetic lives in
// li_scheme.cuh.
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "li_scheme.cuh"
#include "wflow_gb300.h"
#include "wflow_gb300_li.h"

namespace {

using LiDev = wfli::LiNet;

__global__ void li_edge_kernel(LiDev d, double dt) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < d.n_edges;
         k += (int64_t)gridDim.x * blockDim.x)
        wfli::update_edge(d, k, dt);
}

__global__ void li_cell_kernel(LiDev d, double dt) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < d.n_active;
         i += (int64_t)gridDim.x * blockDim.x)
        wfli::update_cell(d, i, dt);
}

// min over the cells of the stable sub-step: one block of LI_DT_THREADS threads (the launch
// uses exactly that many; the shared array is sized for it)
constexpr int LI_DT_THREADS = 256;

__global__ void li_dt_kernel(LiDev d) {
    __shared__ double red[LI_DT_THREADS];
    double m = wfm::from_bits(0x7ff0000000000000ULL);
    for (int64_t i = threadIdx.x; i < d.n; i += blockDim.x) m = wfm::jmin(wfli::cell_timestep(d, i), m);
    red[threadIdx.x] = m;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] = wfm::jmin(red[threadIdx.x + w], red[threadIdx.x]);
        __syncthreads();
    }
    if (threadIdx.x == 0) *d.dt_min = wfli::finish_timestep(red[0]);
}

// q_average = q_cumulative / dt (average_flow_vars!, routing/surface/surface_kinwave.jl:283-290)
__global__ void li_average_kernel(LiDev d, double* q_avg, double dt) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < d.n_edges;
         k += (int64_t)gridDim.x * blockDim.x)
        q_avg[k] = d.q_cum[k] / dt;
}

int grid_of(int64_t n) {
    const int64_t g = (n + 255) / 256;
    return (int)(g < 1 ? 1 : (g > 65535 ? 65535 : g));
}

}  // namespace

struct WfLiRiver {
    LiDev d{};
    double* q_avg = nullptr;                  // q_cumulative / dt of the last wf_li_river_step
    std::vector<double> width, length;        // flow_width and flow_length of the active cells
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<void*> allocs;
    std::string err;
};

namespace {

thread_local std::string g_li_error;

int li_fail(WfLiRiver* r, int code, const std::string& msg) {
    if (r) r->err = msg;
    else g_li_error = msg;
    return code;
}

// device array of count values (at least one allocated), copied from src or zeroed
template <class T>
int li_upload(WfLiRiver* r, T** p, const T* src, size_t count) {
    const size_t bytes = (count ? count : 1) * sizeof(T);
    if (cudaMalloc((void**)p, bytes) != cudaSuccess) return li_fail(r, WF_ERR_NOMEM, "cudaMalloc failed");
    r->allocs.push_back(*p);
    if (cudaMemset(*p, 0, bytes) != cudaSuccess) return li_fail(r, WF_ERR_CUDA, "cudaMemset failed");
    if (src && count && cudaMemcpy(*p, src, count * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
        return li_fail(r, WF_ERR_CUDA, "cudaMemcpy failed");
    return WF_OK;
}

int li_check(WfLiRiver* r, const char* what) {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return li_fail(r, WF_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    return WF_OK;
}

}  // namespace

extern "C" {

const char* wf_li_river_last_error(const WfLiRiver* r) { return r ? r->err.c_str() : g_li_error.c_str(); }

int32_t wf_li_river_create(int64_t n, int64_t n_active, int64_t n_edges, const int64_t* src, const int64_t* dst,
                           const double* zb, const double* flow_length, const double* flow_width,
                           const double* h_init, const double* zb_edge, const double* width_edge,
                           const double* length_edge, const double* mannings_n_sq_edge, double h_thresh,
                           int32_t froude_limit, double alpha, int32_t device, WfLiRiver** out) {
    if (!out) return li_fail(nullptr, WF_ERR_INVALID, "null output");
    *out = nullptr;
    if (n <= 0 || n_active < 0 || n_active > n || n_edges < 0)
        return li_fail(nullptr, WF_ERR_INVALID, "sizes out of range");
    if (!src || !dst || !zb || !flow_length || !flow_width || !h_init || !zb_edge || !width_edge || !length_edge ||
        !mannings_n_sq_edge)
        return li_fail(nullptr, WF_ERR_INVALID, "missing input array");
    if (!(alpha > 0.0)) return li_fail(nullptr, WF_ERR_INVALID, "alpha must be positive");
    for (int64_t k = 0; k < n_edges; ++k)
        if (src[k] < 0 || src[k] >= n || dst[k] < 0 || dst[k] >= n || src[k] == dst[k])
            return li_fail(nullptr, WF_ERR_INVALID, "edge cell index out of range");
    for (int64_t i = 0; i < n_active; ++i)
        if (!(flow_length[i] > 0.0) || !(flow_width[i] > 0.0))
            return li_fail(nullptr, WF_ERR_INVALID, "flow length and width must be positive on active cells");
    std::vector<int64_t> in_cnt, in_edge, out_cnt, out_edge;
    wfli::build_csr(n, n_edges, src, dst, in_cnt, in_edge, out_cnt, out_edge);
    WfLiRiver* r = new WfLiRiver();
    r->device = device;
    auto fail = [&](int rc) {
        g_li_error = r->err;
        wf_li_river_destroy(r);
        return rc;
    };
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking) !=
                                                    cudaSuccess) {
        li_fail(r, WF_ERR_CUDA, "no CUDA device or stream");
        return fail(WF_ERR_CUDA);
    }
    LiDev& d = r->d;
    d.n = n;
    d.n_active = n_active;
    d.n_edges = n_edges;
    d.h_thresh = h_thresh;
    d.alpha = alpha;
    d.froude = froude_limit;
    int rc;
    int64_t *p_src, *p_dst, *p_ip, *p_ie, *p_op, *p_oe;
    double *p_zb, *p_fl, *p_fw, *p_zbe, *p_we, *p_le, *p_ne;
    if ((rc = li_upload(r, &p_src, src, n_edges)) || (rc = li_upload(r, &p_dst, dst, n_edges)) ||
        (rc = li_upload(r, &p_ip, in_cnt.data(), n + 1)) || (rc = li_upload(r, &p_ie, in_edge.data(), n_edges)) ||
        (rc = li_upload(r, &p_op, out_cnt.data(), n + 1)) || (rc = li_upload(r, &p_oe, out_edge.data(), n_edges)) ||
        (rc = li_upload(r, &p_zb, zb, n)) || (rc = li_upload(r, &p_fl, flow_length, n)) ||
        (rc = li_upload(r, &p_fw, flow_width, n)) || (rc = li_upload(r, &p_zbe, zb_edge, n_edges)) ||
        (rc = li_upload(r, &p_we, width_edge, n_edges)) || (rc = li_upload(r, &p_le, length_edge, n_edges)) ||
        (rc = li_upload(r, &p_ne, mannings_n_sq_edge, n_edges)) || (rc = li_upload(r, &d.h, h_init, n)) ||
        (rc = li_upload<double>(r, &d.storage, nullptr, n)) || (rc = li_upload<double>(r, &d.q, nullptr, n_edges)) ||
        (rc = li_upload<double>(r, &d.q_prev, nullptr, n_edges)) ||
        (rc = li_upload<double>(r, &d.q_cum, nullptr, n_edges)) ||
        (rc = li_upload<double>(r, &d.inwater, nullptr, n)) || (rc = li_upload<double>(r, &d.dt_min, nullptr, 1)) ||
        (rc = li_upload<double>(r, &r->q_avg, nullptr, n_edges)))
        return fail(rc);
    // the uploads ran on the legacy stream, which the non-blocking stream does not wait for
    if (cudaDeviceSynchronize() != cudaSuccess) {
        li_fail(r, WF_ERR_CUDA, "upload of the network failed");
        return fail(WF_ERR_CUDA);
    }
    r->width.assign(flow_width, flow_width + n_active);
    r->length.assign(flow_length, flow_length + n_active);
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
    *out = r;
    return WF_OK;
}

void wf_li_river_destroy(WfLiRiver* r) {
    if (!r) return;
    if (r->stream) cudaStreamSynchronize(r->stream);
    for (void* p : r->allocs) cudaFree(p);
    if (r->stream) cudaStreamDestroy(r->stream);
    delete r;
}

int32_t wf_li_river_set_inwater(WfLiRiver* r, const double* inwater) {
    if (!r || !inwater) return li_fail(r, WF_ERR_INVALID, "null argument");
    if (cudaMemcpyAsync(r->d.inwater, inwater, r->d.n * sizeof(double), cudaMemcpyHostToDevice, r->stream) !=
            cudaSuccess ||
        cudaStreamSynchronize(r->stream) != cudaSuccess)
        return li_fail(r, WF_ERR_CUDA, "copy of the inflow failed");
    return WF_OK;
}

int32_t wf_li_river_stable_timestep(WfLiRiver* r, double* dt) {
    if (!r || !dt) return li_fail(r, WF_ERR_INVALID, "null argument");
    li_dt_kernel<<<1, LI_DT_THREADS, 0, r->stream>>>(r->d);
    int rc = li_check(r, "stable time step");
    if (rc) return rc;
    if (cudaMemcpyAsync(dt, r->d.dt_min, sizeof(double), cudaMemcpyDeviceToHost, r->stream) != cudaSuccess ||
        cudaStreamSynchronize(r->stream) != cudaSuccess)
        return li_fail(r, WF_ERR_CUDA, "read of the time step failed");
    return WF_OK;
}

int32_t wf_li_river_substep(WfLiRiver* r, double dt_s) {
    if (!r || !(dt_s > 0.0)) return li_fail(r, WF_ERR_INVALID, "sub-step must be positive");
    if (r->d.n_edges > 0) li_edge_kernel<<<grid_of(r->d.n_edges), 256, 0, r->stream>>>(r->d, dt_s);
    if (r->d.n_active > 0) li_cell_kernel<<<grid_of(r->d.n_active), 256, 0, r->stream>>>(r->d, dt_s);
    int rc = li_check(r, "sub-step");
    if (rc) return rc;
    if (cudaStreamSynchronize(r->stream) != cudaSuccess) return li_fail(r, WF_ERR_CUDA, "sub-step failed");
    return WF_OK;
}

int32_t wf_li_river_step(WfLiRiver* r, double dt, int64_t* substeps) {
    if (!r || !(dt > 0.0)) return li_fail(r, WF_ERR_INVALID, "step must be positive");
    // set_flow_vars!: the cumulative discharge restarts each model step
    if (r->d.n_edges > 0 && cudaMemsetAsync(r->d.q_cum, 0, r->d.n_edges * sizeof(double), r->stream) != cudaSuccess)
        return li_fail(r, WF_ERR_CUDA, "reset of the cumulative discharge failed");
    double t = 0.0;
    int64_t k = 0;
    while (t < dt) {
        double dt_s;
        int rc = wf_li_river_stable_timestep(r, &dt_s);
        if (rc) return rc;
        if (t + dt_s > dt) dt_s = dt - t;  // check_timestepsize (routing/timestepping.jl:30-37)
        if ((rc = wf_li_river_substep(r, dt_s))) return rc;
        t += dt_s;
        if (++k > 10000000) return li_fail(r, WF_ERR_INVALID, "more than 1e7 sub-steps in one step");
    }
    if (r->d.n_edges > 0) {
        li_average_kernel<<<grid_of(r->d.n_edges), 256, 0, r->stream>>>(r->d, r->q_avg, dt);
        const int rc = li_check(r, "average discharge");
        if (rc) return rc;
        if (cudaStreamSynchronize(r->stream) != cudaSuccess) return li_fail(r, WF_ERR_CUDA, "average discharge failed");
    }
    if (substeps) *substeps = k;
    return WF_OK;
}

int32_t wf_li_river_set_state(WfLiRiver* r, const double* h, const double* q) {
    if (!r || !h) return li_fail(r, WF_ERR_INVALID, "null argument");
    const int64_t na = r->d.n_active;
    std::vector<double> storage(r->d.n, 0.0);
    for (int64_t i = 0; i < na; ++i) storage[i] = h[i] * r->width[i] * r->length[i];
    if (cudaMemcpyAsync(r->d.h, h, r->d.n * sizeof(double), cudaMemcpyHostToDevice, r->stream) != cudaSuccess ||
        cudaMemcpyAsync(r->d.storage, storage.data(), r->d.n * sizeof(double), cudaMemcpyHostToDevice, r->stream) !=
            cudaSuccess ||
        (q && r->d.n_edges > 0 &&
         cudaMemcpyAsync(r->d.q, q, r->d.n_edges * sizeof(double), cudaMemcpyHostToDevice, r->stream) != cudaSuccess) ||
        cudaStreamSynchronize(r->stream) != cudaSuccess)
        return li_fail(r, WF_ERR_CUDA, "copy of the state failed");
    return WF_OK;
}

int32_t wf_li_river_get(WfLiRiver* r, int32_t field, double* dst) {
    if (!r || !dst) return li_fail(r, WF_ERR_INVALID, "null argument");
    const double* src = field == 0   ? r->d.h
                        : field == 1 ? r->d.storage
                        : field == 2 ? r->d.q
                        : field == 3 ? r->d.q_cum
                        : field == 4 ? r->q_avg
                                     : nullptr;
    if (!src) return li_fail(r, WF_ERR_INVALID, "unknown field");
    const int64_t cnt = field <= 1 ? r->d.n : r->d.n_edges;
    if (cnt > 0 && (cudaMemcpyAsync(dst, src, cnt * sizeof(double), cudaMemcpyDeviceToHost, r->stream) != cudaSuccess ||
                    cudaStreamSynchronize(r->stream) != cudaSuccess))
        return li_fail(r, WF_ERR_CUDA, "copy failed");
    return WF_OK;
}

}  // extern "C"
