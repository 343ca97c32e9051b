// kernels_snow.cu -- lateral snow transport and the HBV glacier on the GPU
// (include/wflow_gb300_snow.h). The glacier is one element-wise kernel over the cells
// (glacier_hbv in snow_scheme.cuh).
//
// The capacities of all cells come first (from the states before the move); then the cells are
// swept level by level from the leaves (a cell's level is one more than its highest upstream
// level), one launch per level with one thread per cell of the level: every upstream hand-off a
// cell adds is final when its level starts. Each thread adds its upstream hand-offs in the
// topological-sort order of the upstream cells, so the result equals the reference's sequential
// sweep bit for bit. snow_out and snow_in follow in two element-wise passes. The arithmetic is in
// snow_scheme.cuh; the unit is compiled without FMA contraction.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "snow_scheme.cuh"
#include "wflow_gb300.h"
#include "wflow_gb300_snow.h"

namespace {

using wfsn::SnowNet;

__global__ void snow_capacity_kernel(SnowNet d, double dt) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < d.n; i += (int64_t)gridDim.x * blockDim.x)
        wfsn::capacities(d, i, dt);
}

__global__ void snow_level_kernel(SnowNet d, const int64_t* cells, int64_t begin, int64_t end, double dt) {
    for (int64_t k = begin + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < end;
         k += (int64_t)gridDim.x * blockDim.x)
        wfsn::transport_cell(d, cells[k], dt);
}

__global__ void snow_out_kernel(SnowNet d) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < d.n; i += (int64_t)gridDim.x * blockDim.x)
        wfsn::out_cell(d, i);
}

struct GlacierDev {
    int64_t n;
    const double *fraction, *ttm, *cfmax, *sifrac, *temperature;
    double *snow, *store, *melt;
    double max_rate;
};

__global__ void glacier_kernel(GlacierDev g, double dt) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < g.n; i += (int64_t)gridDim.x * blockDim.x) {
        double snow, store, melt;
        wfsn::glacier_hbv(g.fraction[i], g.store[i], g.snow[i], g.temperature[i], g.ttm[i], g.cfmax[i], g.sifrac[i],
                          g.max_rate, dt, &snow, &store, &melt);
        g.snow[i] = snow;
        g.store[i] = store;
        g.melt[i] = melt;
    }
}

__global__ void snow_in_kernel(SnowNet d) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < d.n; i += (int64_t)gridDim.x * blockDim.x)
        wfsn::in_cell(d, i);
}

int grid_of(int64_t n) {
    const int64_t g = (n + 255) / 256;
    return (int)(g < 1 ? 1 : (g > 65535 ? 65535 : g));
}

thread_local std::string g_snow_error;

}  // namespace

struct WfGlacier {
    GlacierDev g{};
    cudaStream_t stream = nullptr;
    std::vector<void*> allocs;
    std::string err;
};

struct WfSnowTransport {
    SnowNet d{};
    int64_t* level_cells = nullptr;    // cells ordered by level
    std::vector<int64_t> level_ptr;    // cells of level l: level_cells[level_ptr[l] .. level_ptr[l + 1])
    cudaStream_t stream = nullptr;
    std::vector<void*> allocs;
    std::string err;
};

namespace {

int snow_fail(WfSnowTransport* t, int code, const std::string& msg) {
    if (t) t->err = msg;
    else g_snow_error = msg;
    return code;
}

template <class T>
int snow_alloc(WfSnowTransport* t, T** p, const T* src, int64_t count) {
    const size_t bytes = (size_t)(count > 0 ? count : 1) * sizeof(T);
    if (cudaMalloc((void**)p, bytes) != cudaSuccess) return snow_fail(t, WF_ERR_NOMEM, "cudaMalloc failed");
    t->allocs.push_back(*p);
    if (cudaMemset(*p, 0, bytes) != cudaSuccess) return snow_fail(t, WF_ERR_CUDA, "cudaMemset failed");
    if (src && count > 0 && cudaMemcpy(*p, src, count * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
        return snow_fail(t, WF_ERR_CUDA, "cudaMemcpy failed");
    return WF_OK;
}

}  // namespace

extern "C" {

const char* wf_snow_transport_last_error(const WfSnowTransport* t) {
    return t ? t->err.c_str() : g_snow_error.c_str();
}

void wf_snow_transport_destroy(WfSnowTransport* t) {
    if (!t) return;
    if (t->stream) cudaStreamSynchronize(t->stream);
    for (void* p : t->allocs) cudaFree(p);
    if (t->stream) cudaStreamDestroy(t->stream);
    delete t;
}

int64_t wf_snow_transport_levels(const WfSnowTransport* t) { return t ? (int64_t)t->level_ptr.size() - 1 : 0; }

int32_t wf_snow_transport_create(int64_t n, const int32_t* ds, const int64_t* order, const int32_t* ups_ds,
                                 const double* slope, int32_t device, WfSnowTransport** out) {
    if (!out) return snow_fail(nullptr, WF_ERR_INVALID, "null output");
    *out = nullptr;
    if (n <= 0 || !ds || !order || !slope) return snow_fail(nullptr, WF_ERR_INVALID, "missing input");
    if (!ups_ds) ups_ds = ds;
    std::vector<int64_t> pos(n, -1);
    for (int64_t k = 0; k < n; ++k) {
        if (order[k] < 0 || order[k] >= n || pos[order[k]] >= 0)
            return snow_fail(nullptr, WF_ERR_INVALID, "order is not a permutation of the cells");
        pos[order[k]] = k;
    }
    for (int64_t i = 0; i < n; ++i) {
        if (ds[i] < -1 || ds[i] >= n || ups_ds[i] < -1 || ups_ds[i] >= n || ds[i] == i || ups_ds[i] == i)
            return snow_fail(nullptr, WF_ERR_INVALID, "downstream index out of range");
        if (ds[i] >= 0 && pos[i] >= pos[ds[i]])
            return snow_fail(nullptr, WF_ERR_INVALID, "order puts a cell after its downstream cell");
    }
    // upstream lists in topological-sort order (the order accucapacityflux! hands material on)
    std::vector<int64_t> up_ptr(n + 1, 0), up_cell(n), in_ptr(n + 1, 0), in_cell;
    for (int64_t i = 0; i < n; ++i)
        if (ds[i] >= 0) up_ptr[ds[i] + 1]++;
    for (int64_t i = 0; i < n; ++i) up_ptr[i + 1] += up_ptr[i];
    std::vector<int64_t> fill(up_ptr.begin(), up_ptr.end() - 1);
    for (int64_t k = 0; k < n; ++k) {
        const int64_t u = order[k];
        if (ds[u] >= 0) up_cell[fill[ds[u]]++] = u;
    }
    // upstream lists for snow_in in ascending cell order
    int64_t n_in = 0;
    for (int64_t i = 0; i < n; ++i)
        if (ups_ds[i] >= 0) {
            in_ptr[ups_ds[i] + 1]++;
            ++n_in;
        }
    for (int64_t i = 0; i < n; ++i) in_ptr[i + 1] += in_ptr[i];
    in_cell.assign(n_in, 0);
    fill.assign(in_ptr.begin(), in_ptr.end() - 1);
    for (int64_t i = 0; i < n; ++i)
        if (ups_ds[i] >= 0) in_cell[fill[ups_ds[i]]++] = i;
    // levels: one more than the highest upstream level, computed along the order
    std::vector<int64_t> level(n, 0);
    int64_t n_levels = 0;
    for (int64_t k = 0; k < n; ++k) {
        const int64_t v = order[k];
        n_levels = std::max(n_levels, level[v] + 1);
        if (ds[v] >= 0) level[ds[v]] = std::max(level[ds[v]], level[v] + 1);
    }
    WfSnowTransport* t = new WfSnowTransport();
    t->level_ptr.assign(n_levels + 1, 0);
    for (int64_t i = 0; i < n; ++i) t->level_ptr[level[i] + 1]++;
    for (int64_t l = 0; l < n_levels; ++l) t->level_ptr[l + 1] += t->level_ptr[l];
    std::vector<int64_t> cells(n);
    fill.assign(t->level_ptr.begin(), t->level_ptr.end() - 1);
    for (int64_t i = 0; i < n; ++i) cells[fill[level[i]]++] = i;

    SnowNet& d = t->d;
    d.n = n;
    int rc;
    int32_t* p_ds;
    int64_t *p_up_ptr, *p_up_cell, *p_in_ptr, *p_in_cell;
    double* p_slope;
    const int64_t *c_up_ptr = up_ptr.data(), *c_up_cell = up_cell.data(), *c_in_ptr = in_ptr.data(),
                  *c_in_cell = in_cell.data(), *c_cells = cells.data();
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&t->stream, cudaStreamNonBlocking) != cudaSuccess)
        rc = snow_fail(t, WF_ERR_CUDA, "no CUDA device or stream");
    else if ((rc = snow_alloc(t, &p_ds, ds, n)) || (rc = snow_alloc(t, &p_up_ptr, c_up_ptr, n + 1)) ||
             (rc = snow_alloc(t, &p_up_cell, c_up_cell, n)) || (rc = snow_alloc(t, &p_in_ptr, c_in_ptr, n + 1)) ||
             (rc = snow_alloc(t, &p_in_cell, c_in_cell, n_in)) || (rc = snow_alloc(t, &p_slope, slope, n)) ||
             (rc = snow_alloc(t, &t->level_cells, c_cells, n)) ||
             (rc = snow_alloc<double>(t, &d.m1, nullptr, n)) || (rc = snow_alloc<double>(t, &d.m2, nullptr, n)) ||
             (rc = snow_alloc<double>(t, &d.cap1, nullptr, n)) || (rc = snow_alloc<double>(t, &d.cap2, nullptr, n)) ||
             (rc = snow_alloc<double>(t, &d.hand1, nullptr, n)) ||
             (rc = snow_alloc<double>(t, &d.hand2, nullptr, n)) || (rc = snow_alloc<double>(t, &d.out1, nullptr, n)) ||
             (rc = snow_alloc<double>(t, &d.out2, nullptr, n)) ||
             (rc = snow_alloc<double>(t, &d.snow_out, nullptr, n)) ||
             (rc = snow_alloc<double>(t, &d.snow_in, nullptr, n)))
        ;
    else if (cudaDeviceSynchronize() != cudaSuccess)  // the uploads ran on the legacy stream
        rc = snow_fail(t, WF_ERR_CUDA, "upload failed");
    if (rc) {
        g_snow_error = t->err;
        wf_snow_transport_destroy(t);
        return rc;
    }
    d.ds = p_ds;
    d.up_ptr = p_up_ptr;
    d.up_cell = p_up_cell;
    d.in_ptr = p_in_ptr;
    d.in_cell = p_in_cell;
    d.slope = p_slope;
    *out = t;
    return WF_OK;
}

int32_t wf_snow_transport_run(WfSnowTransport* t, double dt, double* snow_storage, double* snow_water,
                              double* snow_out, double* snow_in) {
    if (!t || !snow_storage || !snow_water || !snow_out || !snow_in || !(dt > 0.0))
        return snow_fail(t, WF_ERR_INVALID, "null argument or non-positive dt");
    const SnowNet& d = t->d;
    const size_t bytes = (size_t)d.n * sizeof(double);
    if (cudaMemcpyAsync(d.m1, snow_storage, bytes, cudaMemcpyHostToDevice, t->stream) != cudaSuccess ||
        cudaMemcpyAsync(d.m2, snow_water, bytes, cudaMemcpyHostToDevice, t->stream) != cudaSuccess)
        return snow_fail(t, WF_ERR_CUDA, "upload of the snow states failed");
    snow_capacity_kernel<<<grid_of(d.n), 256, 0, t->stream>>>(d, dt);
    for (size_t l = 0; l + 1 < t->level_ptr.size(); ++l) {
        const int64_t b = t->level_ptr[l], e = t->level_ptr[l + 1];
        snow_level_kernel<<<grid_of(e - b), 256, 0, t->stream>>>(d, t->level_cells, b, e, dt);
    }
    snow_out_kernel<<<grid_of(d.n), 256, 0, t->stream>>>(d);
    snow_in_kernel<<<grid_of(d.n), 256, 0, t->stream>>>(d);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return snow_fail(t, WF_ERR_CUDA, std::string("snow transport: ") + cudaGetErrorString(e));
    if (cudaMemcpyAsync(snow_storage, d.m1, bytes, cudaMemcpyDeviceToHost, t->stream) != cudaSuccess ||
        cudaMemcpyAsync(snow_water, d.m2, bytes, cudaMemcpyDeviceToHost, t->stream) != cudaSuccess ||
        cudaMemcpyAsync(snow_out, d.snow_out, bytes, cudaMemcpyDeviceToHost, t->stream) != cudaSuccess ||
        cudaMemcpyAsync(snow_in, d.snow_in, bytes, cudaMemcpyDeviceToHost, t->stream) != cudaSuccess ||
        cudaStreamSynchronize(t->stream) != cudaSuccess)
        return snow_fail(t, WF_ERR_CUDA, "snow transport failed");
    return WF_OK;
}

// ---------------------------------------------------------------- glacier ------------------

namespace {

int glacier_fail(WfGlacier* g, int code, const std::string& msg) {
    if (g) g->err = msg;
    else g_snow_error = msg;
    return code;
}

int glacier_alloc(WfGlacier* g, double** p, const double* src, int64_t n) {
    if (cudaMalloc((void**)p, (size_t)n * sizeof(double)) != cudaSuccess)
        return glacier_fail(g, WF_ERR_NOMEM, "cudaMalloc failed");
    g->allocs.push_back(*p);
    if (src && cudaMemcpy(*p, src, (size_t)n * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
        return glacier_fail(g, WF_ERR_CUDA, "cudaMemcpy failed");
    return WF_OK;
}

}  // namespace

const char* wf_glacier_last_error(const WfGlacier* g) { return g ? g->err.c_str() : g_snow_error.c_str(); }

void wf_glacier_destroy(WfGlacier* g) {
    if (!g) return;
    if (g->stream) cudaStreamSynchronize(g->stream);
    for (void* p : g->allocs) cudaFree(p);
    if (g->stream) cudaStreamDestroy(g->stream);
    delete g;
}

int32_t wf_glacier_create(int64_t n, const double* glacier_fraction, const double* temperature_threshold_melt,
                          const double* degree_day_factor, const double* snow_to_ice_fraction,
                          double maximum_snow_to_ice_rate, int32_t device, WfGlacier** out) {
    if (!out) return glacier_fail(nullptr, WF_ERR_INVALID, "null output");
    *out = nullptr;
    if (n <= 0 || !glacier_fraction || !temperature_threshold_melt || !degree_day_factor || !snow_to_ice_fraction)
        return glacier_fail(nullptr, WF_ERR_INVALID, "missing input");
    WfGlacier* g = new WfGlacier();
    GlacierDev& d = g->g;
    d.n = n;
    d.max_rate = maximum_snow_to_ice_rate;
    double *p_f, *p_t, *p_c, *p_s, *p_temp;
    int rc;
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking) != cudaSuccess)
        rc = glacier_fail(g, WF_ERR_CUDA, "no CUDA device or stream");
    else if ((rc = glacier_alloc(g, &p_f, glacier_fraction, n)) ||
             (rc = glacier_alloc(g, &p_t, temperature_threshold_melt, n)) ||
             (rc = glacier_alloc(g, &p_c, degree_day_factor, n)) ||
             (rc = glacier_alloc(g, &p_s, snow_to_ice_fraction, n)) || (rc = glacier_alloc(g, &p_temp, nullptr, n)) ||
             (rc = glacier_alloc(g, &d.snow, nullptr, n)) || (rc = glacier_alloc(g, &d.store, nullptr, n)) ||
             (rc = glacier_alloc(g, &d.melt, nullptr, n)))
        ;
    else if (cudaDeviceSynchronize() != cudaSuccess)  // the uploads ran on the legacy stream
        rc = glacier_fail(g, WF_ERR_CUDA, "upload failed");
    if (rc) {
        g_snow_error = g->err;
        wf_glacier_destroy(g);
        return rc;
    }
    d.fraction = p_f;
    d.ttm = p_t;
    d.cfmax = p_c;
    d.sifrac = p_s;
    d.temperature = p_temp;
    *out = g;
    return WF_OK;
}

int32_t wf_glacier_run(WfGlacier* g, double dt, const double* temperature, double* snow_storage,
                       double* glacier_store, double* glacier_melt) {
    if (!g || !temperature || !snow_storage || !glacier_store || !glacier_melt || !(dt > 0.0))
        return glacier_fail(g, WF_ERR_INVALID, "null argument or non-positive dt");
    const GlacierDev& d = g->g;
    const size_t bytes = (size_t)d.n * sizeof(double);
    if (cudaMemcpyAsync((void*)d.temperature, temperature, bytes, cudaMemcpyHostToDevice, g->stream) != cudaSuccess ||
        cudaMemcpyAsync(d.snow, snow_storage, bytes, cudaMemcpyHostToDevice, g->stream) != cudaSuccess ||
        cudaMemcpyAsync(d.store, glacier_store, bytes, cudaMemcpyHostToDevice, g->stream) != cudaSuccess)
        return glacier_fail(g, WF_ERR_CUDA, "upload failed");
    glacier_kernel<<<grid_of(d.n), 256, 0, g->stream>>>(d, dt);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return glacier_fail(g, WF_ERR_CUDA, std::string("glacier: ") + cudaGetErrorString(e));
    if (cudaMemcpyAsync(snow_storage, d.snow, bytes, cudaMemcpyDeviceToHost, g->stream) != cudaSuccess ||
        cudaMemcpyAsync(glacier_store, d.store, bytes, cudaMemcpyDeviceToHost, g->stream) != cudaSuccess ||
        cudaMemcpyAsync(glacier_melt, d.melt, bytes, cudaMemcpyDeviceToHost, g->stream) != cudaSuccess ||
        cudaStreamSynchronize(g->stream) != cudaSuccess)
        return glacier_fail(g, WF_ERR_CUDA, "glacier step failed");
    return WF_OK;
}

}  // extern "C"
