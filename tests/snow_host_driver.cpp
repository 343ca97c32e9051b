// Host build of the lateral snow transport's per-cell arithmetic (wflow.jl_gb300/csrc/
// snow_scheme.cuh), driven as the kernels drive it: capacities, then the cells level by level
// (each level's cells in any order, here descending to differ from the oracle's sweep), then
// snow_out and snow_in. Test code: it lets the CPU suite compare the product's arithmetic and its
// level schedule with the oracle without a GPU. Compiled without FMA contraction.
#include <algorithm>
#include <vector>

#include "snow_scheme.cuh"

extern "C" void host_snow_transport(int64_t n, const int32_t* ds, const int64_t* order, const int32_t* ups_ds,
                                    const double* slope, double dt, double* snow_storage, double* snow_water,
                                    double* snow_out, double* snow_in) {
    std::vector<int64_t> up_ptr(n + 1, 0), up_cell(n), in_ptr(n + 1, 0), in_cell, level(n, 0);
    for (int64_t i = 0; i < n; ++i)
        if (ds[i] >= 0) up_ptr[ds[i] + 1]++;
    for (int64_t i = 0; i < n; ++i) up_ptr[i + 1] += up_ptr[i];
    std::vector<int64_t> fill(up_ptr.begin(), up_ptr.end() - 1);
    for (int64_t k = 0; k < n; ++k)
        if (ds[order[k]] >= 0) up_cell[fill[ds[order[k]]]++] = order[k];
    for (int64_t i = 0; i < n; ++i)
        if (ups_ds[i] >= 0) in_ptr[ups_ds[i] + 1]++;
    for (int64_t i = 0; i < n; ++i) in_ptr[i + 1] += in_ptr[i];
    in_cell.assign(in_ptr[n], 0);
    fill.assign(in_ptr.begin(), in_ptr.end() - 1);
    for (int64_t i = 0; i < n; ++i)
        if (ups_ds[i] >= 0) in_cell[fill[ups_ds[i]]++] = i;
    int64_t n_levels = 0;
    for (int64_t k = 0; k < n; ++k) {
        const int64_t v = order[k];
        n_levels = std::max(n_levels, level[v] + 1);
        if (ds[v] >= 0) level[ds[v]] = std::max(level[ds[v]], level[v] + 1);
    }
    std::vector<double> cap1(n), cap2(n), hand1(n), hand2(n), out1(n), out2(n);
    wfsn::SnowNet d{};
    d.n = n;
    d.ds = ds;
    d.up_ptr = up_ptr.data();
    d.up_cell = up_cell.data();
    d.in_ptr = in_ptr.data();
    d.in_cell = in_cell.data();
    d.slope = slope;
    d.m1 = snow_storage;
    d.m2 = snow_water;
    d.cap1 = cap1.data();
    d.cap2 = cap2.data();
    d.hand1 = hand1.data();
    d.hand2 = hand2.data();
    d.out1 = out1.data();
    d.out2 = out2.data();
    d.snow_out = snow_out;
    d.snow_in = snow_in;
    for (int64_t i = 0; i < n; ++i) wfsn::capacities(d, i, dt);
    for (int64_t l = 0; l < n_levels; ++l)
        for (int64_t i = n - 1; i >= 0; --i)
            if (level[i] == l) wfsn::transport_cell(d, i, dt);
    for (int64_t i = 0; i < n; ++i) wfsn::out_cell(d, i);
    for (int64_t i = 0; i < n; ++i) wfsn::in_cell(d, i);
}

// the glacier kernel's loop body over n cells
extern "C" void host_glacier(int64_t n, const double* fraction, const double* ttm, const double* cfmax,
                             const double* sifrac, double max_rate, double dt, const double* temperature,
                             double* snow_storage, double* glacier_store, double* glacier_melt) {
    for (int64_t i = 0; i < n; ++i) {
        double snow, store, melt;
        wfsn::glacier_hbv(fraction[i], glacier_store[i], snow_storage[i], temperature[i], ttm[i], cfmax[i], sifrac[i],
                          max_rate, dt, &snow, &store, &melt);
        snow_storage[i] = snow;
        glacier_store[i] = store;
        glacier_melt[i] = melt;
    }
}
