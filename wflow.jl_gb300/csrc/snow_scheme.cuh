// snow_scheme.cuh -- per-cell arithmetic of the lateral snow transport, written once for the
// kernels of kernels_snow.cu and for a host build of the same code.
//
// lateral_snow_transport! (Wflow/src/routing/surface/surface_process.jl:1-19): the fraction
// min(0.5, slope / tan 80deg) * min(1, snow_storage / 10) of the snow storage and of the snow water
// is the capacity per second of each cell; accucapacityflux! (routing/utils.jl:82-104) walks the
// cells in topological order, each passing on min(material / dt, capacity) and adding what it
// passes to its downstream cell's material. A cell's material is its own plus the hand-offs of
// its upstream cells, added in the order the topological sort visits them, so the sums round as
// the reference's do.
#pragma once

#include <cstdint>

#include "wf_math.cuh"

namespace wfsn {

constexpr double TAN80 = 5.67;             // surface_process.jl:1
constexpr double SNOW_STORAGE_MAX = 10.0;  // surface_process.jl:13

struct SnowNet {
    int64_t n;
    const int32_t* ds;
    const int64_t *up_ptr, *up_cell;  // upstream cells of each cell, in topological-sort order
    const int64_t *in_ptr, *in_cell;  // upstream cells for snow_in, ascending
    const double* slope;
    double *m1, *m2;                  // snow storage and snow water, moved in place
    double *cap1, *cap2;              // capacities [m s-1]
    double *hand1, *hand2;            // what each cell passed on times dt [m]
    double *out1, *out2;              // fluxes [m s-1]
    double *snow_out, *snow_in;
};

// the capacities from the states before the move
WF_HD void capacities(const SnowNet& d, int64_t i, double dt) {
    const double frac = wfm::jmin(0.5, d.slope[i] / TAN80) * wfm::jmin(1.0, d.m1[i] / SNOW_STORAGE_MAX);
    d.cap1[i] = frac * d.m1[i] / dt;
    d.cap2[i] = d.m2[i] * frac / dt;
}

// accucapacityflux! at cell v for one material (m, cap, hand, out)
WF_HD void pass_on(const SnowNet& d, int64_t v, double dt, double* m, const double* cap, double* hand, double* out) {
    double material = m[v];
    for (int64_t o = d.up_ptr[v]; o < d.up_ptr[v + 1]; ++o) material += hand[d.up_cell[o]];
    const double flux = wfm::jmin(material / dt, cap[v]);
    const double update = flux * dt;
    m[v] = material - update;
    out[v] = flux;
    hand[v] = update;
}

WF_HD void transport_cell(const SnowNet& d, int64_t v, double dt) {
    pass_on(d, v, dt, d.m1, d.cap1, d.hand1, d.out1);
    pass_on(d, v, dt, d.m2, d.cap2, d.hand2, d.out2);
}

// snow_out = storage flux + water flux; snow_in = sum of the upstream cells' snow_out
WF_HD void out_cell(const SnowNet& d, int64_t i) { d.snow_out[i] = d.out1[i] + d.out2[i]; }

WF_HD void in_cell(const SnowNet& d, int64_t i) {
    double acc = 0.0;
    for (int64_t o = d.in_ptr[i]; o < d.in_ptr[i + 1]; ++o) acc = acc + d.snow_out[d.in_cell[o]];
    d.snow_in[i] = acc;
}

// glacier_hbv (glacier/glacier_process.jl): firn from the snow on the glacier part, then
// degree-day glacier melt once the snow is below 10 mm. Returns the new snow storage, glacier
// store and melt through the pointers.
WF_HD void glacier_hbv(double glacier_fraction, double glacier_store, double snow_storage, double temperature,
                       double ttm, double cfmax, double sifrac, double max_rate, double dt, double* snow_out,
                       double* store_out, double* melt_out) {
    double snow_to_glacier = glacier_fraction > 0.0 ? sifrac * snow_storage : 0.0;
    snow_to_glacier = wfm::jmin(snow_to_glacier, max_rate);
    snow_storage -= snow_to_glacier * glacier_fraction * dt;
    glacier_store += snow_to_glacier * dt;
    const double potential_melt = temperature > ttm ? cfmax * (temperature - ttm) : 0.0;
    const double melt = snow_storage < 1e-2 ? wfm::jmin(potential_melt, glacier_store / dt) : 0.0;
    glacier_store -= melt * dt;
    *snow_out = snow_storage;
    *store_out = glacier_store;
    *melt_out = melt;
}

}  // namespace wfsn
