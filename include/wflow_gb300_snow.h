/*
 * wflow_gb300_snow.h -- lateral (gravitational) snow transport on the GPU.
 *
 * Wflow's snow_gravitational_transport__flag: after the snow update, a slope- and
 * storage-dependent fraction of each cell's dry snow and of the liquid water in it moves to the
 * downstream cell, limited by a capacity per cell and carried in topological order
 * (lateral_snow_transport!, Wflow/src/routing/surface/surface_process.jl:1-19, on
 * accucapacityflux!, routing/utils.jl:82-104, 144-148). The snow storage and snow water move in
 * place; snow_out is what each cell passed on and snow_in what it received [m s-1]
 * (flux_in!, routing/utils.jl:160-166). FP64 in the reference's operation order.
 *
 * A standalone component: the SBM step of wflow_gb300.h runs without gravitational transport.
 */
#ifndef WFLOW_GB300_SNOW_H
#define WFLOW_GB300_SNOW_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct WfSnowTransport WfSnowTransport;

/* n land cells; ds[i] the downstream cell of i or -1 at a pit; order a topological order of
 * the cells, each before its downstream cell (Wflow's topological_sort_by_dfs order: upstream
 * hand-offs reach a cell in this order); ups_ds the downstream cells whose upstream lists give
 * snow_in (Wflow's upstream_nodes, cut at reservoir outlets; NULL: ds); slope [m m-1]. All
 * 0-based. Returns 0 or a negative WfStatus (wf_snow_transport_last_error). */
int32_t wf_snow_transport_create(int64_t n, const int32_t* ds, const int64_t* order, const int32_t* ups_ds,
                                 const double* slope, int32_t device, WfSnowTransport** out);
void wf_snow_transport_destroy(WfSnowTransport* t);
const char* wf_snow_transport_last_error(const WfSnowTransport* t);
/* One transport over dt [s]: snow_storage and snow_water [m, n, host] move in place;
 * snow_out and snow_in [m s-1, n, host] are written. */
int32_t wf_snow_transport_run(WfSnowTransport* t, double dt, double* snow_storage, double* snow_water,
                              double* snow_out, double* snow_in);
/* Number of topological levels (kernel launches per material sweep). */
int64_t wf_snow_transport_levels(const WfSnowTransport* t);

/* ---- HBV glacier ----------------------------------------------------------------------------
 * update_glacier_model! (Wflow/src/glacier/glacier.jl:122-154, glacier_hbv in
 * glacier/glacier_process.jl): snow on the glacier part of a cell turns into firn at
 * snow_to_ice_fraction of the snow per step (at most maximum_snow_to_ice_rate), and the glacier
 * melts by degree-day above the melt threshold once the snow is nearly gone. Per cell: glacier
 * fraction, melt threshold temperature [K], degree-day factor [m K-1 s-1], snow-to-ice fraction
 * [s-1]; maximum_snow_to_ice_rate [m s-1]. */
typedef struct WfGlacier WfGlacier;
int32_t wf_glacier_create(int64_t n, const double* glacier_fraction, const double* temperature_threshold_melt,
                          const double* degree_day_factor, const double* snow_to_ice_fraction,
                          double maximum_snow_to_ice_rate, int32_t device, WfGlacier** out);
void wf_glacier_destroy(WfGlacier* g);
const char* wf_glacier_last_error(const WfGlacier* g);
/* One step: temperature [K]; snow_storage and glacier_store [m] updated in place; glacier_melt
 * [m s-1] written. Host arrays of n values. */
int32_t wf_glacier_run(WfGlacier* g, double dt, const double* temperature, double* snow_storage,
                       double* glacier_store, double* glacier_melt);

#ifdef __cplusplus
}
#endif

#endif /* WFLOW_GB300_SNOW_H */
