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

#ifdef __cplusplus
}
#endif

#endif /* WFLOW_GB300_SNOW_H */
