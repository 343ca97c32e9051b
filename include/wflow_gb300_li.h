/*
 * wflow_gb300_li.h -- local-inertial river flow on a staggered grid, on the GPU.
 *
 * Wflow's other river routing (river_routing = "local_inertial"): discharge on the edges
 * between river cells from the water-surface slope, friction and the previous discharge
 * (local_inertial_flow, Wflow/src/routing/surface/surface_process.jl:88-115), then water
 * depth on the cells from the edge discharges and the lateral inflow
 * (update_river_channel_flow! and update_water_depth_and_storage!,
 * routing/surface/surface_staggered_scheme.jl:326-385, 723-760), with sub-steps of the
 * stable time step min over cells of alpha dx / sqrt(g h) (:1004-1020, update_river_flow_model!
 * :800-860). Channel only: no floodplain, no reservoirs at edges, no external inflow or
 * abstraction. FP64 in the reference's operation order.
 *
 * A standalone component: it holds its own network and state on the device; the SBM step of
 * wflow_gb300.h routes rivers by the kinematic wave.
 */
#ifndef WFLOW_GB300_LI_H
#define WFLOW_GB300_LI_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct WfLiRiver WfLiRiver;

/* n cells, the first n_active of which are updated (the rest are boundary cells of fixed
 * depth, Wflow's ghost cells at the outlets); n_edges edges, edge k from cell src[k] to cell
 * dst[k] (0-based). Per cell: bed level zb [m], flow_length and flow_width [m], initial depth
 * h [m] (storage starts at zero, as Wflow's state). Per edge: bed level, width, length and
 * Manning's n squared. Returns 0 or a negative WfStatus; wf_li_river_last_error gives the
 * message. */
int32_t wf_li_river_create(int64_t n, int64_t n_active, int64_t n_edges, const int64_t* src, const int64_t* dst,
                           const double* zb, const double* flow_length, const double* flow_width,
                           const double* h_init, const double* zb_edge, const double* width_edge,
                           const double* length_edge, const double* mannings_n_sq_edge, double h_thresh,
                           int32_t froude_limit, double alpha, int32_t device, WfLiRiver** out);
void wf_li_river_destroy(WfLiRiver* r);
const char* wf_li_river_last_error(const WfLiRiver* r);

/* A warm state: depth h of every cell [n] and, unless q is NULL, discharge q of every edge
 * [n_edges]; the storage of the active cells becomes h * flow_width * flow_length (as Wflow sets
 * it after reading a state file, Wflow/src/sbm_model.jl:168-172). */
int32_t wf_li_river_set_state(WfLiRiver* r, const double* h, const double* q);
/* Lateral inflow of every cell [m3 s-1] (inwater). */
int32_t wf_li_river_set_inwater(WfLiRiver* r, const double* inwater);
/* The stable sub-step of the current depths (60 s when every cell is dry). */
int32_t wf_li_river_stable_timestep(WfLiRiver* r, double* dt);
/* One update of edges then cells over dt_s (staggered_scheme_river_update!). */
int32_t wf_li_river_substep(WfLiRiver* r, double dt_s);
/* A model step of dt (update_river_flow_model!): the cumulative discharge restarts at zero,
 * sub-steps of the stable time step run until dt, and the average discharge becomes the
 * cumulative discharge / dt; the number of sub-steps taken goes to *substeps (may be NULL). */
int32_t wf_li_river_step(WfLiRiver* r, double dt, int64_t* substeps);
/* Copy a field to host: 0 depth h [n], 1 storage [n], 2 discharge q [n_edges],
 * 3 cumulative discharge, the sum of q * dt_s [n_edges], 4 average discharge of the last
 * model step [n_edges]. */
int32_t wf_li_river_get(WfLiRiver* r, int32_t field, double* dst);

#ifdef __cplusplus
}
#endif

#endif /* WFLOW_GB300_LI_H */
