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
 * :800-860). Channel only: no floodplain, no reservoirs at edges. FP64 in the reference's
 * operation order.
 *
 * The components hold their own network and state on the device. A land grid with its river
 * (WfLiDomain) can also route an SBM model's land and river inside its step, in place of the
 * kinematic waves (wf_attach_local_inertial).
 */
#ifndef WFLOW_GB300_LI_H
#define WFLOW_GB300_LI_H

#include <stdint.h>

#include "wflow_gb300.h"

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
/* The stable time step is the minimum over cells 0..n_cells-1 (default: all n cells, as the
 * reference's MacDonald test sets its boundary cell inside n; a Wflow model's river has its ghost
 * cells after its RiverFlowStaggeredParameters.n real cells and passes that n). */
int32_t wf_li_river_set_timestep_cells(WfLiRiver* r, int64_t n_cells);
/* Route by Manning's equation on the staggered grid instead (river_routing = "manning_staggered",
 * Wflow/src/routing/surface/surface_staggered_scheme.jl:386-434): each edge takes the upstream
 * cell's depth, q = R^(2/3) sqrt(slope) A / n above the depth threshold, limited to the upstream
 * storage over the sub-step, and the stable sub-step is alpha length / celerity of each edge
 * (:1050-1075). Per edge: slope [-] (Wflow clamps it at 1e-5) and Manning's n [s m-1/3], both
 * positive; the edge bed levels given at create are the upstream cells' (compute_value_at_edge
 * with `first`), the Manning's n squared are unused. Froude limit unused. Before the first step. */
int32_t wf_li_river_set_manning(WfLiRiver* r, const double* slope_edge, const double* mannings_n_edge);
/* External inflow and abstraction of every cell [m3 s-1] (RiverFlowBC.external_inflow and
 * .abstraction; NULL: zero). A negative external inflow is an abstraction limited to 80 % of the
 * storage per step. */
int32_t wf_li_river_set_boundary(WfLiRiver* r, const double* external_inflow, const double* abstraction);
/* Lateral inflow of every cell [m3 s-1] (inwater). */
int32_t wf_li_river_set_inwater(WfLiRiver* r, const double* inwater);
/* The stable sub-step of the current depths (60 s when every cell is dry). */
int32_t wf_li_river_stable_timestep(WfLiRiver* r, double* dt);
/* One update of edges then cells over dt_s (staggered_scheme_river_update!). */
int32_t wf_li_river_substep(WfLiRiver* r, double dt_s);
/* A model step of dt (update_river_flow_model!): the cumulative discharge restarts at zero,
 * sub-steps of the stable time step run until dt, and the average discharge becomes the
 * cumulative discharge / dt; the number of sub-steps taken goes to *substeps (may be NULL).
 * The sub-step loop runs on the device in one cooperative launch (the time step is reduced, the
 * edges and then the cells updated, with grid barriers between; one read-back per step); every
 * barrier wait is bounded, and one that runs out returns WF_ERR_SPIN. */
int32_t wf_li_river_step(WfLiRiver* r, double dt, int64_t* substeps);
/* host_loop != 0: drive the sub-steps of wf_li_river_step from the host instead (one time step
 * read-back and two kernel launches per sub-step; the same results). No counterpart in the
 * reference. */
int32_t wf_li_river_set_host_loop(WfLiRiver* r, int32_t host_loop);
/* Copy a field to host: 0 depth h [n], 1 storage [n], 2 discharge q [n_edges],
 * 3 cumulative discharge, the sum of q * dt_s [n_edges], 4 average discharge of the last
 * model step [n_edges], 5 storage clipped at zero (error) [n], 6 actual abstraction of the
 * model step [m3, n]. */
int32_t wf_li_river_get(WfLiRiver* r, int32_t field, double* dst);

/* ---- Local-inertial overland flow on the land grid coupled with the river ----------------
 *
 * Wflow's land_routing = "local_inertial" with river_routing = "local_inertial"
 * (update_overland_flow_model!, routing/surface/surface_staggered_scheme.jl:1153-1193): per
 * sub-step of min(river, land) stable time step, the x and y discharges on the land cell edges
 * (update_directional_flow!, :1202-1265, local_inertial_flow with theta weighting,
 * surface_process.jl:124-163), the river edge discharges (update_river_channel_flow!), then the
 * storage and depths of every land cell, river cells sharing one storage between channel and
 * floodplain with the spill above bankfull (local_inertial_update_water_depth!, :1322-1546).
 * No reservoirs and no 1D floodplain. FP64 in the reference's operation order. */

typedef struct WfLiDomain WfLiDomain;

/* The land grid: n cells, 0-based neighbour indices (the value n marks outside the grid),
 * river_index[i] the river cell in land cell i or -1. Per cell: x and y length [m], elevation
 * [m], Manning's n squared (mannings_n_sq_at_edge of LocalInertialOverlandFlowParameters), and
 * the effective flow widths at the x and y edges [m] (the cell widths reduced by the river,
 * set_effective_flowwidth!, Wflow/src/utils.jl:604-680). */
typedef struct WfLiLandGrid {
    int64_t n;
    const int64_t* ind_x_up;
    const int64_t* ind_x_down;
    const int64_t* ind_y_up;
    const int64_t* ind_y_down;
    const int64_t* river_index;
    const double* x_length;
    const double* y_length;
    const double* elevation;
    const double* mannings_n_sq;
    const double* xwidth_at_edge;
    const double* ywidth_at_edge;
    double theta;
    double h_thresh;
    double alpha;
    int32_t froude_limit;
} WfLiLandGrid;

/* The river network as for wf_li_river_create, plus the bankfull depth of every cell [m]. */
typedef struct WfLiRiverNetwork {
    int64_t n, n_active, n_edges;
    const int64_t* src;
    const int64_t* dst;
    const double* zb;
    const double* flow_length;
    const double* flow_width;
    const double* bankfull_depth;
    const double* zb_edge;
    const double* width_edge;
    const double* length_edge;
    const double* mannings_n_sq_edge;
    double h_thresh;
    double alpha;
    int32_t froude_limit;
} WfLiRiverNetwork;

/* Fields of wf_li_domain_get. Land: depth, storage (river cells: channel plus floodplain),
 * the storage clipped at zero (error), the x and y discharges and their averages over the last
 * model step [n each]. River: depth, storage, discharge, its average, the cumulative actual
 * abstraction [river n or n_edges]. */
enum WfLiDomainField {
    WF_LI_LAND_H = 0,
    WF_LI_LAND_STORAGE = 1,
    WF_LI_LAND_ERROR = 2,
    WF_LI_LAND_QX = 3,
    WF_LI_LAND_QY = 4,
    WF_LI_LAND_QX_AVERAGE = 5,
    WF_LI_LAND_QY_AVERAGE = 6,
    WF_LI_RIVER_H = 7,
    WF_LI_RIVER_STORAGE = 8,
    WF_LI_RIVER_Q = 9,
    WF_LI_RIVER_Q_AVERAGE = 10,
    WF_LI_RIVER_ABSTRACTION_CUMULATIVE = 11
};

/* Both structs are read during the call only. river_index must map distinct land cells to
 * distinct active river cells, and every active river cell must lie in a land cell. The state
 * starts dry (Wflow's cold start) except for the river depths h_river [river n], which hold
 * the boundary depths of the ghost cells. */
int32_t wf_li_domain_create(const WfLiLandGrid* land, const WfLiRiverNetwork* river, const double* h_river,
                            int32_t device, WfLiDomain** out);
void wf_li_domain_destroy(WfLiDomain* d);
const char* wf_li_domain_last_error(const WfLiDomain* d);
/* A warm state (Wflow/src/sbm_model.jl:135-172): land depths [n], river depths [river n], and
 * unless NULL the x and y discharges [n] and river discharges [n_edges]. The land storage of a
 * river cell is h_land x_length y_length + bankfull storage where h_land > 0, else the river
 * storage; the river storage of an active cell is h_river flow_width flow_length. */
int32_t wf_li_domain_set_state(WfLiDomain* d, const double* h_land, const double* h_river, const double* qx,
                               const double* qy, const double* q_river);
/* Inputs of the coming steps: land runoff [m3 s-1, n]; river external inflow and abstraction
 * [m3 s-1, river n] (NULL: zero). */
int32_t wf_li_domain_set_inputs(WfLiDomain* d, const double* runoff, const double* external_inflow,
                                const double* abstraction);
/* min of the river and land stable time steps, each 60 s where all its cells are dry; the
 * river's over its active cells (not the ghost cells), the land's over cells without a river. */
int32_t wf_li_domain_stable_timestep(WfLiDomain* d, double* dt);
int32_t wf_li_domain_substep(WfLiDomain* d, double dt_s);
/* A model step: cumulative discharges and abstraction restart, sub-steps until dt, averages.
 * The sub-step loop runs on the device in one cooperative launch, as for wf_li_river_step. */
int32_t wf_li_domain_step(WfLiDomain* d, double dt, int64_t* substeps);
/* host_loop != 0: drive the sub-steps of wf_li_domain_step from the host (the same results). */
int32_t wf_li_domain_set_host_loop(WfLiDomain* d, int32_t host_loop);
int32_t wf_li_domain_get(WfLiDomain* d, int32_t field, double* dst);

/* Route an SBM model's land and river by this domain inside wf_step, in place of the kinematic
 * waves: Wflow's surface_routing! for local-inertial land and river routing
 * (Wflow/src/routing/surface/surface_routing.jl:62-89). Every step the land runoff
 * (net_runoff + net_runoff_river) * area, plus the subsurface flow to the river at river cells
 * (update_bc_overland_flow_model!, surface_staggered_scheme.jl:1080-1097), drives the domain's
 * step (update_overland_flow_model!, :1153-1193) on the model's stream; the model's overland and
 * river depths and storages (read by the next step's open-water evaporation and by the total
 * storage) are the domain's, its river discharge that of each river cell's outgoing edge, and its
 * overland balance the domain's per land cell (mass_balance.jl:402-461). Needs the FP64 form, one
 * member, no reservoirs and fixed kinematic-wave settings; the domain's land cells are the
 * model's land cells and its active river cells the model's river cells (river_index of the land
 * cell of river cell r is r). The model takes the domain's state at the call; the domain must
 * outlive the model and is stepped only through it afterwards. No CUDA graph and no
 * wf_step_static for such a model (the loop's status is read back every step). */
int32_t wf_attach_local_inertial(WfHandle* h, WfLiDomain* d);

#ifdef __cplusplus
}
#endif

#endif /* WFLOW_GB300_LI_H */
