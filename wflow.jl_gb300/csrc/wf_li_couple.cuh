// wf_li_couple.cuh -- the local-inertial land and river routing (kernels_li.cu) inside the SBM
// step (wf_api.cu), in place of the kinematic-wave overland and river sweeps.
//
// Wflow's surface_routing! for a model with local-inertial land and river routing
// (Wflow/src/routing/surface/surface_routing.jl:62-89): the land runoff of the step,
// (net_runoff + net_runoff_river) * area plus the subsurface flow to the river at river cells
// (update_bc_overland_flow_model!, surface_staggered_scheme.jl:1080-1097), drives
// update_overland_flow_model! (:1153-1193); the open-water evaporation of the next step and the
// total water storage read the scheme's depths (runoff.jl:74-79, sbm.jl:143-182), and the
// overland balance is the scheme's per land cell (mass_balance.jl:402-461).
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

struct WfLiDomain;

// Device arrays of an attached local-inertial domain (node order: the model's external land and
// river order; the river's ghost cells follow its active cells).
struct WfLiCoupleView {
    int64_t n, nr_total, n_active, n_edges;
    double* runoff;          // [n] land runoff input [m3 s-1] (written by the SBM step)
    double* ext;             // [nr_total] river external inflow [m3 s-1]
    const double* abstraction;      // [nr_total] river abstraction (zero)
    const double* abstraction_cum;  // [nr_total] actual external abstraction of the step [m3]
    const double *h_land, *storage;            // [n]
    const double *h_river, *storage_river;     // [nr_total]
    const double *q, *q_avg;                   // [n_edges]
    const double *qx_avg, *qy_avg;             // [n + 1]
    const int64_t *ixd, *iyd, *river_index;    // [n]
    const int64_t *in_ptr, *in_edge, *out_ptr, *out_edge;  // river CSR (ascending edge order)
};

// The view of a domain, and the land-to-river map on the host [n] (for the checks at attach).
int wf_li_domain_couple_view(WfLiDomain* d, WfLiCoupleView* v, const int64_t** river_index_host);
// One model step of the scheme on `stream` without a host round trip (cumulative discharges
// reset, the device sub-step loop, the averages); wf_li_domain_complete_step after the stream
// synchronised reads the loop's status and sub-step count.
int wf_li_domain_enqueue_step(WfLiDomain* d, double dt, cudaStream_t stream);
int wf_li_domain_complete_step(WfLiDomain* d, int64_t* substeps, const char** err);
