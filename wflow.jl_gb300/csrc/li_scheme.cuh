// li_scheme.cuh -- the local-inertial river scheme's per-edge and per-cell updates, written once
// for the device kernels of kernels_li.cu and for a host build of the same code.
//
// Edge update: discharge from the previous discharge, the water-surface slope and friction
// (local_inertial_flow, Wflow/src/routing/surface/surface_process.jl:88-115, inside the edge
// loop of update_river_channel_flow!, surface_staggered_scheme.jl:326-385). Cell update:
// storage and depth from the edges into and out of the cell and the lateral inflow
// (update_water_depth_and_storage!, :723-760). Stable sub-step of a cell: alpha dx / sqrt(g h)
// (stable_timestep, :1004-1020). FP64 in the reference's operation order.
#pragma once

#include <cstdint>
#include <vector>

#include "wf_math.cuh"

namespace wfli {

constexpr double GRAVITY = 9.80665;  // Wflow.GRAVITATIONAL_ACCELERATION (Wflow.jl:77)

// A river network on a staggered grid, all arrays in device (or, for a host build, host)
// memory. Cells 0..n_active-1 are updated; cells n_active..n-1 are boundary cells of fixed
// depth. Edge k runs from cell src[k] to cell dst[k]; in_ptr/in_edge and out_ptr/out_edge are
// the CSR lists of the edges into and out of each cell, in ascending edge order.
struct LiNet {
    int64_t n, n_active, n_edges;
    const int64_t *src, *dst;
    const int64_t *in_ptr, *in_edge, *out_ptr, *out_edge;
    const double *zb, *flow_length, *flow_width, *zb_e, *width_e, *length_e, *nsq_e;
    double *h, *storage, *q, *q_prev, *q_cum, *inwater, *dt_min;
    double h_thresh, alpha;
    int32_t froude;
};

// local_inertial_flow for a general cross-section of area A and hydraulic radius R
WF_HD double flow(double q0, double zs0, double zs1, double hf, double A, double R, double length, double nsq,
                  bool froude, double dt) {
    const double slope = (zs1 - zs0) / length;
    const double pow_R = wfm::cbrt(R * R * R * R);
    double q = (q0 - GRAVITY * A * dt * slope) / (1.0 + GRAVITY * dt * nsq * wfm::fabs_(q0) / (pow_R * A));
    const double fr = ((q / A) / wfm::sqrt_(GRAVITY * hf)) * (froude ? 1.0 : 0.0);
    if (wfm::fabs_(fr) > 1.0 && q > 0.0) q = wfm::sqrt_(GRAVITY * hf) * A;
    if (wfm::fabs_(fr) > 1.0 && q < 0.0) q = -wfm::sqrt_(GRAVITY * hf) * A;
    return q;
}

// discharge of edge k over dt: keeps the previous discharge, blocks flow out of a dry cell,
// adds q dt to the cumulative discharge
WF_HD void update_edge(const LiNet& d, int64_t k, double dt) {
    const double q_prev = d.q[k];
    d.q_prev[k] = q_prev;
    const int64_t a = d.src[k], b = d.dst[k];
    const double zs_src = d.zb[a] + d.h[a];
    const double zs_dst = d.zb[b] + d.h[b];
    const double zs_e = wfm::jmax(zs_src, zs_dst);
    const double hf = zs_e - d.zb_e[k];
    const double A = d.width_e[k] * hf;
    const double R = A / (2.0 * hf + d.width_e[k]);
    double q = hf > d.h_thresh
                   ? flow(q_prev, zs_src, zs_dst, hf, A, R, d.length_e[k], d.nsq_e[k], d.froude != 0, dt)
                   : 0.0;
    if (d.h[a] <= 0.0) q = wfm::jmin(q, 0.0);
    if (d.h[b] <= 0.0) q = wfm::jmax(q, 0.0);
    d.q[k] = q;
    d.q_cum[k] += q * dt;
}

// storage and depth of active cell i over dt (no external inflow, abstraction or floodplain)
WF_HD void update_cell(const LiNet& d, int64_t i, double dt) {
    double qin = 0.0, qout = 0.0;
    for (int64_t o = d.in_ptr[i]; o < d.in_ptr[i + 1]; ++o) qin = qin + d.q[d.in_edge[o]];
    for (int64_t o = d.out_ptr[i]; o < d.out_ptr[i + 1]; ++o) qout = qout + d.q[d.out_edge[o]];
    double s = d.storage[i] + (qin - qout + d.inwater[i] - 0.0) * dt;
    if (s < 0.0) s = 0.0;
    s += 0.0 * dt;
    d.storage[i] = s;
    d.h[i] = s / (d.flow_length[i] * d.flow_width[i]);
}

// the stable sub-step of cell i (inf for a dry cell)
WF_HD double cell_timestep(const LiNet& d, int64_t i) {
    return d.alpha * d.flow_length[i] / wfm::sqrt_(GRAVITY * d.h[i]);
}

// min over cells of the stable sub-step, 60 s when it is infinite (every cell dry)
WF_HD double finish_timestep(double dt_min) {
    return dt_min == wfm::from_bits(0x7ff0000000000000ULL) ? 60.0 : dt_min;
}

// CSR lists of the edges into and out of each of n cells, each list in ascending edge order
// (the order in which sum_at adds them). Host code; indices must already be checked in range.
inline void build_csr(int64_t n, int64_t n_edges, const int64_t* src, const int64_t* dst, std::vector<int64_t>& in_ptr,
                      std::vector<int64_t>& in_edge, std::vector<int64_t>& out_ptr, std::vector<int64_t>& out_edge) {
    in_ptr.assign(n + 1, 0);
    out_ptr.assign(n + 1, 0);
    for (int64_t k = 0; k < n_edges; ++k) {
        in_ptr[dst[k] + 1]++;
        out_ptr[src[k] + 1]++;
    }
    for (int64_t i = 0; i < n; ++i) {
        in_ptr[i + 1] += in_ptr[i];
        out_ptr[i + 1] += out_ptr[i];
    }
    in_edge.assign(n_edges, 0);
    out_edge.assign(n_edges, 0);
    std::vector<int64_t> fi(in_ptr.begin(), in_ptr.end() - 1), fo(out_ptr.begin(), out_ptr.end() - 1);
    for (int64_t k = 0; k < n_edges; ++k) {
        in_edge[fi[dst[k]]++] = k;
        out_edge[fo[src[k]]++] = k;
    }
}

}  // namespace wfli
