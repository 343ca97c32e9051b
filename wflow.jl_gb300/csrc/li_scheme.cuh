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
// depth; the stable time step is the minimum over cells 0..n_dt-1. Edge k runs from cell src[k] to cell dst[k]; in_ptr/in_edge and out_ptr/out_edge are
// the CSR lists of the edges into and out of each cell, in ascending edge order.
struct LiNet {
    int64_t n, n_active, n_edges, n_dt;
    const int64_t *src, *dst;
    const int64_t *in_ptr, *in_edge, *out_ptr, *out_edge;
    const double *zb, *flow_length, *flow_width, *zb_e, *width_e, *length_e, *nsq_e;
    double *h, *storage, *q, *q_prev, *q_cum, *inwater, *dt_min;
    const double *abstraction, *external_inflow;  // river alone: boundary inflows [m3 s-1]
    double *error, *abstraction_cum;              // river alone: clipped storage, actual abstraction [m3]
    double h_thresh, alpha;
    int32_t froude;
    // Manning's equation on the staggered grid (river_routing = "manning_staggered") instead of
    // the local-inertial edge update: per edge slope and Manning's n, and each edge's last depth
    int32_t manning;
    const double *slope_e, *n_e;
    double* hf_e;
};

constexpr double BETA_KINWAVE = 0.6;  // Wflow.BETA_KINWAVE (routing/surface/surface_kinwave.jl:2)

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

// Manning's equation at edge k over dt (update_river_channel_flow! for ManningStaggered,
// surface_staggered_scheme.jl:386-434): the upstream ("upwind") depth, a rectangular channel,
// manning_flow (surface_process.jl:166-169) above the depth threshold, the discharge limited to
// the upstream storage over dt; q dt into the cumulative discharge
WF_HD void update_edge_manning(const LiNet& d, int64_t k, double dt) {
    const int64_t a = d.src[k];
    const double hf = d.h[a];
    d.hf_e[k] = hf;
    const double A = d.width_e[k] * hf;
    const double R = A / (2.0 * hf + d.width_e[k]);
    double q = hf > d.h_thresh ? ((wfm::cbrt(R * R) * wfm::sqrt_(d.slope_e[k])) * A) / d.n_e[k] : 0.0;
    q = wfm::jmin(q, d.storage[a] / dt);
    d.q[k] = q;
    d.q_cum[k] += q * dt;
}

// the stable sub-step at edge k for Manning's equation (stable_timestep, :1050-1075): the wave
// celerity of a wide rectangular channel at the edge's last depth (inf for a dry edge)
WF_HD double edge_timestep_manning(const LiNet& d, int64_t k) {
    const double hf = d.hf_e[k];
    const double h_r = (d.width_e[k] * hf) / (2.0 * hf + d.width_e[k]);
    const double celerity = ((wfm::cbrt(h_r * h_r) * wfm::sqrt_(d.slope_e[k])) / d.n_e[k]) / BETA_KINWAVE;
    return d.alpha * d.length_e[k] / celerity;
}

// storage and depth of active cell i over dt: edge discharges, lateral inflow and abstraction,
// the storage clipped at zero (the clipped volume counted as error), then the external inflow,
// a negative one limited to 80 % of the storage per step (no floodplain)
WF_HD void update_cell(const LiNet& d, int64_t i, double dt) {
    double qin = 0.0, qout = 0.0;
    for (int64_t o = d.in_ptr[i]; o < d.in_ptr[i + 1]; ++o) qin = qin + d.q[d.in_edge[o]];
    for (int64_t o = d.out_ptr[i]; o < d.out_ptr[i + 1]; ++o) qout = qout + d.q[d.out_edge[o]];
    double s = d.storage[i] + (qin - qout + d.inwater[i] - d.abstraction[i]) * dt;
    if (s < 0.0) {
        d.error[i] = d.error[i] + wfm::fabs_(s);
        s = 0.0;
    }
    const double ext = d.external_inflow[i];
    double inflow = ext;
    if (ext < 0.0) {
        const double taken = wfm::jmin(-ext, s / dt * 0.80);
        d.abstraction_cum[i] += taken * dt;
        inflow = -taken;
    }
    s += inflow * dt;
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

// ---- overland flow on the land grid, coupled with the river --------------------------------

// The land grid of the coupled scheme. Neighbour index n marks outside the grid; the discharge
// arrays hold n + 1 values, the last staying zero. qx0 / qy0 are the discharges of the previous
// sub-step (the device swaps the two buffers each sub-step). river[i] is the river cell in land
// cell i or -1.
struct LiLand {
    int64_t n;
    const int64_t *ixu, *ixd, *iyu, *iyd, *river;
    const double *xl, *yl, *z, *nsq, *xw, *yw, *zx_max, *zy_max;
    const double* runoff;
    double *h, *storage, *error;
    const double *qx0, *qy0;
    double *qx, *qy, *qx_cum, *qy_cum, *dt_min;
    double theta, h_thresh, alpha;
    int32_t froude;
};

// Per river cell boundary data of the coupled scheme.
struct LiRiverBC {
    const double *bankfull_depth, *bankfull_storage, *external_inflow, *abstraction;
    double* abstraction_cum;
};

// local_inertial_flow, rectangular cross-section with the theta weighting
// (surface_process.jl:124-163)
WF_HD double flow_rect(double theta, double q0, double qd, double qu, double zs0, double zs1, double hf, double width,
                       double length, double nsq, bool froude, double dt) {
    const double slope = (zs1 - zs0) / length;
    const double pow_hf = wfm::cbrt(hf * hf * hf * hf * hf * hf * hf);
    double q = ((theta * q0 + 0.5 * (1.0 - theta) * (qu + qd)) - GRAVITY * hf * width * dt * slope) /
               (1.0 + GRAVITY * dt * nsq * wfm::fabs_(q0) / (pow_hf * width));
    if (froude) {
        const double fr = (q / width / hf) / wfm::sqrt_(GRAVITY * hf);
        if (wfm::fabs_(fr) > 1.0 && q > 0.0)
            q = hf * wfm::sqrt_(GRAVITY * hf) * width;
        else if (wfm::fabs_(fr) > 1.0 && q < 0.0)
            q = -hf * wfm::sqrt_(GRAVITY * hf) * width;
    }
    return q;
}

// update_directional_flow! at land cell i (surface_staggered_scheme.jl:1202-1265). An edge
// without an upstream cell or with zero effective width keeps its discharge.
WF_HD void land_direction(const LiLand& L, int64_t i, double dt, bool x_dir) {
    const int64_t u = x_dir ? L.ixu[i] : L.iyu[i];
    const int64_t dn = x_dir ? L.ixd[i] : L.iyd[i];
    const double width = x_dir ? L.yw[i] : L.xw[i];
    const double* q0 = x_dir ? L.qx0 : L.qy0;
    double* q = x_dir ? L.qx : L.qy;
    if (!(u < L.n && width != 0.0)) {
        q[i] = q0[i];
        return;
    }
    const double* len = x_dir ? L.xl : L.yl;
    const double zs_current = L.z[i] + L.h[i];
    const double zs_upstream = L.z[u] + L.h[u];
    const double zs_max = wfm::jmax(zs_current, zs_upstream);
    const double hf = zs_max - (x_dir ? L.zx_max[i] : L.zy_max[i]);
    double qi = 0.0;
    if (hf > L.h_thresh) {
        const double length_e = 0.5 * (len[i] + len[u]);
        qi = flow_rect(L.theta, q0[i], q0[dn], q0[u], zs_current, zs_upstream, hf, width, length_e, L.nsq[i],
                       L.froude != 0, dt);
        if (L.h[i] <= 0.0) qi = wfm::jmin(qi, 0.0);
        if (L.h[u] <= 0.0) qi = wfm::jmax(qi, 0.0);
    }
    q[i] = qi;
    (x_dir ? L.qx_cum : L.qy_cum)[i] += qi * dt;
}

// storage and depths of land cell i (local_inertial_update_water_depth!, :1518-1546): a cell
// without a river from its edge discharges and runoff (:1420-1433, 1481-1503); a river cell
// from those and its river edges, with the external inflow or abstraction, the channel holding
// the storage up to bankfull and the rest spilling over the cell (:1322-1414, 1440-1476)
WF_HD void land_depth(const LiLand& L, const LiNet& R, const LiRiverBC& B, int64_t i, double dt) {
    const int64_t r = L.river[i];
    const int64_t xd = L.ixd[i], yd = L.iyd[i];
    if (r < 0) {
        double s = L.storage[i] + (L.qx[xd] - L.qx[i] + L.qy[yd] - L.qy[i] + L.runoff[i]) * dt;
        if (s < 0.0) {
            L.error[i] += wfm::fabs_(s);
            s = 0.0;
        }
        L.storage[i] = s;
        L.h[i] = s / (L.xl[i] * L.yl[i]);
        return;
    }
    double s_in = 0.0, s_out = 0.0;
    for (int64_t o = R.in_ptr[r]; o < R.in_ptr[r + 1]; ++o) s_in = s_in + R.q[R.in_edge[o]];
    for (int64_t o = R.out_ptr[r]; o < R.out_ptr[r + 1]; ++o) s_out = s_out + R.q[R.out_edge[o]];
    const double net_river = s_in - s_out;
    const double net_land = L.qx[xd] - L.qx[i] + L.qy[yd] - L.qy[i];
    const double net = net_river + net_land + L.runoff[i] - B.abstraction[r];
    double s = L.storage[i] + net * dt;
    if (s < 0.0) {
        L.error[i] += wfm::fabs_(s);
        s = 0.0;
    }
    const double ext = B.external_inflow[r];
    double inflow = ext, taken = 0.0;
    if (ext < 0.0) {
        const double available = s >= B.bankfull_storage[r] ? B.bankfull_storage[r] : R.storage[r];
        taken = wfm::jmin(-ext, available / dt * 0.80);
        inflow = -taken;
    }
    s += inflow * dt;
    B.abstraction_cum[r] += taken * dt;
    L.storage[i] = s;
    if (s >= B.bankfull_storage[r]) {
        const double river_h = B.bankfull_depth[r] + (s - B.bankfull_storage[r]) / (L.xl[i] * L.yl[i]);
        R.h[r] = river_h;
        L.h[i] = river_h - B.bankfull_depth[r];
        R.storage[r] = river_h * R.flow_length[r] * R.flow_width[r];
    } else {
        R.h[r] = s / (R.flow_length[r] * R.flow_width[r]);
        L.h[i] = 0.0;
        R.storage[r] = s;
    }
}

// the stable sub-step of land cell i: cells without a river only (:1022-1040)
WF_HD double land_timestep(const LiLand& L, int64_t i) {
    return L.river[i] < 0 ? L.alpha * wfm::jmin(L.xl[i], L.yl[i]) / wfm::sqrt_(GRAVITY * L.h[i])
                          : wfm::from_bits(0x7ff0000000000000ULL);
}

// Edge elevations of the land grid as LocalInertialOverlandFlowParameters derives them
// (surface_staggered_scheme.jl:929-939): the higher elevation of a cell and its upstream
// neighbour in x and y (0 without one). Host code.
inline void land_edge_parameters(int64_t n, const int64_t* ind_x_up, const int64_t* ind_y_up, const double* elevation,
                                 std::vector<double>& zx_max, std::vector<double>& zy_max) {
    zx_max.assign(n, 0.0);
    zy_max.assign(n, 0.0);
    for (int64_t i = 0; i < n; ++i) {
        if (ind_x_up[i] < n) zx_max[i] = wfm::jmax(elevation[i], elevation[ind_x_up[i]]);
        if (ind_y_up[i] < n) zy_max[i] = wfm::jmax(elevation[i], elevation[ind_y_up[i]]);
    }
}

// bankfull_depth .* flow_width .* flow_length (RiverFlowStaggeredParameters, :118). Host code.
inline void bankfull_storage(int64_t n, const double* bankfull_depth, const double* flow_width,
                             const double* flow_length, std::vector<double>& out) {
    out.assign(n, 0.0);
    for (int64_t r = 0; r < n; ++r) out[r] = bankfull_depth[r] * flow_width[r] * flow_length[r];
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
