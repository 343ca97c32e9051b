// Host build of the local-inertial river scheme (wflow.jl_gb300/csrc/li_scheme.cuh): the same
// per-edge, per-cell and stable-time-step functions the GPU kernels call, driven in the kernels'
// order (all edges, then all active cells; the time step as the 256-thread block reduction of
// li_dt_kernel). Test code: it lets the CPU suite compare the product's scheme arithmetic with
// the oracle without a GPU. Compiled without FMA contraction, as the CUDA unit is.
#include "li_scheme.cuh"

extern "C" {

// one sub-step, with the contract of the oracle's orc_li_river_step
void host_li_substep(int64_t n, int64_t n_active, int64_t n_edges, const int64_t* src, const int64_t* dst,
                     const double* zb, const double* flow_length, const double* flow_width, double* inwater,
                     const double* zb_e, const double* width_e, const double* length_e, const double* nsq_e,
                     double h_thresh, int32_t froude, double dt, double* h, double* storage, double* q, double* q_prev,
                     double* q_cum, const double* abstraction, const double* external_inflow, double* error,
                     double* abstraction_cum) {
    std::vector<int64_t> ip, ie, op, oe;
    wfli::build_csr(n, n_edges, src, dst, ip, ie, op, oe);
    wfli::LiNet d{};
    d.n = n;
    d.n_active = n_active;
    d.n_edges = n_edges;
    d.src = src;
    d.dst = dst;
    d.in_ptr = ip.data();
    d.in_edge = ie.data();
    d.out_ptr = op.data();
    d.out_edge = oe.data();
    d.zb = zb;
    d.flow_length = flow_length;
    d.flow_width = flow_width;
    d.zb_e = zb_e;
    d.width_e = width_e;
    d.length_e = length_e;
    d.nsq_e = nsq_e;
    d.h = h;
    d.storage = storage;
    d.q = q;
    d.q_prev = q_prev;
    d.q_cum = q_cum;
    d.inwater = inwater;
    d.abstraction = abstraction;
    d.external_inflow = external_inflow;
    d.error = error;
    d.abstraction_cum = abstraction_cum;
    d.h_thresh = h_thresh;
    d.froude = froude;
    for (int64_t k = 0; k < n_edges; ++k) wfli::update_edge(d, k, dt);
    for (int64_t i = 0; i < n_active; ++i) wfli::update_cell(d, i, dt);
}

// the stable time step, reduced as li_dt_kernel reduces it
double host_li_stable_timestep(int64_t n, const double* flow_length, double* h, double alpha) {
    wfli::LiNet d{};
    d.n = n;
    d.flow_length = flow_length;
    d.h = h;
    d.alpha = alpha;
    double red[256];
    for (int t = 0; t < 256; ++t) {
        double m = wfm::from_bits(0x7ff0000000000000ULL);
        for (int64_t i = t; i < n; i += 256) m = wfm::jmin(wfli::cell_timestep(d, i), m);
        red[t] = m;
    }
    for (int w = 128; w > 0; w >>= 1)
        for (int t = 0; t < w; ++t) red[t] = wfm::jmin(red[t + w], red[t]);
    return wfli::finish_timestep(red[0]);
}

}  // extern "C"

// ---- the land grid with its river ---------------------------------------------------------

#include "wflow_gb300_li.h"

extern "C" {

// sizes of the two input structs, to check the Python mirrors against
void host_li_struct_sizes(int64_t* out) {
    out[0] = (int64_t)sizeof(WfLiLandGrid);
    out[1] = (int64_t)sizeof(WfLiRiverNetwork);
}

// The state arrays, laid out as the oracle's OrcLiState; qx0 / qy0 hold the previous sub-step's
// discharges and qx / qy receive the new ones (the caller swaps the two each sub-step, as the
// device does).
struct HostLiState {
    double *h_land, *storage, *error, *qx, *qy, *qx0, *qy0, *qx_cum, *qy_cum;
    double *h_river, *storage_river, *q, *q_prev, *q_cum, *abstraction_cum;
};

struct HostDomain {
    wfli::LiLand L{};
    wfli::LiNet R{};
    wfli::LiRiverBC B{};
    std::vector<int64_t> ip, ie, op, oe;
    std::vector<double> zx_max, zy_max, bankfull, zero;
};

static void host_domain(HostDomain& h, const WfLiLandGrid* g, const WfLiRiverNetwork* r, const double* runoff,
                        const double* ext, const double* abstraction, HostLiState* st) {
    wfli::land_edge_parameters(g->n, g->ind_x_up, g->ind_y_up, g->elevation, h.zx_max, h.zy_max);
    wfli::bankfull_storage(r->n, r->bankfull_depth, r->flow_width, r->flow_length, h.bankfull);
    wfli::build_csr(r->n, r->n_edges, r->src, r->dst, h.ip, h.ie, h.op, h.oe);
    h.zero.assign(r->n, 0.0);
    wfli::LiLand& L = h.L;
    L.n = g->n;
    L.ixu = g->ind_x_up;
    L.ixd = g->ind_x_down;
    L.iyu = g->ind_y_up;
    L.iyd = g->ind_y_down;
    L.river = g->river_index;
    L.xl = g->x_length;
    L.yl = g->y_length;
    L.z = g->elevation;
    L.nsq = g->mannings_n_sq;
    L.xw = g->xwidth_at_edge;
    L.yw = g->ywidth_at_edge;
    L.zx_max = h.zx_max.data();
    L.zy_max = h.zy_max.data();
    L.runoff = runoff;
    L.h = st->h_land;
    L.storage = st->storage;
    L.error = st->error;
    L.qx0 = st->qx0;
    L.qy0 = st->qy0;
    L.qx = st->qx;
    L.qy = st->qy;
    L.qx_cum = st->qx_cum;
    L.qy_cum = st->qy_cum;
    L.theta = g->theta;
    L.h_thresh = g->h_thresh;
    L.alpha = g->alpha;
    L.froude = g->froude_limit;
    wfli::LiNet& R = h.R;
    R.n = r->n;
    R.n_active = r->n_active;
    R.n_edges = r->n_edges;
    R.src = r->src;
    R.dst = r->dst;
    R.in_ptr = h.ip.data();
    R.in_edge = h.ie.data();
    R.out_ptr = h.op.data();
    R.out_edge = h.oe.data();
    R.zb = r->zb;
    R.flow_length = r->flow_length;
    R.flow_width = r->flow_width;
    R.zb_e = r->zb_edge;
    R.width_e = r->width_edge;
    R.length_e = r->length_edge;
    R.nsq_e = r->mannings_n_sq_edge;
    R.h = st->h_river;
    R.storage = st->storage_river;
    R.q = st->q;
    R.q_prev = st->q_prev;
    R.q_cum = st->q_cum;
    R.h_thresh = r->h_thresh;
    R.alpha = r->alpha;
    R.froude = r->froude_limit;
    h.B.bankfull_depth = r->bankfull_depth;
    h.B.bankfull_storage = h.bankfull.data();
    h.B.external_inflow = ext ? ext : h.zero.data();
    h.B.abstraction = abstraction ? abstraction : h.zero.data();
    h.B.abstraction_cum = st->abstraction_cum;
}

// one sub-step in the kernels' order: land fluxes, river edges, land depths
void host_li_domain_substep(const WfLiLandGrid* g, const WfLiRiverNetwork* r, const double* runoff, const double* ext,
                            const double* abstraction, double dt, HostLiState* st) {
    HostDomain h;
    host_domain(h, g, r, runoff, ext, abstraction, st);
    for (int64_t i = 0; i < g->n; ++i) {
        wfli::land_direction(h.L, i, dt, true);
        wfli::land_direction(h.L, i, dt, false);
    }
    for (int64_t k = 0; k < r->n_edges; ++k) wfli::update_edge(h.R, k, dt);
    for (int64_t i = 0; i < g->n; ++i) wfli::land_depth(h.L, h.R, h.B, i, dt);
}

// the stable time step reduced as li_domain_dt_kernel reduces it
static double host_block_min(int64_t n, double (*f)(const HostDomain&, int64_t), const HostDomain& h) {
    double red[256];
    for (int t = 0; t < 256; ++t) {
        double m = wfm::from_bits(0x7ff0000000000000ULL);
        for (int64_t i = t; i < n; i += 256) m = wfm::jmin(f(h, i), m);
        red[t] = m;
    }
    for (int w = 128; w > 0; w >>= 1)
        for (int t = 0; t < w; ++t) red[t] = wfm::jmin(red[t + w], red[t]);
    return red[0];
}

double host_li_domain_stable_timestep(const WfLiLandGrid* g, const WfLiRiverNetwork* r, HostLiState* st) {
    HostDomain h;
    host_domain(h, g, r, nullptr, nullptr, nullptr, st);
    const double dt_river = wfli::finish_timestep(
        host_block_min(r->n_active, [](const HostDomain& d, int64_t i) { return wfli::cell_timestep(d.R, i); }, h));
    const double dt_land = wfli::finish_timestep(
        host_block_min(g->n, [](const HostDomain& d, int64_t i) { return wfli::land_timestep(d.L, i); }, h));
    return wfm::jmin(dt_river, dt_land);
}

}  // extern "C"
