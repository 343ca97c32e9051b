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
                     double* q_cum) {
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
