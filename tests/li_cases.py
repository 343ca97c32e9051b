"""Local-inertial river cases shared by the oracle KAT and the GPU parity tests.

`OracleLi` drives the oracle's local-inertial river functions (orc_li_river_step,
orc_li_stable_timestep) with the state layout of the GPU component (wflow_gb300/li_river.py):
cells 0..n_active-1 updated, the rest boundary cells of fixed depth; edge k from src[k] to
dst[k]. Edge attributes follow the reference's construction in its MacDonald test
(Wflow/test/routing_process.jl:1229-1246) and in the RiverFlowStaggeredParameters constructor
(routing/surface/surface_staggered_scheme.jl:99-156): bed level max, width min, length mean,
Manning's n length-weighted, squared.
"""

import ctypes as C

import numpy as np

import oracle_py as O

G = 9.80665


def _pd(v):
    return v.ctypes.data_as(C.POINTER(C.c_double))


def _pl(v):
    return v.ctypes.data_as(C.POINTER(C.c_int64))


def edge_attributes(src, dst, zb, flow_length, width, mannings_n):
    dl = flow_length
    zb_e = np.maximum(zb[src], zb[dst])
    w_e = np.minimum(width[dst], width[src])
    l_e = 0.5 * (dl[dst] + dl[src])
    n_e = (mannings_n[dst] * dl[dst] + mannings_n[src] * dl[src]) / (dl[dst] + dl[src])
    return zb_e, w_e, l_e, n_e * n_e


def random_river(seed, n_active=3000, n_bound=4):
    """A random river tree: each active cell drains to a cell of higher index (a confluence where
    several drain to one), the last n_bound cells are outlets with a fixed depth. Bed levels fall
    downstream; depths start wet, dry and just above and below the threshold."""
    rng = np.random.default_rng(seed)
    n = n_active + n_bound
    down = np.empty(n_active, np.int64)
    for i in range(n_active):
        hi = min(n, i + 1 + int(rng.integers(1, 40)))
        down[i] = int(rng.integers(i + 1, hi)) if i + 1 < n_active else n_active + int(rng.integers(0, n_bound))
    down[n_active - n_bound:] = n_active + np.arange(n_bound)
    flow_length = rng.uniform(200.0, 1200.0, n)
    width = rng.uniform(5.0, 60.0, n)
    mannings_n = rng.uniform(0.02, 0.05, n)
    zb = np.zeros(n)
    zb[n_active:] = rng.uniform(0.0, 2.0, n_bound)
    for i in range(n_active - 1, -1, -1):
        zb[i] = zb[down[i]] + flow_length[i] * rng.uniform(1e-5, 2e-3)
    h = rng.uniform(0.0, 3.0, n)
    kind = rng.integers(0, 10, n)
    h[kind == 0] = 0.0
    h[kind == 1] = 1e-3 * rng.uniform(0.5, 1.5, int((kind == 1).sum()))
    src = np.arange(n_active, dtype=np.int64)
    dst = down.copy()
    order = np.lexsort((dst, src))  # Graphs.jl edge order: by source, then destination
    src, dst = src[order], dst[order]
    zb_e, w_e, l_e, nsq_e = edge_attributes(src, dst, zb, flow_length, width, mannings_n)
    inwater = rng.uniform(0.0, 5.0, n) * (rng.random(n) < 0.7)
    return dict(n=n, n_active=n_active, src=src, dst=dst, zb=zb, flow_length=flow_length, flow_width=width,
                h=h, zb_e=zb_e, w_e=w_e, l_e=l_e, nsq_e=nsq_e, inwater=inwater)


def macdonald_case(a):
    """MacDonald's (1997) long channel (routing_process.jl:1189-1318): bed levels integrate the
    analytical channel slope from each cell to the channel's end, depths start dry with the
    analytical depth at the last cell (the boundary). Returns the network and the analytical
    depths."""
    from scipy.integrate import quad
    Lc, dx = a["L"], a["dx"]
    n = int(Lc / dx)

    def h(x):  # MacDonald's depth profile for a 10 m wide channel, n = 0.03, Q = 20 m3/s
        return np.cbrt(4 / G) * (1.0 + 0.5 * np.exp(-16.0 * (x / Lc - 0.5) ** 2))

    def dh(x):
        return -np.cbrt(4 / G) * 16.0 / Lc * (x / Lc - 0.5) * np.exp(-16 * (x / Lc - 0.5) ** 2)

    def slope(x):
        return (1.0 - 4.0 / (G * h(x) ** 3)) * dh(x) + 0.36 * (2 * h(x) + 10.0) ** (4.0 / 3.0) / (
            (10.0 * h(x)) ** (10.0 / 3.0))

    x = np.arange(1, n + 1) * dx
    h_a = h(x)
    zb = np.array([quad(slope, xi, Lc, epsrel=1e-12, epsabs=0.0)[0] for xi in x])
    src = np.arange(n - 1, dtype=np.int64)
    dst = src + 1
    dl, width, nr = np.full(n, dx), np.full(n, a["width"]), np.full(n, a["mannings_n"])
    zb_e, w_e, l_e, nsq_e = edge_attributes(src, dst, zb, dl, width, nr)
    h0 = np.zeros(n)
    h0[-1] = h_a[-1]
    net = dict(n=n, n_active=n - 1, src=src, dst=dst, zb=zb, flow_length=dl, flow_width=width, h=h0, zb_e=zb_e,
               w_e=w_e, l_e=l_e, nsq_e=nsq_e, inwater=np.zeros(n))
    return net, h_a


class OracleLi:
    """The oracle's local-inertial river over a network dict (random_river / macdonald_case)."""

    def __init__(self, net, h_thresh=1e-3, froude=True, alpha=0.7):
        self.net = net
        self.n, self.na, self.ne = net["n"], net["n_active"], len(net["src"])
        self.h = np.array(net["h"], float)
        self.storage = np.zeros(self.n)
        self.q = np.zeros(self.ne)
        self.q_prev = np.zeros(self.ne)
        self.q_cum = np.zeros(self.ne)
        self.q_avg = np.zeros(self.ne)
        self.inwater = np.zeros(self.n)
        self.h_thresh, self.froude, self.alpha = h_thresh, froude, alpha
        self.L = O.lib()
        self.L.orc_li_stable_timestep.restype = C.c_double

    def set_state(self, h, q=None):
        """Wflow's warm start: storage of active cells = h * flow_width * flow_length."""
        self.h = np.array(h, float)
        if q is not None:
            self.q = np.array(q, float)
        self.storage = np.zeros(self.n)
        na = self.na
        self.storage[:na] = self.h[:na] * self.net["flow_width"][:na] * self.net["flow_length"][:na]

    def set_inwater(self, v):
        self.inwater = np.array(v, float)

    def stable_timestep(self):
        return self.L.orc_li_stable_timestep(C.c_int64(self.n), _pd(self.net["flow_length"]), _pd(self.h),
                                             C.c_double(self.alpha))

    def substep(self, dt):
        t = self.net
        self.L.orc_li_river_step(C.c_int64(self.n), C.c_int64(self.na), C.c_int64(self.ne), _pl(t["src"]),
                                 _pl(t["dst"]), _pd(t["zb"]), _pd(t["flow_length"]), _pd(t["flow_width"]),
                                 _pd(self.inwater), _pd(t["zb_e"]), _pd(t["w_e"]), _pd(t["l_e"]), _pd(t["nsq_e"]),
                                 C.c_double(self.h_thresh), C.c_int32(int(self.froude)), C.c_double(dt), _pd(self.h),
                                 _pd(self.storage), _pd(self.q), _pd(self.q_prev), _pd(self.q_cum))

    def step(self, dt):
        """update_river_flow_model! (surface_staggered_scheme.jl:800-826) without reservoirs or
        floodplain: q_cumulative restarts, sub-steps of the stable time step (cut at dt,
        check_timestepsize) until dt, q_average = q_cumulative / dt. Returns the sub-step count."""
        self.q_cum[:] = 0.0
        t, k = 0.0, 0
        while t < dt:
            dt_s = self.stable_timestep()
            if t + dt_s > dt:
                dt_s = dt - t
            self.substep(dt_s)
            t += dt_s
            k += 1
        self.q_avg = self.q_cum / dt
        return k
