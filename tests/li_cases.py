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
    external_inflow = np.zeros(n)
    pick = rng.choice(n_active, size=max(2, n_active // 50), replace=False)
    external_inflow[pick] = rng.uniform(-20.0, 10.0, len(pick))
    abstraction = np.zeros(n)
    abstraction[rng.choice(n_active, size=max(2, n_active // 100), replace=False)] = rng.uniform(0.0, 8.0)
    return dict(n=n, n_active=n_active, src=src, dst=dst, zb=zb, flow_length=flow_length, flow_width=width,
                h=h, zb_e=zb_e, w_e=w_e, l_e=l_e, nsq_e=nsq_e, inwater=inwater, external_inflow=external_inflow,
                abstraction=abstraction, mannings_n=mannings_n)


def manning_edges(net):
    """Edge slope and Manning's n of the Manning river on the staggered grid, as
    RiverFlowStaggeredParameters derives them (surface_staggered_scheme.jl:96-156): the bed slope
    over the mean edge length, at least 1e-5 (compute_slope_at_edge, routing/utils.jl:194-202), and
    the length-weighted Manning's n (compute_mannings_n_at_edge)."""
    src, dst, zb, fl, n = net["src"], net["dst"], net["zb"], net["flow_length"], net["mannings_n"]
    length_e = 0.5 * (fl[dst] + fl[src])
    slope_e = np.maximum((zb[src] - zb[dst]) / length_e, 1e-5)
    n_e = (n[dst] * fl[dst] + n[src] * fl[src]) / (fl[dst] + fl[src])
    return slope_e, n_e


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
        self.abstraction, self.external_inflow = np.zeros(self.n), np.zeros(self.n)
        self.error, self.abs_cum = np.zeros(self.n), np.zeros(self.n)
        self.h_thresh, self.froude, self.alpha = h_thresh, froude, alpha
        self.n_dt = self.n
        self.L = O.lib()
        self.L.orc_li_stable_timestep.restype = C.c_double

    def set_timestep_cells(self, n_cells):
        self.n_dt = int(n_cells)

    def set_manning(self, slope_e, n_e):
        """Manning's equation on the staggered grid (orc_manning_river_step)."""
        self.manning = (np.array(slope_e, float), np.array(n_e, float))
        self.hf_e = np.zeros(self.ne)
        self.L.orc_manning_stable_timestep.restype = C.c_double

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

    def set_boundary(self, external_inflow=None, abstraction=None):
        self.external_inflow = np.zeros(self.n) if external_inflow is None else np.array(external_inflow, float)
        self.abstraction = np.zeros(self.n) if abstraction is None else np.array(abstraction, float)

    def stable_timestep(self):
        if getattr(self, "manning", None) is not None:
            return self.L.orc_manning_stable_timestep(C.c_int64(self.ne), _pd(self.net["w_e"]), _pd(self.net["l_e"]),
                                                      _pd(self.manning[0]), _pd(self.manning[1]), _pd(self.hf_e),
                                                      C.c_double(self.alpha))
        return self.L.orc_li_stable_timestep(C.c_int64(self.n_dt), _pd(self.net["flow_length"]), _pd(self.h),
                                             C.c_double(self.alpha))

    def substep(self, dt):
        t = self.net
        if getattr(self, "manning", None) is not None:
            self.L.orc_manning_river_step(C.c_int64(self.n), C.c_int64(self.na), C.c_int64(self.ne), _pl(t["src"]),
                                          _pl(t["dst"]), _pd(t["flow_length"]), _pd(t["flow_width"]),
                                          _pd(self.inwater), _pd(t["w_e"]), _pd(self.manning[0]),
                                          _pd(self.manning[1]), C.c_double(self.h_thresh), C.c_double(dt),
                                          _pd(self.h), _pd(self.storage), _pd(self.q), _pd(self.q_cum),
                                          _pd(self.hf_e), _pd(self.abstraction), _pd(self.external_inflow),
                                          _pd(self.error), _pd(self.abs_cum))
            return
        self.L.orc_li_river_step(C.c_int64(self.n), C.c_int64(self.na), C.c_int64(self.ne), _pl(t["src"]),
                                 _pl(t["dst"]), _pd(t["zb"]), _pd(t["flow_length"]), _pd(t["flow_width"]),
                                 _pd(self.inwater), _pd(t["zb_e"]), _pd(t["w_e"]), _pd(t["l_e"]), _pd(t["nsq_e"]),
                                 C.c_double(self.h_thresh), C.c_int32(int(self.froude)), C.c_double(dt), _pd(self.h),
                                 _pd(self.storage), _pd(self.q), _pd(self.q_prev), _pd(self.q_cum),
                                 _pd(self.abstraction), _pd(self.external_inflow), _pd(self.error), _pd(self.abs_cum))

    def step(self, dt):
        """update_river_flow_model! (surface_staggered_scheme.jl:800-826) without reservoirs or
        floodplain: q_cumulative restarts, sub-steps of the stable time step (cut at dt,
        check_timestepsize) until dt, q_average = q_cumulative / dt. Returns the sub-step count."""
        self.q_cum[:] = 0.0
        self.abs_cum[:] = 0.0
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


# ---- the land grid with its river ------------------------------------------------------------

class OrcLiState(C.Structure):
    _fields_ = [(f, C.POINTER(C.c_double)) for f in ("h_land", "storage", "error", "qx", "qy", "qx0", "qy0", "qx_cum",
                                                     "qy_cum", "h_river", "storage_river", "q", "q_prev", "q_cum",
                                                     "abstraction_cum")]


def random_land_domain(seed, nx=36, ny=28):
    """A grid of nx * ny land cells (closed at its sides) with a main river along the middle row
    draining to one ghost cell of fixed depth and a tributary along a column joining it. Land
    cells are 80-160 m, rivers 5-40 m wide with bankfull depths of 1-2.5 m; a few land edges have
    zero effective width. Returns (land, river, h_river) for LiDomain / OracleLiDomain and a warm
    state and inputs with wet, dry, over-bankfull and near-threshold cells."""
    rng = np.random.default_rng(seed)
    n = nx * ny
    row, col = np.divmod(np.arange(n), nx)
    ind_x_up = np.where(col > 0, np.arange(n) - 1, n)
    ind_x_down = np.where(col < nx - 1, np.arange(n) + 1, n)
    ind_y_up = np.where(row > 0, np.arange(n) - nx, n)
    ind_y_down = np.where(row < ny - 1, np.arange(n) + nx, n)
    x_length = np.full(n, rng.uniform(80.0, 160.0))
    y_length = np.full(n, rng.uniform(80.0, 160.0))
    mid, tc = ny // 2, nx // 3
    elevation = 0.002 * (nx - col) * x_length + 0.01 * np.abs(row - mid) * y_length + rng.uniform(0.0, 0.3, n)
    mannings_n = rng.uniform(0.03, 0.1, n)
    # rivers: main channel (mid, 0..nx-1) then the tributary (0..mid-1, tc), one ghost cell
    main = mid * nx + np.arange(nx)
    trib = np.arange(mid) * nx + tc
    cells = np.concatenate([main, trib])
    nra = len(cells)
    river_index = np.full(n, -1, np.int64)
    river_index[cells] = np.arange(nra)
    src = list(range(nx - 1)) + [nx - 1]
    dst = list(range(1, nx)) + [nra]  # the main channel's last cell drains to the ghost cell
    for k in range(mid):
        src.append(nx + k)
        dst.append(nx + k + 1 if k + 1 < mid else tc)
    order = np.lexsort((dst, src))
    src, dst = np.asarray(src, np.int64)[order], np.asarray(dst, np.int64)[order]
    nr = nra + 1
    flow_length = np.concatenate([x_length[main], y_length[trib], [x_length[0]]])
    flow_width = np.concatenate([rng.uniform(15.0, 40.0, nx), rng.uniform(5.0, 15.0, mid), [30.0]])
    bankfull_depth = rng.uniform(1.0, 2.5, nr)
    zb = np.concatenate([elevation[cells], [elevation[main[-1]] - 0.5]]) - bankfull_depth
    nr_manning = rng.uniform(0.025, 0.045, nr)
    zb_e, w_e, l_e, nsq_e = edge_attributes(src, dst, zb, flow_length, flow_width, nr_manning)
    xwidth = x_length.copy()
    ywidth = y_length.copy()
    ywidth[main] = np.maximum(ywidth[main] - flow_width[:nx], 0.0)
    xwidth[trib] = np.maximum(xwidth[trib] - flow_width[nx:nra], 0.0)
    closed = rng.random(n) < 0.03
    xwidth[closed] = 0.0
    ywidth[rng.random(n) < 0.03] = 0.0
    land = dict(ind_x_up=ind_x_up, ind_x_down=ind_x_down, ind_y_up=ind_y_up, ind_y_down=ind_y_down,
                river_index=river_index, x_length=x_length, y_length=y_length, elevation=elevation,
                mannings_n_sq=mannings_n * mannings_n, xwidth_at_edge=xwidth, ywidth_at_edge=ywidth, theta=0.8, h_thresh=1e-3,
                alpha=0.7, froude_limit=True)
    river = dict(n_active=nra, src=src, dst=dst, zb=zb, flow_length=flow_length, flow_width=flow_width,
                 bankfull_depth=bankfull_depth, zb_edge=zb_e, width_edge=w_e, length_edge=l_e,
                 mannings_n_sq_edge=nsq_e, h_thresh=1e-3, alpha=0.7, froude_limit=True)
    h_river = np.zeros(nr)
    h_river[-1] = 1.2
    # warm state and inputs
    h_land = rng.uniform(0.0, 0.25, n) * (rng.random(n) < 0.6)
    h_land[rng.random(n) < 0.05] = 1e-3 * rng.uniform(0.5, 1.5)
    h_land[cells] = 0.0
    over = rng.random(nra) < 0.3
    h_land[cells[over]] = rng.uniform(0.01, 0.3, int(over.sum()))
    h_riv = np.concatenate([rng.uniform(0.3, 2.0, nra), [1.2]])
    h_riv[:nra][over] = bankfull_depth[:nra][over] + h_land[cells[over]]
    qx = rng.uniform(-0.5, 0.5, n) * (rng.random(n) < 0.3)
    qy = rng.uniform(-0.5, 0.5, n) * (rng.random(n) < 0.3)
    q_river = rng.uniform(0.0, 30.0, len(src))
    runoff = rng.uniform(0.0, 0.05, n) * (rng.random(n) < 0.8)
    ext = np.zeros(nr)
    ext[3], ext[nx + 1] = -4.0, 2.5
    abstraction = np.zeros(nr)
    abstraction[5] = 0.3
    state = dict(h_land=h_land, h_river=h_riv, qx=qx, qy=qy, q_river=q_river)
    inputs = dict(runoff=runoff, external_inflow=ext, abstraction=abstraction)
    return land, river, h_river, state, inputs


class OracleLiDomain:
    """The oracle's coupled land + river scheme (orc_li_domain_substep) over the dicts of
    random_land_domain, with the state of wf_li_domain_* (Wflow's warm start and step loop)."""

    def __init__(self, land, river, h_river):
        from wflow_gb300.li_river import land_grid, river_network
        self._keep = []
        self.g, self.r = land_grid(land, self._keep), river_network(river, self._keep)
        self.land, self.river = land, river
        self.n, self.nr, self.ne = self.g.n, self.r.n, self.r.n_edges
        z = np.zeros
        self.a = dict(h_land=z(self.n), storage=z(self.n), error=z(self.n), qx=z(self.n + 1), qy=z(self.n + 1),
                      qx0=z(self.n + 1), qy0=z(self.n + 1), qx_cum=z(self.n + 1), qy_cum=z(self.n + 1),
                      h_river=np.array(h_river, float), storage_river=z(self.nr), q=z(self.ne), q_prev=z(self.ne),
                      q_cum=z(self.ne), abstraction_cum=z(self.nr))
        self.st = OrcLiState(**{k: _pd(v) for k, v in self.a.items()})
        self.runoff, self.ext, self.abs = z(self.n), z(self.nr), z(self.nr)
        self.qx_avg, self.qy_avg, self.q_avg = z(self.n), z(self.n), z(self.ne)
        self.L = O.lib()
        self.L.orc_li_domain_stable_timestep.restype = C.c_double

    def set_state(self, h_land, h_river, qx=None, qy=None, q_river=None):
        """Wflow's warm start (sbm_model.jl:135-172)."""
        a, land, river = self.a, self.land, self.river
        a["h_land"][:] = h_land
        a["h_river"][:] = h_river
        if qx is not None:
            a["qx"][:self.n] = qx
        if qy is not None:
            a["qy"][:self.n] = qy
        if q_river is not None:
            a["q"][:] = q_river
        bankfull = river["bankfull_depth"] * river["flow_width"] * river["flow_length"]
        for i in range(self.n):
            r = land["river_index"][i]
            if r >= 0:
                a["storage"][i] = (h_land[i] * land["x_length"][i] * land["y_length"][i] + bankfull[r]
                                   if h_land[i] > 0.0 else h_river[r] * river["flow_width"][r] * river["flow_length"][r])
            else:
                a["storage"][i] = h_land[i] * land["x_length"][i] * land["y_length"][i]
        na = river["n_active"]
        a["storage_river"][:] = 0.0
        a["storage_river"][:na] = a["h_river"][:na] * river["flow_width"][:na] * river["flow_length"][:na]

    def set_inputs(self, runoff, external_inflow=None, abstraction=None):
        self.runoff[:] = runoff
        self.ext[:] = 0.0 if external_inflow is None else external_inflow
        self.abs[:] = 0.0 if abstraction is None else abstraction

    def stable_timestep(self):
        return self.L.orc_li_domain_stable_timestep(C.byref(self.g), C.byref(self.r), C.byref(self.st))

    def substep(self, dt):
        self.L.orc_li_domain_substep(C.byref(self.g), C.byref(self.r), _pd(self.runoff), _pd(self.ext), _pd(self.abs),
                                     C.c_double(dt), C.byref(self.st))

    def step(self, dt):
        """update_overland_flow_model! (surface_staggered_scheme.jl:1153-1193) without reservoirs."""
        for k in ("q_cum", "abstraction_cum", "qx_cum", "qy_cum"):
            self.a[k][:] = 0.0
        t, k = 0.0, 0
        while t < dt:
            dt_s = self.stable_timestep()
            if t + dt_s > dt:
                dt_s = dt - t
            self.substep(dt_s)
            t += dt_s
            k += 1
        self.q_avg = self.a["q_cum"] / dt
        self.qx_avg = self.a["qx_cum"][:self.n] / dt
        self.qy_avg = self.a["qy_cum"][:self.n] / dt
        return k

    def get(self, field):
        a = self.a
        return {"h_land": a["h_land"], "storage": a["storage"], "error": a["error"], "qx": a["qx"][:self.n],
                "qy": a["qy"][:self.n], "qx_average": self.qx_avg, "qy_average": self.qy_avg,
                "h_river": a["h_river"], "storage_river": a["storage_river"], "q_river": a["q"],
                "q_river_average": self.q_avg, "abstraction_cumulative": a["abstraction_cum"]}[field].copy()
