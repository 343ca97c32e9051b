"""Local-inertial routing on the GPU (include/wflow_gb300_li.h), over ctypes.

`LiRiver` holds a river network on a staggered grid (cells and the edges between them) with
its state on the device; `substep`, `stable_timestep` and `step` mirror Wflow's
staggered_scheme_river_update!, stable_timestep and update_river_flow_model! for a channel
without floodplain (Wflow/src/routing/surface/surface_staggered_scheme.jl).

`LiDomain` adds the land grid: overland flow on the x and y cell edges coupled with the river
(update_overland_flow_model!, surface_staggered_scheme.jl:1153-1193), river cells sharing one
storage between channel and floodplain.
"""

import ctypes as C

import numpy as np

from . import abi

_declared = False


def _lib():
    global _declared
    lib = abi.load_library(required=True)
    if not _declared:
        P, i32, i64, d = C.c_void_p, C.c_int32, C.c_int64, C.c_double
        pd, pl = C.POINTER(C.c_double), C.POINTER(C.c_int64)
        sig = {
            "wf_li_river_create": (i32, [i64, i64, i64, pl, pl, pd, pd, pd, pd, pd, pd, pd, pd, d, i32, d, i32,
                                         C.POINTER(P)]),
            "wf_li_river_destroy": (None, [P]),
            "wf_li_river_last_error": (C.c_char_p, [P]),
            "wf_li_river_set_state": (i32, [P, pd, pd]),
            "wf_li_river_set_timestep_cells": (i32, [P, i64]),
            "wf_li_river_set_boundary": (i32, [P, pd, pd]),
            "wf_li_river_set_inwater": (i32, [P, pd]),
            "wf_li_river_stable_timestep": (i32, [P, pd]),
            "wf_li_river_substep": (i32, [P, d]),
            "wf_li_river_step": (i32, [P, d, pl]),
            "wf_li_river_set_host_loop": (i32, [P, i32]),
            "wf_li_river_get": (i32, [P, i32, pd]),
            "wf_li_domain_create": (i32, [C.POINTER(WfLiLandGrid), C.POINTER(WfLiRiverNetwork), pd, i32,
                                          C.POINTER(P)]),
            "wf_li_domain_destroy": (None, [P]),
            "wf_li_domain_last_error": (C.c_char_p, [P]),
            "wf_li_domain_set_state": (i32, [P, pd, pd, pd, pd, pd]),
            "wf_li_domain_set_inputs": (i32, [P, pd, pd, pd]),
            "wf_li_domain_stable_timestep": (i32, [P, pd]),
            "wf_li_domain_substep": (i32, [P, d]),
            "wf_li_domain_step": (i32, [P, d, pl]),
            "wf_li_domain_set_host_loop": (i32, [P, i32]),
            "wf_li_domain_get": (i32, [P, i32, pd]),
        }
        for name, (res, args) in sig.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _declared = True
    return lib


def _pd(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _pl(a):
    return a.ctypes.data_as(C.POINTER(C.c_int64))


_PL, _PD = C.POINTER(C.c_int64), C.POINTER(C.c_double)


class WfLiLandGrid(C.Structure):
    _fields_ = [("n", C.c_int64)] + [(f, _PL) for f in ("ind_x_up", "ind_x_down", "ind_y_up", "ind_y_down",
                                                         "river_index")] + \
               [(f, _PD) for f in ("x_length", "y_length", "elevation", "mannings_n_sq", "xwidth_at_edge",
                                   "ywidth_at_edge")] + \
               [("theta", C.c_double), ("h_thresh", C.c_double), ("alpha", C.c_double), ("froude_limit", C.c_int32)]


class WfLiRiverNetwork(C.Structure):
    _fields_ = [("n", C.c_int64), ("n_active", C.c_int64), ("n_edges", C.c_int64), ("src", _PL), ("dst", _PL)] + \
               [(f, _PD) for f in ("zb", "flow_length", "flow_width", "bankfull_depth", "zb_edge", "width_edge",
                                   "length_edge", "mannings_n_sq_edge")] + \
               [("h_thresh", C.c_double), ("alpha", C.c_double), ("froude_limit", C.c_int32)]


LAND_INT = ("ind_x_up", "ind_x_down", "ind_y_up", "ind_y_down", "river_index")
LAND_DBL = ("x_length", "y_length", "elevation", "mannings_n_sq", "xwidth_at_edge", "ywidth_at_edge")
RIVER_INT = ("src", "dst")
RIVER_CELL = ("zb", "flow_length", "flow_width", "bankfull_depth")
RIVER_EDGE = ("zb_edge", "width_edge", "length_edge", "mannings_n_sq_edge")


def land_grid(land, keep):
    """A WfLiLandGrid over the arrays of `land` (a dict; the arrays are kept alive in `keep`)."""
    n = len(land["x_length"])
    g = WfLiLandGrid()
    g.n = n
    for f in LAND_INT:
        a = np.ascontiguousarray(land[f], np.int64)
        if a.shape != (n,):
            raise ValueError(f"{f} must have {n} values")
        keep.append(a)
        setattr(g, f, _pl(a))
    for f in LAND_DBL:
        a = np.ascontiguousarray(land[f], np.float64)
        if a.shape != (n,):
            raise ValueError(f"{f} must have {n} values")
        keep.append(a)
        setattr(g, f, _pd(a))
    g.theta, g.h_thresh, g.alpha = float(land["theta"]), float(land["h_thresh"]), float(land["alpha"])
    g.froude_limit = int(bool(land["froude_limit"]))
    return g


def river_network(river, keep):
    """A WfLiRiverNetwork over the arrays of `river` (a dict)."""
    n, ne = len(river["zb"]), len(river["src"])
    r = WfLiRiverNetwork()
    r.n, r.n_active, r.n_edges = n, int(river["n_active"]), ne
    for f in RIVER_INT + RIVER_CELL + RIVER_EDGE:
        dt = np.int64 if f in RIVER_INT else np.float64
        a = np.ascontiguousarray(river[f], dt)
        m = n if f in RIVER_CELL else ne
        if a.shape != (m,):
            raise ValueError(f"{f} must have {m} values")
        keep.append(a)
        setattr(r, f, _pl(a) if f in RIVER_INT else _pd(a))
    r.h_thresh, r.alpha = float(river["h_thresh"]), float(river["alpha"])
    r.froude_limit = int(bool(river["froude_limit"]))
    return r


class LiRiver:
    FIELDS = {"h": 0, "storage": 1, "q": 2, "q_cumulative": 3, "q_average": 4, "error": 5,
              "abstraction_cumulative": 6}

    def __init__(self, src, dst, zb, flow_length, flow_width, h_init, zb_edge, width_edge, length_edge,
                 mannings_n_sq_edge, n_active, h_thresh=1e-3, froude_limit=True, alpha=0.7, device=0):
        self.lib = _lib()
        self._keep = [np.ascontiguousarray(a, np.int64) for a in (src, dst)] + [
            np.ascontiguousarray(a, np.float64) for a in (zb, flow_length, flow_width, h_init, zb_edge, width_edge,
                                                          length_edge, mannings_n_sq_edge)]
        s, d_, zb_, fl, fw, h0, zbe, we, le, ne = self._keep
        self.n, self.n_edges = len(zb_), len(s)
        for name, a, m in (("dst", d_, self.n_edges), ("flow_length", fl, self.n), ("flow_width", fw, self.n),
                           ("h_init", h0, self.n), ("zb_edge", zbe, self.n_edges), ("width_edge", we, self.n_edges),
                           ("length_edge", le, self.n_edges), ("mannings_n_sq_edge", ne, self.n_edges)):
            if a.shape != (m,):
                raise ValueError(f"{name} must have {m} values, got shape {a.shape}")
        self.h = C.c_void_p()
        pl = lambda a: a.ctypes.data_as(C.POINTER(C.c_int64))  # noqa: E731
        st = self.lib.wf_li_river_create(self.n, int(n_active), self.n_edges, pl(s), pl(d_), _pd(zb_), _pd(fl), _pd(fw),
                                         _pd(h0), _pd(zbe), _pd(we), _pd(le), _pd(ne), float(h_thresh),
                                         int(bool(froude_limit)), float(alpha), int(device), C.byref(self.h))
        if st != 0:
            msg = self.lib.wf_li_river_last_error(None)
            raise RuntimeError(f"wf_li_river_create failed ({st}): {msg.decode() if msg else ''}")

    def _check(self, st, what):
        if st != 0:
            msg = self.lib.wf_li_river_last_error(self.h)
            raise RuntimeError(f"{what} failed ({st}): {msg.decode() if msg else ''}")

    def close(self):
        if getattr(self, "h", None):
            self.lib.wf_li_river_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, h, q=None):
        """Depth of every cell and (optionally) discharge of every edge; storage = h w l."""
        hv = np.ascontiguousarray(h, np.float64)
        if hv.shape != (self.n,):
            raise ValueError(f"h must have {self.n} values")
        qv = None if q is None else np.ascontiguousarray(q, np.float64)
        if qv is not None and qv.shape != (self.n_edges,):
            raise ValueError(f"q must have {self.n_edges} values")
        self._check(self.lib.wf_li_river_set_state(self.h, _pd(hv), None if qv is None else _pd(qv)),
                    "wf_li_river_set_state")

    def set_timestep_cells(self, n_cells):
        """The stable time step over cells 0..n_cells-1 (default all; a Wflow model's river
        passes its real cells, the ghost cells coming after them)."""
        self._check(self.lib.wf_li_river_set_timestep_cells(self.h, int(n_cells)), "wf_li_river_set_timestep_cells")

    def set_manning(self, slope_edge, mannings_n_edge):
        """Manning's equation on the staggered grid instead of the local-inertial edge update
        (river_routing = "manning_staggered"): per edge slope and Manning's n."""
        s_ = np.ascontiguousarray(slope_edge, np.float64)
        n_ = np.ascontiguousarray(mannings_n_edge, np.float64)
        if s_.shape != (self.n_edges,) or n_.shape != (self.n_edges,):
            raise ValueError(f"edge arrays must have {self.n_edges} values")
        self._check(self.lib.wf_li_river_set_manning(self.h, _pd(s_), _pd(n_)), "wf_li_river_set_manning")

    def set_boundary(self, external_inflow=None, abstraction=None):
        """External inflow and abstraction of every cell [m3 s-1] (None: zero)."""
        v = [None if a is None else np.ascontiguousarray(a, np.float64) for a in (external_inflow, abstraction)]
        if any(a is not None and a.shape != (self.n,) for a in v):
            raise ValueError(f"boundary arrays must have {self.n} values")
        self._check(self.lib.wf_li_river_set_boundary(self.h, *[None if a is None else _pd(a) for a in v]),
                    "wf_li_river_set_boundary")

    def set_inwater(self, inwater):
        v = np.ascontiguousarray(inwater, np.float64)
        if v.shape != (self.n,):
            raise ValueError(f"inwater must have {self.n} values")
        self._check(self.lib.wf_li_river_set_inwater(self.h, _pd(v)), "wf_li_river_set_inwater")

    def stable_timestep(self):
        dt = C.c_double()
        self._check(self.lib.wf_li_river_stable_timestep(self.h, C.byref(dt)), "wf_li_river_stable_timestep")
        return dt.value

    def substep(self, dt_s):
        self._check(self.lib.wf_li_river_substep(self.h, float(dt_s)), "wf_li_river_substep")

    def step(self, dt):
        """update_river_flow_model! over dt: the sub-step loop on the device (one cooperative
        launch); returns the number of sub-steps."""
        k = C.c_int64()
        self._check(self.lib.wf_li_river_step(self.h, float(dt), C.byref(k)), "wf_li_river_step")
        return k.value

    def set_host_loop(self, on=True):
        """Drive the sub-steps of step() from the host instead (the same results)."""
        self._check(self.lib.wf_li_river_set_host_loop(self.h, int(bool(on))), "wf_li_river_set_host_loop")

    def get(self, field):
        f = self.FIELDS[field]
        out = np.empty(self.n if (f <= 1 or f >= 5) else self.n_edges)
        self._check(self.lib.wf_li_river_get(self.h, f, _pd(out)), "wf_li_river_get")
        return out


class LiDomain:
    """The land grid with its river (wf_li_domain_*). `land` and `river` are dicts with the
    fields of WfLiLandGrid and WfLiRiverNetwork; h_river the starting river depths (the ghost
    cells' boundary depths)."""

    FIELDS = {"h_land": 0, "storage": 1, "error": 2, "qx": 3, "qy": 4, "qx_average": 5, "qy_average": 6,
              "h_river": 7, "storage_river": 8, "q_river": 9, "q_river_average": 10, "abstraction_cumulative": 11}

    def __init__(self, land, river, h_river, device=0):
        self.lib = _lib()
        self._keep = []
        g, r = land_grid(land, self._keep), river_network(river, self._keep)
        self.n, self.nr, self.ne = g.n, r.n, r.n_edges
        hr = np.ascontiguousarray(h_river, np.float64)
        if hr.shape != (self.nr,):
            raise ValueError(f"h_river must have {self.nr} values")
        self.h = C.c_void_p()
        st = self.lib.wf_li_domain_create(C.byref(g), C.byref(r), _pd(hr), int(device), C.byref(self.h))
        if st != 0:
            msg = self.lib.wf_li_domain_last_error(None)
            raise RuntimeError(f"wf_li_domain_create failed ({st}): {msg.decode() if msg else ''}")

    def _check(self, st, what):
        if st != 0:
            msg = self.lib.wf_li_domain_last_error(self.h)
            raise RuntimeError(f"{what} failed ({st}): {msg.decode() if msg else ''}")

    def _vec(self, a, m, name):
        if a is None:
            return None
        v = np.ascontiguousarray(a, np.float64)
        if v.shape != (m,):
            raise ValueError(f"{name} must have {m} values")
        return v

    def close(self):
        if getattr(self, "h", None):
            self.lib.wf_li_domain_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, h_land, h_river, qx=None, qy=None, q_river=None):
        v = [self._vec(h_land, self.n, "h_land"), self._vec(h_river, self.nr, "h_river"), self._vec(qx, self.n, "qx"),
             self._vec(qy, self.n, "qy"), self._vec(q_river, self.ne, "q_river")]
        self._check(self.lib.wf_li_domain_set_state(self.h, *[None if a is None else _pd(a) for a in v]),
                    "wf_li_domain_set_state")

    def set_inputs(self, runoff, external_inflow=None, abstraction=None):
        v = [self._vec(runoff, self.n, "runoff"), self._vec(external_inflow, self.nr, "external_inflow"),
             self._vec(abstraction, self.nr, "abstraction")]
        self._check(self.lib.wf_li_domain_set_inputs(self.h, *[None if a is None else _pd(a) for a in v]),
                    "wf_li_domain_set_inputs")

    def stable_timestep(self):
        dt = C.c_double()
        self._check(self.lib.wf_li_domain_stable_timestep(self.h, C.byref(dt)), "wf_li_domain_stable_timestep")
        return dt.value

    def substep(self, dt_s):
        self._check(self.lib.wf_li_domain_substep(self.h, float(dt_s)), "wf_li_domain_substep")

    def step(self, dt):
        """update_overland_flow_model! over dt: the sub-step loop on the device; returns the
        number of sub-steps."""
        k = C.c_int64()
        self._check(self.lib.wf_li_domain_step(self.h, float(dt), C.byref(k)), "wf_li_domain_step")
        return k.value

    def set_host_loop(self, on=True):
        """Drive the sub-steps of step() from the host instead (the same results)."""
        self._check(self.lib.wf_li_domain_set_host_loop(self.h, int(bool(on))), "wf_li_domain_set_host_loop")

    def get(self, field):
        f = self.FIELDS[field]
        m = self.n if f <= 6 else (self.ne if f in (9, 10) else self.nr)
        out = np.empty(m)
        self._check(self.lib.wf_li_domain_get(self.h, f, _pd(out)), "wf_li_domain_get")
        return out
