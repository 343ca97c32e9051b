"""Local-inertial river flow on the GPU (include/wflow_gb300_li.h), over ctypes.

`LiRiver` holds a river network on a staggered grid (cells and the edges between them) with
its state on the device; `substep`, `stable_timestep` and `step` mirror Wflow's
staggered_scheme_river_update!, stable_timestep and update_river_flow_model! for a channel
without floodplain (Wflow/src/routing/surface/surface_staggered_scheme.jl).
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
            "wf_li_river_set_inwater": (i32, [P, pd]),
            "wf_li_river_stable_timestep": (i32, [P, pd]),
            "wf_li_river_substep": (i32, [P, d]),
            "wf_li_river_step": (i32, [P, d, pl]),
            "wf_li_river_get": (i32, [P, i32, pd]),
        }
        for name, (res, args) in sig.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _declared = True
    return lib


def _pd(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class LiRiver:
    FIELDS = {"h": 0, "storage": 1, "q": 2, "q_cumulative": 3, "q_average": 4}

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
        k = C.c_int64()
        self._check(self.lib.wf_li_river_step(self.h, float(dt), C.byref(k)), "wf_li_river_step")
        return k.value

    def get(self, field):
        f = self.FIELDS[field]
        out = np.empty(self.n if f <= 1 else self.n_edges)
        self._check(self.lib.wf_li_river_get(self.h, f, _pd(out)), "wf_li_river_get")
        return out
