"""ctypes binding of the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg, as the checker of the CUDA path. Product code never imports it.
"""

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

ORACLE_DIR = Path(__file__).resolve().parent
LIB_PATH = ORACLE_DIR / "_build" / "liboracle.so"
MAXL = 8

_lib = None
_d, _i32, _i64, _pd = C.c_double, C.c_int32, C.c_int64, C.POINTER(C.c_double)


def build():
    subprocess.run(["make", "-C", str(ORACLE_DIR)], check=True, capture_output=True)


def lib():
    global _lib
    if _lib is None:
        srcs = [ORACLE_DIR / "wflow_oracle.cpp", ORACLE_DIR / "oracle_math.h", ORACLE_DIR / "wflow_oracle.h"]
        if not LIB_PATH.exists() or any(s.stat().st_mtime > LIB_PATH.stat().st_mtime for s in srcs):
            build()
        L = C.CDLL(str(LIB_PATH))
        for name in ["orc_exp", "orc_log", "orc_cbrt"]:
            getattr(L, name).restype = _d
            getattr(L, name).argtypes = [_d]
        L.orc_pow.restype = _d
        L.orc_pow.argtypes = [_d, _d]
        L.orc_cld.restype = _d
        L.orc_cld.argtypes = [_d, _d]
        L.orc_round_sigdigits.restype = _d
        L.orc_round_sigdigits.argtypes = [_d, _i32]
        L.orc_soil_layout.restype = C.c_char_p
        L.orc_soil_sizeof.restype = _i32
        L.orc_model_error.restype = C.c_char_p
        L.orc_model_error.argtypes = [C.c_void_p]
        L.orc_model_create.restype = _i32
        L.orc_model_create.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p)]
        L.orc_model_destroy.argtypes = [C.c_void_p]
        L.orc_model_set_forcing.argtypes = [C.c_void_p, _pd, _pd, _pd]
        L.orc_model_step.argtypes = [C.c_void_p, _i32]
        L.orc_model_get.argtypes = [C.c_void_p, _i32, _i32, _pd]
        L.orc_model_set.argtypes = [C.c_void_p, _i32, _i32, _pd]
        L.orc_model_outlets.argtypes = [C.c_void_p, _i32, _pd, C.POINTER(_i64)]
        L.orc_model_substeps.argtypes = [C.c_void_p, C.POINTER(_i64), C.POINTER(_i64), C.POINTER(_i64)]
        L.orc_model_substep_signature.restype = _i32
        L.orc_model_substep_signature.argtypes = [C.c_void_p, _i32, _pd]
        L.orc_topo_order_dfs.restype = _i32
        L.orc_topo_order_dfs.argtypes = [_i64, C.POINTER(_i32), C.POINTER(_i64)]
        for name in ["orc_head_brooks_corey", "orc_vwc_brooks_corey", "orc_feddes_h3", "orc_rwu_reduction_feddes",
                     "orc_soil_temperature", "orc_infiltration_reduction_factor",
                     "orc_soil_evaporation_unsaturated_store", "orc_soil_evaporation_saturated_store", "orc_scurve",
                     "orc_ssf_celerity", "orc_kw_ssf_newton_raphson", "orc_kinwave_stable_timestep", "orc_quantile"]:
            getattr(L, name).restype = _d
        _lib = L
    return _lib


# ---------------------------------------------------------------- OrcSoil mirror --------
class Soil:
    """A single OrcSoil column in a raw buffer, addressed by the C layout string."""

    def __init__(self, **fields):
        L = lib()
        self.size = L.orc_soil_sizeof()
        self.buf = (C.c_char * self.size)()
        self.layout = {}
        for item in L.orc_soil_layout().decode().strip(";").split(";"):
            name, off, kind = item.split(":")
            self.layout[name] = (int(off), kind)
        # reference-like defaults: NaN-free zeros
        for k, v in fields.items():
            self[k] = v

    def ptr(self):
        return C.cast(self.buf, C.c_void_p)

    def __setitem__(self, name, value):
        off, kind = self.layout[name]
        if kind == "i":
            C.c_int32.from_buffer(self.buf, off).value = int(value)
        elif kind == "d":
            C.c_double.from_buffer(self.buf, off).value = float(value)
        else:
            n = int(kind[1:])
            arr = (C.c_double * n).from_buffer(self.buf, off)
            vals = list(value)
            for i in range(n):
                arr[i] = float(vals[i]) if i < len(vals) else 0.0

    def __getitem__(self, name):
        off, kind = self.layout[name]
        if kind == "i":
            return C.c_int32.from_buffer(self.buf, off).value
        if kind == "d":
            return C.c_double.from_buffer(self.buf, off).value
        n = int(kind[1:])
        return np.array((C.c_double * n).from_buffer(self.buf, off)[:])


class Reservoir(C.Structure):
    """OrcReservoir (wflow_oracle.cpp): one reservoir's parameters, boundary conditions of the
    step and state."""
    _fields_ = [("outflow_type", C.c_int32)] + [(n, C.c_double) for n in (
        "area", "maximum_storage", "threshold", "rating_curve_coefficient", "rating_curve_exponent",
        "maximum_release", "demand", "target_minimum_fraction", "target_full_fraction",
        "external_inflow", "precipitation", "evaporation", "inflow_overland", "inflow_subsurface", "outflow_obs",
        "storage", "waterlevel", "outflow",
        "inflow_cumulative", "outflow_cumulative", "actevap_cumulative", "abstraction_cumulative")] + [
        ("storage_curve_type", C.c_int32), ("lower", C.c_int32), ("sh_n", C.c_int64), ("hq_n", C.c_int64),
        ("sh_h", C.POINTER(C.c_double)), ("sh_s", C.POINTER(C.c_double)), ("hq_h", C.POINTER(C.c_double)),
        ("hq_q", C.POINTER(C.c_double)), ("hq_day", C.c_int32)]

    def __init__(self, **kw):
        super().__init__()
        self.storage_curve_type = 1
        self.hq_day = 1
        nan = float("nan")
        for n in ("maximum_storage", "threshold", "rating_curve_coefficient", "rating_curve_exponent",
                  "maximum_release", "demand", "target_minimum_fraction", "target_full_fraction", "outflow_obs"):
            setattr(self, n, nan)
        for k, v in kw.items():
            setattr(self, k, v)


def reservoir_update(r, q, dt):
    lib().orc_reservoir_update(C.byref(r), C.c_double(q), C.c_double(dt))


def reservoir_update_model(res, i, inflow, dt):
    """update_reservoir_model!(reservoir_model, i, inflow, dt) on reservoir i (0-based) of the
    ctypes array `res` (Reservoir * n), whose `lower` fields are 1-based indices into it."""
    lib().orc_reservoir_update_model(res, C.c_int64(i), C.c_double(inflow), C.c_double(dt))


def interpolate_linear(x, xp, fp):
    xp = np.ascontiguousarray(xp, np.float64)
    fp = np.ascontiguousarray(fp, np.float64)
    f = lib().orc_interpolate_linear
    f.restype = C.c_double
    return f(C.c_double(x), xp.ctypes.data_as(_pd), fp.ctypes.data_as(_pd), C.c_int64(xp.size))


def call_out(fname, *args, nout):
    out = (C.c_double * nout)()
    fn = getattr(lib(), fname)
    fn(*[a if isinstance(a, (C.c_void_p,)) else (C.c_double(a) if isinstance(a, float) else a) for a in args], out)
    return list(out)


def fcall(fname, *args, types=None):
    fn = getattr(lib(), fname)
    conv = []
    for i, a in enumerate(args):
        t = types[i] if types else ("d" if isinstance(a, float) else "i")
        conv.append(C.c_double(a) if t == "d" else C.c_int32(int(a)) if t == "i" else a)
    return fn(*conv)


# ------------------------------------------------------------------------- model -------
class OracleModel:
    """The oracle's full model on one synthetic domain (the CPU reference of a wf_create handle)."""

    def __init__(self, cfg, dom, params=None, reservoirs=None):
        import sys
        sys.path.insert(0, str(ORACLE_DIR.parent / "wflow.jl_gb300"))
        from wflow_gb300 import synthetic
        self.dom = dom
        self.cfg = cfg
        self._params = params if params is not None else dom.params
        self._d, self._p = synthetic.c_structs(dom, self._params)
        h = C.c_void_p()
        self._reservoirs = reservoirs
        if reservoirs is not None:
            self._r = synthetic.c_reservoirs(reservoirs)
            self._rt = synthetic.c_reservoir_tables(reservoirs)
            st = lib().orc_model_create_with_reservoir_tables(
                C.byref(cfg), C.byref(self._d), C.byref(self._p), C.byref(self._r),
                C.byref(self._rt) if self._rt is not None else None, C.byref(h))
        else:
            st = lib().orc_model_create(C.byref(cfg), C.byref(self._d), C.byref(self._p), C.byref(h))
        self.h = h
        if st != 0:
            msg = lib().orc_model_error(h)
            raise RuntimeError(f"oracle create failed {st}: {msg}")
        self.n = dom.n_land
        self.nr = dom.n_river
        self.M = max(1, cfg.n_members)
        self.nres = 0 if reservoirs is None else int(reservoirs["river_index"].size)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_model_destroy(self.h)
            self.h = None

    def set_forcing(self, P, PET, T):
        P, PET, T = (np.ascontiguousarray(x, dtype=np.float64) for x in (P, PET, T))
        lib().orc_model_set_forcing(self.h, P.ctypes.data_as(_pd), PET.ctypes.data_as(_pd), T.ctypes.data_as(_pd))

    def set_rating_curve_day(self, day):
        if lib().orc_model_set_rating_curve_day(self.h, int(day)) != 0:
            raise ValueError(day)

    def step(self, threads=1):
        lib().orc_model_step(self.h, threads)

    def get(self, field, layer=0):
        nn = (self.nres if field >= 200 else self.nr if field >= 100 else self.n) * self.M
        out = np.empty(nn)
        st = lib().orc_model_get(self.h, field, layer, out.ctypes.data_as(_pd))
        if st != 0:
            raise KeyError(field)
        return out

    def set(self, field, values, layer=0):
        v = np.ascontiguousarray(values, dtype=np.float64)
        lib().orc_model_set(self.h, field, layer, v.ctypes.data_as(_pd))

    def attach_li(self, land, river, h_land, h_river):
        """orc_model_attach_li: local-inertial land and river routing in the step (the dicts of
        wflow_gb300.li_river's structs)."""
        from wflow_gb300.li_river import land_grid, river_network
        keep = []
        g, r = land_grid(land, keep), river_network(river, keep)
        hl = np.ascontiguousarray(h_land, np.float64)
        hr = np.ascontiguousarray(h_river, np.float64)
        st = lib().orc_model_attach_li(self.h, C.byref(g), C.byref(r), hl.ctypes.data_as(_pd), hr.ctypes.data_as(_pd))
        if st != 0:
            raise RuntimeError(f"orc_model_attach_li failed {st}: {lib().orc_model_error(self.h)}")
        self.n_river_total = len(river["zb"])
        self.n_edges = len(river["src"])

    def li_get(self, field):
        """A WfLiDomainField of the coupled scheme (-1: the sub-steps of the last step)."""
        n = {-1: 1, 7: self.n_river_total, 8: self.n_river_total, 11: self.n_river_total, 9: self.n_edges,
             10: self.n_edges}.get(field, self.n)
        out = np.empty(n)
        if lib().orc_model_li_get(self.h, field, out.ctypes.data_as(_pd)) != 0:
            raise KeyError(field)
        return out

    def outlets(self, which=0):
        out = np.empty(max(1, self.nr * self.M))
        n = C.c_int64()
        lib().orc_model_outlets(self.h, which, out.ctypes.data_as(_pd), C.byref(n))
        return out[: n.value].copy()

    def substep_signature(self, kind):
        """Per member, the sum of the squared sub-step sizes of the last step (0 subsurface, 1 land,
        2 river)."""
        out = np.empty(self.M)
        if lib().orc_model_substep_signature(self.h, int(kind), out.ctypes.data_as(_pd)) != 0:
            raise RuntimeError("no sub-step signature")
        return out

    def substeps(self):
        a, b, c = C.c_int64(), C.c_int64(), C.c_int64()
        lib().orc_model_substeps(self.h, C.byref(a), C.byref(b), C.byref(c))
        return a.value, b.value, c.value
