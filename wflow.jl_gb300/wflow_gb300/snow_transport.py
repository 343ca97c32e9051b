"""Lateral snow transport on the GPU (include/wflow_gb300_snow.h), over ctypes.

`SnowTransport(ds, order, slope, ups_ds=None)` holds the land graph; `run(dt, snow_storage,
snow_water)` moves the two states in place as lateral_snow_transport! does
(Wflow/src/routing/surface/surface_process.jl:1-19) and returns (snow_out, snow_in) [m s-1].
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
        pd, pl, pi = C.POINTER(C.c_double), C.POINTER(C.c_int64), C.POINTER(C.c_int32)
        for name, res, args in (("wf_snow_transport_create", i32, [i64, pi, pl, pi, pd, i32, C.POINTER(P)]),
                                ("wf_snow_transport_destroy", None, [P]),
                                ("wf_snow_transport_last_error", C.c_char_p, [P]),
                                ("wf_snow_transport_run", i32, [P, d, pd, pd, pd, pd]),
                                ("wf_snow_transport_levels", i64, [P])):
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _declared = True
    return lib


class SnowTransport:
    def __init__(self, ds, order, slope, ups_ds=None, device=0):
        self.lib = _lib()
        self.ds = np.ascontiguousarray(ds, np.int32)
        self.n = len(self.ds)
        self.order = np.ascontiguousarray(order, np.int64)
        self.slope = np.ascontiguousarray(slope, np.float64)
        self.ups = None if ups_ds is None else np.ascontiguousarray(ups_ds, np.int32)
        for name, a in (("order", self.order), ("slope", self.slope), ("ups_ds", self.ups)):
            if a is not None and a.shape != (self.n,):
                raise ValueError(f"{name} must have {self.n} values")
        pi = C.POINTER(C.c_int32)
        self.h = C.c_void_p()
        st = self.lib.wf_snow_transport_create(
            self.n, self.ds.ctypes.data_as(pi), self.order.ctypes.data_as(C.POINTER(C.c_int64)),
            None if self.ups is None else self.ups.ctypes.data_as(pi),
            self.slope.ctypes.data_as(C.POINTER(C.c_double)), int(device), C.byref(self.h))
        if st != 0:
            msg = self.lib.wf_snow_transport_last_error(None)
            raise RuntimeError(f"wf_snow_transport_create failed ({st}): {msg.decode() if msg else ''}")

    @property
    def levels(self):
        return int(self.lib.wf_snow_transport_levels(self.h))

    def run(self, dt, snow_storage, snow_water):
        """Moves snow_storage and snow_water (float64 arrays of n values) in place; returns
        (snow_out, snow_in)."""
        for name, a in (("snow_storage", snow_storage), ("snow_water", snow_water)):
            if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.shape == (self.n,)
                    and a.flags.c_contiguous):
                raise ValueError(f"{name} must be a contiguous float64 array of {self.n} values")
        out, inn = np.empty(self.n), np.empty(self.n)
        pd = C.POINTER(C.c_double)
        st = self.lib.wf_snow_transport_run(self.h, float(dt), snow_storage.ctypes.data_as(pd),
                                            snow_water.ctypes.data_as(pd), out.ctypes.data_as(pd),
                                            inn.ctypes.data_as(pd))
        if st != 0:
            msg = self.lib.wf_snow_transport_last_error(self.h)
            raise RuntimeError(f"wf_snow_transport_run failed ({st}): {msg.decode() if msg else ''}")
        return out, inn

    def close(self):
        if getattr(self, "h", None):
            self.lib.wf_snow_transport_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _glacier_lib():
    lib = _lib()
    if not getattr(lib, "_glacier_declared", False):
        P, i32, i64, d = C.c_void_p, C.c_int32, C.c_int64, C.c_double
        pd = C.POINTER(C.c_double)
        for name, res, args in (("wf_glacier_create", i32, [i64, pd, pd, pd, pd, d, i32, C.POINTER(P)]),
                                ("wf_glacier_destroy", None, [P]),
                                ("wf_glacier_last_error", C.c_char_p, [P]),
                                ("wf_glacier_run", i32, [P, d, pd, pd, pd, pd])):
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        lib._glacier_declared = True
    return lib


class Glacier:
    """The HBV glacier of every cell (wf_glacier_*, update_glacier_model!,
    Wflow/src/glacier/glacier.jl:122-154)."""

    def __init__(self, glacier_fraction, temperature_threshold_melt, degree_day_factor, snow_to_ice_fraction,
                 maximum_snow_to_ice_rate, device=0):
        self.lib = _glacier_lib()
        self._keep = [np.ascontiguousarray(a, np.float64) for a in (glacier_fraction, temperature_threshold_melt,
                                                                    degree_day_factor, snow_to_ice_fraction)]
        self.n = len(self._keep[0])
        if any(a.shape != (self.n,) for a in self._keep):
            raise ValueError(f"the glacier parameters must have {self.n} values each")
        pd = C.POINTER(C.c_double)
        self.h = C.c_void_p()
        st = self.lib.wf_glacier_create(self.n, *[a.ctypes.data_as(pd) for a in self._keep],
                                        float(maximum_snow_to_ice_rate), int(device), C.byref(self.h))
        if st != 0:
            msg = self.lib.wf_glacier_last_error(None)
            raise RuntimeError(f"wf_glacier_create failed ({st}): {msg.decode() if msg else ''}")

    def run(self, dt, temperature, snow_storage, glacier_store):
        """Updates snow_storage and glacier_store in place; returns the glacier melt [m s-1]."""
        t = np.ascontiguousarray(temperature, np.float64)
        for name, a in (("snow_storage", snow_storage), ("glacier_store", glacier_store)):
            if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.shape == (self.n,)
                    and a.flags.c_contiguous):
                raise ValueError(f"{name} must be a contiguous float64 array of {self.n} values")
        if t.shape != (self.n,):
            raise ValueError(f"temperature must have {self.n} values")
        melt = np.empty(self.n)
        pd = C.POINTER(C.c_double)
        st = self.lib.wf_glacier_run(self.h, float(dt), t.ctypes.data_as(pd), snow_storage.ctypes.data_as(pd),
                                     glacier_store.ctypes.data_as(pd), melt.ctypes.data_as(pd))
        if st != 0:
            msg = self.lib.wf_glacier_last_error(self.h)
            raise RuntimeError(f"wf_glacier_run failed ({st}): {msg.decode() if msg else ''}")
        return melt

    def close(self):
        if getattr(self, "h", None):
            self.lib.wf_glacier_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
