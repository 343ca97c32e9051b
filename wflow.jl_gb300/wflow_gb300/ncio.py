"""netCDF classic-format files (CDF-1, CDF-2, CDF-5) over the library's native reader/writer.

`NcFile` wraps the C ABI of include/wflow_gb300_nc.h (wf_netcdf.cpp in the step library). It
is what the static-map and state helpers (`wflow_gb300.states`) read and write; arrays come
back in the file's C order (record dimension first), as Wflow's files store them: a Julia
variable of dimensions (x, y, layer, time) is (time, layer, y, x) here.
"""

import ctypes as C

import numpy as np

from . import abi

NC_BYTE, NC_CHAR, NC_SHORT, NC_INT, NC_FLOAT, NC_DOUBLE = 1, 2, 3, 4, 5, 6
NC_UBYTE, NC_USHORT, NC_UINT, NC_INT64, NC_UINT64 = 7, 8, 9, 10, 11
NC_GLOBAL = -1
TYPE_OF_DTYPE = {np.dtype("int8"): NC_BYTE, np.dtype("int16"): NC_SHORT, np.dtype("int32"): NC_INT,
                 np.dtype("float32"): NC_FLOAT, np.dtype("float64"): NC_DOUBLE, np.dtype("uint8"): NC_UBYTE,
                 np.dtype("uint16"): NC_USHORT, np.dtype("uint32"): NC_UINT, np.dtype("int64"): NC_INT64,
                 np.dtype("uint64"): NC_UINT64}

_declared = False


def _lib():
    global _declared
    lib = abi.load_library(required=True)
    if not _declared:
        P, i32, i64, pd, pi64 = C.c_void_p, C.c_int32, C.c_int64, C.POINTER(C.c_double), C.POINTER(C.c_int64)
        sig = {
            "wf_nc_open": (i32, [C.c_char_p, C.POINTER(P)]),
            "wf_nc_close": (None, [P]),
            "wf_nc_last_error": (C.c_char_p, [P]),
            "wf_nc_format": (i32, [P]),
            "wf_nc_numrecs": (i64, [P]),
            "wf_nc_ndims": (i32, [P]),
            "wf_nc_nvars": (i32, [P]),
            "wf_nc_dim": (i32, [P, i32, C.c_char_p, i32, pi64, C.POINTER(i32)]),
            "wf_nc_var": (i32, [P, i32, C.c_char_p, i32, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32)]),
            "wf_nc_varid": (i32, [P, C.c_char_p]),
            "wf_nc_natts": (i32, [P, i32]),
            "wf_nc_att_name": (i32, [P, i32, i32, C.c_char_p, i32]),
            "wf_nc_att": (i32, [P, i32, C.c_char_p, C.POINTER(i32), pi64]),
            "wf_nc_att_get": (i32, [P, i32, C.c_char_p, pd, i64]),
            "wf_nc_att_text": (i32, [P, i32, C.c_char_p, C.c_char_p, i64]),
            "wf_nc_get": (i32, [P, i32, pi64, pi64, pd, i32]),
            "wf_nc_create": (i32, [C.c_char_p, i32, C.POINTER(P)]),
            "wf_nc_def_dim": (i32, [P, C.c_char_p, i64]),
            "wf_nc_def_var": (i32, [P, C.c_char_p, i32, i32, C.POINTER(i32)]),
            "wf_nc_put_att_text": (i32, [P, i32, C.c_char_p, C.c_char_p]),
            "wf_nc_put_att": (i32, [P, i32, C.c_char_p, i32, pd, i64]),
            "wf_nc_enddef": (i32, [P]),
            "wf_nc_put": (i32, [P, i32, pi64, pi64, pd]),
        }
        for name, (res, args) in sig.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _declared = True
    return lib


class NcFile:
    """A netCDF classic-format file: mode "r" reads, mode "w" creates (format 1, 2 or 5)."""

    def __init__(self, path, mode="r", format=2):
        self.lib = _lib()
        self.h = C.c_void_p()
        self.path = str(path)
        if mode == "r":
            st = self.lib.wf_nc_open(self.path.encode(), C.byref(self.h))
        elif mode == "w":
            st = self.lib.wf_nc_create(self.path.encode(), int(format), C.byref(self.h))
        else:
            raise ValueError(mode)
        if st != 0:
            msg = self.lib.wf_nc_last_error(None)
            raise OSError(f"{self.path}: {msg.decode() if msg else st}")
        self.mode = mode
        self._define = mode == "w"

    def _check(self, st, what):
        if st < 0:
            msg = self.lib.wf_nc_last_error(self.h)
            raise ValueError(f"{what}: {msg.decode() if msg else st}")
        return st

    def close(self):
        if self.h:
            if self._define:
                self.enddef()
            self.lib.wf_nc_close(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- reading
    @property
    def format(self):
        return self.lib.wf_nc_format(self.h)

    @property
    def numrecs(self):
        return self.lib.wf_nc_numrecs(self.h)

    @property
    def dimensions(self):
        """name -> (length, is_record) (the record dimension's length is the record count)."""
        out = {}
        buf = C.create_string_buffer(1024)
        n, rec = C.c_int64(), C.c_int32()
        for i in range(self.lib.wf_nc_ndims(self.h)):
            self.lib.wf_nc_dim(self.h, i, buf, 1024, C.byref(n), C.byref(rec))
            out[buf.value.decode(errors="replace")] = (n.value, bool(rec.value))
        return out

    @property
    def variables(self):
        """name -> (nc type, dimension names)."""
        dims = list(self.dimensions)
        out = {}
        buf = C.create_string_buffer(1024)
        t, nd = C.c_int32(), C.c_int32()
        ids = (C.c_int32 * 16)()
        for i in range(self.lib.wf_nc_nvars(self.h)):
            self.lib.wf_nc_var(self.h, i, buf, 1024, C.byref(t), C.byref(nd), ids)
            out[buf.value.decode(errors="replace")] = (t.value, tuple(dims[ids[k]] for k in range(nd.value)))
        return out

    def _varid(self, name):
        if name is None:
            return NC_GLOBAL
        v = self.lib.wf_nc_varid(self.h, name.encode())
        if v < 0:
            raise KeyError(name)
        return v

    def attrs(self, name=None):
        """Attributes of a variable (or the file's with name=None): text or float arrays."""
        vid = self._varid(name)
        out = {}
        for key in self._att_names(vid):
            t, n = C.c_int32(), C.c_int64()
            self.lib.wf_nc_att(self.h, vid, key.encode(), C.byref(t), C.byref(n))
            if t.value == NC_CHAR:
                buf = C.create_string_buffer(n.value + 1)
                self.lib.wf_nc_att_text(self.h, vid, key.encode(), buf, n.value + 1)
                out[key] = buf.value.decode(errors="replace")
            else:
                a = np.zeros(n.value)
                self.lib.wf_nc_att_get(self.h, vid, key.encode(), abi.as_ptr(a), n.value)
                out[key] = a
        return out

    def _att_names(self, vid):
        buf = C.create_string_buffer(1024)
        out = []
        for i in range(max(0, self.lib.wf_nc_natts(self.h, vid))):
            self.lib.wf_nc_att_name(self.h, vid, i, buf, 1024)
            out.append(buf.value.decode(errors="replace"))
        return out

    def shape(self, name):
        dims = self.dimensions
        return tuple(dims[d][0] for d in self.variables[name][1])

    def read(self, name, decode=True, start=None, count=None):
        """Variable (or hyperslab) as float64, CF-decoded unless decode=False."""
        vid = self._varid(name)
        shape = self.shape(name)
        start = [0] * len(shape) if start is None else list(start)
        count = [s - a for s, a in zip(shape, start)] if count is None else list(count)
        out = np.empty(int(np.prod(count)) if count else 1)
        st = np.asarray(start, np.int64)
        ct = np.asarray(count, np.int64)
        self._check(self.lib.wf_nc_get(self.h, vid, st.ctypes.data_as(C.POINTER(C.c_int64)),
                                       ct.ctypes.data_as(C.POINTER(C.c_int64)), abi.as_ptr(out), int(bool(decode))),
                    f"read {name}")
        return out.reshape(count) if count else out[0]

    # ---- writing
    def def_dim(self, name, length):
        """length 0 (or None) defines the record dimension."""
        return self._check(self.lib.wf_nc_def_dim(self.h, name.encode(), int(length or 0)), f"dimension {name}")

    def def_var(self, name, nctype, dims, attrs=None):
        names = self._defined_dims()
        ids = (C.c_int32 * max(1, len(dims)))(*[names.index(d) for d in dims])
        vid = self._check(self.lib.wf_nc_def_var(self.h, name.encode(), int(nctype), len(dims), ids), f"variable {name}")
        for k, v in (attrs or {}).items():
            self.put_att(name, k, v, nctype)
        return vid

    def _defined_dims(self):
        out = []
        buf = C.create_string_buffer(1024)
        for i in range(self.lib.wf_nc_ndims(self.h)):
            self.lib.wf_nc_dim(self.h, i, buf, 1024, None, None)
            out.append(buf.value.decode(errors="replace"))
        return out

    def put_att(self, var, key, value, nctype=NC_DOUBLE):
        vid = self._varid(var)
        if isinstance(value, str):
            self._check(self.lib.wf_nc_put_att_text(self.h, vid, key.encode(), value.encode()), f"attribute {key}")
        else:
            a = np.atleast_1d(np.asarray(value, np.float64))
            t = nctype if key in ("_FillValue", "missing_value", "valid_min", "valid_max") else NC_DOUBLE
            self._check(self.lib.wf_nc_put_att(self.h, vid, key.encode(), int(t), abi.as_ptr(a), a.size),
                        f"attribute {key}")

    def enddef(self):
        if self._define:
            self._check(self.lib.wf_nc_enddef(self.h), "enddef")
            self._define = False

    def write(self, name, values, start=None):
        self.enddef()
        vid = self._varid(name)
        v = np.ascontiguousarray(values, np.float64)
        shape = v.shape if v.ndim else ()
        start = [0] * len(shape) if start is None else list(start)
        st = np.asarray(start, np.int64)
        ct = np.asarray(shape, np.int64)
        self._check(self.lib.wf_nc_put(self.h, vid, st.ctypes.data_as(C.POINTER(C.c_int64)),
                                       ct.ctypes.data_as(C.POINTER(C.c_int64)), abi.as_ptr(v)), f"write {name}")
