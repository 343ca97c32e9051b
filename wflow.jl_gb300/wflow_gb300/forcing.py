"""Wflow forcing files: the step's precipitation, potential evaporation and temperature from a
netCDF forcing file, as Wflow's `update_forcing!` reads them (Wflow/src/io.jl:108-160).

For a model time t the record is the first one at or after t (backward fill, `get_at`,
io.jl:9-29: a forcing time stamps the end of its interval); the grid is standardised (x and y
increasing, io.jl:1346-1352); the TOML-style mapping names the file variables and may add a
scale and offset (apply_affine_transform!); values are converted to SI as the standard-name
tables say (precipitation and potential evaporation in mm per model step, temperature in
degC; units.jl:271). With reservoirs, precipitation and potential evaporation over each
reservoir's area are averaged into the reservoir's inputs and set to zero on the land cells
there (io.jl:128-137). Missing values on active cells are an error, as in the reference.
"""

import datetime as _dt
import re

import numpy as np

from . import ncio
from .staticmaps import _Maps

PRECIP = "atmosphere_water__precipitation_volume_flux"
PET = "land_surface_water__potential_evaporation_volume_flux"
TEMP = "atmosphere_air__temperature"
_UNIT_SECONDS = {"second": 1.0, "seconds": 1.0, "s": 1.0, "minute": 60.0, "minutes": 60.0, "hour": 3600.0,
                 "hours": 3600.0, "h": 3600.0, "day": 86400.0, "days": 86400.0, "d": 86400.0}


def to_si_factor_per_step(dt, length_factor=1e-3):
    """Factor of a unit "length per model step" to SI (units.jl:256-269): the length's factor
    times dt^-1 (mm per step by default)."""
    return length_factor * (1.0 / float(dt))


def parse_time_units(units):
    """CF time units "<unit> since <date>[ <time>]" -> (seconds per unit, epoch datetime)."""
    m = re.match(r"\s*(\w+)\s+since\s+(\d{1,4})-(\d{1,2})-(\d{1,2})(?:[ T](\d{1,2}):(\d{1,2})(?::(\d{1,2}(?:\.\d*)?))?)?",
                 units)
    if not m or m.group(1).lower() not in _UNIT_SECONDS:
        raise ValueError(f"unsupported time units: {units!r}")
    y, mo, d = int(m.group(2)), int(m.group(3)), int(m.group(4))
    hh = int(m.group(5) or 0)
    mm = int(m.group(6) or 0)
    ss = float(m.group(7) or 0.0)
    epoch = _dt.datetime(y, mo, d, hh, mm) + _dt.timedelta(seconds=ss)
    return _UNIT_SECONDS[m.group(1).lower()], epoch


class ForcingFile:
    """Forcing of a domain (land cells of `grid`) from a netCDF file."""

    def __init__(self, path, grid, dt, mapping=None, reservoirs=None):
        self.maps = _Maps(path, mapping)
        self.nc = self.maps.nc
        self.grid = grid
        self.dt = float(dt)
        self.mapping = mapping or {}
        tname = next((d for d, (_, rec) in self.nc.dimensions.items() if rec), "time")
        units = self.nc.attrs(tname).get("units", "days since 1970-01-01")
        cal = self.nc.attrs(tname).get("calendar", "standard")
        if cal not in ("standard", "gregorian", "proleptic_gregorian"):
            raise ValueError(f"calendar {cal!r} is not supported")
        scale, epoch = parse_time_units(units)
        raw = self.nc.read(tname)
        self.times = [epoch + _dt.timedelta(seconds=float(v) * scale) for v in np.atleast_1d(raw)]
        self.tname = tname
        self.cells = grid.row * grid.nx + grid.col
        self.reservoirs = reservoirs

    def _entry(self, sn):
        from .config import _entry
        e = _entry(self.mapping.get(sn, sn))
        if "value" in e:
            raise ValueError(f"forcing `{sn}` must be a netCDF variable")
        return e["name"], float(np.ravel(e.get("scale", 1.0))[0]), float(np.ravel(e.get("offset", 0.0))[0])

    def index(self, t):
        """The record used at model time t: the first at or after t (io.jl:9-22)."""
        if t < self.times[0]:
            raise ValueError(f"time {t} before dataset begin {self.times[0]}")
        for i, ti in enumerate(self.times):
            if ti >= t:
                return i
        raise ValueError(f"time {t} after dataset end {self.times[-1]}")

    def _grid_at(self, sn, i):
        name, scale, offset = self._entry(sn)
        if name not in self.maps.vars:
            raise KeyError(f"forcing `{sn}` ({name}) not in the file")
        dims = self.maps.vars[name][1]
        start = [i if d == self.tname else 0 for d in dims]
        count = [1 if d == self.tname else self.nc.dimensions[d][0] for d in dims]
        a = self.nc.read(name, start=start, count=count)
        a = a.reshape([c for d, c in zip(dims, count) if d != self.tname])
        other = [d for d in dims if d != self.tname]
        ren = {self.maps.xname: "x", self.maps.yname: "y"}
        other = [ren.get(d, d) for d in other]
        a = np.transpose(a, [other.index("y"), other.index("x")])
        if self.maps.flip_y:
            a = a[::-1, :]
        if self.maps.flip_x:
            a = a[:, ::-1]
        return a * scale + offset if (scale != 1.0 or offset != 0.0) else a

    def at(self, t):
        """(P, PET, T) in SI on the land cells for the step ending at model time t, and with
        reservoirs the reservoirs' precipitation and evaporation (both [m s-1])."""
        i = self.index(t)
        f = to_si_factor_per_step(self.dt)  # Unit(mm = 1, dt = -1)
        to_si = {PRECIP: f, PET: f}
        out, res_out = {}, {}
        for sn in (PRECIP, PET, TEMP):
            g = self._grid_at(sn, i)
            g = g + 273.15 if sn == TEMP else g * to_si[sn]
            flat = g.reshape(-1).copy()
            if self.reservoirs is not None and sn in to_si:
                cov = self.reservoirs.get("coverage_cells")
                vals = []
                for cells in cov:
                    vals.append(float(np.mean(flat[cells])))
                    flat[cells] = 0.0
                res_out[sn] = np.array(vals)
            v = flat[self.cells]
            if np.isnan(v).any():
                raise ValueError(f"forcing at {t} has missing values on active cells for `{sn}`")
            out[sn] = np.ascontiguousarray(v)
        if self.reservoirs is not None:
            return out[PRECIP], out[PET], out[TEMP], res_out[PRECIP], res_out[PET]
        return out[PRECIP], out[PET], out[TEMP]

    def close(self):
        self.nc.close()


def write_forcing(path, grid, times, precip, pet, temp, dt, time_units="days since 2000-01-01 00:00:00", format=2,
                  names=None):
    """Write SI forcing arrays ([steps, n_land]) as a Wflow forcing file (mm per step, degC)."""
    names = names or {PRECIP: "precip", PET: "pet", TEMP: "temp"}
    scale, epoch = parse_time_units(time_units)
    nc = ncio.NcFile(path, "w", format=format)
    nc.def_dim("time", 0)
    nc.def_dim("x", grid.nx)
    nc.def_dim("y", grid.ny)
    nc.def_var("x", ncio.NC_DOUBLE, ("x",), {"axis": "X"})
    nc.def_var("y", ncio.NC_DOUBLE, ("y",), {"axis": "Y"})
    nc.def_var("time", ncio.NC_DOUBLE, ("time",), {"units": time_units, "calendar": "proleptic_gregorian"})
    for sn, unit in ((PRECIP, "mm"), (PET, "mm"), (TEMP, "degC")):
        nc.def_var(names[sn], ncio.NC_DOUBLE, ("time", "y", "x"), {"_FillValue": np.nan, "units": unit})
    nc.enddef()
    nc.write("x", grid.xc)
    nc.write("y", grid.yc)
    nc.write("time", np.array([(t - epoch).total_seconds() / scale for t in times]))
    for k in range(len(times)):
        f = to_si_factor_per_step(dt)
        for sn, arr, conv in ((PRECIP, precip, lambda v: v / f), (PET, pet, lambda v: v / f),
                              (TEMP, temp, lambda v: v - 273.15)):
            buf = np.full((grid.ny, grid.nx), np.nan)
            buf[grid.row, grid.col] = conv(np.asarray(arr[k]))
            nc.write(names[sn], buf[None], start=[k, 0, 0])
    nc.close()
