"""Wflow state files: write a model's states and start a model from them.

Wflow saves the states of a run in a netCDF file on the model grid (Wflow/src/io.jl:735-760
`setup_grid_netcdf` with Float64 variables, `write_netcdf_timestep` :849-885) and starts a warm
run from such a file (`set_states!`, Wflow/src/utils.jl:150-213, then sbm_model.jl:104-193 for
the quantities derived from the states). The variables are the states of the model's
components, named by their standard names (or by the names the TOML maps them to), in the
units of the standard-name tables (standard_name_sbm.jl, standard_name_routing.jl), with
dimensions (x, y[, layer], time) in Julia order -- (time[, layer], y, x) in the file -- and NaN
outside the active cells.

`write_states` / `read_states` do the same for a model of this library (`model.Model`, or the
CPU oracle's model through the same calls): the file is a netCDF classic-format file written
by the library's own writer (`ncio`), which Wflow's reader (NCDatasets) opens as well.
"""

import numpy as np

from . import abi, ncio

# standard name -> (field, layered, file unit, domain part)
# units: file value * factor = SI value (units.jl to_SI), degC shifted by 273.15 (ABSOLUTE_DEGREES)
UNITS = {"mm": 1e-3, "m": 1.0, "m3 s-1": 1.0, "m3 d-1": 1.0 / 86400.0, "degC": None}
STATES = {
    "vegetation_canopy_water__depth": ("CANOPY_STORAGE", False, "mm", "land"),
    "snowpack_dry_snow__leq_depth": ("SNOW_STORAGE", False, "mm", "land"),
    "snowpack_liquid_water__depth": ("SNOW_WATER", False, "mm", "land"),
    "soil_surface__temperature": ("SOIL_SURFACE_TEMPERATURE", False, "degC", "land"),
    "soil_water_saturated_zone__depth": ("SATURATED_WATER_DEPTH", False, "mm", "land"),
    "soil_layer_water_unsaturated_zone__depth": ("UNSATURATED_LAYER_DEPTH", True, "mm", "land"),
    "subsurface_water__instantaneous_volume_flow_rate": ("SSF_Q", False, "m3 d-1", "land"),
    "land_surface_water__instantaneous_volume_flow_rate": ("LAND_Q", False, "m3 s-1", "land"),
    "land_surface_water__depth": ("LAND_H", False, "m", "land"),
    "river_water__instantaneous_volume_flow_rate": ("RIVER_Q", False, "m3 s-1", "river"),
    "river_water__depth": ("RIVER_H", False, "m", "river"),
    "reservoir_water_surface__elevation": ("RESERVOIR_WATERLEVEL", False, "m", "reservoir"),
}


def required_states(config, reservoirs=False):
    """The states a model needs (extract_required_states, Wflow/src/states.jl:139-170 for the
    `sbm` type with kinematic-wave routing)."""
    names = ["vegetation_canopy_water__depth", "soil_water_saturated_zone__depth",
             "soil_layer_water_unsaturated_zone__depth"]
    if config.snow:
        names = (["snowpack_dry_snow__leq_depth", "snowpack_liquid_water__depth"] + names +
                 ["soil_surface__temperature"])
    names += ["subsurface_water__instantaneous_volume_flow_rate",
              "land_surface_water__instantaneous_volume_flow_rate", "land_surface_water__depth",
              "river_water__instantaneous_volume_flow_rate", "river_water__depth"]
    if reservoirs:
        names.append("reservoir_water_surface__elevation")
    return names


def to_si(x, unit):
    return x + 273.15 if unit == "degC" else x * UNITS[unit]


def from_si(x, unit):
    return x - 273.15 if unit == "degC" else x / UNITS[unit]


class Grid:
    """The model grid of a domain: nx * ny cells, land cell i at column x[i], row y[i], with
    the coordinates of the columns and rows (Wflow's `indices` and the x/y variables)."""

    def __init__(self, nx, ny, col, row, xc=None, yc=None, cell_length_in_meter=True):
        self.nx, self.ny = int(nx), int(ny)
        self.col = np.asarray(col, np.int64)
        self.row = np.asarray(row, np.int64)
        self.xc = np.arange(self.nx, dtype=float) if xc is None else np.asarray(xc, float)
        self.yc = np.arange(self.ny, dtype=float) if yc is None else np.asarray(yc, float)
        self.metres = bool(cell_length_in_meter)

    @classmethod
    def of_domain(cls, dom):
        """Grid of a synthetic single-catchment domain (land index = row * nx + column)."""
        i = np.arange(dom.n_land)
        return cls(dom.nx, dom.ny, i % dom.nx, i // dom.nx, xc=(np.arange(dom.nx) + 0.5) * dom.cell_size,
                   yc=(np.arange(dom.ny) + 0.5) * dom.cell_size)


class _Access:
    """get / set of a field for the library's Model or the oracle's model, member-major."""

    def __init__(self, model):
        self.m = model
        self.gpu = hasattr(model, "get_value")

    def get(self, name, layer=0):
        if self.gpu:
            return self.m.get_value(name, layer=layer)
        return self.m.get(abi.FIELD[name], layer)

    def set(self, name, values, layer=0):
        if self.gpu:
            self.m.set_value(name, values, layer=layer)
        else:
            self.m.set(abi.FIELD[name], values, layer)


def _cells(dom, part, reservoirs):
    if part == "land":
        return np.arange(dom.n_land)
    if part == "river":
        return np.asarray(dom.river["river_land_index"], np.int64)
    return np.asarray(dom.river["river_land_index"], np.int64)[reservoirs["river_index"]]


def write_states(model, dom, path, grid=None, names=None, ncnames=None, member=0, time=0.0,
                 time_units="days since 2000-01-01 00:00:00", calendar="proleptic_gregorian",
                 reservoirs=None, format=2):
    """Write member `member`'s states to a Wflow state file. `names` defaults to the states the
    model needs; `ncnames` maps standard names to variable names (the TOML's [state.variables])."""
    grid = Grid.of_domain(dom) if grid is None else grid
    acc = _Access(model)
    M = max(1, getattr(model, "M", 1))
    names = required_states(model.config if hasattr(model, "config") else model.cfg, reservoirs is not None) \
        if names is None else names
    ncnames = ncnames or {}
    N = model.N if hasattr(model, "N") else model.cfg.n_soil_layer_thickness + 1
    xname, yname = ("x", "y") if grid.metres else ("lon", "lat")
    nc = ncio.NcFile(path, "w", format=format)
    nc.def_dim("time", 0)
    nc.def_dim(xname, grid.nx)
    nc.def_dim(yname, grid.ny)
    nc.def_dim("layer", N)
    nc.def_var(xname, ncio.NC_DOUBLE, (xname,), {"axis": "X", "units": "m" if grid.metres else "degrees_east"})
    nc.def_var(yname, ncio.NC_DOUBLE, (yname,), {"axis": "Y", "units": "m" if grid.metres else "degrees_north"})
    nc.def_var("layer", ncio.NC_DOUBLE, ("layer",), {"long_name": "layer_index", "standard_name": "layer_index",
                                                     "axis": "Z"})
    nc.def_var("time", ncio.NC_DOUBLE, ("time",), {"units": time_units, "calendar": calendar})
    for sn in names:
        field, layered, unit, _ = STATES[sn]
        dims = ("time", "layer", yname, xname) if layered else ("time", yname, xname)
        nc.def_var(ncnames.get(sn, sn), ncio.NC_DOUBLE, dims, {"_FillValue": np.nan, "units": unit})
    nc.enddef()
    nc.write(xname, grid.xc)
    nc.write(yname, grid.yc)
    nc.write("layer", np.arange(1, N + 1, dtype=float))
    nc.write("time", np.array([float(time)]))
    for sn in names:
        field, layered, unit, part = STATES[sn]
        cells = _cells(dom, part, reservoirs)
        n_part = len(cells)
        for k in range(N if layered else 1):
            v = acc.get(field, layer=k).reshape(M, n_part)[member]
            buf = np.full((grid.ny, grid.nx), np.nan)
            buf[grid.row[cells], grid.col[cells]] = from_si(v, unit)
            if layered:
                nc.write(ncnames.get(sn, sn), buf[None, None], start=[0, k, 0, 0])
            else:
                nc.write(ncnames.get(sn, sn), buf[None], start=[0, 0, 0])
    nc.close()


def interpolate_linear(x, xp, fp):
    """interpolate_linear (routing/surface/reservoir.jl:363-375): the bounds are the columns'
    extremes, between them the last row at or below x and the next."""
    if x <= min(xp):
        return min(fp)
    if x >= max(xp):
        return max(fp)
    i1 = max(i for i in range(len(xp)) if xp[i] <= x)
    i2 = i1 + 1
    return fp[i1] * (1.0 - (x - xp[i1]) / (xp[i2] - xp[i1])) + fp[i2] * (x - xp[i1]) / (xp[i2] - xp[i1])


def reservoir_storage(reservoirs, waterlevel):
    """initialize_storage (reservoir.jl:343-360) of every reservoir at `waterlevel` ([members,
    reservoirs]): A H for the linear profile, the S-H table interpolated at H otherwise."""
    wl = np.asarray(waterlevel, float)
    out = reservoirs["area"] * wl
    prof = reservoirs.get("storage_curve_type")
    if prof is not None:
        for k in np.flatnonzero(np.asarray(prof) == 2):
            a, b = reservoirs["sh_offset"][k], reservoirs["sh_offset"][k + 1]
            h = [float(v) for v in reservoirs["sh_h"][a:b]]
            sv = [float(v) for v in reservoirs["sh_s"][a:b]]
            for m in range(wl.shape[0]):
                out[m, k] = interpolate_linear(float(wl[m, k]), h, sv)
    return out


def read_states(model, dom, path, grid=None, names=None, ncnames=None, reservoirs=None, time_index=0):
    """Set a model's states from a Wflow state file (every member gets the file's states) and
    derive what set_states! derives from them (sbm_model.jl:120-190): q and h zero on land cells
    without a surface flow width, overland and river storage from the depths, total soil water
    storage from the saturated and unsaturated stores, reservoir storage from the water level."""
    grid = Grid.of_domain(dom) if grid is None else grid
    acc = _Access(model)
    M = max(1, getattr(model, "M", 1))
    cfg = model.config if hasattr(model, "config") else model.cfg
    names = required_states(cfg, reservoirs is not None) if names is None else names
    ncnames = ncnames or {}
    N = model.N if hasattr(model, "N") else cfg.n_soil_layer_thickness + 1
    nc = ncio.NcFile(path)
    variables = nc.variables
    got = {}
    for sn in names:
        field, layered, unit, part = STATES[sn]
        vname = ncnames.get(sn, sn)
        if vname not in variables:
            raise KeyError(f"state variable `{sn}` ({vname}) not in {path}")
        dims = variables[vname][1]
        a = nc.read(vname)
        # order the axes as (time, layer, y, x) whatever the file's order (read_standardized)
        order = [d for d in dims]
        want = ["time"] + (["layer"] if layered else []) + [d for d in dims if d in ("y", "lat")] + \
            [d for d in dims if d in ("x", "lon")]
        a = np.transpose(a, [order.index(d) for d in want])[time_index]
        cells = _cells(dom, part, reservoirs)
        if layered:
            vals = [a[k][grid.row[cells], grid.col[cells]] for k in range(min(N, a.shape[0]))]
            vals = [np.where(np.isnan(v), 0.0, to_si(v, unit)) for v in vals]  # inactive layers
        else:
            v = a[grid.row[cells], grid.col[cells]]
            if np.isnan(v).any():
                raise ValueError(f"state `{sn}` has missing values on active cells")
            vals = [to_si(v, unit)]
        got[sn] = vals
        for k, v in enumerate(vals):
            acc.set(field, np.tile(v, M), layer=k)
    nc.close()
    # derived quantities (sbm_model.jl:120-190)
    sfw = dom.land["surface_flow_width"]
    if "land_surface_water__depth" in got or "land_surface_water__instantaneous_volume_flow_rate" in got:
        h = acc.get("LAND_H").reshape(M, -1)
        q = acc.get("LAND_Q").reshape(M, -1)
        dry = sfw <= 0.0
        h[:, dry] = 0.0
        q[:, dry] = 0.0
        acc.set("LAND_Q", q.reshape(-1))
        acc.set("LAND_H", h.reshape(-1))
        acc.set("LAND_STORAGE", (h * sfw * dom.land["flow_length"]).reshape(-1))
    if "river_water__depth" in got and dom.n_river:
        h = acc.get("RIVER_H").reshape(M, -1)
        acc.set("RIVER_STORAGE", (h * dom.river["river_width"] * dom.river["river_length"]).reshape(-1))
    if "soil_water_saturated_zone__depth" in got:
        sat = acc.get("SATURATED_WATER_DEPTH")
        ust = np.zeros_like(sat)
        for k in range(N):
            ust = ust + acc.get("UNSATURATED_LAYER_DEPTH", layer=k)
        acc.set("TOTAL_SOIL_WATER_STORAGE", sat + ust)
    if reservoirs is not None and "reservoir_water_surface__elevation" in got:
        # the storage is re-initialised from the water level (sbm_model.jl:181-190)
        wl = acc.get("RESERVOIR_WATERLEVEL").reshape(M, -1)
        acc.set("RESERVOIR_STORAGE", reservoir_storage(reservoirs, wl).reshape(-1))
