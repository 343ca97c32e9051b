"""Wflow static maps: build the step library's domain and parameters from a staticmaps file.

Restates the part of Wflow's model construction that the SBM + kinematic-wave path needs, from
a netCDF file of the standard-name variables (or the names a TOML [input.static] section maps
them to):
  active cells      subbasin_location__count not missing (network.jl:87-112, utils.jl:85-99)
  drainage graph    basin__local_drain_direction with PCRaster codes (utils.jl:3-13,
                    routing/utils.jl:6-33: a direction leaving the active cells becomes a pit)
  river network     river_location__mask; a river cell draining to a non-river cell is a pit
                    (network.jl:214-258)
  geometry          cell lengths in metres or from latitude (utils.jl:114-150,
                    domain.jl:350-360), flow width and length (utils.jl:418-449), river and
                    open-water fractions, surface flow width, flow fraction to the river
                    (domain.jl:220-347, utils.jl:458-510), slopes clamped at 1e-5
  parameters        the SBM, snow, vegetation and lateral-subsurface inputs of the standard-
                    name tables with their units and defaults (standard_name_sbm.jl,
                    standard_name_routing.jl), converted to SI as to_SI does (units.jl:271)
Axes are standardised as read_standardized does (io.jl:1346-1384): x and y increasing, so the
land cells are numbered x fastest, then y. Reservoir maps are read when asked for.
"""

from pathlib import Path

import numpy as np

from . import ncio
from .states import Grid
from .synthetic import Domain

MM = 1e-3
CM = 1e-2
MM_D = 1e-3 / 86400.0

# WfParams field -> (standard name, factor to SI (None: degC absolute), default, layered)
PARAMS = {
    "canopy_gap_fraction": ("vegetation_canopy__gap_fraction", 1.0, None, False),
    "maximum_canopy_storage": ("vegetation_water__storage_capacity", MM, 1.0, False),
    "crop_coefficient": ("vegetation__crop_factor", 1.0, 1.0, False),
    "rooting_depth": ("vegetation_root__depth", MM, None, False),
    "evaporation_to_precipitation_ratio": ("vegetation_canopy_water__mean_evaporation_to_mean_precipitation_ratio",
                                           1.0, 0.1, False),
    "degree_day_factor": ("snowpack__degree_day_coefficient", MM_D, 3.75, False),
    "temperature_threshold_snowfall": ("atmosphere_air__snowfall_temperature_threshold", None, 0.0, False),
    "temperature_interval_snowfall": ("atmosphere_air__snowfall_temperature_interval", 1.0, 1.0, False),
    "temperature_threshold_melt": ("snowpack__melting_temperature_threshold", None, 0.0, False),
    "water_holding_capacity": ("snowpack__liquid_water_holding_capacity", 1.0, 0.1, False),
    "theta_s": ("soil_water__saturated_volume_fraction", 1.0, None, False),
    "theta_r": ("soil_water__residual_volume_fraction", 1.0, None, False),
    "kv_0": ("soil_surface_water__vertical_saturated_hydraulic_conductivity", MM_D, None, False),
    "f": ("soil_water__vertical_saturated_hydraulic_conductivity_scale_parameter", 1.0 / MM, None, False),
    "soil_thickness": ("soil__thickness", MM, None, False),
    "air_entry_pressure": ("soil_water__air_entry_pressure_head", CM, -10.0, False),
    "h1": ("vegetation_root__feddes_critical_pressure_head_h1", CM, 0.0, False),
    "h2": ("vegetation_root__feddes_critical_pressure_head_h2", CM, -100.0, False),
    "h3_high": ("vegetation_root__feddes_critical_pressure_head_h3_high", CM, -400.0, False),
    "h3_low": ("vegetation_root__feddes_critical_pressure_head_h3_low", CM, -1000.0, False),
    "h4": ("vegetation_root__feddes_critical_pressure_head_h4", CM, -16000.0, False),
    "alpha_h1": ("vegetation_root__feddes_critical_pressure_head_h1_reduction_coefficient", 1.0, 1.0, False),
    "infiltration_capacity_compacted_soil": ("compacted_soil_surface_water__infiltration_capacity", MM_D, 10.0, False),
    "compacted_soil_area_fraction": ("compacted_soil__area_fraction", 1.0, None, False),
    "wet_root_distribution_parameter": ("soil_wet_root__sigmoid_function_shape_parameter", 1.0 / MM, -500.0, False),
    "cap_hmax": ("soil_water_saturated_zone_top__capillary_rise_max_water_table_depth", MM, 2000.0, False),
    "cap_n": ("soil_water_saturated_zone_top__capillary_rise_averianov_exponent", 1.0, 2.0, False),
    "maximum_leakage": ("soil_water_saturated_zone_bottom__max_leakage_volume_flux", MM_D, 0.0, False),
    "w_soil": ("soil_surface_temperature__weight_coefficient", 1.0, 0.1125, False),
    "cf_soil": ("soil_surface_water__infiltration_reduction_parameter", 1.0, 0.038, False),
    "brooks_corey_exponent": ("soil_layer_water__brooks_corey_exponent", 1.0, None, True),
    "kv_factor": ("soil_layer_water__vertical_saturated_hydraulic_conductivity_factor", 1.0, 1.0, True),
    "horizontal_to_vertical_ratio": ("subsurface_water__horizontal_to_vertical_saturated_hydraulic_conductivity_ratio",
                                     1.0, None, False),
    "z_exp": ("soil_exponential_vertical_saturated_hydraulic_conductivity_profile_below_surface__depth", MM, None,
              False),
    # HBV glacier (glacier.jl:58-98, standard_name_sbm.jl:70-108)
    "glacier_fraction": ("glacier_surface__area_fraction", 1.0, 0.0, False),
    "glacier_temperature_threshold_melt": ("glacier_ice__melting_temperature_threshold", None, 0.0, False),
    "glacier_degree_day_factor": ("glacier_ice__degree_day_coefficient", MM_D, 3.0, False),
    "glacier_snow_to_ice_fraction": ("glacier_firn_accumulation__snowpack_dry_snow_leq_depth_fraction",
                                     1.0 / 86400.0, 0.001, False),
    "glacier_initial_store": ("glacier_ice__initial_leq_depth", MM, 5500.0, False),
}
# read only when present: the snow parameters all have defaults; z_exp only serves the
# exponential_constant Kv profile; the glacier parameters only the glacier model (the library
# applies the reference's defaults to the ones not given)
OPTIONAL_PARAMS = {"z_exp", "glacier_fraction", "glacier_temperature_threshold_melt", "glacier_degree_day_factor",
                   "glacier_snow_to_ice_fraction", "glacier_initial_store"}

# PCRaster local drain direction -> (dx, dy) on the standardised grid (utils.jl:3-13)
PCR_DX = np.array([0, -1, 0, 1, -1, 0, 1, -1, 0, 1])
PCR_DY = np.array([0, -1, -1, -1, 0, 0, 0, 1, 1, 1])
LDD_PIT = 5


def lattometres(lat):
    """Lengths of a degree of longitude and latitude in metres at latitude `lat` (utils.jl:114-128)."""
    lat = np.asarray(lat, float)
    c = lambda d: np.cos(np.deg2rad(d))  # noqa: E731
    latlen = 111132.92 + (-559.82 * c(2.0 * lat)) + (1.175 * c(4.0 * lat)) + (-0.0023 * c(6.0 * lat))
    longlen = (111412.84 * c(lat)) + (-93.5 * c(3.0 * lat)) + (0.118 * c(5.0 * lat))
    return longlen, latlen


def apply_affine_transform(a, scale=1.0, offset=0.0):
    """a * scale + offset as apply_affine_transform! does (utils.jl:239-256): the scaling only
    when a scale differs from 1, the offset only when one differs from 0; a vector of several
    scales or offsets applies along the first axis (the layers of a layered map)."""
    a = np.asarray(a, float)
    scale = np.asarray(scale, float)
    offset = np.asarray(offset, float)
    if scale.ndim:
        scale = scale.reshape((-1,) + (1,) * (a.ndim - 1)) if scale.size > 1 else scale.reshape(())
    if offset.ndim:
        offset = offset.reshape((-1,) + (1,) * (a.ndim - 1)) if offset.size > 1 else offset.reshape(())
    if np.any(scale != 1.0):
        a = a * scale
    if np.any(offset != 0.0):
        a = a + offset
    return a


class _Maps:
    """Variables of a static-map file on the standardised grid, by standard name."""

    def __init__(self, path, mapping=None):
        self.nc = ncio.NcFile(path)
        self.vars = self.nc.variables
        self.mapping = mapping or {}
        dims = self.nc.dimensions
        self.xname = next((d for d in ("x", "lon", "longitude") if d in dims), None)
        self.yname = next((d for d in ("y", "lat", "latitude") if d in dims), None)
        if self.xname is None or self.yname is None:
            raise ValueError(f"no x or y axis in {path}")
        xc, yc = self.nc.read(self.xname), self.nc.read(self.yname)
        self.flip_x = len(xc) > 1 and xc[0] > xc[-1]
        self.flip_y = len(yc) > 1 and yc[0] > yc[-1]
        self.xc = np.sort(xc)
        self.yc = np.sort(yc)

    def _entry(self, sn):
        """The mapping's entry for a standard name: {"name", "scale", "offset"} or {"value"}
        (the three forms of a TOML [input] entry, config_init.jl:113-156)."""
        from .config import _entry
        m = self.mapping.get(sn, sn)
        e = _entry(m)
        if "layer" in e:
            raise ValueError(f"`layer` selections of [input] entries are not supported ({sn})")
        return e

    def has(self, sn):
        e = self._entry(sn)
        return "value" in e or e["name"] in self.vars

    def read(self, sn, default=None, layered=False, n_layers=None):
        """(ny, nx) or (layer, ny, nx) array; a constant from the mapping ({"value": v}) or the
        default when the variable is absent; KeyError when neither exists. The entry's scale
        and offset are applied as apply_affine_transform! does (utils.jl:239-256)."""
        e = self._entry(sn)
        shape = (len(self.yc), len(self.xc))
        if "value" in e:
            v = np.asarray(e["value"], float)
            if layered:
                return np.broadcast_to(v.reshape(-1, 1, 1), (v.size if v.ndim else n_layers,) + shape).copy()
            return np.full(shape, float(v))
        m = e["name"]
        if m not in self.vars:
            if default is None:
                raise KeyError(f"static map `{sn}` not found")
            return np.full(((n_layers,) if layered else ()) + shape, float(default))
        a = self._standardise(m, self.nc.read(m))
        return apply_affine_transform(a, e.get("scale", 1.0), e.get("offset", 0.0))

    def _standardise(self, m, a):
        dims = list(self.vars[m][1])
        ren = {self.xname: "x", self.yname: "y"}
        dims = [ren.get(d, d) for d in dims]
        keep = [d for d in dims if d in ("x", "y", "layer")]
        # drop length-1 axes other than the grid's (time of a one-time map)
        idx = tuple(slice(None) if d in keep else 0 for d in dims)
        a = a[idx]
        want = (["layer"] if "layer" in keep else []) + ["y", "x"]
        a = np.transpose(a, [keep.index(d) for d in want])
        if self.flip_y:
            a = a[..., ::-1, :]
        if self.flip_x:
            a = a[..., ::-1]
        return np.ascontiguousarray(a)


def load_staticmaps(path, mapping=None, cell_length_in_meter=True, n_layers=4, reservoirs=False):
    """Domain (land/river arrays and SI parameters, the `synthetic.Domain` layout), its Grid,
    and, with reservoirs=True, the reservoir dict of `wf_create_with_reservoirs` (None when the
    file has no reservoir locations). The number of soil layers is the file's `layer` dimension
    (n_layers when the file has none)."""
    S = _Maps(path, mapping)
    ny, nx = len(S.yc), len(S.xc)
    n_layers = S.nc.dimensions.get("layer", (n_layers, False))[0]
    sub = S.read("subbasin_location__count")
    active = ~np.isnan(sub).reshape(-1)
    cells = np.flatnonzero(active)
    n = len(cells)
    if n == 0:
        raise ValueError("no active cells")
    rev = np.full(nx * ny, -1, np.int64)
    rev[cells] = np.arange(n)
    col, row = cells % nx, cells // nx

    def at(a):
        return a.reshape(-1)[cells]

    ldd_f = at(S.read("basin__local_drain_direction"))
    if np.isnan(ldd_f).any():
        raise ValueError("local drain direction missing on active cells")
    ldd = ldd_f.astype(np.int64)
    if ((ldd < 1) | (ldd > 9)).any():
        raise ValueError("local drain direction outside 1-9")
    tx, ty = col + PCR_DX[ldd], row + PCR_DY[ldd]
    inside = (tx >= 0) & (tx < nx) & (ty >= 0) & (ty < ny)
    target = np.where(inside, rev[np.where(inside, ty * nx + tx, 0)], -1)
    pit = (ldd == LDD_PIT) | (target < 0)
    ldd = np.where(pit, LDD_PIT, ldd)
    ds = np.where(pit, -1, target).astype(np.int32)
    order = _topological_order(ds)
    # geometry
    celllength = float(abs(np.mean(np.diff(S.xc)))) if nx > 1 else float(abs(np.mean(np.diff(S.yc))))
    if cell_length_in_meter:
        xl = np.full(n, celllength)
        yl = np.full(n, celllength)
    else:
        longlen, latlen = lattometres(S.yc[row])
        xl, yl = longlen * celllength, latlen * celllength
    area = xl * yl
    straight_y = (ldd == 2) | (ldd == 8)
    straight_x = (ldd == 4) | (ldd == 6)
    hyp = np.hypot(xl, yl)
    flow_width = np.where(straight_y, xl, np.where(straight_x, yl, (xl * yl) / hyp))
    flow_length = np.where(straight_y, yl, np.where(straight_x, xl, hyp))
    slope = np.maximum(at(S.read("land_surface__slope")), 1e-5)
    rmask = at(S.read("river_location__mask", default=0.0))
    is_river = np.where(np.isnan(rmask), False, rmask != 0)
    rw_all = at(S.read("river__width", default=0.0))
    rl_all = at(S.read("river__length", default=0.0))
    river_fraction = np.where(is_river, np.minimum((rl_all * rw_all) / area, 1.0), 0.0)
    wf = at(S.read("land_water_covered__area_fraction", default=0.0))
    water_fraction = np.maximum(wf - river_fraction, 0.0)
    land_area = (1.0 - river_fraction) * area
    sfw = np.where(is_river, land_area / flow_length, flow_width)
    frac = np.zeros(n)
    j = np.flatnonzero(ds >= 0)
    to = ds[j]
    sel = is_river[to] & (ldd[j] != ldd[to])
    jj, ii = j[sel], to[sel]
    frac[jj] = slope[jj] / (slope[ii] + slope[jj])
    land = dict(land_downstream=ds, area=area, flow_width=flow_width, flow_length=flow_length,
                surface_flow_width=sfw, slope=slope, flow_fraction_to_river=frac, river_fraction=river_fraction,
                water_fraction=water_fraction, elevation=at(S.read("land_surface__elevation", default=0.0)),
                land_manning_n=at(S.read("land_surface_water_flow__manning_n_parameter", default=0.072)))
    # river network: a river cell draining to a non-river cell is a pit
    river_land = np.flatnonzero(is_river).astype(np.int32)
    rindex = np.full(n, -1, np.int64)
    rindex[river_land] = np.arange(len(river_land))
    d_land = ds[river_land]
    rds = np.where((d_land >= 0) & is_river[np.maximum(d_land, 0)], rindex[np.maximum(d_land, 0)], -1).astype(np.int32)
    r_width, r_length = rw_all[river_land], rl_all[river_land]
    if len(river_land) and (not (r_length > 0).all() or not (r_width > 0).all()):
        raise ValueError("river length and width must be positive on river cells")
    river = dict(river_land_index=river_land, river_downstream=rds, river_width=r_width.copy(),
                 river_length=r_length.copy(),
                 river_slope=np.maximum(at(S.read("river__slope", default=np.nan))[river_land], 1e-5),
                 river_manning_n=at(S.read("river_water_flow__manning_n_parameter", default=0.036))[river_land],
                 river_bankfull_depth=at(S.read("river_bank_water__depth", default=1.0))[river_land],
                 river_external_inflow=at(S.read("river_water__external_inflow_volume_flow_rate",
                                                 default=0.0))[river_land])
    params = {}
    for field, (sn, factor, default, layered) in PARAMS.items():
        if field in OPTIONAL_PARAMS and not S.has(sn):
            continue
        a = S.read(sn, default=default, layered=layered, n_layers=n_layers)
        if layered:
            v = np.stack([lay.reshape(-1)[cells] for lay in a], axis=1)  # cell-major [i * N + k]
        else:
            v = at(a)
        if np.isnan(v).any():
            raise ValueError(f"static map `{sn}` has missing values on active cells")
        v = v + 273.15 if factor is None else v * factor
        params[field] = np.ascontiguousarray(v.reshape(-1))
    ups = _upstream_cells(ds, order)
    dom = Domain(nx=nx, ny=ny, cell_size=celllength, ldd=ldd.astype(np.uint8), land=land, river=river, params=params,
                 upstream_cells=ups)
    dom.outlets = [int(r) for r in np.flatnonzero(rds < 0)]
    grid = Grid(nx, ny, col, row, xc=S.xc, yc=S.yc, cell_length_in_meter=cell_length_in_meter)
    res = _reservoirs(S, cells, river_land, Path(path).parent) if reservoirs else None
    S.nc.close()
    return dom, grid, res


def _topological_order(ds):
    n = len(ds)
    indeg = np.zeros(n, np.int64)
    np.add.at(indeg, ds[ds >= 0], 1)
    order = list(np.flatnonzero(indeg == 0))
    k = 0
    while k < len(order):
        v = order[k]
        d = ds[v]
        if d >= 0:
            indeg[d] -= 1
            if indeg[d] == 0:
                order.append(d)
        k += 1
    if len(order) != n:
        raise ValueError("one or more cycles in the flow graph (routing/utils.jl:26-31)")
    return np.array(order, np.int64)


def _upstream_cells(ds, order):
    ups = np.ones(len(ds), np.int64)
    for v in order:
        d = ds[v]
        if d >= 0:
            ups[d] += ups[v]
    return ups


def read_sh_csv(path):
    """An S-H table (read_sh_csv, io.jl:1129-1140): the columns headed H and S (any case) of a
    comma-separated file with one header line."""
    with open(path) as f:
        names = [c.strip().strip('"').upper() for c in f.readline().split(",")]
        data = np.loadtxt(f, delimiter=",", ndmin=2)
    if "H" not in names or "S" not in names:
        raise ValueError(f"{path} needs to provide H and S columns, got {names}")
    return data[:, names.index("H")].copy(), data[:, names.index("S")].copy()


def read_hq_csv(path):
    """An H-Q table (read_hq_csv, io.jl:1143-1147): after one header line, the level in the first
    column and the discharge of each of the 365 days of the year in the next 365."""
    data = np.loadtxt(path, delimiter=",", skiprows=1, ndmin=2)
    return data[:, 0].copy(), np.ascontiguousarray(data[:, 1:366])


def write_sh_csv(path, h, s):
    np.savetxt(path, np.column_stack([h, s]), delimiter=",", header="H,S", comments="", fmt="%.17g")


def write_hq_csv(path, h, q):
    header = "H," + ",".join(str(d) for d in range(1, 366))
    np.savetxt(path, np.column_stack([h, q]), delimiter=",", header=header, comments="", fmt="%.17g")


def _reservoirs(S, cells, river_land, folder):
    """Reservoirs at the river cells where reservoir_location__count > 0, in river order
    (network.jl:314-350), with their parameters (reservoir.jl:40-200), initial water level, storage
    profile, link to a lower reservoir and the S-H / H-Q tables of the CSV files
    reservoir_sh_<id>.csv and reservoir_hq_<id>.csv beside the static maps (reservoir.jl:152-192)."""
    if not S.has("reservoir_location__count"):
        return None
    loc = S.read("reservoir_location__count", default=0.0).reshape(-1)[cells][river_land]
    ids = np.where(np.isnan(loc), 0.0, loc)
    ri = np.flatnonzero(ids > 0).astype(np.int32)
    if len(ri) == 0:
        return None
    at = lambda sn, d=None: S.read(sn, default=d).reshape(-1)[cells][river_land][ri]  # noqa: E731
    res = dict(river_index=ri,
               outflow_curve_type=at("reservoir_water__rating_curve_type_count").astype(np.int32),
               area=at("reservoir_surface__area"),
               waterlevel=at("reservoir_water_surface__initial_elevation"))
    nan = np.nan
    for key, sn in [("maximum_storage", "reservoir_water__max_volume"),
                    ("threshold", "reservoir_water_flow_threshold_level__elevation"),
                    ("rating_curve_coefficient", "reservoir_water__rating_curve_coefficient"),
                    ("rating_curve_exponent", "reservoir_water__rating_curve_exponent"),
                    ("maximum_release", "reservoir_water_release_below_spillway__max_volume_flow_rate"),
                    ("demand", "reservoir_water_demand__required_downstream_volume_flow_rate"),
                    ("target_minimum_fraction", "reservoir_water__target_min_volume_fraction"),
                    ("target_full_fraction", "reservoir_water__target_full_volume_fraction")]:
        res[key] = at(sn, nan)
    ids_r = ids[ri]
    k = len(ri)
    prof = at("reservoir_water__storage_curve_type_count", 1.0)
    prof = np.where(np.isnan(prof), 1.0, prof).astype(np.int32)
    linked = at("reservoir_lower_location__count", 0.0)
    linked = np.where(np.isnan(linked), 0.0, linked)
    lower = np.full(k, -1, np.int32)
    for i in range(k):
        if linked[i] > 0:
            match = np.flatnonzero(ids_r == linked[i])
            if len(match) != 1:
                raise ValueError(f"reservoir {ids_r[i]:g}: lower reservoir {linked[i]:g} not found once")
            lower[i] = match[0]
    tables = any(prof == 2) or any(res["outflow_curve_type"] == 1) or any(lower >= 0)
    if tables:
        sh_h, sh_s, hq_h, hq_q, sh_off, hq_off = [], [], [], [], [0], [0]
        for i in range(k):
            rid = int(ids_r[i])
            if prof[i] == 2:
                h, sv = read_sh_csv(Path(folder) / f"reservoir_sh_{rid}.csv")
                sh_h.append(h)
                sh_s.append(sv)
            sh_off.append(sh_off[-1] + (len(sh_h[-1]) if prof[i] == 2 else 0))
            if res["outflow_curve_type"][i] == 1:
                h, q = read_hq_csv(Path(folder) / f"reservoir_hq_{rid}.csv")
                hq_h.append(h)
                hq_q.append(q.reshape(-1))
            hq_off.append(hq_off[-1] + (len(hq_h[-1]) if res["outflow_curve_type"][i] == 1 else 0))
        cat = lambda xs: np.concatenate(xs) if xs else np.zeros(0)  # noqa: E731
        res.update(storage_curve_type=prof, sh_offset=np.array(sh_off, np.int64), sh_h=cat(sh_h), sh_s=cat(sh_s),
                   hq_offset=np.array(hq_off, np.int64), hq_h=cat(hq_h), hq_q=cat(hq_q), lower_reservoir=lower)
    out = {k: np.ascontiguousarray(v) for k, v in res.items()}
    # the reservoirs' areas: grid cells (flat y * nx + x, active or not) of each reservoir id
    # (network.jl:325-347), for averaging the forcing over them
    if S.has("reservoir_area__count"):
        area_map = S.read("reservoir_area__count").reshape(-1)
        out["coverage_cells"] = [np.flatnonzero(area_map == v) for v in ids_r]
    else:
        out["coverage_cells"] = [np.array([cells[river_land[k]]]) for k in ri]
    return out


# ------------------------------------------------------------------ writing ------------------
def write_staticmaps(dom, path, grid=None, reservoirs=None, format=2, names=None):
    """Write a domain's land, river and parameter arrays as a Wflow static-map file (standard
    names, or the file names `names` maps them to; file units): the inverse of
    `load_staticmaps` for cell_length_in_meter grids."""
    names = names or {}
    grid = Grid.of_domain(dom) if grid is None else grid
    n = dom.n_land
    nc = ncio.NcFile(path, "w", format=format)
    nc.def_dim("x", grid.nx)
    nc.def_dim("y", grid.ny)
    N = len(dom.params["brooks_corey_exponent"]) // n
    nc.def_dim("layer", N)
    nc.def_var("x", ncio.NC_DOUBLE, ("x",), {"axis": "X", "units": "m"})
    nc.def_var("y", ncio.NC_DOUBLE, ("y",), {"axis": "Y", "units": "m"})
    nc.def_var("layer", ncio.NC_DOUBLE, ("layer",), {"axis": "Z"})
    maps = {}

    def grid_of(values, cells, fill=np.nan):
        buf = np.full((grid.ny, grid.nx), fill)
        buf[grid.row[cells], grid.col[cells]] = values
        return buf

    land_cells = np.arange(n)
    rl = np.asarray(dom.river["river_land_index"], np.int64)
    maps["subbasin_location__count"] = (ncio.NC_INT, grid_of(np.ones(n), land_cells), -999.0)
    maps["basin__local_drain_direction"] = (ncio.NC_BYTE, grid_of(dom.ldd.astype(float), land_cells), -1.0)
    maps["river_location__mask"] = (ncio.NC_BYTE, grid_of(np.isin(land_cells, rl).astype(float), land_cells, 0.0),
                                    -1.0)
    maps["land_surface__slope"] = (ncio.NC_DOUBLE, grid_of(dom.land["slope"], land_cells), np.nan)
    maps["land_surface__elevation"] = (ncio.NC_DOUBLE, grid_of(dom.land["elevation"], land_cells), np.nan)
    maps["land_surface_water_flow__manning_n_parameter"] = (ncio.NC_DOUBLE, grid_of(dom.land["land_manning_n"],
                                                                                    land_cells), np.nan)
    wf = dom.land["water_fraction"] + dom.land["river_fraction"]  # the map holds rivers as well
    maps["land_water_covered__area_fraction"] = (ncio.NC_DOUBLE, grid_of(np.where(wf > 0, wf, 0.0), land_cells), np.nan)
    for sn, key in [("river__width", "river_width"), ("river__length", "river_length"), ("river__slope", "river_slope"),
                    ("river_water_flow__manning_n_parameter", "river_manning_n"),
                    ("river_bank_water__depth", "river_bankfull_depth"),
                    ("river_water__external_inflow_volume_flow_rate", "river_external_inflow")]:
        maps[sn] = (ncio.NC_DOUBLE, grid_of(dom.river[key], rl), np.nan)
    for field, (sn, factor, default, layered) in PARAMS.items():
        if field not in dom.params or dom.params[field] is None:
            continue
        v = np.asarray(dom.params[field], float)
        v = v - 273.15 if factor is None else v / factor
        if layered:
            v = v.reshape(n, N)
            maps[sn] = (ncio.NC_DOUBLE, np.stack([grid_of(v[:, k], land_cells) for k in range(N)]), np.nan)
        else:
            maps[sn] = (ncio.NC_DOUBLE, grid_of(v[:n], land_cells), np.nan)
    if reservoirs is not None:
        cells = rl[reservoirs["river_index"]]
        k = len(cells)
        maps["reservoir_location__count"] = (ncio.NC_INT, grid_of(np.arange(1, k + 1), cells, 0.0), -999.0)
        maps["reservoir_area__count"] = (ncio.NC_INT, grid_of(np.arange(1, k + 1), cells, 0.0), -999.0)
        maps["reservoir_water__rating_curve_type_count"] = (ncio.NC_INT, grid_of(reservoirs["outflow_curve_type"],
                                                                                 cells), -999.0)
        prof = reservoirs.get("storage_curve_type", np.ones(k))
        maps["reservoir_water__storage_curve_type_count"] = (ncio.NC_INT, grid_of(prof, cells), -999.0)
        if "lower_reservoir" in reservoirs:  # ids are 1..k in reservoir order
            lo = np.asarray(reservoirs["lower_reservoir"])
            maps["reservoir_lower_location__count"] = (ncio.NC_INT, grid_of(np.where(lo >= 0, lo + 1, 0), cells, 0.0),
                                                       -999.0)
        folder = Path(path).parent
        for i in range(k):  # the CSV tables beside the static maps (reservoir.jl:152-192)
            if "sh_offset" in reservoirs and prof[i] == 2:
                a, b = reservoirs["sh_offset"][i], reservoirs["sh_offset"][i + 1]
                write_sh_csv(folder / f"reservoir_sh_{i + 1}.csv", reservoirs["sh_h"][a:b], reservoirs["sh_s"][a:b])
            if "hq_offset" in reservoirs and reservoirs["outflow_curve_type"][i] == 1:
                a, b = reservoirs["hq_offset"][i], reservoirs["hq_offset"][i + 1]
                write_hq_csv(folder / f"reservoir_hq_{i + 1}.csv", reservoirs["hq_h"][a:b],
                             reservoirs["hq_q"][a * 365:b * 365].reshape(-1, 365))
        for key, sn in [("area", "reservoir_surface__area"), ("waterlevel", "reservoir_water_surface__initial_elevation"),
                        ("maximum_storage", "reservoir_water__max_volume"),
                        ("threshold", "reservoir_water_flow_threshold_level__elevation"),
                        ("rating_curve_coefficient", "reservoir_water__rating_curve_coefficient"),
                        ("rating_curve_exponent", "reservoir_water__rating_curve_exponent"),
                        ("maximum_release", "reservoir_water_release_below_spillway__max_volume_flow_rate"),
                        ("demand", "reservoir_water_demand__required_downstream_volume_flow_rate"),
                        ("target_minimum_fraction", "reservoir_water__target_min_volume_fraction"),
                        ("target_full_fraction", "reservoir_water__target_full_volume_fraction")]:
            maps[sn] = (ncio.NC_DOUBLE, grid_of(reservoirs[key], cells), np.nan)
    for sn, (t, a, fill) in maps.items():
        dims = ("layer", "y", "x") if a.ndim == 3 else ("y", "x")
        nc.def_var(names.get(sn, sn), t, dims, {"_FillValue": fill})
    nc.enddef()
    nc.write("x", grid.xc)
    nc.write("y", grid.yc)
    nc.write("layer", np.arange(1, N + 1, dtype=float))
    for sn, (t, a, fill) in maps.items():
        nc.write(names.get(sn, sn), a)
    nc.close()
