"""Seeded synthetic SBM domains and forcing.

Stands in for Wflow's staticmaps/forcing netCDF files (no such data ships with the reference
test suite in this environment): a square raster catchment with a fractal DEM (Hurst 0.8,
0-1000 m), a depression-free D8 drainage network draining to one corner outlet, a river
network where more than 20 cells drain through a cell, and per-cell soil, vegetation and snow
parameters drawn from the distributions of the benchmark configurations. Parameters that the
reference gives defaults for use those defaults (Wflow/src/standard_name/standard_name_sbm.jl,
standard_name_routing.jl). Units are SI, as after Wflow's `to_SI` (Wflow/src/units.jl:271).

Derived geometry follows the reference initialisation:
  flow length / width          Wflow/src/utils.jl:418-449
  river fraction               Wflow/src/domain.jl:311-347
  surface flow width           Wflow/src/utils.jl:458-466, domain.jl:231-233
  flow fraction to river       Wflow/src/utils.jl:493-510
  river graph (pit where the downstream cell is not a river cell)  Wflow/src/network.jl:214-258
"""

from dataclasses import dataclass, field

import numpy as np

from . import abi

MM = 1e-3
MM_PER_DAY = (1.0 / 86400.0) * 1e-3   # Wflow's mm d-1 to m s-1 factor
HURST = 0.8
SCALE_RATIO_H08 = float.fromhex("0x1.2611186bae674p-1")  # 2**-0.8, passed to the generator (no pow on the host)


@dataclass
class Domain:
    nx: int
    ny: int
    cell_size: float
    ldd: np.ndarray
    land: dict          # WfDomain land arrays + "land_downstream"
    river: dict         # WfDomain river arrays + "river_land_index", "river_downstream"
    params: dict        # WfParams arrays
    upstream_cells: np.ndarray
    catchment_of_cell: np.ndarray = None   # ragged batches: catchment id of each land cell
    outlets: list = field(default_factory=list)

    @property
    def n_land(self):
        return len(self.ldd)

    @property
    def n_river(self):
        return len(self.river["river_land_index"])


DEM_TILT = float(__import__("os").environ.get("WF_SYNTH_TILT", "1.0"))


def _d8(nx, ny, seed, cell_size, min_slope=1e-4, tilt=None):
    tilt = DEM_TILT if tilt is None else tilt
    lib = abi.load_synth()
    n = nx * ny
    dem = np.zeros(n)
    ldd = np.zeros(n, np.uint8)
    ds = np.zeros(n, np.int32)
    slope = np.zeros(n)
    ups = np.zeros(n, np.int64)
    fl = np.zeros(n)
    fw = np.zeros(n)
    import ctypes as C
    st = lib.wf_synth_dem_d8(nx, ny, C.c_uint64(seed), SCALE_RATIO_H08, 1000.0, float(cell_size), min_slope, tilt,
                             abi.as_ptr(dem), abi.as_ptr(ldd, C.c_uint8), abi.as_ptr(ds, C.c_int32),
                             abi.as_ptr(slope), abi.as_ptr(ups, C.c_int64), abi.as_ptr(fl), abi.as_ptr(fw))
    if st != 0:
        raise RuntimeError(f"wf_synth_dem_d8 failed ({st})")
    return dem, ldd, ds, slope, ups, fl, fw


def make_domain(nx, cell_size, seed=1, ny=None, river_min_cells=20, n_layers_cfg=(100.0, 300.0, 800.0)):
    """One square catchment of nx*ny cells (cells of `cell_size` metres)."""
    ny = nx if ny is None else ny
    dem, ldd, ds, slope, ups, fl, fw = _d8(nx, ny, seed, cell_size)
    n = nx * ny
    area = np.full(n, float(cell_size) * float(cell_size))
    is_river = ups > river_min_cells
    amax = float(ups.max())
    river_width_all = np.where(is_river, 10.0 + 90.0 * np.sqrt(ups / amax), 0.0)
    river_length_all = np.where(is_river, fl, 0.0)
    river_fraction = np.where(is_river, np.minimum((river_length_all * river_width_all) / area, 1.0), 0.0)
    water_fraction = np.maximum(np.zeros(n) - river_fraction, 0.0)
    land_area = (1.0 - river_fraction) * area
    sfw = np.where(is_river, land_area / fl, fw)
    # flow fraction to river (utils.jl:493-510)
    frac = np.zeros(n)
    j = np.nonzero(ds >= 0)[0]
    dsj = ds[j]
    sel = is_river[dsj] & (ldd[j] != ldd[dsj])
    jj, ii = j[sel], dsj[sel]
    frac[jj] = slope[jj] / (slope[ii] + slope[jj])
    land = dict(
        land_downstream=ds.astype(np.int32), area=area, flow_width=fw, flow_length=fl, surface_flow_width=sfw,
        slope=slope, flow_fraction_to_river=frac, river_fraction=river_fraction, water_fraction=water_fraction,
        elevation=dem, land_manning_n=np.full(n, 0.072))
    river_land = np.nonzero(is_river)[0].astype(np.int32)
    rindex = np.full(n, -1, np.int64)
    rindex[river_land] = np.arange(len(river_land))
    rds_land = ds[river_land]
    rds = np.where((rds_land >= 0) & is_river[np.maximum(rds_land, 0)], rindex[np.maximum(rds_land, 0)], -1)
    nr = len(river_land)
    river = dict(
        river_land_index=river_land, river_downstream=rds.astype(np.int32),
        river_width=river_width_all[river_land].copy(), river_length=river_length_all[river_land].copy(),
        river_slope=slope[river_land].copy(), river_manning_n=np.full(nr, 0.036),
        river_bankfull_depth=np.full(nr, 1.0), river_external_inflow=np.zeros(nr))
    params = make_params(n, seed, n_layers=len(n_layers_cfg) + 1)
    dom = Domain(nx=nx, ny=ny, cell_size=float(cell_size), ldd=ldd, land=land, river=river, params=params,
                 upstream_cells=ups)
    dom.outlets = [int(r) for r in np.nonzero(rds < 0)[0]]
    return dom


def make_params(n, seed, n_layers=4):
    """Per-cell SBM parameters (SI). Distributions of the benchmark configurations; reference
    defaults elsewhere (standard_name_sbm.jl line refs in the comments)."""
    rng = np.random.default_rng([int(seed), 7])
    p = {}
    p["theta_s"] = rng.uniform(0.45, 0.6, n)
    p["theta_r"] = rng.uniform(0.05, 0.1, n)
    ksat_mm_d = np.clip(np.exp(np.log(200.0) + 0.8 * rng.standard_normal(n)), 50.0, 500.0)
    p["kv_0"] = ksat_mm_d * MM_PER_DAY
    p["f"] = rng.uniform(0.001, 0.01, n) * 1000.0              # mm-1 -> m-1
    p["brooks_corey_exponent"] = rng.uniform(8.0, 12.0, n * n_layers)
    p["soil_thickness"] = np.full(n, 2000.0 * MM)
    p["air_entry_pressure"] = np.full(n, -0.1)                # -10 cm (:452-453)
    p["h1"] = np.zeros(n)                                     # 0 cm (:668-669)
    p["h2"] = np.full(n, -1.0)                                # -100 cm
    p["h3_high"] = np.full(n, -4.0)                           # -400 cm
    p["h3_low"] = np.full(n, -10.0)                           # -1000 cm
    p["h4"] = np.full(n, -160.0)                              # -16000 cm
    p["alpha_h1"] = np.ones(n)
    p["infiltration_capacity_compacted_soil"] = np.full(n, 10.0 * MM_PER_DAY)  # 10 mm d-1 (:38-39)
    p["compacted_soil_area_fraction"] = np.zeros(n)           # PathFrac 0
    p["wet_root_distribution_parameter"] = np.full(n, -500.0 * 1000.0)  # -500 mm-1 (:497)
    p["cap_hmax"] = np.full(n, 2000.0 * MM)                   # (:483)
    p["cap_n"] = np.full(n, 2.0)
    p["maximum_leakage"] = np.zeros(n)
    p["w_soil"] = np.full(n, 0.1125)
    p["cf_soil"] = np.full(n, 0.038)
    p["z_exp"] = np.full(n, 0.0)
    p["kv_factor"] = np.ones(n * n_layers)
    p["horizontal_to_vertical_ratio"] = np.full(n, 100.0)     # no reference default: fixed here
    # vegetation
    p["canopy_gap_fraction"] = rng.uniform(0.1, 0.6, n)       # no reference default: fixed here
    p["maximum_canopy_storage"] = np.full(n, 1.0 * MM)        # 1 mm (:711)
    p["crop_coefficient"] = np.ones(n)
    p["rooting_depth"] = rng.uniform(300.0, 800.0, n) * MM    # no reference default: fixed here
    p["evaporation_to_precipitation_ratio"] = np.full(n, 0.1)  # (:651)
    # snow (:8-19, :326-342)
    p["degree_day_factor"] = np.full(n, 3.75 * MM_PER_DAY)
    p["temperature_threshold_snowfall"] = np.full(n, 273.15)
    p["temperature_interval_snowfall"] = np.full(n, 1.0)
    p["temperature_threshold_melt"] = np.full(n, 273.15)
    p["water_holding_capacity"] = np.full(n, 0.1)
    return {k: np.ascontiguousarray(v, dtype=np.float64) for k, v in p.items()}


def perturb_members(params, n_members, seed):
    """Ensemble members: KsatVer x 10^U(-0.5, 0.5) and f x U(0.5, 2) per member; returns
    member-major kv_0/f arrays and the per-member precipitation factors lognormal(0, 0.3)."""
    rng = np.random.default_rng([int(seed), 11])
    kfac = 10.0 ** rng.uniform(-0.5, 0.5, n_members)
    ffac = rng.uniform(0.5, 2.0, n_members)
    pfac = np.exp(0.3 * rng.standard_normal(n_members))
    kv0 = np.concatenate([params["kv_0"] * k for k in kfac])
    f = np.concatenate([params["f"] * x for x in ffac])
    return kv0, f, pfac


def make_ragged(n_catchments, seed=3, cell_size=1000.0, log10_min=3.0, log10_max=6.0):
    """Uneven batch: independent square catchments of log-uniform size packed into one domain."""
    rng = np.random.default_rng([int(seed), 5])
    sides = np.maximum(np.round(np.sqrt(10.0 ** rng.uniform(log10_min, log10_max, n_catchments))), 4).astype(int)
    parts = [make_domain(int(s), cell_size, seed=int(seed) * 1000 + k) for k, s in enumerate(sides)]
    return concat_domains(parts)


def concat_domains(parts):
    land, river, params = {}, {}, {}
    off_l = off_r = 0
    cat = []
    outlets = []
    for k, d in enumerate(parts):
        for key, v in d.land.items():
            if key == "land_downstream":
                v = np.where(v >= 0, v + off_l, -1).astype(np.int32)
            land.setdefault(key, []).append(v)
        for key, v in d.river.items():
            if key == "river_land_index":
                v = (v + off_l).astype(np.int32)
            elif key == "river_downstream":
                v = np.where(v >= 0, v + off_r, -1).astype(np.int32)
            river.setdefault(key, []).append(v)
        for key, v in d.params.items():
            params.setdefault(key, []).append(v)
        cat.append(np.full(d.n_land, k, np.int32))
        outlets += [o + off_r for o in d.outlets]
        off_l += d.n_land
        off_r += d.n_river
    cat_arr = np.concatenate(cat)
    out = Domain(nx=off_l, ny=1, cell_size=parts[0].cell_size,
                 ldd=np.concatenate([d.ldd for d in parts]),
                 land={k: np.ascontiguousarray(np.concatenate(v)) for k, v in land.items()},
                 river={k: np.ascontiguousarray(np.concatenate(v)) for k, v in river.items()},
                 params={k: np.ascontiguousarray(np.concatenate(v)) for k, v in params.items()},
                 upstream_cells=np.concatenate([d.upstream_cells for d in parts]), catchment_of_cell=cat_arr)
    out.outlets = outlets
    return out


def forcing(step, dt, n, seed=1, precip_scale=1.0):
    """Forcing of model step `step` (0-based) in SI: precipitation and potential evaporation
    [m s-1], temperature [K]. Daily rates are divided by the number of steps per day."""
    rng = np.random.default_rng([int(seed), 1000003, int(step)])
    steps_per_day = 86400.0 / dt
    t_days = (step + 1) * dt / 86400.0
    season = np.sin(2.0 * np.pi * t_days / 365.0)
    dry = rng.random(n) < 0.4
    p_mm_day = np.where(dry, 0.0, rng.gamma(0.4, 10.0, n)) * precip_scale
    temp_c = 10.0 + 10.0 * season + 3.0 * rng.standard_normal(n)
    pet_mm_day = np.full(n, 2.5 + 2.5 * season)
    to_si = 1e-3 * (1.0 / dt)   # mm dt-1 -> m s-1
    P = (p_mm_day / steps_per_day) * to_si
    PET = (pet_mm_day / steps_per_day) * to_si
    T = temp_c + 273.15
    return np.ascontiguousarray(P), np.ascontiguousarray(PET), np.ascontiguousarray(T)


def make_config(dt, n_members=1, form=abi.WF_FORM_FP64, snow=True, adaptive=False, mass_balance=True,
                layers=(100.0, 300.0, 800.0), per_member_soil=False):
    c = abi.WfConfig()
    c.dt = float(dt)
    c.n_soil_layer_thickness = len(layers)
    for i, t in enumerate(layers):
        c.soil_layer_thickness[i] = t * MM
    c.snow = int(snow)
    c.soil_infiltration_reduction = 0
    c.water_mass_balance = int(mass_balance)
    c.adaptive_timestep = int(adaptive)
    c.kv_profile = abi.WF_KV_EXPONENTIAL
    c.land_dt_fixed = 3600.0
    c.river_dt_fixed = 900.0
    c.subsurface_dt_fixed = 86400.0
    c.subsurface_alpha = 1.0
    c.form = int(form)
    c.n_members = int(n_members)
    c.per_member_soil = int(per_member_soil)
    return c


def c_structs(dom, params=None):
    """WfDomain and WfParams structs pointing into the domain's arrays (keep `dom` alive)."""
    import ctypes as C
    params = dom.params if params is None else params
    d = abi.WfDomain()
    d.n_land = dom.n_land
    d.land_downstream = abi.as_ptr(dom.land["land_downstream"], C.c_int32)
    for k in abi.DOMAIN_LAND_ARRAYS:
        setattr(d, k, abi.as_ptr(dom.land[k]))
    d.n_river = dom.n_river
    d.river_land_index = abi.as_ptr(dom.river["river_land_index"], C.c_int32)
    d.river_downstream = abi.as_ptr(dom.river["river_downstream"], C.c_int32)
    for k in abi.DOMAIN_RIVER_ARRAYS:
        setattr(d, k, abi.as_ptr(dom.river[k]))
    p = abi.WfParams()
    for k in abi.PARAM_FIELDS:
        setattr(p, k, abi.as_ptr(params.get(k)))
    return d, p


def make_reservoirs(dom, n, seed=1, types=(abi.WF_RES_SIMPLE, abi.WF_RES_MODIFIED_PULS, abi.WF_RES_FREE_WEIR)):
    """`n` reservoirs on river cells of the domain (outflow types cycling through `types`), at
    cells with a downstream river cell, no two draining into the same cell. Parameters are of the
    scale of the reference's reservoir unit test (test/routing_process.jl:310-331) with the area
    scaled down so that a step's inflow moves the water level noticeably."""
    rng = np.random.default_rng([int(seed), 77])
    rds = dom.river["river_downstream"]
    rland = dom.river["river_land_index"]
    up = np.asarray(dom.upstream_cells)[rland]
    order = np.argsort(-up, kind="stable")
    cand = [int(v) for v in order if rds[v] >= 0][: max(4 * n, n)]
    rng.shuffle(cand)
    chosen, fed = [], set()
    for v in cand:
        if len(chosen) == n:
            break
        if v in chosen or int(rds[v]) in fed:
            continue
        chosen.append(v)
        fed.add(int(rds[v]))
    k = len(chosen)
    t = np.array([types[i % len(types)] for i in range(k)], np.int32)
    area = rng.uniform(2.0e4, 2.0e5, k)
    wl = rng.uniform(2.0, 8.0, k)
    nan = np.full(k, np.nan)
    simple = t == abi.WF_RES_SIMPLE
    weir = (t == abi.WF_RES_FREE_WEIR) | (t == abi.WF_RES_MODIFIED_PULS)
    res = dict(
        river_index=np.array(chosen, np.int32), outflow_curve_type=t, area=area, waterlevel=wl,
        maximum_storage=np.where(simple, area * wl * rng.uniform(1.05, 1.4, k), nan),
        threshold=np.where(weir, wl - rng.uniform(0.1, 1.0, k), nan),
        rating_curve_coefficient=np.where(weir, rng.uniform(0.5, 5.0, k), nan),
        rating_curve_exponent=np.where(t == abi.WF_RES_FREE_WEIR, rng.uniform(1.2, 2.0, k), nan),
        maximum_release=np.where(simple, rng.uniform(0.5, 5.0, k), nan),
        demand=np.where(simple, rng.uniform(0.01, 0.3, k), nan),
        target_minimum_fraction=np.where(simple, rng.uniform(0.05, 0.2, k), nan),
        target_full_fraction=np.where(simple, rng.uniform(0.6, 0.9, k), nan),
    )
    return {key: np.ascontiguousarray(v) for key, v in res.items()}


TABLE_KEYS = ("storage_curve_type", "sh_offset", "sh_h", "sh_s", "hq_offset", "hq_h", "hq_q", "lower_reservoir")


def _sh_table(area, wl, rng, rows=9):
    """An S-H table around water level `wl`: storage grows a little faster than linearly with
    the level (a basin widening upward), zero at the lowest level."""
    h = wl + np.linspace(-3.0, 4.0, rows)
    s = area * (h - h[0]) ** rng.uniform(1.05, 1.3) + np.arange(rows) * 1e-3 * area
    return h, s


def _hq_table(wl, threshold, rng, rows=7):
    """An H-Q table: no outflow up to `threshold`, then a weir-like rise; the discharge of each
    day of the year varies seasonally by +-30 %."""
    h = np.sort(np.concatenate([[threshold], wl + np.linspace(-2.5, 4.5, rows - 1)]))
    h = np.unique(h)
    base = np.where(h > threshold, rng.uniform(0.5, 2.0) * np.maximum(h - threshold, 0.0) ** 1.5, 0.0)
    season = 1.0 + 0.3 * np.sin(2.0 * np.pi * (np.arange(365) + rng.uniform(0, 365)) / 365.0)
    return h, np.ascontiguousarray(np.outer(base, season))


def make_linked_reservoirs(dom, seed=1, extra=2):
    """Reservoirs with tables and a link (ReservoirParameters, reservoir.jl:5-44): an upper free
    weir linked to a lower reservoir a few river cells downstream on the main stem (both with
    interpolated S-H profiles, the lower one released by a rating curve), the lower reservoir's
    level above the upper one's at the start so that water first flows back; plus `extra`
    reservoirs elsewhere (a modified Puls with the linear profile and a simple reservoir with an
    interpolated profile, cycling)."""
    rng = np.random.default_rng([int(seed), 91])
    rds = dom.river["river_downstream"]
    nr = rds.size
    rland = dom.river["river_land_index"]
    up = np.asarray(dom.upstream_cells)[rland]
    # main stem: from the outlet upward, always into the upstream neighbour of largest area
    children = [[] for _ in range(nr)]
    for v in range(nr):
        if rds[v] >= 0:
            children[rds[v]].append(v)
    outlet = int(np.argmax(np.where(rds < 0, up, -1)))
    stem = [outlet]
    while children[stem[-1]]:
        stem.append(max(children[stem[-1]], key=lambda c: up[c]))
    lo_v, up_v = stem[len(stem) // 3], stem[len(stem) // 3 + 4]  # four river cells apart
    others = [int(v) for v in np.argsort(-up, kind="stable")
              if rds[v] >= 0 and v not in stem and rds[v] not in stem][: 8 * extra]
    rng.shuffle(others)
    chosen, fed = [up_v, lo_v], {int(rds[up_v]), int(rds[lo_v])}
    for v in others:
        if len(chosen) == 2 + extra:
            break
        if int(rds[v]) in fed or v in chosen:
            continue
        chosen.append(v)
        fed.add(int(rds[v]))
    k = len(chosen)
    t = np.array([abi.WF_RES_FREE_WEIR, abi.WF_RES_RATING_CURVE]
                 + [(abi.WF_RES_MODIFIED_PULS, abi.WF_RES_SIMPLE)[i % 2] for i in range(k - 2)], np.int32)
    area = rng.uniform(5.0e4, 2.0e5, k)
    wl = np.concatenate([[5.0, 5.3], rng.uniform(2.0, 8.0, k - 2)])
    prof = np.array([2, 2] + [(1, 2)[i % 2] for i in range(k - 2)], np.int32)
    nan = np.full(k, np.nan)
    simple = t == abi.WF_RES_SIMPLE
    weir = (t == abi.WF_RES_FREE_WEIR) | (t == abi.WF_RES_MODIFIED_PULS)
    thr = np.where(weir | (t == abi.WF_RES_RATING_CURVE), wl - rng.uniform(0.2, 0.8, k), nan)
    sh_h, sh_s, sh_off, hq_h, hq_q, hq_off = [], [], [0], [], [], [0]
    s0 = area * wl
    for i in range(k):
        if prof[i] == 2:
            h, sv = _sh_table(area[i], wl[i], rng)
            sh_h.append(h)
            sh_s.append(sv)
            s0[i] = np.interp(wl[i], h, sv)
        sh_off.append(sh_off[-1] + (len(sh_h[-1]) if prof[i] == 2 else 0))
        if t[i] == abi.WF_RES_RATING_CURVE:
            h, q = _hq_table(wl[i], thr[i], rng)
            hq_h.append(h)
            hq_q.append(q)
        hq_off.append(hq_off[-1] + (len(hq_h[-1]) if t[i] == abi.WF_RES_RATING_CURVE else 0))
    lower = np.full(k, -1, np.int32)
    lower[0] = 1
    res = dict(
        river_index=np.array(chosen, np.int32), outflow_curve_type=t, area=area, waterlevel=wl,
        maximum_storage=np.where(simple, s0 * rng.uniform(1.05, 1.4, k), nan),
        threshold=np.where(weir, thr, nan),
        rating_curve_coefficient=np.where(weir, rng.uniform(0.5, 5.0, k), nan),
        rating_curve_exponent=np.where(t == abi.WF_RES_FREE_WEIR, rng.uniform(1.2, 2.0, k), nan),
        maximum_release=np.where(simple, rng.uniform(0.5, 5.0, k), nan),
        demand=np.where(simple, rng.uniform(0.01, 0.3, k), nan),
        target_minimum_fraction=np.where(simple, rng.uniform(0.05, 0.2, k), nan),
        target_full_fraction=np.where(simple, rng.uniform(0.6, 0.9, k), nan),
        storage_curve_type=prof, sh_offset=np.array(sh_off, np.int64),
        sh_h=np.concatenate(sh_h) if sh_h else np.zeros(0), sh_s=np.concatenate(sh_s) if sh_s else np.zeros(0),
        hq_offset=np.array(hq_off, np.int64), hq_h=np.concatenate(hq_h) if hq_h else np.zeros(0),
        hq_q=np.concatenate(hq_q).reshape(-1) if hq_q else np.zeros(0), lower_reservoir=lower,
    )
    return {key: np.ascontiguousarray(v) for key, v in res.items()}


def c_reservoir_tables(res):
    """WfReservoirTables struct pointing into a reservoir dict's table arrays (keep `res` alive),
    or None when the dict has no tables or links."""
    import ctypes as C
    if res is None or not any(k in res for k in TABLE_KEYS):
        return None
    t = abi.WfReservoirTables()
    for k in TABLE_KEYS:
        a = res.get(k)
        if a is None:
            continue
        ct = C.c_int32 if k in ("storage_curve_type", "lower_reservoir") else C.c_int64 if k.endswith("offset") \
            else C.c_double
        setattr(t, k, abi.as_ptr(a, ct))
    return t


def reservoir_forcing(dom, res, P, PET, M=1):
    """Reservoir precipitation and evaporation of a step [m s-1], member-major, taken from the
    land forcing at each reservoir's outlet cell (a one-cell reservoir area; Wflow averages the
    forcing over the reservoir's area cells, io.jl:128-137)."""
    cells = dom.river["river_land_index"][res["river_index"]]
    n = dom.n_land
    P = np.asarray(P).reshape(-1)
    PET = np.asarray(PET).reshape(-1)
    mp = P.size // n
    rp = np.concatenate([P[(m if mp > 1 else 0) * n + cells] for m in range(M)])
    re = np.concatenate([PET[(m if PET.size // n > 1 else 0) * n + cells] for m in range(M)])
    return np.ascontiguousarray(rp), np.ascontiguousarray(re)


def c_reservoirs(res):
    """WfReservoirs struct pointing into the arrays of a reservoir dict (keep `res` alive)."""
    import ctypes as C
    r = abi.WfReservoirs()
    if res is None:
        r.n = 0
        return r
    r.n = int(res["river_index"].size)
    r.river_index = abi.as_ptr(res["river_index"], C.c_int32)
    r.outflow_curve_type = abi.as_ptr(res["outflow_curve_type"], C.c_int32)
    for k in abi.RESERVOIR_PARAMS:
        setattr(r, k, abi.as_ptr(res.get(k)))
    return r


def li_grid(nx, ny, seed=1, river_every=64, cell=100.0):
    """A local-inertial land grid with its river (include/wflow_gb300_li.h) for throughput runs: a
    square grid of `cell` m cells, elevation falling east and toward the river rows, a river along
    every `river_every`-th row draining east into one ghost cell per row, a warm state and 5 mm/h
    of runoff on every cell. Returns (land, river, h_river, h_land, runoff) for
    li_river.LiDomain."""
    rng = np.random.default_rng(seed)
    n = nx * ny
    idx = np.arange(n)
    row, col = np.divmod(idx, nx)
    land = dict(ind_x_up=np.where(col > 0, idx - 1, n), ind_x_down=np.where(col < nx - 1, idx + 1, n),
                ind_y_up=np.where(row > 0, idx - nx, n), ind_y_down=np.where(row < ny - 1, idx + nx, n),
                x_length=np.full(n, cell), y_length=np.full(n, cell))
    rows = np.arange(river_every // 2, ny, river_every)
    r = (row - river_every // 2) % river_every
    dist = np.minimum(r, river_every - r)  # rows to the nearest river row
    land["elevation"] = 0.001 * (nx - col) * cell + 0.002 * dist * cell + rng.uniform(0.0, 0.05, n)
    land["mannings_n_sq"] = rng.uniform(0.03, 0.08, n) ** 2
    cells = (rows[:, None] * nx + np.arange(nx)[None, :]).ravel()  # river cells, row by row
    nra, nrow = len(cells), len(rows)
    river_index = np.full(n, -1, np.int64)
    river_index[cells] = np.arange(nra)
    land["river_index"] = river_index
    width = rng.uniform(10.0, 40.0, nra + nrow)
    land["xwidth_at_edge"] = land["x_length"].copy()
    land["ywidth_at_edge"] = land["y_length"].copy()
    land["ywidth_at_edge"][cells] = np.maximum(cell - width[:nra], 0.0)
    land.update(theta=0.8, h_thresh=1e-3, alpha=0.7, froude_limit=True)
    k = np.arange(nra)
    last = (k % nx) == nx - 1
    src = k.astype(np.int64)
    dst = np.where(last, nra + k // nx, k + 1).astype(np.int64)
    bankfull = rng.uniform(1.0, 2.0, nra + nrow)
    zb = np.concatenate([land["elevation"][cells], land["elevation"][cells[last]] - 0.5]) - bankfull
    fl = np.full(nra + nrow, cell)
    n_manning = rng.uniform(0.025, 0.04, nra + nrow)
    n_e = (n_manning[dst] * fl[dst] + n_manning[src] * fl[src]) / (fl[dst] + fl[src])
    river = dict(n_active=nra, src=src, dst=dst, zb=zb, flow_length=fl, flow_width=width, bankfull_depth=bankfull,
                 zb_edge=np.maximum(zb[src], zb[dst]), width_edge=np.minimum(width[dst], width[src]),
                 length_edge=0.5 * (fl[dst] + fl[src]), mannings_n_sq_edge=n_e * n_e, h_thresh=1e-3, alpha=0.7,
                 froude_limit=True)
    h_river = np.concatenate([rng.uniform(0.3, 1.5, nra), np.full(nrow, 1.0)])
    h_land = rng.uniform(0.0, 0.1, n) * (rng.random(n) < 0.5)
    h_land[cells] = 0.0
    runoff = np.full(n, 5e-3 / 3600.0 * cell * cell)  # 5 mm/h over every cell [m3 s-1]
    return land, river, h_river, h_land, runoff


def li_coupling(dom, seed=1, warm=True, theta=0.8, alpha=0.7, h_thresh=1e-3):
    """The local-inertial land grid with its river for the cells of `dom` (a square grid from
    make_domain), as Wflow builds it for land_routing = river_routing = "local_inertial":
    edge_indices of the staggered grid (network.jl:136-154: ind_x_up the cell at x + 1, ind_x_down
    at x - 1, likewise y; n outside), land edge widths reduced by the river widths along the river's
    D8 directions (set_effective_flowwidth!, utils.jl:604-680), a ghost cell after the active river
    cells at every pit with the pit's width, length, Manning's n and bed (get_river_parameters,
    surface_staggered_scheme.jl:40-74), bed level = bank elevation - bankfull depth, edge values as
    RiverFlowStaggeredParameters derives them (:96-156). Returns (land, river, h_land, h_river) for
    li_river.LiDomain / OracleModel.attach_li; `warm` starts the river 0.2-1 m deep and a few land
    cells ponded, else dry (the ghost cells stay at 0 m)."""
    rng = np.random.default_rng([seed, 77])
    nx, ny, n = dom.nx, dom.ny, dom.n_land
    idx = np.arange(n)
    row, col = np.divmod(idx, nx)
    cell = dom.cell_size
    land = dict(ind_x_up=np.where(col < nx - 1, idx + 1, n), ind_x_down=np.where(col > 0, idx - 1, n),
                ind_y_up=np.where(row < ny - 1, idx + nx, n), ind_y_down=np.where(row > 0, idx - nx, n),
                x_length=np.full(n, cell), y_length=np.full(n, cell),
                elevation=np.asarray(dom.land["elevation"], float).copy(),
                mannings_n_sq=np.asarray(dom.land["land_manning_n"], float) ** 2,
                theta=theta, h_thresh=h_thresh, alpha=alpha, froude_limit=True)
    rl = np.asarray(dom.river["river_land_index"], np.int64)
    rds = np.asarray(dom.river["river_downstream"], np.int64)
    nra = len(rl)
    river_index = np.full(n, -1, np.int64)
    river_index[rl] = np.arange(nra)
    land["river_index"] = river_index
    pits = np.nonzero(rds < 0)[0]
    ghost = np.full(nra, -1, np.int64)
    ghost[pits] = nra + np.arange(len(pits))
    width = np.concatenate([dom.river["river_width"], dom.river["river_width"][pits]])
    length = np.concatenate([dom.river["river_length"], dom.river["river_length"][pits]])
    mann = np.concatenate([dom.river["river_manning_n"], dom.river["river_manning_n"][pits]])
    bankfull = np.concatenate([dom.river["river_bankfull_depth"], dom.river["river_bankfull_depth"][pits]])
    bank_elev = np.concatenate([land["elevation"][rl], land["elevation"][rl[pits]]])
    zb = bank_elev - bankfull
    src = np.arange(nra, dtype=np.int64)  # one outgoing edge per river cell, in cell order
    dst = np.where(rds >= 0, rds, ghost).astype(np.int64)
    n_e = (mann[dst] * length[dst] + mann[src] * length[src]) / (length[dst] + length[src])
    river = dict(n_active=nra, src=src, dst=dst, zb=zb, flow_length=length, flow_width=width,
                 bankfull_depth=bankfull, zb_edge=np.maximum(zb[src], zb[dst]),
                 width_edge=np.minimum(width[dst], width[src]), length_edge=0.5 * (length[dst] + length[src]),
                 mannings_n_sq_edge=n_e * n_e, h_thresh=h_thresh, alpha=alpha, froude_limit=True)
    # effective land edge widths along the river's D8 directions (PCRaster codes: x right, y down
    # the rows; code -> (dx, dy) as Wflow's PCR_DIR)
    pcr = {1: (-1, -1), 2: (0, -1), 3: (1, -1), 4: (-1, 0), 6: (1, 0), 7: (-1, 1), 8: (0, 1), 9: (1, 1)}
    we_x, we_y = land["x_length"].copy(), land["y_length"].copy()
    ldd = np.asarray(dom.ldd).reshape(-1)
    xd, yd = land["ind_x_down"], land["ind_y_down"]
    for v in range(nra):
        if rds[v] < 0:
            continue
        w = min(width[v], width[rds[v]])
        i = rl[v]
        d = pcr.get(int(ldd[i]))
        if d is None:
            continue
        half = 0.5 * w
        if d == (1, 1):
            we_x[i] = max(we_x[i] - half, 0.0)
            we_y[i] = max(we_y[i] - half, 0.0)
        elif d == (-1, -1):
            if xd[i] < n:
                we_y[xd[i]] = max(we_y[xd[i]] - half, 0.0)
            if yd[i] < n:
                we_x[yd[i]] = max(we_x[yd[i]] - half, 0.0)
        elif d == (1, 0):
            we_y[i] = max(we_y[i] - w, 0.0)
        elif d == (0, 1):
            we_x[i] = max(we_x[i] - w, 0.0)
        elif d == (-1, 0):
            if xd[i] < n:
                we_y[xd[i]] = max(we_y[xd[i]] - w, 0.0)
        elif d == (0, -1):
            if yd[i] < n:
                we_x[yd[i]] = max(we_x[yd[i]] - w, 0.0)
        elif d == (1, -1):
            we_y[i] = max(we_y[i] - half, 0.0)
            if yd[i] < n:
                we_x[yd[i]] = max(we_x[yd[i]] - half, 0.0)
        elif d == (-1, 1):
            if xd[i] < n:
                we_y[xd[i]] = max(we_y[xd[i]] - half, 0.0)
            we_x[i] = max(we_x[i] - half, 0.0)
    land["xwidth_at_edge"], land["ywidth_at_edge"] = we_x, we_y
    h_river = np.zeros(nra + len(pits))
    h_land = np.zeros(n)
    if warm:
        h_river[:nra] = rng.uniform(0.2, 1.0, nra)
        pond = (rng.random(n) < 0.05) & (river_index < 0)
        h_land[pond] = rng.uniform(0.0, 0.05, int(pond.sum()))
    return land, river, h_land, h_river
