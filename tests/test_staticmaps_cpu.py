"""Wflow static maps (wflow_gb300.staticmaps) on the CPU.

`load_staticmaps` restates the part of Wflow's model construction the path needs (active cells,
PCRaster drainage graph with pits where a direction leaves the active cells, river network,
cell geometry in metres or from latitude, fractions, slopes, parameters in file units with the
standard-name defaults). Checked here: a domain written as a static-map file loads back to the
same arrays and the same model results; hand-made grids pin the graph rules, axis
standardisation (a decreasing y axis), latitude geometry (utils.jl:114-150) and the TOML-style
name mapping and constants; reservoir maps load back to the reservoir set.
"""

import numpy as np
import pytest

from wflow_gb300 import abi, staticmaps, synthetic
import oracle_py as O

netcdf = pytest.importorskip("scipy.io").netcdf_file
F = abi.FIELD


def test_round_trip_domain_and_model(tmp_path):
    dom = synthetic.make_domain(20, 250.0, seed=8, ny=16)
    path = tmp_path / "staticmaps.nc"
    staticmaps.write_staticmaps(dom, path)
    got, grid, _ = staticmaps.load_staticmaps(path)
    assert got.n_land == dom.n_land and got.n_river == dom.n_river
    for k in ("land_downstream",):
        assert np.array_equal(got.land[k], dom.land[k])
    for k in ("river_land_index", "river_downstream"):
        assert np.array_equal(got.river[k], dom.river[k])
    for part_got, part_ref in ((got.land, dom.land), (got.river, dom.river)):
        for k, v in part_ref.items():
            np.testing.assert_allclose(part_got[k], v, rtol=2e-16, atol=0, err_msg=k)
    for k, v in dom.params.items():
        if v is None:
            continue
        np.testing.assert_allclose(got.params[k], v, rtol=4e-16, atol=0, err_msg=k)
    assert np.array_equal(grid.col, np.arange(dom.n_land) % 20) and np.array_equal(grid.row, np.arange(dom.n_land) // 20)
    # the model built from the file runs like the model built from the arrays
    cfg = synthetic.make_config(86400.0)
    a, b = O.OracleModel(cfg, dom), O.OracleModel(cfg, got)
    for s in range(4):
        P, PET, T = synthetic.forcing(s, cfg.dt, dom.n_land, seed=1)
        for m in (a, b):
            m.set_forcing(P, PET, T)
            m.step()
    for f in ("RIVER_Q", "SSF_Q", "SATURATED_WATER_DEPTH", "LAND_Q"):
        x, y = a.get(F[f]), b.get(F[f])
        assert np.max(np.abs(x - y) / np.maximum(np.abs(x), 1e-300)) <= 1e-12, f


def _tiny(path, y_descending=False, latlon=False, extra=None):
    """A 4 x 3 grid: one inactive cell, a direction into it, one leaving the grid, a river."""
    ny, nx = 3, 4
    sub = np.array([[1, 1, 1, 1], [1, 1, -999, 1], [1, 1, 1, 1]], np.int32)
    # PCRaster codes (x right, y up the array): 6 east, 4 west, 2 y-1, 8 y+1, 5 pit
    ldd = np.array([[6, 6, 6, 5], [6, 6, 5, 2], [6, 6, 2, 2]], np.int8)
    river = np.array([[0, 1, 1, 1], [0, 0, 0, 1], [0, 0, 0, 1]], np.int8)
    slope = np.full((ny, nx), 0.01)
    slope[0, 0] = 1e-7  # clamped to 1e-5
    xc = np.arange(nx) * (0.25 if latlon else 100.0)
    yc = (np.arange(ny) * (0.25 if latlon else 100.0)) + (50.0 if latlon else 0.0)
    if y_descending:
        sub, ldd, river, slope, yc = sub[::-1], ldd[::-1].copy(), river[::-1], slope[::-1], yc[::-1]
    f = netcdf(str(path), "w", version=2)
    xn, yn = ("lon", "lat") if latlon else ("x", "y")
    f.createDimension(xn, nx)
    f.createDimension(yn, ny)
    f.createVariable(xn, "d", (xn,))[:] = xc
    f.createVariable(yn, "d", (yn,))[:] = yc
    v = f.createVariable("wflow_subcatch", "i", (yn, xn))
    v[:] = sub
    v._FillValue = np.int32(-999)
    f.createVariable("basin__local_drain_direction", "b", (yn, xn))[:] = ldd
    f.createVariable("river_location__mask", "b", (yn, xn))[:] = river
    f.createVariable("land_surface__slope", "d", (yn, xn))[:] = slope
    for sn in ("river__width", "river__length", "river__slope"):
        f.createVariable(sn, "d", (yn, xn))[:] = np.full((ny, nx), 20.0 if sn != "river__slope" else 0.001)
    for field, (sn, factor, default, layered) in staticmaps.PARAMS.items():
        if default is None and not layered and sn != "soil_water__residual_volume_fraction":
            f.createVariable(sn, "d", (yn, xn))[:] = np.full((ny, nx), 0.3)
    f.createVariable("soil_water__residual_volume_fraction", "d", (yn, xn))[:] = np.full((ny, nx), 0.05)
    f.createDimension("layer", 2)
    f.createVariable("soil_layer_water__brooks_corey_exponent", "d", ("layer", yn, xn))[:] = np.full((2, ny, nx), 10.0)
    for k, val in (extra or {}).items():
        f.createVariable(k, "d", (yn, xn))[:] = val
    f.close()


MAPPING = {"subbasin_location__count": "wflow_subcatch"}


def test_graph_rules_on_a_hand_made_grid(tmp_path):
    p = tmp_path / "t.nc"
    _tiny(p)
    dom, grid, _ = staticmaps.load_staticmaps(p, mapping=MAPPING)
    # active cells x fastest, y slowest; (x=2, y=1) inactive
    assert dom.n_land == 11
    cell = {(int(c), int(r)): i for i, (c, r) in enumerate(zip(grid.col, grid.row))}
    ds = dom.land["land_downstream"]
    assert ds[cell[(0, 0)]] == cell[(1, 0)] and ds[cell[(2, 0)]] == cell[(3, 0)]
    assert ds[cell[(3, 0)]] == -1                      # code 5: pit
    assert ds[cell[(1, 1)]] == -1                      # east into the inactive cell: pit
    assert dom.ldd[cell[(1, 1)]] == 5
    assert ds[cell[(3, 1)]] == cell[(3, 0)]            # code 2: y - 1
    assert ds[cell[(3, 2)]] == cell[(3, 1)]
    assert ds[cell[(2, 2)]] == -1                      # y - 1 into the inactive cell: pit
    # river network: (1,0) -> (2,0) -> (3,0) pit, (3,2) -> (3,1) -> (3,0)
    rl = list(dom.river["river_land_index"])
    rds = dom.river["river_downstream"]
    r = {(int(grid.col[i]), int(grid.row[i])): k for k, i in enumerate(rl)}
    assert rds[r[(1, 0)]] == r[(2, 0)] and rds[r[(2, 0)]] == r[(3, 0)] and rds[r[(3, 0)]] == -1
    assert rds[r[(3, 2)]] == r[(3, 1)]
    # geometry: straight directions take the cell length, pits and diagonals the hypotenuse
    fl, fw = dom.land["flow_length"], dom.land["flow_width"]
    assert fl[cell[(0, 0)]] == 100.0 and fw[cell[(0, 0)]] == 100.0
    assert fl[cell[(3, 0)]] == np.hypot(100.0, 100.0)
    assert dom.land["slope"][cell[(0, 0)]] == 1e-5
    # flow fraction to the river (utils.jl:493-510): (0,0) drains into the river cell (1,0) in
    # the same direction as that cell drains, fraction 0; (3,1) is itself a river cell
    assert dom.land["flow_fraction_to_river"][cell[(0, 0)]] == 0.0
    assert dom.params["brooks_corey_exponent"].size == 11 * 2
    assert np.all(dom.params["kv_factor"] == 1.0)                 # default, per layer
    np.testing.assert_allclose(dom.params["air_entry_pressure"], -0.1)  # default -10 cm
    np.testing.assert_allclose(dom.params["kv_0"], 0.3 * 1e-3 / 86400.0)  # mm d-1


def test_decreasing_y_axis_is_standardised(tmp_path):
    a, b = tmp_path / "a.nc", tmp_path / "b.nc"
    _tiny(a)
    _tiny(b, y_descending=True)
    da, ga, _ = staticmaps.load_staticmaps(a, mapping=MAPPING)
    db, gb, _ = staticmaps.load_staticmaps(b, mapping=MAPPING)
    assert np.array_equal(da.land["land_downstream"], db.land["land_downstream"])
    assert np.array_equal(ga.yc, gb.yc)
    for k in da.land:
        assert np.array_equal(da.land[k], db.land[k]), k


def test_latitude_geometry(tmp_path):
    p = tmp_path / "ll.nc"
    _tiny(p, latlon=True)
    dom, grid, _ = staticmaps.load_staticmaps(p, mapping=MAPPING, cell_length_in_meter=False)
    lat = grid.yc[grid.row]
    d = np.deg2rad
    latlen = 111132.92 - 559.82 * np.cos(d(2 * lat)) + 1.175 * np.cos(d(4 * lat)) - 0.0023 * np.cos(d(6 * lat))
    lonlen = 111412.84 * np.cos(d(lat)) - 93.5 * np.cos(d(3 * lat)) + 0.118 * np.cos(d(5 * lat))
    np.testing.assert_allclose(dom.land["area"], (lonlen * 0.25) * (latlen * 0.25), rtol=1e-14)
    assert dom.land["area"][grid.row == 0][0] > dom.land["area"][grid.row == 2][0]  # cells shrink poleward


def test_mapping_constants_and_missing_values(tmp_path):
    p = tmp_path / "m.nc"
    _tiny(p, extra={"my_kc": np.full((3, 4), 0.8)})
    mapping = dict(MAPPING, **{"vegetation__crop_factor": "my_kc", "vegetation_root__depth": {"value": 450.0}})
    dom, _, _ = staticmaps.load_staticmaps(p, mapping=mapping)
    assert np.all(dom.params["crop_coefficient"] == 0.8)
    np.testing.assert_allclose(dom.params["rooting_depth"], 0.45)
    q = tmp_path / "q.nc"
    bad = np.full((3, 4), 0.3)
    bad[0, 1] = np.nan
    _tiny(q, extra={"theta_bad": bad})
    with pytest.raises(ValueError, match="missing values"):
        staticmaps.load_staticmaps(q, mapping=dict(MAPPING, soil_water__saturated_volume_fraction="theta_bad"))
    with pytest.raises(KeyError, match="soil__thickness"):
        staticmaps.load_staticmaps(q, mapping=dict(MAPPING, soil__thickness="absent"))


def test_reservoir_maps_round_trip(tmp_path):
    dom = synthetic.make_domain(24, 1000.0, seed=5)
    res = synthetic.make_reservoirs(dom, 3, seed=2)
    p = tmp_path / "r.nc"
    staticmaps.write_staticmaps(dom, p, reservoirs=res)
    got, _, gres = staticmaps.load_staticmaps(p, reservoirs=True)
    order = np.argsort(res["river_index"])  # the file gives reservoirs in river order
    for k, v in res.items():
        np.testing.assert_array_equal(gres[k], v[order], err_msg=k)
    cfg = synthetic.make_config(86400.0)
    m = O.OracleModel(cfg, got, reservoirs=gres)
    P, PET, T = synthetic.forcing(0, cfg.dt, got.n_land, seed=1)
    m.set_forcing(P, PET, T)
    m.step()
    assert np.all(np.isfinite(m.get(F["RESERVOIR_STORAGE"])))


def test_reservoir_tables_and_links_round_trip(tmp_path):
    # storage profiles, rating curves and a link in the maps, the tables in reservoir_sh_<id>.csv
    # and reservoir_hq_<id>.csv beside them (reservoir.jl:152-192; read_sh_csv / read_hq_csv,
    # io.jl:1129-1147): the oracle fed the loaded set follows the one fed the original set
    dom = synthetic.make_domain(48, 1000.0, seed=3)
    res = synthetic.make_linked_reservoirs(dom, seed=3)
    p = tmp_path / "r.nc"
    staticmaps.write_staticmaps(dom, p, reservoirs=res)
    assert (tmp_path / "reservoir_hq_2.csv").exists() and (tmp_path / "reservoir_sh_1.csv").exists()
    got, _, gres = staticmaps.load_staticmaps(p, reservoirs=True)
    order = np.argsort(res["river_index"])
    np.testing.assert_array_equal(gres["river_index"], res["river_index"][order])
    np.testing.assert_array_equal(gres["storage_curve_type"], res["storage_curve_type"][order])
    inv = np.argsort(order)
    lo = res["lower_reservoir"][order]
    np.testing.assert_array_equal(gres["lower_reservoir"], np.where(lo >= 0, inv[np.maximum(lo, 0)], -1))
    cfg = synthetic.make_config(86400.0)
    a = O.OracleModel(cfg, dom, reservoirs=res)
    b = O.OracleModel(cfg, got, reservoirs=gres)
    for s in range(6):
        P, PET, T = synthetic.forcing(s, cfg.dt, dom.n_land, seed=3)
        for m, r in ((a, res), (b, gres)):
            m.set_forcing(P * 3.0, PET, T)
            rp, re = synthetic.reservoir_forcing(dom, r, P * 3.0, PET)
            m.set(F["RESERVOIR_PRECIPITATION"], rp)
            m.set(F["RESERVOIR_EVAPORATION"], re)
            m.set_rating_curve_day(100 + s)
            m.step()
    for f in ("RESERVOIR_STORAGE", "RESERVOIR_WATERLEVEL", "RESERVOIR_OUTFLOW_AVERAGE"):
        np.testing.assert_allclose(b.get(F[f]), a.get(F[f])[order], rtol=1e-12, err_msg=f)
    np.testing.assert_allclose(b.outlets(0), a.outlets(0), rtol=1e-12)
