"""Wflow state files (wflow_gb300.states) on the CPU, with the oracle's model.

A warm start from a state file written by `write_states` continues like the run that wrote it
(the reference's restart path: set_states!, Wflow/src/utils.jl:150-213 and
sbm_model.jl:104-193); the file has Wflow's layout (standard names, file units, dimensions
(time[, layer], y, x) in C order, NaN outside the active cells, a layer coordinate) as read by
scipy; a state file whose grid axes are stored in another order is read by dimension names.
"""

import numpy as np
import pytest

from wflow_gb300 import abi, states, synthetic
import oracle_py as O

netcdf = pytest.importorskip("scipy.io").netcdf_file
F = abi.FIELD


def forcing(dom, s, dt):
    return synthetic.forcing(s, dt, dom.n_land, seed=1, precip_scale=3.0)


def step(m, dom, s, dt, res=None):
    P, PET, T = forcing(dom, s, dt)
    if res is not None:
        rp, re = synthetic.reservoir_forcing(dom, res, P, PET)
        m.set(F["RESERVOIR_PRECIPITATION"], rp)
        m.set(F["RESERVOIR_EVAPORATION"], re)
    m.set_forcing(P, PET, T)
    m.step()


FIELDS = ["RIVER_Q", "RIVER_Q_AVERAGE", "LAND_Q", "SSF_Q", "SATURATED_WATER_DEPTH", "CANOPY_STORAGE",
          "SNOW_STORAGE", "TOTAL_STORAGE", "BALANCE_LAND_ERROR", "BALANCE_RIVER_ERROR"]


@pytest.mark.parametrize("with_reservoirs", [False, True, "tables"])
def test_warm_start_continues_the_run(tmp_path, with_reservoirs):
    # "tables": interpolated S-H profiles, a rating curve and a linked pair; the storage read
    # back is the S-H table at the stored level (initialize_storage), which inverts the level the
    # run reached from its storage to within rounding
    dom = synthetic.make_domain(24, 1000.0, seed=5)
    if with_reservoirs == "tables":
        dom = synthetic.make_domain(48, 1000.0, seed=3)
        res = synthetic.make_linked_reservoirs(dom, seed=3)
    else:
        res = synthetic.make_reservoirs(dom, 2, seed=2) if with_reservoirs else None
    cfg = synthetic.make_config(86400.0)
    a = O.OracleModel(cfg, dom, reservoirs=res)
    for s in range(6):
        step(a, dom, s, cfg.dt, res)
    path = tmp_path / "outstates.nc"
    states.write_states(a, dom, path, reservoirs=res)
    b = O.OracleModel(cfg, dom, reservoirs=res)
    states.read_states(b, dom, path, reservoirs=res)
    worst = 0.0
    for s in range(6, 10):
        step(a, dom, s, cfg.dt, res)
        step(b, dom, s, cfg.dt, res)
        for f in FIELDS + (["RESERVOIR_STORAGE", "RESERVOIR_OUTFLOW_AVERAGE"] if res is not None else []):
            x, y = a.get(F[f]), b.get(F[f])
            scale = np.maximum(np.abs(x), 1e-300) if "BALANCE" not in f else np.max(np.abs(a.get(F["RIVER_Q"]))) + 1
            worst = max(worst, float(np.max(np.abs(x - y) / scale)))
    # the file stores depths in mm: x / 1e-3 * 1e-3 may move a state by an ulp, nothing more
    assert worst <= 1e-10, worst


def test_state_file_layout(tmp_path):
    dom = synthetic.make_domain(12, 500.0, seed=9, ny=10)
    cfg = synthetic.make_config(3600.0)
    m = O.OracleModel(cfg, dom)
    for s in range(3):
        step(m, dom, s, cfg.dt)
    path = tmp_path / "s.nc"
    states.write_states(m, dom, path, time=3.0 / 24.0)
    N = cfg.n_soil_layer_thickness + 1
    with netcdf(str(path), "r", mmap=False) as f:
        assert set(states.required_states(cfg)) <= set(f.variables)
        sat = f.variables["soil_water_saturated_zone__depth"]
        assert sat.dimensions == ("time", "y", "x") and sat.units == b"mm"
        ust = f.variables["soil_layer_water_unsaturated_zone__depth"]
        assert ust.dimensions == ("time", "layer", "y", "x")
        assert np.array_equal(f.variables["layer"][:], np.arange(1, N + 1))
        assert f.variables["layer"].axis == b"Z"
        assert f.variables["time"][0] == 3.0 / 24.0
        # values in file units on the grid (land index = row * nx + column)
        grid_sat = sat[0].copy()
        assert grid_sat.shape == (10, 12)
        np.testing.assert_array_equal(grid_sat.reshape(-1), m.get(F["SATURATED_WATER_DEPTH"]) / 1e-3)
        ssf = f.variables["subsurface_water__instantaneous_volume_flow_rate"]
        assert ssf.units == b"m3 d-1"
        np.testing.assert_array_equal(ssf[0].reshape(-1), m.get(F["SSF_Q"]) / (1.0 / 86400.0))
        tsoil = f.variables["soil_surface__temperature"][0].reshape(-1)
        np.testing.assert_array_equal(tsoil, m.get(F["SOIL_SURFACE_TEMPERATURE"]) - 273.15)
        # river states only on river cells, NaN (the fill value) elsewhere
        rq = f.variables["river_water__instantaneous_volume_flow_rate"][0].reshape(-1)
        rl = dom.river["river_land_index"]
        assert np.array_equal(rq[rl], m.get(F["RIVER_Q"]))
        off = np.ones(dom.n_land, bool)
        off[rl] = False
        assert np.isnan(rq[off]).all()


def test_reads_states_stored_in_another_axis_order(tmp_path):
    # a state file whose grid is stored as (x, y) rows, written by another tool
    dom = synthetic.make_domain(8, 1000.0, seed=4, ny=6)
    cfg = synthetic.make_config(86400.0, snow=False)
    src = O.OracleModel(cfg, dom)
    for s in range(2):
        step(src, dom, s, cfg.dt)
    path = tmp_path / "t.nc"
    N = cfg.n_soil_layer_thickness + 1
    grid = states.Grid.of_domain(dom)
    f = netcdf(str(path), "w", version=2)
    f.createDimension("time", None)
    f.createDimension("x", dom.nx)
    f.createDimension("y", dom.ny)
    f.createDimension("layer", N)
    acc = states._Access(src)
    for sn in states.required_states(cfg):
        field, layered, unit, part = states.STATES[sn]
        cells = states._cells(dom, part, None)
        dims = ("time", "x", "y", "layer") if layered else ("time", "x", "y")
        v = f.createVariable(sn, "d", dims)
        v._FillValue = np.nan
        arr = np.full((1, dom.nx, dom.ny) + ((N,) if layered else ()), np.nan)
        for k in range(N if layered else 1):
            val = states.from_si(acc.get(field, layer=k), unit)
            if layered:
                arr[0, grid.col[cells], grid.row[cells], k] = val
            else:
                arr[0, grid.col[cells], grid.row[cells]] = val
        v[:] = arr
    f.close()
    dst = O.OracleModel(cfg, dom)
    states.read_states(dst, dom, path)
    for fld in ["SATURATED_WATER_DEPTH", "SSF_Q", "LAND_Q", "RIVER_Q", "RIVER_H", "CANOPY_STORAGE"]:
        np.testing.assert_allclose(dst.get(F[fld]), src.get(F[fld]), rtol=1e-15, atol=0)
    for k in range(N):
        np.testing.assert_allclose(dst.get(F["UNSATURATED_LAYER_DEPTH"], k), src.get(F["UNSATURATED_LAYER_DEPTH"], k),
                                   rtol=1e-15, atol=0)


def test_missing_state_is_an_error(tmp_path):
    dom = synthetic.make_domain(6, 1000.0, seed=4)
    cfg = synthetic.make_config(86400.0)
    m = O.OracleModel(cfg, dom)
    path = tmp_path / "m.nc"
    names = [n for n in states.required_states(cfg) if n != "river_water__depth"]
    states.write_states(m, dom, path, names=names)
    with pytest.raises(KeyError, match="river_water__depth"):
        states.read_states(O.OracleModel(cfg, dom), dom, path)
