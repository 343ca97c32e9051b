"""Wflow forcing files (wflow_gb300.forcing) on the CPU.

The record of a step is the first at or after the model time (backward fill, io.jl:9-22);
precipitation and potential evaporation are in mm per model step and temperature in degC in
the file (standard_name_sbm.jl), converted as to_SI does; over a reservoir's area the forcing
becomes the reservoir's input and is zeroed on the land (io.jl:128-137).
"""

import datetime as dt

import numpy as np
import pytest

from wflow_gb300 import abi, forcing, states, synthetic
import oracle_py as O

netcdf = pytest.importorskip("scipy.io").netcdf_file
F = abi.FIELD
T0 = dt.datetime(2000, 1, 1)


def test_forcing_file_drives_the_model_like_the_arrays(tmp_path):
    dom = synthetic.make_domain(16, 1000.0, seed=3)
    grid = states.Grid.of_domain(dom)
    step = 86400.0
    steps = 5
    arrs = [synthetic.forcing(s, step, dom.n_land, seed=1) for s in range(steps)]
    times = [T0 + dt.timedelta(seconds=step * (k + 1)) for k in range(steps)]  # right-labelled
    path = tmp_path / "inmaps.nc"
    forcing.write_forcing(path, grid, times, [a[0] for a in arrs], [a[1] for a in arrs], [a[2] for a in arrs], step)
    ff = forcing.ForcingFile(path, grid, step, mapping={forcing.PRECIP: "precip", forcing.PET: "pet",
                                                          forcing.TEMP: "temp"})
    cfg = synthetic.make_config(step)
    a, b = O.OracleModel(cfg, dom), O.OracleModel(cfg, dom)
    for k in range(steps):
        P, PET, T = ff.at(T0 + dt.timedelta(seconds=step * (k + 1)))
        for x, y in zip((P, PET, T), arrs[k]):
            np.testing.assert_allclose(x, y, rtol=4e-16, atol=0)
        a.set_forcing(*arrs[k])
        a.step()
        b.set_forcing(P, PET, T)
        b.step()
    for f in ("RIVER_Q", "SATURATED_WATER_DEPTH", "SNOW_STORAGE"):
        x, y = a.get(F[f]), b.get(F[f])
        assert np.max(np.abs(x - y) / np.maximum(np.abs(x), 1e-300)) <= 1e-12, f


def test_backward_fill_and_time_units(tmp_path):
    p = tmp_path / "f.nc"
    f = netcdf(str(p), "w", version=2)
    f.createDimension("time", None)
    f.createDimension("lon", 2)
    f.createDimension("lat", 2)
    f.createVariable("lon", "d", ("lon",))[:] = [5.0, 5.1]
    f.createVariable("lat", "d", ("lat",))[:] = [51.1, 51.0]  # north-up: decreasing
    t = f.createVariable("time", "d", ("time",))
    t.units = "hours since 2001-03-01 06:00:00"
    t[:] = [0.0, 6.0, 12.0]
    for name, base in (("P", 1.0), ("E", 2.0), ("Tair", 10.0)):
        v = f.createVariable(name, "d", ("time", "lat", "lon"))
        v[:] = base + np.arange(12, dtype=float).reshape(3, 2, 2)
    f.close()
    grid = states.Grid(2, 2, [0, 1, 0, 1], [0, 0, 1, 1])
    mapping = {forcing.PRECIP: "P", forcing.PET: "E", forcing.TEMP: {"name": "Tair", "scale": 2.0, "offset": -1.0}}
    ff = forcing.ForcingFile(p, grid, 6 * 3600.0, mapping=mapping)
    base = dt.datetime(2001, 3, 1, 6)
    assert ff.index(base) == 0
    assert ff.index(base + dt.timedelta(hours=1)) == 1   # between records: the next one
    assert ff.index(base + dt.timedelta(hours=12)) == 2
    with pytest.raises(ValueError, match="before"):
        ff.index(base - dt.timedelta(hours=1))
    with pytest.raises(ValueError, match="after"):
        ff.index(base + dt.timedelta(hours=13))
    P, PET, T = ff.at(base + dt.timedelta(hours=6))
    raw = 1.0 + np.arange(12, dtype=float).reshape(3, 2, 2)[1]
    std = raw[::-1]  # latitude increasing
    np.testing.assert_array_equal(P, std.reshape(-1) * (1e-3 * (1.0 / (6 * 3600.0))))
    traw = (10.0 + np.arange(12, dtype=float).reshape(3, 2, 2)[1])[::-1].reshape(-1)
    np.testing.assert_array_equal(T, traw * 2.0 - 1.0 + 273.15)


def test_reservoir_areas_take_the_forcing(tmp_path):
    dom = synthetic.make_domain(10, 1000.0, seed=3)
    grid = states.Grid.of_domain(dom)
    step = 86400.0
    arr = synthetic.forcing(0, step, dom.n_land, seed=1, precip_scale=3.0)
    path = tmp_path / "r.nc"
    forcing.write_forcing(path, grid, [T0 + dt.timedelta(days=1)], [arr[0]], [arr[1]], [arr[2]], step)
    cov = [np.array([0, 1, 10]), np.array([55])]  # grid cells of two reservoirs' areas
    res = {"coverage_cells": cov}
    ff = forcing.ForcingFile(path, grid, step, mapping={forcing.PRECIP: "precip", forcing.PET: "pet",
                                                          forcing.TEMP: "temp"}, reservoirs=res)
    P, PET, T, rp, re = ff.at(T0 + dt.timedelta(days=1))
    np.testing.assert_allclose(rp, [np.mean(arr[0][c]) for c in cov], rtol=1e-15)
    np.testing.assert_allclose(re, [np.mean(arr[1][c]) for c in cov], rtol=1e-15)
    for c in cov:
        assert np.all(P[c] == 0.0) and np.all(PET[c] == 0.0)
    np.testing.assert_allclose(T, arr[2], rtol=1e-15)  # temperature is not moved
