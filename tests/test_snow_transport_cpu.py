"""Lateral snow transport in the oracle (routing/surface/surface_process.jl:1-19).

The transport rests on accucapacityflux!, pinned exactly by the reference's accucapacity unit
test (test_oracle_kats.py). Here, on a synthetic drainage graph: every cell passes on at most
its capacity (a slope- and storage-dependent fraction of its snow per second), the transported
snow is conserved (what leaves all cells either enters a cell downstream or leaves through a
pit), flat or snow-free cells pass nothing on, and the snow storage and snow water move in
place (accucapacityflux hands its material to accucapacityflux!, routing/utils.jl:144-148): the
domain's snow falls by exactly what left through the pits.
"""

import ctypes as C

import numpy as np

from wflow_gb300 import synthetic
import oracle_py as O


def transport(dom, slope, snow, water, dt):
    ds = np.ascontiguousarray(dom.land["land_downstream"], np.int32)
    n = len(ds)
    indeg = np.zeros(n, np.int64)
    np.add.at(indeg, ds[ds >= 0], 1)
    order = list(np.flatnonzero(indeg == 0))
    k = 0
    while k < len(order):
        d = ds[order[k]]
        if d >= 0:
            indeg[d] -= 1
            if indeg[d] == 0:
                order.append(d)
        k += 1
    order = np.asarray(order, np.int64)
    out, inn = np.zeros(n), np.zeros(n)
    p = lambda a, t=C.c_double: a.ctypes.data_as(C.POINTER(t))  # noqa: E731
    snow_after, water_after = np.array(snow, float), np.array(water, float)
    O.lib().orc_lateral_snow_transport(p(ds, C.c_int32), p(ds, C.c_int32), p(order, C.c_int64), C.c_int64(n),
                                       C.c_double(dt), p(slope), p(snow_after), p(water_after), p(out), p(inn))
    return out, inn, snow_after, water_after


def test_snow_transport_conserves_and_respects_capacity():
    dom = synthetic.make_domain(24, 250.0, seed=6)
    rng = np.random.default_rng(1)
    n = dom.n_land
    slope = np.ascontiguousarray(dom.land["slope"] * 50.0)  # steep enough for transport
    snow = rng.uniform(0.0, 20.0, n)
    snow[::7] = 0.0
    water = snow * rng.uniform(0.0, 0.1, n)
    dt = 86400.0
    out, inn, snow_after, water_after = transport(dom, slope, snow, water, dt)
    frac = np.minimum(0.5, slope / 5.67) * np.minimum(1.0, snow / 10.0)
    assert np.all(out >= 0.0)
    # a cell passes on at most its capacity plus what it received (the sweep runs downstream)
    assert np.all(out <= frac * (snow + water) / dt + inn + 1e-18)
    ds = dom.land["land_downstream"]
    pits = ds < 0
    assert abs((out.sum() - inn.sum()) - out[pits].sum()) <= 1e-12 * out.sum()
    # snow-free cells with nothing from upstream pass nothing on
    quiet = (snow == 0.0) & (inn == 0.0)
    assert np.all(out[quiet] == 0.0)
    # the states move: the domain loses what leaves through the pits, no cell goes negative
    assert np.all(snow_after >= 0.0) and np.all(water_after >= 0.0)
    lost = (snow.sum() + water.sum()) - (snow_after.sum() + water_after.sum())
    assert abs(lost - out[pits].sum() * dt) <= 1e-9 * (snow.sum() + water.sum())
    assert not np.array_equal(snow_after, snow)
