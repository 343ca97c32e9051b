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
import pytest

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


def _setup(seed, size=24):
    dom = synthetic.make_domain(size, 250.0, seed=seed)
    rng = np.random.default_rng(seed)
    n = dom.n_land
    slope = np.ascontiguousarray(dom.land["slope"] * 50.0)
    snow = rng.uniform(0.0, 20.0, n)
    snow[::7] = 0.0
    water = snow * rng.uniform(0.0, 0.1, n)
    return dom, slope, snow, water


def _order(ds):
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
    return np.asarray(order, np.int64)


@pytest.fixture(scope="module")
def snow_host_lib(tmp_path_factory):
    import shutil
    import subprocess
    from pathlib import Path
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    repo = Path(__file__).resolve().parent.parent
    out = tmp_path_factory.mktemp("snow_host") / "snow_host.so"
    subprocess.run([cxx, "-O2", "-ffp-contract=off", "-std=c++17", "-shared", "-fPIC",
                    "-I", str(repo / "wflow.jl_gb300" / "csrc"), str(repo / "tests" / "snow_host_driver.cpp"),
                    "-o", str(out)], check=True)
    return C.CDLL(str(out))


@pytest.mark.parametrize("seed", [3, 4])
def test_host_build_bit_identical(snow_host_lib, seed):
    """The product's per-cell arithmetic (snow_scheme.cuh) on its level schedule equals the
    oracle's sequential sweep bit for bit: states, snow_out and snow_in."""
    dom, slope, snow, water = _setup(seed)
    ds = np.ascontiguousarray(dom.land["land_downstream"], np.int32)
    order = _order(ds)
    n, dt = len(ds), 86400.0
    out_o, in_o, s_o, w_o = transport(dom, slope, snow, water, dt)
    s_h, w_h, out_h, in_h = np.array(snow), np.array(water), np.zeros(n), np.zeros(n)
    p = lambda a, t=C.c_double: a.ctypes.data_as(C.POINTER(t))  # noqa: E731
    snow_host_lib.host_snow_transport(C.c_int64(n), p(ds, C.c_int32), p(order, C.c_int64), p(ds, C.c_int32),
                                      p(slope), C.c_double(dt), p(s_h), p(w_h), p(out_h), p(in_h))
    for a, b in ((s_o, s_h), (w_o, w_h), (out_o, out_h), (in_o, in_h)):
        assert np.array_equal(a, b)


def test_create_rejects_bad_orders():
    from wflow_gb300 import build
    from wflow_gb300.snow_transport import SnowTransport
    build.build_all()
    dom, slope, _, _ = _setup(5, size=12)
    ds = np.ascontiguousarray(dom.land["land_downstream"], np.int32)
    order = _order(ds)
    with pytest.raises(RuntimeError, match="not a permutation"):
        SnowTransport(ds, np.concatenate([order[:-1], order[:1]]), slope)
    with pytest.raises(RuntimeError, match="after its downstream cell"):
        SnowTransport(ds, order[::-1].copy(), slope)
    bad = ds.copy()
    bad[0] = len(ds)
    with pytest.raises(RuntimeError, match="out of range"):
        SnowTransport(bad, order, slope)


def glacier_case(seed, n=5000):
    """Glacier inputs with the branches of glacier_hbv: no glacier, the snow-to-ice rate capped,
    temperatures below and above the melt threshold, snow above and below 10 mm."""
    rng = np.random.default_rng(seed)
    frac = rng.uniform(0.0, 1.0, n) * (rng.random(n) < 0.7)
    ttm = 273.15 + rng.uniform(-1.0, 1.0, n)
    cfmax = rng.uniform(2.0, 6.0, n) * 1e-3 / 86400.0
    sifrac = rng.uniform(0.0, 0.005, n) / 86400.0
    temp = 273.15 + rng.uniform(-10.0, 10.0, n)
    snow = rng.uniform(0.0, 0.5, n) * (rng.random(n) < 0.6)
    store = rng.uniform(0.0, 50.0, n)
    return frac, ttm, cfmax, sifrac, 8e-3 / 86400.0, temp, snow, store


def oracle_glacier(frac, ttm, cfmax, sifrac, max_rate, dt, temp, snow, store):
    out = np.empty(4)
    s, g, m = np.empty_like(snow), np.empty_like(store), np.empty_like(snow)
    for i in range(len(snow)):
        O.lib().orc_glacier_hbv(C.c_double(frac[i]), C.c_double(store[i]), C.c_double(snow[i]), C.c_double(temp[i]),
                                C.c_double(ttm[i]), C.c_double(cfmax[i]), C.c_double(sifrac[i]), C.c_double(max_rate),
                                C.c_double(dt), out.ctypes.data_as(C.POINTER(C.c_double)))
        s[i], g[i], m[i] = out[0], out[2], out[3]
    return s, g, m


def test_glacier_host_build_bit_identical(snow_host_lib):
    frac, ttm, cfmax, sifrac, max_rate, temp, snow, store = glacier_case(1)
    dt = 86400.0
    s_o, g_o, m_o = oracle_glacier(frac, ttm, cfmax, sifrac, max_rate, dt, temp, snow, store)
    s_h, g_h, m_h = snow.copy(), store.copy(), np.zeros_like(snow)
    p = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
    snow_host_lib.host_glacier(C.c_int64(len(snow)), p(frac), p(ttm), p(cfmax), p(sifrac), C.c_double(max_rate),
                               C.c_double(dt), p(temp), p(s_h), p(g_h), p(m_h))
    for a, b in ((s_o, s_h), (g_o, g_h), (m_o, m_h)):
        assert np.array_equal(a, b)
    assert (m_o > 0).any() and (m_o == 0).any() and (frac == 0).any()
