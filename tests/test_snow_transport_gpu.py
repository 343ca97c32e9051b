"""Lateral snow transport on the GPU (include/wflow_gb300_snow.h) against the oracle.

lateral_snow_transport! (Wflow/src/routing/surface/surface_process.jl:1-19): the snow storage
and snow water move downhill in place, limited by a slope- and storage-dependent capacity per
cell, in topological order (accucapacityflux!, routing/utils.jl:82-104). The GPU sweeps the
cells level by level, each cell adding its upstream hand-offs in the topological-sort order, so
states, snow_out and snow_in equal the oracle's to relative 1e-12 (the arithmetic is the same,
operation for operation).
"""

import numpy as np
import pytest

from test_snow_transport_cpu import _order, _setup, transport

pytestmark = pytest.mark.gpu


def _max_rel(a, b):
    return float(np.max(np.abs(a - b) / np.maximum(np.maximum(np.abs(a), np.abs(b)), 1e-300)))


@pytest.mark.parametrize("seed,size", [(3, 24), (8, 96)])
def test_snow_transport_matches_oracle(gpu_lib, seed, size):
    from wflow_gb300.snow_transport import SnowTransport
    dom, slope, snow, water = _setup(seed, size)
    ds = np.ascontiguousarray(dom.land["land_downstream"], np.int32)
    order = _order(ds)
    dt = 86400.0
    out_o, in_o, s_o, w_o = transport(dom, slope, snow, water, dt)
    t = SnowTransport(ds, order, slope)
    assert t.levels > 1
    s_g, w_g = np.array(snow), np.array(water)
    out_g, in_g = t.run(dt, s_g, w_g)
    for name, a, b in (("snow_storage", s_o, s_g), ("snow_water", w_o, w_g), ("snow_out", out_o, out_g),
                       ("snow_in", in_o, in_g)):
        assert _max_rel(a, b) <= 1e-12, name
    t.close()


def test_glacier_matches_oracle(gpu_lib):
    from test_snow_transport_cpu import glacier_case, oracle_glacier
    from wflow_gb300.snow_transport import Glacier
    frac, ttm, cfmax, sifrac, max_rate, temp, snow, store = glacier_case(2, n=20000)
    dt = 86400.0
    s_o, g_o, m_o = oracle_glacier(frac, ttm, cfmax, sifrac, max_rate, dt, temp, snow, store)
    g = Glacier(frac, ttm, cfmax, sifrac, max_rate)
    s_g, g_g = snow.copy(), store.copy()
    m_g = g.run(dt, temp, s_g, g_g)
    for name, a, b in (("snow_storage", s_o, s_g), ("glacier_store", g_o, g_g), ("glacier_melt", m_o, m_g)):
        assert _max_rel(a, b) <= 1e-12, name
    g.close()
