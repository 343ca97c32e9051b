"""Gravitational snow transport and the HBV glacier in the oracle's model step, and the C ABI's
checks of their options (CPU).

The oracle's step runs them where Wflow does (sbm.jl:95-102) and keeps the land balance closed
with snow_in / snow_out and the glacier storage in it (mass_balance.jl:96-113, 236-244). The
transport hands material on in the order of Graphs.jl's topological_sort_by_dfs of the land graph
(Wflow's network.order); the order is checked here against that definition on small graphs.
"""

import ctypes as C

import numpy as np
import pytest

from wflow_gb300 import abi, build, synthetic
import oracle_py as O

F = abi.FIELD


def dfs_order(ds):
    """topological_sort_by_dfs of a graph of out-degree <= 1, written from its definition: a
    depth-first search from every unvisited vertex in index order, vertices appended when they
    finish, the result reversed."""
    n = len(ds)
    color = [0] * n
    finished = []

    def visit(v):
        color[v] = 1
        w = ds[v]
        if w >= 0 and color[w] == 0:
            visit(w)
        color[v] = 2
        finished.append(v)

    for v in range(n):
        if color[v] == 0:
            visit(v)
    return finished[::-1]


def cold_run(dom, cfg, params, steps=60, seed=41):
    o = O.OracleModel(cfg, dom, params=params)
    for s in range(steps):
        P, PET, T = synthetic.forcing(230 + s, cfg.dt, dom.n_land, seed=seed)
        o.set_forcing(P, PET, T - 2.0)
        o.step()
    return o


def glacier_params(dom):
    rng = np.random.default_rng(3)
    n = dom.n_land
    p = dict(dom.params)
    p.update(glacier_fraction=np.where(rng.random(n) < 0.3, rng.uniform(0.05, 0.6, n), 0.0),
             glacier_temperature_threshold_melt=np.full(n, 273.15),
             glacier_degree_day_factor=np.full(n, 3e-3 / 86400.0),
             glacier_snow_to_ice_fraction=np.full(n, 0.002 / 86400.0),
             glacier_initial_store=rng.uniform(0.5, 6.0, n))
    return p


@pytest.fixture(scope="module")
def dom():
    return synthetic.make_domain(24, 1000.0, seed=41)


def test_balance_closes_with_transport_and_glacier(dom):
    cfg = synthetic.make_config(86400.0)
    cfg.snow_gravitational_transport = 1
    cfg.glacier = 1
    o = cold_run(dom, cfg, glacier_params(dom))
    assert np.abs(o.get(F["BALANCE_LAND_RELATIVE_ERROR"])).max() < 1e-9
    snow_out, snow_in = o.get(F["SNOW_OUT"]), o.get(F["SNOW_IN"])
    assert snow_out.max() > 0.0
    # what leaves the cells arrives downstream, except at the pits
    ds = dom.land["land_downstream"]
    assert abs(snow_in.sum() - snow_out[ds >= 0].sum()) <= 1e-12 * snow_out.sum()
    assert o.get(F["GLACIER_MELT"]).max() > 0.0


def test_options_change_the_result_only_when_on(dom):
    base = cold_run(dom, synthetic.make_config(86400.0), dom.params, steps=30)
    cfg = synthetic.make_config(86400.0)
    cfg.glacier = 1
    p = dict(dom.params, glacier_fraction=np.zeros(dom.n_land))
    zero_fraction = cold_run(dom, cfg, p, steps=30)
    # a glacier flag without glacier area leaves the land states as they were
    for f in ["SNOW_STORAGE", "SATURATED_WATER_DEPTH", "LAND_Q"]:
        assert np.array_equal(base.get(F[f]), zero_fraction.get(F[f])), f
    cfg.snow_gravitational_transport = 1
    moved = cold_run(dom, cfg, p, steps=30)
    assert not np.array_equal(base.get(F["SNOW_STORAGE"]), moved.get(F["SNOW_STORAGE"]))


def test_topological_order_definition():
    rng = np.random.default_rng(5)
    for n in (1, 7, 40):
        # a random forest: each vertex drains to a higher-numbered one or is a pit
        ds = np.array([rng.integers(v + 1, n) if v + 1 < n and rng.random() < 0.8 else -1 for v in range(n)])
        perm = rng.permutation(n)
        inv = np.argsort(perm)
        ds_p = np.array([inv[ds[perm[i]]] if ds[perm[i]] >= 0 else -1 for i in range(n)], np.int32)
        order = dfs_order(list(ds_p))
        pos = {v: k for k, v in enumerate(order)}
        assert sorted(order) == list(range(n))
        assert all(pos[v] < pos[ds_p[v]] for v in range(n) if ds_p[v] >= 0)
        # the oracle's order (the one its snow transport and the GPU's hand-off order follow)
        out = np.empty(n, np.int64)
        assert O.lib().orc_topo_order_dfs(n, ds_p.ctypes.data_as(C.POINTER(C.c_int32)),
                                          out.ctypes.data_as(C.POINTER(C.c_int64))) == 0
        assert list(out) == order
    cyc = np.array([1, 0], np.int32)
    assert O.lib().orc_topo_order_dfs(2, cyc.ctypes.data_as(C.POINTER(C.c_int32)),
                                      np.empty(2, np.int64).ctypes.data_as(C.POINTER(C.c_int64))) == abi.WF_ERR_CYCLE


def _create(dom, cfg, res=None):
    lib = abi.load_library()
    d, p = synthetic.c_structs(dom)
    h = C.c_void_p()
    if res is None:
        st = lib.wf_create(C.byref(cfg), C.byref(d), C.byref(p), 0, C.byref(h))
    else:
        r = synthetic.c_reservoirs(res)
        st = lib.wf_create_with_reservoirs(C.byref(cfg), C.byref(d), C.byref(p), C.byref(r), 0, C.byref(h))
    msg = lib.wf_last_error(None)
    return st, (msg.decode() if msg else "")


def test_abi_rejects_glacier_or_transport_without_snow(dom):
    build.build_all()
    for flag in ("glacier", "snow_gravitational_transport"):
        cfg = synthetic.make_config(86400.0, snow=False)
        setattr(cfg, flag, 1)
        st, msg = _create(dom, cfg)
        assert st == abi.WF_ERR_INVALID and "snow" in msg, (st, msg)
        with pytest.raises(RuntimeError):
            O.OracleModel(cfg, dom)


def test_abi_rejects_transport_with_reservoirs():
    build.build_all()
    d = synthetic.make_domain(48, 1000.0, seed=3)
    res = synthetic.make_reservoirs(d, 2, seed=3)
    cfg = synthetic.make_config(86400.0)
    cfg.snow_gravitational_transport = 1
    st, msg = _create(d, cfg, res)
    assert st == abi.WF_ERR_UNSUPPORTED and "reservoirs" in msg, (st, msg)
    with pytest.raises(RuntimeError):
        O.OracleModel(cfg, d, reservoirs=res)
