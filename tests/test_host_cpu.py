"""Host-side checks that need no GPU: the C ABI library loads and exports what the header
declares, struct layouts agree with the ctypes mirror, the wavefront planner's invariants hold
on drainage forests of every shape, and the synthetic domains are valid D8 forests."""

import ctypes as C

import numpy as np
import pytest

from wflow_gb300 import abi, build, synthetic


@pytest.fixture(scope="module")
def lib():
    build.build_all()
    return abi.load_library()


@pytest.mark.parametrize("header,must", [("wflow_gb300.h", ("wf_create", "wf_step")),
                                          ("wflow_gb300_nc.h", ("wf_nc_open", "wf_nc_get")),
                                          ("wflow_gb300_li.h", ("wf_li_river_create", "wf_li_river_step")),
                                          ("wflow_gb300_snow.h", ("wf_snow_transport_create", "wf_snow_transport_run", "wf_glacier_run"))])
def test_header_symbols_exported(lib, header, must):
    names = abi.header_symbols(header)
    assert all(m in names for m in must)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_synth_header_symbols_exported():
    s = abi.load_synth()
    text = (abi.REPO_ROOT / "include" / "wflow_gb300_synth.h").read_text()
    assert "wf_synth_dem_d8" in text
    assert hasattr(s, "wf_synth_dem_d8")


def test_struct_sizes_match(lib):
    for i, cls in enumerate([abi.WfConfig, abi.WfDomain, abi.WfParams, abi.WfMetrics, abi.WfTuning,
                             abi.WfReservoirs, abi.WfReservoirTables]):
        assert lib.wf_struct_size(i) == C.sizeof(cls), cls.__name__


def _plan(lib, ds, members):
    ds = np.ascontiguousarray(ds, np.int32)
    counts = np.zeros(4, np.int64)
    slot = np.zeros(max(1, len(ds)), np.int64)
    ok = C.c_int32()
    g = C.c_int32()
    st = lib.wf_plan_routing(len(ds), ds.ctypes.data_as(C.POINTER(C.c_int32)), members,
                             counts.ctypes.data_as(C.POINTER(C.c_int64)), slot.ctypes.data_as(C.POINTER(C.c_int64)),
                             C.byref(ok), C.byref(g))
    return st, counts, slot[: len(ds)], ok.value, g.value


def _random_forest(n, rng, n_roots=1):
    ds = np.full(n, -1, np.int32)
    for i in range(n_roots, n):
        ds[i] = rng.integers(0, i)
    perm = rng.permutation(n)
    inv = np.empty(n, np.int64)
    inv[perm] = np.arange(n)
    out = np.full(n, -1, np.int32)
    out[inv] = np.where(ds >= 0, inv[np.maximum(ds, 0)], -1)
    return out


def _long_forest(rng, trunk, n_side):
    """A trunk path with side chains of random length (up to the trunk's) joining it: long
    chains, which the plan gives a chunk of their own."""
    ds = [i + 1 for i in range(trunk - 1)] + [-1]
    for _ in range(n_side):
        length = int(rng.integers(1, trunk))
        join = int(rng.integers(length, trunk))  # a chain of this length joins at height >= length
        start = len(ds)
        ds += [start + i + 1 for i in range(length - 1)] + [join]
    return np.array(ds, np.int32)


@pytest.mark.parametrize("members", [1, 2, 8, 32, 64])
def test_plan_invariants(lib, members):
    rng = np.random.default_rng(members)
    cases = [np.array([-1]), np.array([1, 2, -1]), np.array([2, 2, -1]), np.array([-1, -1, -1]),
             np.array([1, 2, 3, -1, 3, 4])]
    cases += [_random_forest(n, rng, r) for n, r in [(50, 1), (500, 3), (3000, 1)]]
    cases += [_long_forest(rng, 400, 60), _long_forest(rng, 150, 300)]
    for ds in cases:
        st, counts, slot, ok, G = _plan(lib, ds, members)
        assert st == 0
        assert ok == 1, ds
        assert G == max(1, 32 // members)
        n_chains, n_chunks, n_slots, max_len = counts
        assert n_slots >= len(ds)
        assert len(set(slot.tolist())) == len(ds)
        assert n_chunks <= n_chains


def test_plan_rejects_cycles(lib):
    st, *_ = _plan(lib, np.array([1, 0], np.int32), 1)
    assert st == abi.WF_ERR_CYCLE
    st, *_ = _plan(lib, np.array([0], np.int32), 1)
    assert st == abi.WF_ERR_CYCLE
    st, *_ = _plan(lib, np.array([5], np.int32), 1)
    assert st != 0


def test_plan_real_domain_height(lib):
    dom = synthetic.make_domain(64, 1000.0, seed=3)
    st, counts, slot, ok, G = _plan(lib, dom.land["land_downstream"], 1)
    assert st == 0 and ok == 1
    # chain length of the longest chain = height of the outlet + 1
    ds = dom.land["land_downstream"]
    order = np.argsort(-dom.land["elevation"], kind="stable")
    h = np.zeros(len(ds), np.int64)
    for v in order:
        if ds[v] >= 0:
            h[ds[v]] = max(h[ds[v]], h[v] + 1)
    assert counts[3] == h.max() + 1


def test_synthetic_domain_is_valid_d8():
    dom = synthetic.make_domain(48, 250.0, seed=5)
    ds = dom.land["land_downstream"]
    assert (ds == -1).sum() == 1 and ds[0] == -1  # one corner outlet
    z = dom.land["elevation"]
    assert np.all(z[ds[ds >= 0]] < z[ds >= 0] + 1e-9)
    assert np.all(dom.land["slope"] >= 1e-4)
    assert dom.n_river > 0
    rds = dom.river["river_downstream"]
    assert (rds == -1).sum() == 1
    assert np.all(dom.land["river_fraction"] <= 1.0)
    # identical on a second call (seeded)
    dom2 = synthetic.make_domain(48, 250.0, seed=5)
    assert np.array_equal(dom.land["elevation"], dom2.land["elevation"])


def test_forcing_distribution():
    P, PET, T = synthetic.forcing(10, 86400.0, 20000, seed=2)
    dry = (P == 0).mean()
    assert 0.37 < dry < 0.43
    mm_day = P * 86400.0 * 1000.0
    assert abs(mm_day[mm_day > 0].mean() - 4.0) < 0.3   # gamma(0.4, 10) mean
    assert np.all(T > 250) and np.all(PET >= 0)


@pytest.mark.parametrize("members", [1, 64])
def test_heavy_hints_keep_a_path_on_one_chain(lib, members):
    # the planner's hints for linked reservoirs: the river path from an upper node to a lower one
    # lies on one chain (one lane walks both in order), and the plan's invariants still hold
    rng = np.random.default_rng(7)
    for trial in range(20):
        n = int(rng.integers(20, 400))
        ds = _random_forest(n, rng, n_roots=int(rng.integers(1, 4)))
        # a path: start at a leaf-ish node, go down a few links
        u = int(rng.integers(0, n))
        path = [u]
        while ds[path[-1]] >= 0 and len(path) < 12:
            path.append(int(ds[path[-1]]))
        hint = np.full(n, -1, np.int64)
        for a, b in zip(path[:-1], path[1:]):
            hint[b] = a
        counts = np.zeros(4, np.int64)
        chain = np.zeros(n, np.int64)
        ok, g = C.c_int32(), C.c_int32()
        st = lib.wf_plan_routing_hinted(n, ds.ctypes.data_as(C.POINTER(C.c_int32)), members,
                                        hint.ctypes.data_as(C.POINTER(C.c_int64)),
                                        counts.ctypes.data_as(C.POINTER(C.c_int64)),
                                        chain.ctypes.data_as(C.POINTER(C.c_int64)), C.byref(ok), C.byref(g))
        assert st == 0 and ok.value == 1, (trial, st, ok.value)
        assert len(set(chain[path].tolist())) == 1, (trial, path, chain[path])
    # a hint that is not a child of its node is refused
    ds = np.array([1, 2, -1, 2], np.int32)
    bad = np.array([-1, -1, 0, -1], np.int64)  # node 0 drains into 1, not into 2
    counts = np.zeros(4, np.int64)
    ok, g = C.c_int32(), C.c_int32()
    st = lib.wf_plan_routing_hinted(4, ds.ctypes.data_as(C.POINTER(C.c_int32)), members,
                                    bad.ctypes.data_as(C.POINTER(C.c_int64)),
                                    counts.ctypes.data_as(C.POINTER(C.c_int64)), None, C.byref(ok), C.byref(g))
    assert st != 0
