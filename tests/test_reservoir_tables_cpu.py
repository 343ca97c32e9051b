"""Reservoir tables and links in the oracle, and the C ABI's checks of them (CPU).

The S-H storage profile, the H-Q rating curve and the free weir linked to a lower reservoir
(Wflow/src/routing/surface/reservoir.jl:306-375, 455-521) are restated here in Python from the
reference's definitions, independently of the oracle's C++, and the two are compared on
synthetic tables. The reference's own tests of these options (test/reservoir.jl:223-345) read
CSV tables that the checkout does not hold, so no known answers pin them; the outflow functions
the tables feed are pinned by the reservoir.jl known-answer tests (test_oracle_kats.py).
"""

import ctypes as C

import numpy as np
import pytest

from wflow_gb300 import abi, build, synthetic
import oracle_py as O

F = abi.FIELD


def interp_ref(x, xp, fp):
    """interpolate_linear (reservoir.jl:363-375), statement for statement."""
    if x <= min(xp):
        return min(fp)
    if x >= max(xp):
        return max(fp)
    i1 = max(i for i in range(len(xp)) if xp[i] <= x)
    i2 = i1 + 1
    return fp[i1] * (1.0 - (x - xp[i1]) / (xp[i2] - xp[i1])) + fp[i2] * (x - xp[i1]) / (xp[i2] - xp[i1])


def test_interpolate_linear_matches_the_definition():
    rng = np.random.default_rng(4)
    for n in (1, 2, 5, 17):
        xp = np.cumsum(rng.uniform(0.1, 2.0, n)) + 100.0
        fp = rng.uniform(-5.0, 50.0, n)  # not monotonic: the bounds are the column's extremes
        xs = np.concatenate([xp, xp - 1e-9, xp + 1e-9, rng.uniform(xp[0] - 3, xp[-1] + 3, 40)])
        for x in xs:
            assert O.interpolate_linear(float(x), xp, fp) == interp_ref(float(x), list(xp), list(fp)), (n, x)


def _linked_pair():
    """Two reservoirs: an upper free weir linked to a lower reservoir released by a rating curve,
    both with S-H tables; ctypes records plus the tables they point into."""
    h1 = np.array([390.0, 392.0, 394.0, 395.0, 396.0, 398.0])
    s1 = np.array([0.0, 2.0e8, 6.0e8, 9.0e8, 1.25e9, 2.0e9])
    h2 = np.array([391.0, 393.0, 394.5, 395.5, 397.0])
    s2 = np.array([0.0, 5.0e7, 1.4e8, 2.2e8, 3.8e8])
    hq_h = np.array([393.0, 394.0, 395.0, 396.0, 397.5])
    day = np.arange(365)
    hq_q = np.outer(np.array([0.0, 40.0, 180.0, 420.0, 900.0]), 1.0 + 0.25 * np.sin(2 * np.pi * day / 365.0))
    keep = [h1, s1, h2, s2, hq_h, np.ascontiguousarray(hq_q)]
    pd = C.POINTER(C.c_double)
    up = O.Reservoir(outflow_type=2, area=4.7e8, threshold=393.7, rating_curve_coefficient=140.0,
                     rating_curve_exponent=1.5, precipitation=1.1574074074074074e-7,
                     evaporation=2.3148148148148148e-8, storage_curve_type=2, lower=2, sh_n=len(h1),
                     sh_h=h1.ctypes.data_as(pd), sh_s=s1.ctypes.data_as(pd))
    lo = O.Reservoir(outflow_type=1, area=6.1e7, precipitation=1.1574074074074074e-7,
                     evaporation=2.3148148148148148e-8, storage_curve_type=2, sh_n=len(h2),
                     sh_h=h2.ctypes.data_as(pd), sh_s=s2.ctypes.data_as(pd), hq_n=len(hq_h),
                     hq_h=hq_h.ctypes.data_as(pd), hq_q=keep[-1].ctypes.data_as(pd), hq_day=15)
    lo.maximum_storage = interp_ref(hq_h.max(), list(h2), list(s2))  # get_maximum_storage
    return up, lo, (h1, s1, h2, s2, hq_h, keep[-1]), keep


def _update_ref(st, i, inflow, dt, tables):
    """update_reservoir_model! (reservoir.jl:583-628) with the rating curve (:455-479) and the
    linked free weir (:482-521), on a list of dicts (0-based `lower`, -1 none)."""
    h1, s1, h2, s2, hq_h, hq_q = tables
    sh = {0: (h1, s1), 1: (h2, s2)}
    r = st[i]
    precipitation = r["precipitation"] * r["area"]
    available = r["storage"] + (inflow + precipitation) * dt
    evaporation = min(available / dt, r["evaporation"] * r["area"])
    if r["type"] == 1:
        storage_input = r["storage"] / dt + precipitation - evaporation + inflow
        outflow = interp_ref(r["waterlevel"], list(hq_h), list(hq_q[:, r["day"] - 1]))
        outflow = min(outflow, storage_input)
        storage = (storage_input - outflow) * dt
        overflow = max(0.0, (storage - r["maximum_storage"]) / dt)
        storage = min(storage, r["maximum_storage"])
        outflow += overflow
    else:
        lo = r["lower"]
        diff_wl = r["waterlevel"] - st[lo]["waterlevel"] if lo >= 0 else 0.0
        storage_input = max(r["storage"] / dt + precipitation - evaporation + inflow, 0.0)
        if diff_wl >= 0.0:
            if r["waterlevel"] > r["threshold"]:
                dh = r["waterlevel"] - r["threshold"]
                outflow = min(r["coef"] * dh ** r["exp"], dh * r["area"] / dt)
            else:
                outflow = 0.0
        else:
            if st[lo]["waterlevel"] > r["threshold"]:
                dh = st[lo]["waterlevel"] - r["threshold"]
                outflow = max(-r["coef"] * dh ** r["exp"], -(dh * st[lo]["area"] / dt))
            else:
                outflow = 0.0
        storage = (storage_input - outflow) * dt
        if diff_wl < 0.0:
            lower_storage = st[lo]["storage"] + outflow * dt
            st[lo]["waterlevel"] = interp_ref(lower_storage, list(sh[lo][1]), list(sh[lo][0]))
            st[lo]["outflow"] = -outflow
            st[lo]["outflow_cumulative"] -= outflow * dt
            st[lo]["storage"] = lower_storage
    r["waterlevel"] = interp_ref(storage, list(sh[i][1]), list(sh[i][0]))
    r["storage"] = storage
    r["outflow"] = outflow
    r["outflow_cumulative"] += outflow * dt


@pytest.mark.parametrize("levels", [(395.03027, 394.87833), (394.6, 395.2), (393.5, 393.4)])
def test_linked_free_weir_and_rating_curve(levels):
    up, lo, tables, keep = _linked_pair()
    h1, s1, h2, s2 = tables[:4]
    up.waterlevel, lo.waterlevel = levels
    up.storage = interp_ref(levels[0], list(h1), list(s1))  # initialize_storage
    lo.storage = interp_ref(levels[1], list(h2), list(s2))
    res = (O.Reservoir * 2)(up, lo)
    st = [dict(type=2, area=up.area, threshold=up.threshold, coef=140.0, exp=1.5, lower=1),
          dict(type=1, area=lo.area, maximum_storage=lo.maximum_storage, day=15, lower=-1)]
    for d, r in zip(st, (up, lo)):
        d.update(precipitation=r.precipitation, evaporation=r.evaporation, storage=r.storage,
                 waterlevel=r.waterlevel, outflow=0.0, outflow_cumulative=0.0)
    dt = 86400.0
    for step in range(6):
        for i, inflow in ((0, 500.0), (1, 500.0)):
            O.reservoir_update_model(res, i, inflow, dt)
            _update_ref(st, i, inflow, dt, tables)
        for i in range(2):
            for key, attr in (("storage", "storage"), ("waterlevel", "waterlevel"), ("outflow", "outflow"),
                              ("outflow_cumulative", "outflow_cumulative")):
                # the weir's power is Julia's ^ in the oracle and Python's ** here
                assert np.isclose(getattr(res[i], attr), st[i][key], rtol=1e-13, atol=0.0), (step, i, key)


def test_oracle_model_with_linked_reservoirs_closes_its_balances():
    dom = synthetic.make_domain(48, 1000.0, seed=3)
    res = synthetic.make_linked_reservoirs(dom, seed=3)
    cfg = synthetic.make_config(86400.0)
    o = O.OracleModel(cfg, dom, reservoirs=res)
    outs = []
    for s in range(10):
        P, PET, T = synthetic.forcing(s, cfg.dt, dom.n_land, seed=3)
        o.set_forcing(P * 3.0, PET, T)
        rp, re = synthetic.reservoir_forcing(dom, res, P * 3.0, PET)
        o.set(F["RESERVOIR_PRECIPITATION"], rp)
        o.set(F["RESERVOIR_EVAPORATION"], re)
        o.set_rating_curve_day(1 + 30 * s)
        o.step()
        outs.append(o.get(F["RESERVOIR_OUTFLOW"]))
        assert np.abs(o.get(F["BALANCE_RESERVOIR_RELATIVE_ERROR"])).max() < 1e-12
    outs = np.array(outs)
    assert outs[:, 0].min() < 0.0 < outs[:, 0].max()  # the linked weir ran both ways
    # the interpolated profile keeps every level inside its table
    hi = [res["sh_h"][res["sh_offset"][k]:res["sh_offset"][k + 1]].max() for k in (0, 1)]
    assert all(o.get(F["RESERVOIR_WATERLEVEL"])[k] <= hi[k] for k in (0, 1))
    with pytest.raises(ValueError):
        o.set_rating_curve_day(366)


def _create(dom, res):
    lib = abi.load_library()
    cfg = synthetic.make_config(86400.0)
    d, p = synthetic.c_structs(dom)
    r, t = synthetic.c_reservoirs(res), synthetic.c_reservoir_tables(res)
    h = C.c_void_p()
    st = lib.wf_create_with_reservoir_tables(C.byref(cfg), C.byref(d), C.byref(p), C.byref(r),
                                             C.byref(t) if t is not None else None, 0, C.byref(h))
    msg = lib.wf_last_error(None)
    return st, (msg.decode() if msg else "")


@pytest.fixture(scope="module")
def linked():
    build.build_all()
    dom = synthetic.make_domain(48, 1000.0, seed=3)
    return dom, synthetic.make_linked_reservoirs(dom, seed=3)


def test_abi_rejects_bad_tables_and_links(linked):
    dom, res = linked
    cases = []
    r = dict(res, sh_h=res["sh_h"].copy())
    r["sh_h"][1] = r["sh_h"][0]  # a level repeated
    cases.append((r, abi.WF_ERR_INVALID, "not strictly increasing"))
    r = dict(res, hq_offset=None, hq_h=None, hq_q=None)
    cases.append((r, abi.WF_ERR_INVALID, "H-Q tables missing"))
    r = dict(res, lower_reservoir=np.array([0, -1, -1, -1], np.int32))
    cases.append((r, abi.WF_ERR_INVALID, "out of range"))
    r = dict(res, lower_reservoir=np.array([-1, 0, -1, -1], np.int32))  # the lower one upstream
    cases.append((r, abi.WF_ERR_UNSUPPORTED, "downstream"))
    r = dict(res, storage_curve_type=np.array([3, 2, 1, 2], np.int32))
    cases.append((r, abi.WF_ERR_INVALID, "storage curve type"))
    for r, code, words in cases:
        r = {k: v for k, v in r.items() if v is not None}
        st, msg = _create(dom, r)
        assert st == code and words in msg, (st, msg, words)


def test_abi_rejects_joining_links(linked):
    dom, _ = linked
    # two upper reservoirs on different tributaries linked to one lower reservoir below their
    # confluence: the two river paths join at the confluence
    rds = dom.river["river_downstream"]
    nr = rds.size
    children = [[] for _ in range(nr)]
    for v in range(nr):
        if rds[v] >= 0:
            children[rds[v]].append(v)
    junction = next(v for v in range(nr) if len(children[v]) >= 2 and rds[v] >= 0 and rds[rds[v]] >= 0
                    and all(children[c] for c in children[v][:2]))
    a, b = children[junction][:2]
    u1, u2, low = children[a][0], children[b][0], int(rds[junction])
    k = 3
    res = dict(river_index=np.array([u1, u2, low], np.int32),
               outflow_curve_type=np.full(k, abi.WF_RES_FREE_WEIR, np.int32), area=np.full(k, 1e5),
               waterlevel=np.full(k, 5.0), threshold=np.full(k, 4.5), rating_curve_coefficient=np.full(k, 1.0),
               rating_curve_exponent=np.full(k, 1.5), lower_reservoir=np.array([2, 2, -1], np.int32))
    st, msg = _create(dom, res)
    assert st == abi.WF_ERR_UNSUPPORTED and "join" in msg, (st, msg)
    # one of the two links alone is accepted as far as the checks before the device go
    res["lower_reservoir"] = np.array([2, -1, -1], np.int32)
    st, msg = _create(dom, res)
    assert "join" not in msg and "downstream" not in msg, (st, msg)
