"""Reservoirs on the CPU: the oracle's model-level coupling and the C ABI's rejections.

The reservoir update at a node is pinned by the reference's kinwave_river_update! unit test
(test_oracle_kats.py). Here the oracle's coupling of reservoirs into the model step is checked
against the properties the reference's code implies (routing/surface/surface_kinwave.jl:441-489,
:771-802, domain.jl:95-121, mass_balance.jl:261-284):
  * the river cell below a reservoir receives the reservoir outflow, not the discharge of the
    reservoir's cell, plus the discharge of its other upstream cells;
  * the reservoir's outlet cell is a pit of the land upstream lists: the land cell below it gets
    nothing from it, and its overland and subsurface discharge feed the reservoir;
  * each reservoir closes its own water balance;
  * an observed outflow replaces the outflow function.
The C ABI rejects invalid reservoir sets before it touches a device, so those checks run here.
"""

import ctypes as C

import numpy as np
import pytest

from wflow_gb300 import abi, build, synthetic
import oracle_py as O

F = abi.FIELD


@pytest.fixture(scope="module")
def domain():
    dom = synthetic.make_domain(40, 1000.0, seed=12)
    res = synthetic.make_reservoirs(dom, 6, seed=3)
    return dom, res


def drive(model, dom, res, cfg, steps, obs=None, ext=None, precip_scale=3.0):
    M = max(1, cfg.n_members)
    for s in range(steps):
        P, PET, T = synthetic.forcing(s, cfg.dt, dom.n_land, seed=1, precip_scale=precip_scale)
        if M > 1:
            P, PET, T = np.tile(P, M), np.tile(PET, M), np.tile(T, M)
        rp, re = synthetic.reservoir_forcing(dom, res, P, PET, M)
        model.set(F["RESERVOIR_PRECIPITATION"], rp)
        model.set(F["RESERVOIR_EVAPORATION"], re)
        if ext is not None:
            model.set(F["RESERVOIR_EXTERNAL_INFLOW"], np.tile(ext, M))
        if obs is not None:
            model.set(F["RESERVOIR_OUTFLOW_OBS"], np.tile(obs(s), M))
        model.set_forcing(P, PET, T)
        model.step()


def test_every_outflow_type_is_present(domain):
    dom, res = domain
    assert len(res["river_index"]) == 6
    assert set(res["outflow_curve_type"].tolist()) == {abi.WF_RES_FREE_WEIR, abi.WF_RES_MODIFIED_PULS,
                                                       abi.WF_RES_SIMPLE}
    rds = dom.river["river_downstream"]
    assert np.all(rds[res["river_index"]] >= 0)
    assert len(set(rds[res["river_index"]].tolist())) == len(res["river_index"])


def test_oracle_reservoir_coupling(domain):
    dom, res = domain
    cfg = synthetic.make_config(86400.0)
    orc = O.OracleModel(cfg, dom, reservoirs=res)
    ext = np.zeros(len(res["river_index"]))
    ext[0], ext[1] = -0.05, 0.02
    drive(orc, dom, res, cfg, 8, ext=ext)
    rds = dom.river["river_downstream"]
    ri = res["river_index"]
    qin = orc.get(F["RIVER_QIN_AVERAGE"])
    qa = orc.get(F["RIVER_Q_AVERAGE"])
    out = orc.get(F["RESERVOIR_OUTFLOW_AVERAGE"])
    assert np.all(np.isfinite(out)) and np.all(out >= 0.0)
    for k, v in enumerate(ri):
        j = rds[v]
        others = [u for u in np.where(rds == j)[0] if u != v]
        expect = out[k] + sum(qa[u] for u in others)
        assert abs(qin[j] - expect) <= 1e-12 * max(1.0, abs(expect)), (k, qin[j], expect)
    # reservoir balance (mass_balance.jl:261-284)
    rel = np.abs(orc.get(F["BALANCE_RESERVOIR_RELATIVE_ERROR"]))
    assert rel.max() <= 1e-10, rel
    # abstraction limited and accounted, positive external inflow enters the net inflow
    assert orc.get(F["RESERVOIR_ABSTRACTION_AVERAGE"])[0] > 0.0
    # inflow from the outlet cell's land routing
    cells = dom.river["river_land_index"][ri]
    assert np.array_equal(orc.get(F["RESERVOIR_INFLOW_OVERLAND"]), orc.get(F["LAND_Q_AVERAGE"])[cells])
    assert np.array_equal(orc.get(F["RESERVOIR_INFLOW_SUBSURFACE"]), orc.get(F["SSF_Q_AVERAGE"])[cells])


def test_oracle_land_cut_at_reservoir_outlets(domain):
    dom, res = domain
    cfg = synthetic.make_config(86400.0)
    orc = O.OracleModel(cfg, dom, reservoirs=res)
    drive(orc, dom, res, cfg, 4)
    lds = dom.land["land_downstream"]
    cells = set(dom.river["river_land_index"][res["river_index"]].tolist())
    fr = dom.land["flow_fraction_to_river"]
    sfw = dom.land["surface_flow_width"]
    qavg = orc.get(F["LAND_Q_AVERAGE"])
    qin = orc.get(F["LAND_QIN_AVERAGE"])
    checked = 0
    for c in cells:
        d = int(lds[c])
        if d < 0 or not sfw[d] > 0.0:
            continue
        ups = np.where(lds == d)[0]
        cut = sum(qavg[u] * (1.0 - fr[u]) for u in ups if u not in cells)
        full = sum(qavg[u] * (1.0 - fr[u]) for u in ups)
        assert abs(qin[d] - cut) <= 1e-12 * max(1.0, cut), (d, qin[d], cut, full)
        checked += 1
    assert checked > 0


def test_oracle_observed_outflow_overrides(domain):
    dom, res = domain
    cfg = synthetic.make_config(86400.0)
    orc = O.OracleModel(cfg, dom, reservoirs=res)
    n = len(res["river_index"])

    def obs(s):
        v = np.full(n, np.nan)
        v[2] = 0.01  # a small observed release, below what the reservoir holds
        return v

    drive(orc, dom, res, cfg, 3, obs=obs)
    out = orc.get(F["RESERVOIR_OUTFLOW_AVERAGE"])
    smax = res["maximum_storage"][2]
    if np.isnan(smax) or orc.get(F["RESERVOIR_STORAGE"])[2] < smax:
        assert abs(out[2] - 0.01) <= 1e-15
    assert np.abs(orc.get(F["BALANCE_RESERVOIR_RELATIVE_ERROR"])).max() <= 1e-10


def test_oracle_without_reservoirs_is_unchanged(domain):
    dom, _ = domain
    cfg = synthetic.make_config(86400.0)
    a = O.OracleModel(cfg, dom)
    b = O.OracleModel(cfg, dom, reservoirs={k: v[:0] for k, v in synthetic.make_reservoirs(dom, 1).items()})
    for s in range(3):
        P, PET, T = synthetic.forcing(s, cfg.dt, dom.n_land, seed=1)
        for m in (a, b):
            m.set_forcing(P, PET, T)
            m.step()
    assert np.array_equal(a.get(F["RIVER_Q"]), b.get(F["RIVER_Q"]))
    assert np.array_equal(a.outlets(0), b.outlets(0))


def _create_status(dom, res):
    """wf_create_with_reservoirs on an invalid reservoir set: rejected before any device use."""
    lib = abi.load_library()
    cfg = synthetic.make_config(86400.0)
    d, p = synthetic.c_structs(dom)
    r = synthetic.c_reservoirs(res)
    h = C.c_void_p()
    st = lib.wf_create_with_reservoirs(C.byref(cfg), C.byref(d), C.byref(p), C.byref(r), 0, C.byref(h))
    msg = lib.wf_last_error(None)
    return st, (msg.decode() if msg else "")


@pytest.mark.parametrize("case", ["pit", "two_into_one", "bad_type", "rating_curve_without_table", "bad_area",
                                  "missing_param", "out_of_range"])
def test_abi_rejects_invalid_reservoirs(domain, case):
    build.build_all()
    dom, res = domain
    res = {k: v.copy() for k, v in res.items()}
    rds = dom.river["river_downstream"]
    if case == "pit":
        res["river_index"][0] = int(np.where(rds < 0)[0][0])
        expect = (abi.WF_ERR_INVALID, "downstream")
    elif case == "two_into_one":
        j = rds[res["river_index"][0]]
        sib = [u for u in np.where(rds == j)[0] if u != res["river_index"][0]]
        if not sib:
            pytest.skip("no sibling at the first reservoir")
        res["river_index"][1] = sib[0]
        expect = (abi.WF_ERR_UNSUPPORTED, "drain into one")
    elif case == "bad_type":
        res["outflow_curve_type"][0] = 5
        expect = (abi.WF_ERR_UNSUPPORTED, "outflow type")
    elif case == "rating_curve_without_table":
        res["outflow_curve_type"][0] = abi.WF_RES_RATING_CURVE
        expect = (abi.WF_ERR_INVALID, "H-Q tables missing")
    elif case == "bad_area":
        res["area"][0] = 0.0
        expect = (abi.WF_ERR_INVALID, "area")
    elif case == "missing_param":
        res.pop("threshold")
        expect = (abi.WF_ERR_INVALID, "parameter")
    else:
        res["river_index"][0] = dom.n_river
        expect = (abi.WF_ERR_INVALID, "out of range")
    st, msg = _create_status(dom, res)
    assert st == expect[0] and expect[1] in msg, (st, msg)
    # the oracle refuses the same sets (the sibling case included)
    if case in ("pit", "two_into_one", "bad_type", "rating_curve_without_table", "bad_area", "out_of_range"):
        with pytest.raises(RuntimeError):
            O.OracleModel(synthetic.make_config(86400.0), dom, reservoirs=res)
