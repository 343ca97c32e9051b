"""Reservoirs through the C ABI against the CPU oracle.

A model created with wf_create_with_reservoirs cuts the land and river upstream lists at the
reservoir outlets (domain.jl:95-121), feeds each reservoir from its outlet cell's overland and
subsurface discharge (surface_kinwave.jl:771-802), updates it inside the river sweep after its
cell's kinematic wave and hands its outflow to the downstream river cell
(surface_kinwave.jl:441-489, reservoir.jl:583-628). The reservoirs here cover the four outflow
functions (simple, modified Puls, free weir, rating curve), both storage profiles, a free weir
linked to a lower reservoir (water flowing back when the lower one is higher), a negative and a
positive external inflow and an observed outflow on alternate steps.

FP64 form: every land, river and reservoir field within relative 1e-9 of the oracle (the
drop-in bar; the arithmetic is the oracle's, operation for operation). Split form: the outlet
discharge within 1e-4 (the benchmark's bar), reservoir storage within 1e-5 and reservoir
outflow within 1e-4 of the largest reservoir outflow, reservoir balance closure 1e-9; the
reservoir arithmetic itself is FP64, its inputs carry the split form's discharge error.
"""

import numpy as np
import pytest

from wflow_gb300 import abi, synthetic
from wflow_gb300.model import Model
import oracle_py as O
from test_gpu_parity import LAND, RIVER, assert_parity, compare

pytestmark = pytest.mark.gpu

F = abi.FIELD
RES = ["RESERVOIR_STORAGE", "RESERVOIR_WATERLEVEL", "RESERVOIR_OUTFLOW", "RESERVOIR_OUTFLOW_AVERAGE",
       "RESERVOIR_INFLOW_AVERAGE", "RESERVOIR_ACTEVAP_AVERAGE", "RESERVOIR_ABSTRACTION_AVERAGE",
       "RESERVOIR_INFLOW_OVERLAND", "RESERVOIR_INFLOW_SUBSURFACE"]


def step_inputs(dom, res, s, dt, M, pfac, precip_scale):
    """Forcing of step s and the reservoirs' inputs: precipitation and evaporation at the outlet
    cell, external inflow (reservoir 0 abstracts, reservoir 1 receives), an observed outflow for
    reservoir 2 on even steps."""
    P, PET, T = synthetic.forcing(s, dt, dom.n_land, seed=1, precip_scale=precip_scale)
    if M > 1:
        P = np.concatenate([P * pfac[m] for m in range(M)])
        PET, T = np.tile(PET, M), np.tile(T, M)
    n = len(res["river_index"])
    rp, re = synthetic.reservoir_forcing(dom, res, P, PET, M)
    ext = np.zeros(n)
    ext[0], ext[1] = -0.05, 0.02
    obs = np.full(n, np.nan)
    if s % 2 == 0:
        obs[2] = 0.01
    inputs = {"RESERVOIR_PRECIPITATION": rp, "RESERVOIR_EVAPORATION": re,
              "RESERVOIR_EXTERNAL_INFLOW": np.tile(ext, M), "RESERVOIR_OUTFLOW_OBS": np.tile(obs, M)}
    return (P, PET, T), inputs


def rating_day(s):
    """The H-Q tables' column of step s: a different day of the year every step."""
    return 1 + (40 + 37 * s) % 365


def run_res_pair(dom, res, cfg, steps, params=None, pfac=None, precip_scale=3.0, check_every=1, trace=None):
    gpu = Model(cfg, dom, params=params, reservoirs=res)
    orc = O.OracleModel(cfg, dom, params=params, reservoirs=res)
    M = max(1, cfg.n_members)
    pfac = np.ones(M) if pfac is None else pfac
    results, counts = [], []
    prev = gpu.metrics()
    for s in range(steps):
        (P, PET, T), inputs = step_inputs(dom, res, s, cfg.dt, M, pfac, precip_scale)
        for name, v in inputs.items():
            gpu.set_value(name, v)
            orc.set(F[name], v)
        gpu.set_rating_curve_day(rating_day(s))
        orc.set_rating_curve_day(rating_day(s))
        gpu.run_timestep(P, PET, T)
        orc.set_forcing(P, PET, T)
        orc.step()
        now = gpu.metrics()
        counts.append(((now["substeps_land"] - prev["substeps_land"], now["substeps_river"] - prev["substeps_river"]),
                       orc.substeps()[:2]))
        prev = now
        if trace is not None:
            trace.append({f: gpu.get_value(f) for f in ("RESERVOIR_OUTFLOW", "RESERVOIR_OUTFLOW_AVERAGE",
                                                         "RESERVOIR_WATERLEVEL")})
        if (s + 1) % check_every == 0 or s == steps - 1:
            results.append(compare(gpu, orc, LAND + ["LAND_QIN_AVERAGE", "UNSATURATED_LAYER_DEPTH"] + RIVER + RES,
                                   layers=gpu.N))
    return gpu, orc, results, counts


def reservoir_closure(gpu):
    return float(np.abs(gpu.get_value("BALANCE_RESERVOIR_RELATIVE_ERROR")).max())


def test_reservoirs_fp64_daily_match_oracle(gpu_lib):
    dom = synthetic.make_domain(48, 1000.0, seed=12)
    res = synthetic.make_reservoirs(dom, 6, seed=3)
    cfg = synthetic.make_config(86400.0)
    gpu, orc, results, _ = run_res_pair(dom, res, cfg, 10, check_every=5)
    assert_parity(results)
    assert np.array_equal(gpu.outlets(0), orc.outlets(0))
    assert reservoir_closure(gpu) <= 1e-9
    assert gpu.get_value("RESERVOIR_ABSTRACTION_AVERAGE")[0] > 0.0


def test_reservoirs_fp64_hourly_ensemble(gpu_lib):
    # four river sub-steps per step; members differ in rain and soil
    dom = synthetic.make_domain(32, 250.0, seed=13)
    res = synthetic.make_reservoirs(dom, 4, seed=5)
    M = 4
    kv0, f, pfac = synthetic.perturb_members(dom.params, M, seed=13)
    params = dict(dom.params, kv_0=kv0, f=f)
    cfg = synthetic.make_config(3600.0, n_members=M, per_member_soil=True)
    gpu, orc, results, _ = run_res_pair(dom, res, cfg, 8, params=params, pfac=pfac * 3.0, check_every=4)
    assert_parity(results)
    assert reservoir_closure(gpu) <= 1e-9


def test_reservoirs_fp64_adaptive(gpu_lib):
    dom = synthetic.make_domain(48, 1000.0, seed=12)
    res = synthetic.make_reservoirs(dom, 6, seed=3)
    cfg = synthetic.make_config(86400.0, adaptive=True)
    gpu, orc, results, counts = run_res_pair(dom, res, cfg, 6, check_every=3)
    assert_parity(results)
    for g, o in counts:
        assert g == o, counts


def test_reservoir_state_roundtrip(gpu_lib):
    dom = synthetic.make_domain(32, 1000.0, seed=12)
    res = synthetic.make_reservoirs(dom, 3, seed=3)
    cfg = synthetic.make_config(86400.0)
    gpu = Model(cfg, dom, reservoirs=res)

    def step(s):
        (P, PET, T), inputs = step_inputs(dom, res, s, cfg.dt, 1, np.ones(1), 3.0)
        for name, v in inputs.items():
            gpu.set_value(name, v)
        gpu.run_timestep(P, PET, T)

    for s in range(3):
        step(s)
    blob = gpu.save_state()
    for s in range(3, 5):
        step(s)
    a = [gpu.get_value(f) for f in ("RESERVOIR_STORAGE", "RESERVOIR_OUTFLOW_AVERAGE", "RIVER_Q")]
    gpu.load_state(blob)
    for s in range(3, 5):
        step(s)
    b = [gpu.get_value(f) for f in ("RESERVOIR_STORAGE", "RESERVOIR_OUTFLOW_AVERAGE", "RIVER_Q")]
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


# Reservoir tables and links (synthetic.make_linked_reservoirs): an upper free weir linked to a
# lower reservoir four river cells downstream (interpolated S-H profiles; the lower one released
# by a rating curve read in a different day's column every step), a modified Puls reservoir with
# the linear profile and a simple reservoir with an interpolated profile. The lower reservoir
# starts above the upper one, so water first runs back (a negative outflow of the upper one).
def test_linked_reservoirs_and_tables_fp64_daily(gpu_lib):
    dom = synthetic.make_domain(48, 1000.0, seed=12)
    res = synthetic.make_linked_reservoirs(dom, seed=3)
    cfg = synthetic.make_config(86400.0)
    trace = []
    gpu, orc, results, _ = run_res_pair(dom, res, cfg, 12, check_every=4, trace=trace)
    assert_parity(results)
    assert np.array_equal(gpu.outlets(0), orc.outlets(0))
    assert reservoir_closure(gpu) <= 1e-9
    upper = np.array([t["RESERVOIR_OUTFLOW"][0] for t in trace])
    assert upper.min() < 0.0 < upper.max(), upper  # back flow and forward flow both happened


def test_linked_reservoirs_fp64_hourly_ensemble(gpu_lib):
    # four river sub-steps per step, each its own launch (linked reservoirs); members differ
    dom = synthetic.make_domain(32, 250.0, seed=13)
    res = synthetic.make_linked_reservoirs(dom, seed=5)
    M = 4
    kv0, f, pfac = synthetic.perturb_members(dom.params, M, seed=13)
    params = dict(dom.params, kv_0=kv0, f=f)
    cfg = synthetic.make_config(3600.0, n_members=M, per_member_soil=True)
    gpu, orc, results, _ = run_res_pair(dom, res, cfg, 8, params=params, pfac=pfac * 3.0, check_every=4)
    assert_parity(results)
    assert reservoir_closure(gpu) <= 1e-9


def split_res_errors(dom, res, cfg, steps, precip_scale=3.0, models=None):
    import copy
    cfg64 = copy.copy(cfg)
    cfg64.form = abi.WF_FORM_FP64
    gpu = Model(cfg, dom, reservoirs=res)
    orc = O.OracleModel(cfg64, dom, reservoirs=res)
    w = {"outlet_q": 0.0, "storage": 0.0, "outflow": 0.0, "closure": 0.0, "res_closure": 0.0}
    for s in range(steps):
        (P, PET, T), inputs = step_inputs(dom, res, s, cfg.dt, 1, np.ones(1), precip_scale)
        for name, v in inputs.items():
            gpu.set_value(name, v)
            orc.set(F[name], v)
        gpu.set_rating_curve_day(rating_day(s))
        orc.set_rating_curve_day(rating_day(s))
        gpu.run_timestep(P, PET, T)
        orc.set_forcing(P, PET, T)
        orc.step()
        qo, qg = orc.outlets(0), gpu.outlets(0)
        w["outlet_q"] = max(w["outlet_q"], float(np.max(np.abs(qg - qo) / np.maximum(np.abs(qo), 1e-12))))
        so, sg = orc.get(F["RESERVOIR_STORAGE"]), gpu.get_value("RESERVOIR_STORAGE")
        w["storage"] = max(w["storage"], float(np.max(np.abs(sg - so) / np.maximum(np.abs(so), 1e-12))))
        oo, og = orc.get(F["RESERVOIR_OUTFLOW_AVERAGE"]), gpu.get_value("RESERVOIR_OUTFLOW_AVERAGE")
        w["outflow"] = max(w["outflow"], float(np.max(np.abs(og - oo)) / max(float(np.max(np.abs(oo))), 1e-12)))
        w["closure"] = max(w["closure"], float(np.abs(gpu.get_value("BALANCE_LAND_RELATIVE_ERROR")).max()))
        w["res_closure"] = max(w["res_closure"], reservoir_closure(gpu))
    if models is not None:
        models.extend([gpu, orc])
    return w


# Measured on a GB300 (fixed and adaptive alike): outlet 3.4e-7, reservoir storage 1.1e-7,
# reservoir outflow 3.8e-7, reservoir closure 6.5e-13, land closure 5.5e-7. The land closure
# involves no reservoir quantity; it is the reference's relative balance error (error over the
# mean of in- and outflow), which peaks in cells with tiny fluxes (the FP64 form itself reaches
# 1.4e-5 on the benchmark's 64-member ensemble). At this test's triple daily rain it exceeds the
# 1e-7 the split tests meet at the benchmark's rain; the same case without reservoirs has not
# been measured, so the bar here is 1e-6.
@pytest.mark.parametrize("adaptive", [False, True])
def test_reservoirs_split_accuracy(gpu_lib, adaptive):
    dom = synthetic.make_domain(48, 1000.0, seed=12)
    res = synthetic.make_reservoirs(dom, 6, seed=3)
    cfg = synthetic.make_config(86400.0, form=abi.WF_FORM_SPLIT, adaptive=adaptive)
    w = split_res_errors(dom, res, cfg, 12)
    print(f"split reservoirs (adaptive={adaptive}) errors", w)
    assert w["outlet_q"] <= 1e-4, w
    assert w["storage"] <= 1e-5, w
    assert w["outflow"] <= 1e-4, w
    assert w["closure"] <= 1e-6, w
    assert w["res_closure"] <= 1e-9, w


def test_linked_reservoirs_split_accuracy(gpu_lib):
    dom = synthetic.make_domain(48, 1000.0, seed=12)
    res = synthetic.make_linked_reservoirs(dom, seed=3)
    cfg = synthetic.make_config(86400.0, form=abi.WF_FORM_SPLIT)
    models = []
    w = split_res_errors(dom, res, cfg, 12, models=models)
    print("split linked reservoirs with tables, errors", w)
    assert w["outlet_q"] <= 1e-4, w
    assert w["storage"] <= 1e-5, w
    assert w["outflow"] <= 1e-4, w
    assert w["res_closure"] <= 1e-9, w
    # the river cells below the reservoirs receive each reservoir's own outflow: the water the
    # upper reservoir draws back from the lower one leaves the lower reservoir but does not flow
    # down the river (reservoir.jl:482-521, surface_kinwave.jl:441-489)
    gpu, orc = models
    below = dom.river["river_downstream"][res["river_index"]]
    qo = orc.get(F["RIVER_QIN_AVERAGE"])[below]
    qg = gpu.get_value("RIVER_QIN_AVERAGE")[below]
    scale = max(float(np.max(np.abs(qo))), 1e-12)
    assert float(np.max(np.abs(qg - qo))) <= 1e-4 * scale, (qg, qo)
