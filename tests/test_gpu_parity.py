"""FP64 plain form on the GPU against the CPU oracle, through the C ABI.

The FP64 form computes every operation in the same order as the oracle with the same
elementary-function implementations, so results are expected to agree bit for bit; the
acceptance bar asserted here is the drop-in tolerance, relative 1e-9 (absolute 1e-300 for
exact zeros), and the exact-equality fraction is asserted separately.
"""

import numpy as np
import pytest

from wflow_gb300 import abi, synthetic
from wflow_gb300.model import Model
import oracle_py as O

pytestmark = pytest.mark.gpu

RTOL = 1e-9

LAND = ["CANOPY_STORAGE", "SNOW_STORAGE", "SNOW_WATER", "SOIL_SURFACE_TEMPERATURE", "SATURATED_WATER_DEPTH",
        "SSF_Q", "LAND_Q", "LAND_H", "WATER_TABLE_DEPTH", "UNSATURATED_STORE_DEPTH", "TOTAL_SOIL_WATER_STORAGE",
        "RECHARGE", "NET_RUNOFF", "RUNOFF", "ACTUAL_EVAPOTRANSPIRATION", "ACTUAL_LEAKAGE", "TRANSPIRATION",
        "SOIL_EVAPORATION", "ACTUAL_INFILTRATION", "EXFILTRATION_SATURATED_WATER", "INTERCEPTION_RATE",
        "NET_RUNOFF_RIVER", "SSF_Q_AVERAGE", "SSF_WATER_TABLE_DEPTH", "SSF_STORAGE", "SSF_TO_RIVER_AVERAGE",
        "LAND_Q_AVERAGE", "LAND_STORAGE", "LAND_TO_RIVER_AVERAGE", "LAND_INWATER", "TOTAL_STORAGE",
        "BALANCE_LAND_ERROR", "BALANCE_OVERLAND_ERROR", "BALANCE_SUBSURFACE_ERROR"]
RIVER = ["RIVER_Q", "RIVER_H", "RIVER_STORAGE", "RIVER_Q_AVERAGE", "RIVER_QIN_AVERAGE", "RIVER_INWATER",
         "BALANCE_RIVER_ERROR"]


def rel_err(a, b):
    a, b = np.asarray(a), np.asarray(b)
    both_nan = np.isnan(a) & np.isnan(b)
    d = np.abs(a - b)
    scale = np.maximum(np.abs(a), np.abs(b))
    r = np.where(scale > 1e-300, d / np.maximum(scale, 1e-300), d)
    r[both_nan] = 0.0
    return r


# Balance errors are differences of nearly equal totals: they are compared in absolute terms
# against the scale of the fluxes that enter them.
BALANCE_SCALE = {"BALANCE_LAND_ERROR": "ACTUAL_EVAPOTRANSPIRATION", "BALANCE_OVERLAND_ERROR": "LAND_Q_AVERAGE",
                 "BALANCE_SUBSURFACE_ERROR": "SSF_Q_AVERAGE", "BALANCE_RIVER_ERROR": "RIVER_Q_AVERAGE"}


def compare(gpu, orc, fields, layers=0):
    worst = {}
    exact = 0
    total = 0
    inexact = {}
    for f in fields:
        fid = abi.FIELD[f]
        for k in (range(layers) if f in abi.LAYERED_FIELDS else [0]):
            g = gpu.get_value(fid, layer=k)
            o = orc.get(fid, layer=k)
            name = f if k == 0 else f"{f}[{k}]"
            if f in BALANCE_SCALE:
                scale = np.max(np.abs(orc.get(abi.FIELD[BALANCE_SCALE[f]]))) + 1e-300
                r = np.abs(g - o) / scale
            else:
                r = rel_err(g, o)
            worst[name] = float(r.max()) if r.size else 0.0
            eq = (g == o) | (np.isnan(g) & np.isnan(o))
            exact += int(np.sum(eq))
            total += g.size
            if not eq.all():
                inexact[name] = round(float(1.0 - eq.mean()), 5)
    return worst, exact / max(total, 1), inexact


def run_pair(dom, cfg, steps, seed=1, params=None, check_every=1, precip_scale=None):
    gpu = Model(cfg, dom, params=params)
    orc = O.OracleModel(cfg, dom, params=params)
    M = max(1, cfg.n_members)
    results = []
    for s in range(steps):
        P, PET, T = synthetic.forcing(s, cfg.dt, dom.n_land, seed=seed)
        if M > 1:
            scale = precip_scale if precip_scale is not None else np.ones(M)
            P = np.concatenate([P * scale[m] for m in range(M)])
            PET = np.tile(PET, M)
            T = np.tile(T, M)
        gpu.run_timestep(P, PET, T)
        orc.set_forcing(P, PET, T)
        orc.step()
        if (s + 1) % check_every == 0 or s == steps - 1:
            results.append(compare(gpu, orc, LAND + ["UNSATURATED_LAYER_DEPTH", "VOLUMETRIC_WATER_CONTENT"] +
                                   (RIVER if dom.n_river else []), layers=gpu.N))
    return gpu, orc, results


def assert_parity(results, min_exact=0.999):
    for worst, exact_frac, inexact in results:
        bad = {k: v for k, v in worst.items() if v > RTOL}
        assert not bad, (bad, inexact)
        assert exact_frac >= min_exact, (exact_frac, inexact)


def test_daily_gash_64(gpu_lib):
    dom = synthetic.make_domain(64, 1000.0, seed=1)
    cfg = synthetic.make_config(86400.0)
    gpu, orc, res = run_pair(dom, cfg, 30, check_every=5)
    assert_parity(res)
    assert np.array_equal(gpu.outlets(0), orc.outlets(0))


def test_hourly_rutter_48(gpu_lib):
    dom = synthetic.make_domain(48, 250.0, seed=2)
    cfg = synthetic.make_config(3600.0)
    gpu, orc, res = run_pair(dom, cfg, 48, check_every=12)
    assert_parity(res)


def test_snow_off_and_kv_exponential_constant(gpu_lib):
    dom = synthetic.make_domain(24, 1000.0, seed=4)
    params = dict(dom.params)
    params["z_exp"] = np.full(dom.n_land, 0.6)
    cfg = synthetic.make_config(86400.0, snow=False)
    cfg.kv_profile = abi.WF_KV_EXPONENTIAL_CONSTANT
    gpu, orc, res = run_pair(dom, cfg, 10, params=params, check_every=5)
    assert_parity(res)


def test_single_cell_and_no_river(gpu_lib):
    dom = synthetic.make_domain(2, 1000.0, seed=6, ny=1)
    assert dom.n_river == 0
    cfg = synthetic.make_config(86400.0)
    gpu, orc, res = run_pair(dom, cfg, 5)
    worst, _, _ = res[-1]
    assert all(v <= RTOL for v in worst.values()), worst


def test_ensemble_members_match_oracle(gpu_lib):
    dom = synthetic.make_domain(32, 1000.0, seed=7)
    M = 4
    kv0, f, pfac = synthetic.perturb_members(dom.params, M, seed=7)
    params = dict(dom.params, kv_0=kv0, f=f)
    cfg = synthetic.make_config(86400.0, n_members=M, per_member_soil=True)
    gpu, orc, res = run_pair(dom, cfg, 8, params=params, precip_scale=pfac, check_every=4)
    assert_parity(res)
    q = gpu.outlets(0)
    assert q.size == M and len(set(np.round(q, 12))) > 1  # members differ


def test_restart_equivalence(gpu_lib):
    # test/run.jl: a cold run equals a run interrupted, checkpointed and resumed
    dom = synthetic.make_domain(32, 1000.0, seed=8)
    cfg = synthetic.make_config(86400.0)
    a = Model(cfg, dom)
    b = Model(cfg, dom)
    for s in range(12):
        P, PET, T = synthetic.forcing(s, cfg.dt, dom.n_land, seed=8)
        a.run_timestep(P, PET, T)
        if s < 5:
            b.run_timestep(P, PET, T)
        if s == 4:
            blob = b.save_state()
            b.close()
            b = Model(cfg, dom)
            b.load_state(blob)
        if s > 4:
            b.run_timestep(P, PET, T)
    for f in ["SATURATED_WATER_DEPTH", "SSF_Q", "LAND_Q", "RIVER_Q", "RIVER_Q_AVERAGE", "SNOW_STORAGE"]:
        assert np.array_equal(a.get_value(f), b.get_value(f)), f


def test_graph_and_eager_paths_agree(gpu_lib):
    dom = synthetic.make_domain(32, 1000.0, seed=9)
    cfg = synthetic.make_config(86400.0)
    a = Model(cfg, dom)
    b = Model(cfg, dom)
    b.set_tuning(use_graph=0, routing_warps=2)
    for s in range(4):
        P, PET, T = synthetic.forcing(s, cfg.dt, dom.n_land, seed=9)
        a.run_timestep(P, PET, T)
        b.run_timestep(P, PET, T)
    for f in ["SSF_Q", "LAND_Q", "RIVER_Q", "TOTAL_STORAGE"]:
        assert np.array_equal(a.get_value(f), b.get_value(f)), f
    assert a.metrics()["kernel_launches"] > 0


def test_launch_tuning_leaves_split_results_unchanged(gpu_lib):
    # the launch shapes the autotuner picks (resident warps, sub-step lanes, staged or register
    # sweep inputs, the vertical kernel's block and grid, the overland and river sweeps in one
    # launch or two) change no arithmetic of the split form
    dom = synthetic.make_domain(48, 1000.0, seed=12)
    M = 32
    cfg = synthetic.make_config(3600.0, n_members=M, form=abi.WF_FORM_SPLIT)
    a = Model(cfg, dom)
    b = Model(cfg, dom)
    b.set_tuning(routing_warps=2, routing_blocks_per_sm=3, substep_lanes=4, sweep_inputs=5,
                 vertical_block=128, vertical_blocks_per_sm=1, separate_overland_river=1)
    for s in range(4):
        P, PET, T = synthetic.forcing(s, cfg.dt, dom.n_land, seed=12)
        P, PET, T = (np.tile(x, M) for x in (P, PET, T))
        a.run_timestep(P, PET, T)
        b.run_timestep(P, PET, T)
    for f in ["SATURATED_WATER_DEPTH", "SSF_Q", "LAND_Q", "RIVER_Q", "TOTAL_STORAGE"]:
        assert np.array_equal(a.get_value(f), b.get_value(f)), f
    for bad in (dict(vertical_blocks_per_sm=-1), dict(vertical_blocks_per_sm=65), dict(sweep_inputs=8),
                dict(separate_overland_river=2)):
        with pytest.raises(RuntimeError):
            b.set_tuning(**bad)


@pytest.mark.parametrize("M,lanes", [(1, 0), (1, 1), (64, 0), (64, 1)])
def test_shared_overland_river_launch_matches_separate_launches(gpu_lib, M, lanes):
    # hourly steps: one overland sub-step and four river sub-steps, all in the shared launch
    # (lanes 0: the river's first-dispatched chains on the diagonal schedule, 1: all node-major);
    # a stale lateral inflow (a river node not waiting for the overland walker) would show here
    dom = synthetic.make_domain(64, 250.0, seed=15)
    cfg = synthetic.make_config(3600.0, n_members=M, form=abi.WF_FORM_SPLIT)
    a = Model(cfg, dom)
    a.set_tuning(substep_lanes=lanes)
    b = Model(cfg, dom)
    b.set_tuning(separate_overland_river=1)
    for s in range(6):
        P, PET, T = synthetic.forcing(s, cfg.dt, dom.n_land, seed=15, precip_scale=2.0 + s)
        P, PET, T = (np.tile(x, M) for x in (P, PET, T))
        a.run_timestep(P, PET, T)
        b.run_timestep(P, PET, T)
        for f in ["RIVER_Q", "RIVER_INWATER", "LAND_Q", "BALANCE_RIVER_ERROR"]:
            assert np.array_equal(a.get_value(f), b.get_value(f)), (s, f)
    assert np.abs(a.get_value("RIVER_INWATER")).max() > 0.0


def test_bounded_wait_reports_error_and_recovers(gpu_lib):
    # a wait on an epoch nothing publishes must end within its budget with WF_ERR_SPIN
    dom = synthetic.make_domain(16, 1000.0, seed=10)
    cfg = synthetic.make_config(86400.0)
    m = Model(cfg, dom)
    m.set_tuning(use_graph=0, wait_budget_us=20000, wait_offset=1000)
    P, PET, T = synthetic.forcing(0, cfg.dt, dom.n_land, seed=10)
    with pytest.raises(RuntimeError, match="status -5"):
        m.run_timestep(P, PET, T)
    m.set_tuning(use_graph=1)
    m.run_timestep(P, PET, T)  # the context stays usable
    assert np.all(np.isfinite(m.get_value("SSF_Q")))


def test_set_value_and_get_value_at_indices(gpu_lib):
    dom = synthetic.make_domain(16, 1000.0, seed=11)
    cfg = synthetic.make_config(86400.0)
    m = Model(cfg, dom)
    v = m.get_value("SATURATED_WATER_DEPTH")
    m.set_value("SATURATED_WATER_DEPTH", v[10:20] * 0.5, offset=10)
    w = m.get_value("SATURATED_WATER_DEPTH", offset=5, count=20)
    assert np.array_equal(w[5:15], v[10:20] * 0.5)
    assert np.array_equal(w[:5], v[5:10])
    with pytest.raises(RuntimeError):
        m.set_value("RECHARGE", v[:3])


# ---------------------------------------------------------------- split form ----------
def split_errors(dom, cfg_split, steps, seed=1, params=None, precip_scale=None):
    """Run the split form and the FP64 oracle side by side; return the worst relative errors
    of outlet discharge, per-cell discharge and storages, and the split form's own worst
    relative balance closure."""
    import copy
    cfg64 = copy.copy(cfg_split)
    cfg64.form = abi.WF_FORM_FP64
    gpu = Model(cfg_split, dom, params=params)
    orc = O.OracleModel(cfg64, dom, params=params)
    M = max(1, cfg_split.n_members)
    worst = {"outlet_q": 0.0, "river_q": 0.0, "soil_storage": 0.0, "snow_storage": 0.0, "closure": 0.0}
    for s in range(steps):
        P, PET, T = synthetic.forcing(s, cfg_split.dt, dom.n_land, seed=seed)
        if M > 1:
            scale = precip_scale if precip_scale is not None else np.ones(M)
            P = np.concatenate([P * scale[m] for m in range(M)])
            PET, T = np.tile(PET, M), np.tile(T, M)
        gpu.run_timestep(P, PET, T)
        orc.set_forcing(P, PET, T)
        orc.step()
        qo, qg = orc.outlets(0), gpu.outlets(0)
        worst["outlet_q"] = max(worst["outlet_q"], float(np.max(np.abs(qg - qo) / np.maximum(np.abs(qo), 1e-12))))
        rq_o, rq_g = orc.get(abi.FIELD["RIVER_Q"]), gpu.get_value("RIVER_Q")
        big = rq_o > 1e-3 * rq_o.max()
        worst["river_q"] = max(worst["river_q"], float(np.max(np.abs(rq_g - rq_o)[big] / rq_o[big])))
        so, sg = orc.get(abi.FIELD["TOTAL_SOIL_WATER_STORAGE"]), gpu.get_value("TOTAL_SOIL_WATER_STORAGE")
        worst["soil_storage"] = max(worst["soil_storage"], float(np.max(np.abs(sg - so) / so)))
        wo, wg = orc.get(abi.FIELD["SNOW_STORAGE"]), gpu.get_value("SNOW_STORAGE")
        wbig = wo > 1e-4
        if wbig.any():
            worst["snow_storage"] = max(worst["snow_storage"], float(np.max(np.abs(wg - wo)[wbig] / wo[wbig])))
        rel = np.abs(gpu.get_value("BALANCE_LAND_RELATIVE_ERROR"))
        worst["closure"] = max(worst["closure"], float(rel.max()))
    return worst


def test_split_form_accuracy_daily(gpu_lib):
    dom = synthetic.make_domain(48, 1000.0, seed=12)
    cfg = synthetic.make_config(86400.0, form=abi.WF_FORM_SPLIT)
    w = split_errors(dom, cfg, 40)
    print("split daily errors", w)
    assert w["outlet_q"] <= 1e-4, w
    assert w["soil_storage"] <= 1e-4, w
    assert w["closure"] <= 1e-7, w


def test_split_form_accuracy_hourly_ensemble(gpu_lib):
    dom = synthetic.make_domain(32, 250.0, seed=13)
    M = 32
    kv0, f, pfac = synthetic.perturb_members(dom.params, M, seed=13)
    params = dict(dom.params, kv_0=kv0, f=f)
    cfg = synthetic.make_config(3600.0, n_members=M, form=abi.WF_FORM_SPLIT, per_member_soil=True)
    w = split_errors(dom, cfg, 48, params=params, precip_scale=pfac)
    print("split hourly ensemble errors", w)
    assert w["outlet_q"] <= 1e-4, w
    assert w["closure"] <= 1e-7, w


def test_async_forcing_pipeline_matches_synchronous_steps(gpu_lib):
    # wf_set_forcing_async of step k+1 issued while step k runs (wf_step_async) gives the same
    # state as wf_set_forcing + wf_step, for both forms
    import torch
    dom = synthetic.make_domain(32, 1000.0, seed=21)
    for form in (abi.WF_FORM_FP64, abi.WF_FORM_SPLIT):
        cfg = synthetic.make_config(86400.0, form=form)
        a, b = Model(cfg, dom), Model(cfg, dom)
        forc = [[torch.from_numpy(x).pin_memory() for x in synthetic.forcing(s, cfg.dt, dom.n_land, seed=21)]
                for s in range(5)]
        b.set_forcing_async(*[x.numpy() for x in forc[0]])
        for s in range(5):
            a.run_timestep(*[x.numpy() for x in forc[s]])
            b.step_async()
            if s + 1 < 5:
                b.set_forcing_async(*[x.numpy() for x in forc[s + 1]])
            b.synchronize()
        for f in ["SSF_Q", "LAND_Q", "RIVER_Q", "TOTAL_STORAGE", "SATURATED_WATER_DEPTH"]:
            assert np.array_equal(a.get_value(f), b.get_value(f)), (form, f)
        assert np.array_equal(a.outlets(0), b.outlets(0))


def test_six_soil_layers_and_constant_kv_both_forms(gpu_lib):
    # more than four soil layers (the kernels' 8-layer instantiation) with the
    # exponential_constant conductivity profile
    layers = (50.0, 100.0, 200.0, 400.0, 600.0)
    dom = synthetic.make_domain(24, 1000.0, seed=22, n_layers_cfg=layers)
    params = dict(dom.params)
    params["z_exp"] = np.full(dom.n_land, 0.8)
    cfg = synthetic.make_config(86400.0, layers=layers)
    cfg.kv_profile = abi.WF_KV_EXPONENTIAL_CONSTANT
    gpu, orc, res = run_pair(dom, cfg, 10, params=params, check_every=5)
    assert gpu.N == 6
    assert_parity(res)
    cfgs = synthetic.make_config(86400.0, form=abi.WF_FORM_SPLIT, layers=layers)
    cfgs.kv_profile = abi.WF_KV_EXPONENTIAL_CONSTANT
    w = split_errors(dom, cfgs, 20, params=params)
    print("split six layers errors", w)
    assert w["outlet_q"] <= 1e-4, w
    assert w["soil_storage"] <= 1e-4, w
    assert w["closure"] <= 1e-7, w


def test_fp32_forcing_matches_fp64_forcing(gpu_lib):
    # wf_set_forcing_f32 / wf_set_forcing_async_f32: the split form computes with FP32 forcing, so
    # FP32 arrays give the same state as FP64 ones; the FP64 form widens them exactly
    dom = synthetic.make_domain(32, 1000.0, seed=23)
    for form in (abi.WF_FORM_SPLIT, abi.WF_FORM_FP64):
        cfg = synthetic.make_config(86400.0, form=form)
        a, b = Model(cfg, dom), Model(cfg, dom)
        for s in range(4):
            P, PET, T = (x.astype(np.float32).astype(np.float64) for x in synthetic.forcing(s, cfg.dt, dom.n_land, seed=23))
            a.run_timestep(P, PET, T)
            b.set_forcing_f32(P, PET, T, asynchronous=s % 2 == 1)
            b.update_model()
        for f in ["SSF_Q", "LAND_Q", "RIVER_Q", "TOTAL_STORAGE", "SATURATED_WATER_DEPTH", "SNOW_STORAGE"]:
            assert np.array_equal(a.get_value(f), b.get_value(f)), (form, f)


def test_fp32_forcing_with_shared_arrays(gpu_lib):
    # wf_set_forcing_counts_(async_)f32: per-member precipitation with the potential evaporation
    # and temperature given once for every member equals the tiled arrays
    dom = synthetic.make_domain(24, 1000.0, seed=29)
    M = 4
    cfg = synthetic.make_config(86400.0, form=abi.WF_FORM_SPLIT, n_members=M)
    a, b = Model(cfg, dom), Model(cfg, dom)
    for s in range(3):
        P, PET, T = (x.astype(np.float32).astype(np.float64) for x in synthetic.forcing(s, cfg.dt, dom.n_land, seed=29))
        Pm = np.concatenate([P * f for f in (0.5, 1.0, 1.5, 2.0)])
        a.run_timestep(Pm, np.tile(PET, M), np.tile(T, M))
        b.set_forcing_f32(Pm, PET, T, asynchronous=s == 1)
        b.update_model()
    for f in ["SSF_Q", "LAND_Q", "RIVER_Q", "TOTAL_STORAGE", "SNOW_STORAGE"]:
        assert np.array_equal(a.get_value(f), b.get_value(f)), f
