"""Sub-stepping and batching cases through the C ABI against the CPU oracle.

* adaptive (Courant) sub-steps (kinematic_wave__adaptive_time_step_flag = true): the overland
  and river sub-step is the type-7 quantile of the cells' Courant times (p = 0.02 land, 0.05
  river), the subsurface one the minimum times the alpha coefficient
  (routing/surface/surface_kinwave.jl:674-704, routing/subsurface/lateral_subsurface_flow.jl:
  314-344); members step independently;
* fixed sub-steps shorter than the model step for all three sweeps (routing/timestepping.jl);
* an uneven batch of independent catchments packed into one model.

The FP64 form must match the oracle to relative 1e-9 with the same sub-step counts; the split
form is held to the accuracy bar of the benchmark (outlet discharge 1e-4, closure 1e-7), except
where the adaptive sub-step itself depends on rounding (see the ensemble case below).
"""

import copy

import numpy as np
import pytest

from wflow_gb300 import abi, synthetic
from wflow_gb300.model import Model
import oracle_py as O
from test_gpu_parity import LAND, RIVER, assert_parity, compare, split_errors

pytestmark = pytest.mark.gpu


def member_forcing(s, dt, n, M, pfac, seed=1, precip_scale=1.0):
    P, PET, T = synthetic.forcing(s, dt, n, seed=seed, precip_scale=precip_scale)
    if M > 1:
        P = np.concatenate([P * pfac[m] for m in range(M)])
        PET, T = np.tile(PET, M), np.tile(T, M)
    return P, PET, T


def run_substep_pair(dom, cfg, steps, params=None, pfac=None, precip_scale=1.0, check_every=1):
    """FP64 form and oracle side by side; per step the sub-step counts of both (land, river,
    subsurface) and the field comparison."""
    gpu = Model(cfg, dom, params=params)
    orc = O.OracleModel(cfg, dom, params=params)
    M = max(1, cfg.n_members)
    pfac = np.ones(M) if pfac is None else pfac
    results, counts = [], []
    prev = gpu.metrics()
    for s in range(steps):
        P, PET, T = member_forcing(s, cfg.dt, dom.n_land, M, pfac, precip_scale=precip_scale)
        gpu.run_timestep(P, PET, T)
        orc.set_forcing(P, PET, T)
        orc.step()
        now = gpu.metrics()
        g = (now["substeps_land"] - prev["substeps_land"], now["substeps_river"] - prev["substeps_river"],
             now["substeps_subsurface"] - prev["substeps_subsurface"])
        prev = now
        counts.append((g, orc.substeps()))
        if (s + 1) % check_every == 0 or s == steps - 1:
            results.append(compare(gpu, orc, LAND + ["UNSATURATED_LAYER_DEPTH", "VOLUMETRIC_WATER_CONTENT"] +
                                   (RIVER if dom.n_river else []), layers=gpu.N))
    return gpu, orc, results, counts


def test_adaptive_fp64_daily_matches_oracle(gpu_lib):
    dom = synthetic.make_domain(48, 1000.0, seed=12)
    cfg = synthetic.make_config(86400.0, adaptive=True)
    gpu, orc, res, counts = run_substep_pair(dom, cfg, 8, precip_scale=3.0, check_every=2)
    assert_parity(res)
    for g, o in counts:
        assert g[:2] == o[:2], counts
    assert max(g[1] for g, _ in counts) > 4  # the river really sub-steps


def test_adaptive_fp64_hourly_ensemble_with_subsurface_substeps(gpu_lib):
    # alpha 1e-3 gives about ten subsurface sub-steps per hour; members differ in rain and soil,
    # so their sub-step sequences differ
    dom = synthetic.make_domain(32, 250.0, seed=13)
    M = 4
    kv0, f, pfac = synthetic.perturb_members(dom.params, M, seed=13)
    params = dict(dom.params, kv_0=kv0, f=f)
    cfg = synthetic.make_config(3600.0, n_members=M, adaptive=True, per_member_soil=True)
    cfg.subsurface_alpha = 1e-3
    gpu, orc, res, counts = run_substep_pair(dom, cfg, 6, params=params, pfac=pfac * 3.0, check_every=3)
    assert_parity(res)
    assert all(g[2] >= o[2] > 1 for g, o in counts), counts  # GPU count is the maximum over members


def test_adaptive_split_accuracy(gpu_lib):
    dom = synthetic.make_domain(48, 1000.0, seed=12)
    cfg = synthetic.make_config(86400.0, form=abi.WF_FORM_SPLIT, adaptive=True)
    w = split_errors(dom, cfg, 12)
    print("split adaptive daily errors", w)
    assert w["outlet_q"] <= 1e-4, w
    assert w["soil_storage"] <= 1e-4, w
    assert w["closure"] <= 1e-7, w


# The reference's Courant quantile counts every cell with Q > 1e-30 (surface_kinwave.jl:687), so
# its rank, and with it the sub-step, moves with the number of cells holding a tiny flow. A
# river cell that evaporation drains within a step ends at a tiny flow or at the 1e-30 floor
# depending on the sign of a cancellation (its storage minus its evaporation) that the reference
# itself decides at the level of FP64 rounding. The split form reproduces the floor and the
# Newton early stop of the reference (kw_node_ff) but cannot reproduce that rounding, so now and
# then a member takes a different sequence of sub-steps than the oracle. The test identifies
# those members from the sub-step signature (the sum of the squared sub-step sizes of every
# step, wf_get_substep_signature, against the oracle's) and holds every member whose sub-steps
# matched to the benchmark's 1e-4 on outlet discharge; the others are reported and bounded at
# 1e-2 (their discharge follows a different but equally valid time discretisation).
@pytest.mark.parametrize("rain", [1.0, 3.0])
def test_adaptive_split_ensemble_accuracy(gpu_lib, rain):
    dom = synthetic.make_domain(32, 250.0, seed=14)
    M = 32
    kv0, f, pfac = synthetic.perturb_members(dom.params, M, seed=14)
    params = dict(dom.params, kv_0=kv0, f=f)
    cfg = synthetic.make_config(3600.0, n_members=M, form=abi.WF_FORM_SPLIT, adaptive=True, per_member_soil=True)
    cfg.subsurface_alpha = 1e-3
    cfg64 = copy.copy(cfg)
    cfg64.form = abi.WF_FORM_FP64
    gpu = Model(cfg, dom, params=params)
    orc = O.OracleModel(cfg64, dom, params=params)
    n_out = len(dom.outlets)
    matched = np.ones(M, bool)
    err = np.zeros(M)
    soil = closure = 0.0
    for s in range(12):
        P, PET, T = synthetic.forcing(s, cfg.dt, dom.n_land, seed=1)
        P = np.concatenate([P * (pfac[m] * rain) for m in range(M)])
        PET, T = np.tile(PET, M), np.tile(T, M)
        gpu.run_timestep(P, PET, T)
        orc.set_forcing(P, PET, T)
        orc.step()
        for kind in (1, 2):
            sg, so = gpu.substep_signature(kind), orc.substep_signature(kind)
            matched &= np.abs(sg - so) <= 1e-6 * so
        qo, qg = orc.outlets(0).reshape(M, n_out), gpu.outlets(0).reshape(M, n_out)
        err = np.maximum(err, np.max(np.abs(qg - qo) / np.maximum(np.abs(qo), 1e-12), axis=1))
        so_, sg_ = orc.get(abi.FIELD["TOTAL_SOIL_WATER_STORAGE"]), gpu.get_value("TOTAL_SOIL_WATER_STORAGE")
        soil = max(soil, float(np.max(np.abs(sg_ - so_) / so_)))
        rel = np.abs(gpu.get_value("BALANCE_LAND_RELATIVE_ERROR"))
        closure = max(closure, float(rel.max()))
    print(f"split adaptive hourly ensemble (rain x{rain}): members with the oracle's sub-steps "
          f"{int(matched.sum())}/{M}, their outlet error {err[matched].max() if matched.any() else 0.0:.2e}; "
          f"other members {err[~matched].round(6).tolist()}; soil {soil:.2e}; closure {closure:.2e}")
    assert matched.sum() >= M // 2, matched
    assert err[matched].max() <= 1e-4, err[matched]
    assert err.max() <= 1e-2, err
    assert soil <= 1e-4
    assert closure <= 1e-7


def fixed_short_substeps(cfg):
    cfg.subsurface_dt_fixed = 1800.0
    cfg.land_dt_fixed = 1200.0
    cfg.river_dt_fixed = 300.0
    return cfg


def test_fixed_substeps_shorter_than_step_fp64(gpu_lib):
    dom = synthetic.make_domain(32, 250.0, seed=15)
    cfg = fixed_short_substeps(synthetic.make_config(3600.0))
    gpu, orc, res, counts = run_substep_pair(dom, cfg, 12, precip_scale=3.0, check_every=4)
    assert_parity(res)
    assert all(g == (3, 12, 2) for g, _ in counts), counts


def test_fixed_substeps_shorter_than_step_split(gpu_lib):
    dom = synthetic.make_domain(32, 250.0, seed=15)
    cfg = fixed_short_substeps(synthetic.make_config(3600.0, form=abi.WF_FORM_SPLIT))
    w = split_errors(dom, cfg, 24)
    print("split fixed short sub-steps errors", w)
    assert w["outlet_q"] <= 1e-4, w
    assert w["closure"] <= 1e-7, w


def ragged_domain():
    # 12 catchments of 10^2 - 10^3.5 cells (the uneven-batch generator at a scale the oracle
    # runs in seconds)
    return synthetic.make_ragged(12, seed=3, cell_size=1000.0, log10_min=2.0, log10_max=3.5)


def test_ragged_batch_fp64_matches_oracle(gpu_lib):
    dom = ragged_domain()
    assert len(dom.outlets) >= 12
    cfg = synthetic.make_config(86400.0)
    gpu, orc, res, _ = run_substep_pair(dom, cfg, 10, check_every=5)
    assert_parity(res)
    assert np.array_equal(gpu.outlets(0), orc.outlets(0))


def test_ragged_batch_split_per_catchment_outlets(gpu_lib):
    dom = ragged_domain()
    cfg = synthetic.make_config(86400.0, form=abi.WF_FORM_SPLIT)
    cfg64 = copy.copy(cfg)
    cfg64.form = abi.WF_FORM_FP64
    gpu = Model(cfg, dom)
    orc = O.OracleModel(cfg64, dom)
    worst = 0.0
    for s in range(20):
        P, PET, T = synthetic.forcing(s, cfg.dt, dom.n_land, seed=1)
        gpu.run_timestep(P, PET, T)
        orc.set_forcing(P, PET, T)
        orc.step()
        qg, qo = gpu.outlets(0), orc.outlets(0)
        assert qg.shape == qo.shape and qg.size >= 12
        worst = max(worst, float(np.max(np.abs(qg - qo) / np.maximum(np.abs(qo), 1e-12))))
    print("ragged split worst per-catchment outlet error", worst)
    assert worst <= 1e-4
    rel = np.abs(gpu.get_value("BALANCE_LAND_RELATIVE_ERROR"))
    assert rel.max() <= 1e-7
