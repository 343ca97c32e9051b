"""The benchmark configurations against the FP64 oracle, at their stated sizes.

* 64 x 64 cells of 1000 m, daily, 365 steps (the FP64 parity run): the FP64 plain form over the
  whole year, outlet discharge compared every step, every land and river field every 73 steps, at
  relative 1e-9; the split form's errors over the same year.
* 1024 x 1024 cells of 250 m, hourly: both forms against the oracle. The default run takes the
  first 48 of the configuration's 720 steps (the oracle needs about 0.7 s per step of the
  1M-cell domain on 16 host threads); WF_CONFIG1_STEPS=720 runs the whole month.
* The frozen-soil infiltration reduction (soil_infiltration_reduction__flag with snow, the
  branch of soil.jl:711-729 consumed at :750) through a cold autumn and winter, both forms.

Closure is reported two ways. The reference's relative balance error (mass_balance.jl:84-93,
error / mean of in- and outflow) peaks in cells whose fluxes are ~1e-12 m s-1, for the FP64
oracle as well. The closure bar of the split form is the balance error over
max(local mean flux, median mean flux over the cells): the reference's relative error wherever
the flux is at least the median, bounded by the median flux elsewhere.
"""

import copy
import os

import numpy as np
import pytest

from wflow_gb300 import abi, synthetic
from wflow_gb300.model import Model
import oracle_py as O

from test_gpu_parity import LAND, RIVER, compare

pytestmark = pytest.mark.gpu

RTOL = 1e-9
THREADS = os.cpu_count() or 1


def closure(err, rel):
    """(max |relative error| as the reference defines it, max |error| / max(flux, median flux))
    of one balance; the local mean flux is |error / relative error| where the latter is non-zero."""
    err, rel = np.asarray(err), np.asarray(rel)
    nz = rel != 0.0
    flux = np.zeros_like(err)
    flux[nz] = np.abs(err[nz] / rel[nz])
    med = float(np.median(flux[nz])) if nz.any() else 1.0
    return float(np.max(np.abs(rel))), float(np.max(np.abs(err) / np.maximum(flux, med)))


def land_closure(src, get):
    return closure(get(src, "BALANCE_LAND_ERROR"), get(src, "BALANCE_LAND_RELATIVE_ERROR"))


def gpu_get(m, f):
    return m.get_value(f)


def orc_get(o, f):
    return o.get(abi.FIELD[f])


def run_config(dom, cfg, steps, seed=1, full_every=None, temp_offset=0.0, split=True, step0=0):
    """FP64 form and (optionally) split form against the oracle over `steps` steps; returns the
    worst FP64 errors of the full-field comparisons, the FP64 outlet error of every step and the
    split form's errors."""
    cfg64 = copy.copy(cfg)
    cfg64.form = abi.WF_FORM_FP64
    g64 = Model(cfg64, dom)
    orc = O.OracleModel(cfg64, dom)
    gsp = None
    if split:
        cfgs = copy.copy(cfg)
        cfgs.form = abi.WF_FORM_SPLIT
        gsp = Model(cfgs, dom)
    full = []
    out64 = 0.0
    sp = {"outlet_q": 0.0, "river_q": 0.0, "soil_storage": 0.0, "snow_storage": 0.0,
          "closure_rel": 0.0, "closure_flux": 0.0, "oracle_closure_rel": 0.0, "oracle_closure_flux": 0.0}
    for s in range(steps):
        P, PET, T = synthetic.forcing(step0 + s, cfg.dt, dom.n_land, seed=seed)
        T = T + temp_offset
        orc.set_forcing(P, PET, T)
        orc.step(THREADS)
        g64.run_timestep(P, PET, T)
        qo = orc.outlets(0)
        q64 = g64.outlets(0)
        out64 = max(out64, float(np.max(np.abs(q64 - qo) / np.maximum(np.abs(qo), 1e-300))))
        if full_every and ((s + 1) % full_every == 0 or s == steps - 1):
            full.append(compare(g64, orc, LAND + ["UNSATURATED_LAYER_DEPTH"] + (RIVER if dom.n_river else []),
                                layers=g64.N))
        if gsp is None:
            continue
        gsp.run_timestep(P, PET, T)
        qs = gsp.outlets(0)
        sp["outlet_q"] = max(sp["outlet_q"], float(np.max(np.abs(qs - qo) / np.maximum(np.abs(qo), 1e-12))))
        rq_o, rq_g = orc_get(orc, "RIVER_Q"), gsp.get_value("RIVER_Q")
        big = rq_o > 1e-3 * rq_o.max()
        if big.any():
            sp["river_q"] = max(sp["river_q"], float(np.max(np.abs(rq_g - rq_o)[big] / rq_o[big])))
        so, sg = orc_get(orc, "TOTAL_SOIL_WATER_STORAGE"), gsp.get_value("TOTAL_SOIL_WATER_STORAGE")
        sp["soil_storage"] = max(sp["soil_storage"], float(np.max(np.abs(sg - so) / so)))
        wo, wg = orc_get(orc, "SNOW_STORAGE"), gsp.get_value("SNOW_STORAGE")
        wbig = wo > 1e-4
        if wbig.any():
            sp["snow_storage"] = max(sp["snow_storage"], float(np.max(np.abs(wg - wo)[wbig] / wo[wbig])))
        r, f = land_closure(gsp, gpu_get)
        ro, fo = land_closure(orc, orc_get)
        sp["closure_rel"] = max(sp["closure_rel"], r)
        sp["closure_flux"] = max(sp["closure_flux"], f)
        sp["oracle_closure_rel"] = max(sp["oracle_closure_rel"], ro)
        sp["oracle_closure_flux"] = max(sp["oracle_closure_flux"], fo)
    return full, out64, sp


def assert_fp64(full, out64):
    assert out64 <= RTOL, out64
    for worst, exact_frac, inexact in full:
        bad = {k: v for k, v in worst.items() if v > RTOL}
        assert not bad, (bad, inexact)
        assert exact_frac >= 0.999, (exact_frac, inexact)


def assert_split(sp, soil=1e-4):
    assert sp["outlet_q"] <= 1e-4, sp
    assert sp["soil_storage"] <= soil, sp
    assert sp["closure_flux"] <= 1e-7, sp


def test_config_64_daily_full_year(gpu_lib):
    dom = synthetic.make_domain(64, 1000.0, seed=1)
    cfg = synthetic.make_config(86400.0)
    full, out64, sp = run_config(dom, cfg, 365, full_every=73)
    print("64x64 daily, 365 steps: FP64 outlet", out64, "split", sp)
    assert_fp64(full, out64)
    # a year of daily steps: the split form's FP32 rates move the slowest soil stores by up to
    # 7.3e-4 relative over the year (2e-6 after 40 days); the outlet discharge stays within 1e-4
    assert_split(sp, soil=1e-3)


def test_config_1024_hourly(gpu_lib):
    steps = int(os.environ.get("WF_CONFIG1_STEPS", "48"))
    dom = synthetic.make_domain(1024, 250.0, seed=1)
    cfg = synthetic.make_config(3600.0)
    full, out64, sp = run_config(dom, cfg, steps, full_every=max(steps // 2, 1))
    print(f"1024x1024 hourly, {steps} steps: FP64 outlet", out64, "split", sp)
    assert_fp64(full, out64)
    assert_split(sp)


def test_frozen_soil_infiltration_reduction(gpu_lib):
    # autumn and winter of the benchmark forcing (from day 231), 2 K colder: the soil surface
    # freezes and thaws, so the infiltration reduction factor (soil_process.jl:229-244) changes
    # the infiltration of about an eighth of the cell-steps
    dom = synthetic.make_domain(32, 1000.0, seed=31)
    cfg = synthetic.make_config(86400.0)
    cfg.soil_infiltration_reduction = 1
    full, out64, sp = run_config(dom, cfg, 120, seed=31, full_every=30, temp_offset=-2.0, step0=230)
    print("frozen soil: FP64 outlet", out64, "split", sp)
    assert_fp64(full, out64)
    assert_split(sp)
    # the flag changes the result: the same run without it differs
    cfg0 = synthetic.make_config(86400.0)
    a, b = Model(cfg, dom), Model(cfg0, dom)
    for s in range(40):
        P, PET, T = synthetic.forcing(230 + s, cfg.dt, dom.n_land, seed=31)
        a.run_timestep(P, PET, T - 2.0)
        b.run_timestep(P, PET, T - 2.0)
    assert not np.array_equal(a.get_value("ACTUAL_INFILTRATION"), b.get_value("ACTUAL_INFILTRATION"))
