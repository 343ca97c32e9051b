"""The GPU model fed from Wflow's files: a TOML configuration, its static maps, forcing and state
files (wflow_gb300.config, staticmaps, forcing, states), against the oracle fed from the same
files and against the GPU model built from the arrays the files were written from.

The files hold parameters and forcing in file units (mm, mm per step, degC) and the helpers
convert them as Wflow's to_SI does, so a value read back may differ from the array it was
written from by an ulp; the models built from files and from arrays therefore agree to 1e-12,
while the GPU and the oracle fed the same files agree to the FP64 form's 1e-9 (bit-identical
in practice). A warm start from a state file written by the GPU model (or by the oracle)
continues the run it was written from (set_states!, Wflow/src/utils.jl:150-213; the file
stores depths in mm, so a state may move by an ulp).
"""

import copy

import numpy as np
import pytest

from wflow_gb300 import abi, forcing, staticmaps, states, synthetic
from wflow_gb300.config import WflowConfig
from wflow_gb300.model import Model
import oracle_py as O

from test_config_cpu import FILE_NAMES, TOML

pytestmark = pytest.mark.gpu

FIELDS = ["RIVER_Q", "LAND_Q", "SSF_Q", "SATURATED_WATER_DEPTH", "SNOW_STORAGE", "CANOPY_STORAGE",
          "TOTAL_STORAGE"]


def rel(x, y):
    return float(np.max(np.abs(x - y) / np.maximum(np.abs(x), 1e-300)))


@pytest.fixture()
def files(tmp_path):
    (tmp_path / "data" / "input").mkdir(parents=True)
    (tmp_path / "data" / "output").mkdir(parents=True)
    (tmp_path / "sbm.toml").write_text(TOML)
    dom = synthetic.make_domain(32, 1000.0, seed=3)
    dom.params["crop_coefficient"] = np.ones(dom.n_land)
    staticmaps.write_staticmaps(dom, tmp_path / "data" / "input" / "staticmaps.nc", names=FILE_NAMES)
    cfg = WflowConfig(tmp_path / "sbm.toml")
    got, grid, _ = staticmaps.load_staticmaps(cfg.path_static, mapping=cfg.static)
    times = cfg.times()
    arrs = [synthetic.forcing(s, cfg.dt, dom.n_land, seed=1) for s in range(len(times))]
    forcing.write_forcing(cfg.path_forcing, grid, times, [a[0] for a in arrs], [a[1] for a in arrs],
                          [a[2] for a in arrs], cfg.dt, time_units=cfg.time_units)
    ff = forcing.ForcingFile(cfg.path_forcing, grid, cfg.dt, mapping=cfg.forcing)
    return cfg, dom, got, grid, times, arrs, ff


def test_gpu_model_from_toml_and_files(files):
    cfg, dom, got, grid, times, arrs, ff = files
    wcfg = cfg.wf_config()
    wcfg.form = abi.WF_FORM_FP64
    from_files = Model(wcfg, got)
    from_arrays = Model(wcfg, dom)
    orc = O.OracleModel(wcfg, got)
    for k, t in enumerate(times):
        P, PET, T = ff.at(t)
        from_files.run_timestep(P, PET, T)
        orc.set_forcing(P, PET, T)
        orc.step()
        from_arrays.run_timestep(*arrs[k])
        qo, qg = orc.outlets(0), from_files.outlets(0)
        assert np.all(np.abs(qg - qo) <= 1e-9 * np.abs(qo) + 1e-300), k
    for f in FIELDS:
        g = from_files.get_value(f)
        assert rel(orc.get(abi.FIELD[f]), g) <= 1e-9, f
        assert rel(from_arrays.get_value(f), g) <= 1e-12, f
    # the split form from the same files, within its stated error of the FP64 oracle
    scfg = copy.copy(wcfg)
    scfg.form = abi.WF_FORM_SPLIT
    sp = Model(scfg, got)
    for t in times:
        sp.run_timestep(*ff.at(t))
    qo, qs = orc.outlets(0), sp.outlets(0)
    assert np.max(np.abs(qs - qo) / np.maximum(np.abs(qo), 1e-12)) <= 1e-4


@pytest.mark.parametrize("writer", ["gpu", "oracle"])
def test_warm_start_from_a_state_file(files, writer):
    cfg, dom, got, grid, times, arrs, ff = files
    wcfg = cfg.wf_config()
    wcfg.form = abi.WF_FORM_FP64
    a = Model(wcfg, got)
    o = O.OracleModel(wcfg, got)
    for t in times[:3]:
        P, PET, T = ff.at(t)
        a.run_timestep(P, PET, T)
        o.set_forcing(P, PET, T)
        o.step()
    src = a if writer == "gpu" else o
    states.write_states(src, got, cfg.state_output, grid=grid, ncnames=cfg.state_ncnames, time=3.0)
    b = Model(wcfg, got)
    states.read_states(b, got, cfg.state_output, grid=grid, ncnames=cfg.state_ncnames)
    for f in ("SATURATED_WATER_DEPTH", "SNOW_STORAGE", "RIVER_Q", "SSF_Q"):
        assert rel(src.get_value(f) if writer == "gpu" else src.get(abi.FIELD[f]), b.get_value(f)) <= 1e-15, f
    # continue both: the restarted model follows the run that wrote the file
    for k in range(3, len(times)):
        P, PET, T = arrs[k]
        a.run_timestep(P, PET, T)
        b.run_timestep(P, PET, T)
    for f in FIELDS:
        assert rel(a.get_value(f), b.get_value(f)) <= 1e-10, f
