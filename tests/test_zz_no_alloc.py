"""wf_step_static, the allocation-free model step, against wf_step through the C ABI.

This file is collected last on purpose: it must pass after every other test (the static
scratch keeps the contents of earlier calls) as well as alone in a fresh process (the first
call on the device looks the scratch address up).
"""

import numpy as np
import pytest

from wflow_gb300 import abi, synthetic
from wflow_gb300.model import Model

pytestmark = pytest.mark.gpu

RTOL = 1e-9  # the tolerance of the FP64 parity tests
FIELDS = ["RIVER_Q", "RIVER_STORAGE", "LAND_Q", "LAND_H", "SSF_Q", "WATER_TABLE_DEPTH", "TOTAL_SOIL_WATER_STORAGE",
          "SNOW_STORAGE", "CANOPY_STORAGE", "RECHARGE", "BALANCE_LAND_ERROR", "BALANCE_RIVER_ERROR"]


def close(a, b):
    scale = np.maximum(np.maximum(np.abs(a), np.abs(b)), 1e-300)
    return np.abs(a - b) / scale <= RTOL


@pytest.mark.parametrize("form,dt", [(abi.WF_FORM_FP64, 3600.0), (abi.WF_FORM_SPLIT, 3600.0),
                                     (abi.WF_FORM_FP64, 86400.0)])
def test_static_step_matches_step(gpu_lib, form, dt):
    dom = synthetic.make_domain(32, 1000.0, seed=5)
    cfg = synthetic.make_config(dt, form=form)
    ref = Model(cfg, dom)
    sta = Model(cfg, dom)
    for s in range(2):  # two calls in a row on the same static scratch
        P, PET, T = synthetic.forcing(s, dt, dom.n_land, seed=3, precip_scale=3.0)
        ref.set_forcing(P, PET, T)
        sta.set_forcing(P, PET, T)
        ref.update_model()
        rc = sta.lib.wf_step_static(sta.h)
        assert rc == abi.WF_OK, sta.lib.wf_last_error(sta.h)
        qo_ref, qo_sta = ref.outlets(0), sta.outlets(0)
        assert np.all(close(qo_ref, qo_sta)), (s, qo_ref, qo_sta)
        for f in FIELDS:
            a, b = ref.get_value(f), sta.get_value(f)
            if f.startswith("BALANCE"):
                assert np.max(np.abs(a - b)) <= RTOL * (np.max(np.abs(ref.get_value("RECHARGE"))) + 1e-300), f
            else:
                assert np.all(close(a, b)), (s, f)
    m = sta.metrics()
    assert m["steps"] == 2


def test_static_step_leaves_device_memory_unchanged(gpu_lib):
    # after the first call (set-up: the scratch address lookup), further calls allocate nothing
    import torch
    dom = synthetic.make_domain(32, 1000.0, seed=7)
    cfg = synthetic.make_config(3600.0, form=abi.WF_FORM_SPLIT)
    sta = Model(cfg, dom)
    P, PET, T = synthetic.forcing(0, 3600.0, dom.n_land, seed=7)
    sta.set_forcing(P, PET, T)
    assert sta.lib.wf_step_static(sta.h) == abi.WF_OK
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info(0)[0]
    for s in range(1, 4):
        P, PET, T = synthetic.forcing(s, 3600.0, dom.n_land, seed=7)
        sta.set_forcing(P, PET, T)
        assert sta.lib.wf_step_static(sta.h) == abi.WF_OK
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info(0)[0] == free0
    assert sta.metrics()["steps"] == 4


def test_static_step_rejects_models_beyond_the_scratch(gpu_lib):
    # daily steps with 3600 s overland sub-steps: 24 published discharges per land chain end and
    # member in one launch
    dom = synthetic.make_domain(96, 1000.0, seed=6)
    members = 32
    cfg = synthetic.make_config(86400.0, n_members=members, form=abi.WF_FORM_FP64)
    model = Model(cfg, dom)
    m = model.metrics()

    def need(chains, substeps):  # scratch of one sweep launch (see wf_step_static)
        slots = chains * members
        return 256 + (slots * 4 + 255) // 256 * 256 + slots * substeps * 8

    # land launches carry 24 overland sub-steps (3600 s), river launches 32 of the 96 (900 s):
    # the FP64 walker takes at most 32 sub-steps per launch
    need_max = max(need(m["n_chains_land"], 24), need(m["n_chains_river"], 32))
    assert need_max > abi.WF_STATIC_SCRATCH_BYTES, need_max
    rc = model.lib.wf_step_static(model.h)
    assert rc == abi.WF_ERR_UNSUPPORTED
    msg = model.lib.wf_last_error(model.h)
    msg = msg.decode() if isinstance(msg, bytes) else msg
    assert "static scratch" in msg and str(need_max) in msg, msg
    # the model is untouched and still steps through the regular entry point
    P, PET, T = synthetic.forcing(0, 86400.0, dom.n_land * members, seed=1)
    model.run_timestep(P, PET, T)
    assert model.metrics()["steps"] == 1
