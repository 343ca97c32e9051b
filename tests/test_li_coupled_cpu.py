"""Local-inertial land and river routing inside the oracle's model step (CPU).

With land_routing = river_routing = "local_inertial", Wflow's surface_routing!
(Wflow/src/routing/surface/surface_routing.jl:62-89) sets the land runoff of the step to
(net_runoff + net_runoff_river) * area plus the subsurface flow to the river at river cells
(update_bc_overland_flow_model!, surface_staggered_scheme.jl:1080-1097) and runs
update_overland_flow_model! (:1153-1193). Checked here: the oracle's coupled step equals the
standalone scheme (tests/li_cases.OracleLiDomain) driven by that runoff, bit for bit; the model
takes the scheme's depths and storages; the overland balance of mass_balance.jl:402-461 closes;
the options the coupling cannot take are refused.
"""

import numpy as np
import pytest

from wflow_gb300 import abi, synthetic
import oracle_py as O
from li_cases import OracleLiDomain

F = abi.FIELD


def coupled(dom, dt, warm=True, seed=1):
    cfg = synthetic.make_config(dt, form=abi.WF_FORM_FP64)
    o = O.OracleModel(cfg, dom)
    land, river, h_land, h_river = synthetic.li_coupling(dom, seed=seed, warm=warm)
    o.attach_li(land, river, h_land, h_river)
    ref = OracleLiDomain(land, river, h_river)
    ref.set_state(h_land, h_river)
    return cfg, o, ref, land, river


@pytest.mark.parametrize("dt,warm", [(86400.0, True), (3600.0, False)])
def test_coupled_step_is_the_scheme_driven_by_the_runoff(dt, warm):
    dom = synthetic.make_domain(20, 250.0, seed=6)
    cfg, o, ref, land, river = coupled(dom, dt, warm)
    rl = np.asarray(dom.river["river_land_index"])
    area = dom.land["area"]
    for s in range(4):
        P, PET, T = synthetic.forcing(s, dt, dom.n_land, seed=6, precip_scale=4.0)
        o.set_forcing(P, PET, T)
        o.step()
        runoff = (o.get(F["NET_RUNOFF"]) + o.get(F["NET_RUNOFF_RIVER"])) * area
        runoff[rl] += o.get(F["SSF_TO_RIVER_AVERAGE"])[rl]
        ref.set_inputs(runoff, np.concatenate([dom.river["river_external_inflow"],
                                               np.zeros(len(river["zb"]) - dom.n_river)]))
        k = ref.step(dt)
        assert o.li_get(-1)[0] == k
        for name, field in (("h_land", 0), ("storage", 1), ("h_river", 7), ("q_river", 9),
                            ("q_river_average", 10), ("qx_average", 5)):
            assert np.array_equal(ref.get(name), o.li_get(field)[:len(ref.get(name))]), (s, name)
        # the model's overland and river variables are the scheme's
        assert np.array_equal(o.get(F["LAND_H"]), ref.get("h_land"))
        assert np.array_equal(o.get(F["RIVER_H"]), ref.get("h_river")[:dom.n_river])
        q_out = ref.get("q_river")[river["src"] >= 0][:dom.n_river]
        assert np.array_equal(o.get(F["RIVER_Q"]), q_out)
    # closure over max(local mean flux, median mean flux): the reference's relative error reads
    # up to 2 in cells whose fluxes are ~1e-36 m3 s-1 (an error of 5e-36)
    for err_f, rel_f in (("BALANCE_OVERLAND_ERROR", "BALANCE_OVERLAND_RELATIVE_ERROR"),
                         ("BALANCE_LAND_ERROR", "BALANCE_LAND_RELATIVE_ERROR")):
        err, rel = o.get(F[err_f]), o.get(F[rel_f])
        nz = rel != 0.0
        flux = np.zeros_like(err)
        flux[nz] = np.abs(err[nz] / rel[nz])
        med = float(np.median(flux[nz])) if nz.any() else 1.0
        assert float(np.max(np.abs(err) / np.maximum(flux, med))) < 1e-9, err_f
    assert np.all(o.get(F["BALANCE_RIVER_ERROR"]) == 0.0)
    assert ref.get("h_land").max() > 0.0


def test_coupling_refuses_what_it_cannot_take():
    dom = synthetic.make_domain(16, 250.0, seed=7)
    land, river, h_land, h_river = synthetic.li_coupling(dom)
    cfg = synthetic.make_config(86400.0, n_members=2)
    with pytest.raises(RuntimeError):
        O.OracleModel(cfg, dom).attach_li(land, river, h_land, h_river)
    cfg = synthetic.make_config(86400.0, adaptive=True)
    with pytest.raises(RuntimeError):
        O.OracleModel(cfg, dom).attach_li(land, river, h_land, h_river)
    bad = dict(land, river_index=np.roll(land["river_index"], 1))
    with pytest.raises(RuntimeError):
        O.OracleModel(synthetic.make_config(86400.0), dom).attach_li(bad, river, h_land, h_river)
