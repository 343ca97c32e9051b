"""The local-inertial river on the GPU (include/wflow_gb300_li.h) against the CPU oracle.

The component runs Wflow's river_routing = "local_inertial" for a channel without floodplain:
edge discharge from local_inertial_flow (routing/surface/surface_process.jl:88-115), cell
storage and depth (surface_staggered_scheme.jl:326-385, 723-760), sub-steps of the stable time
step (:1004-1020) inside a model step (update_river_flow_model!, :800-826). The arithmetic is
FP64 in the oracle's order, so every field is held to relative 1e-9 (the drop-in bar); the
sub-step counts must be equal. MacDonald's long channel (routing_process.jl:1189-1318) run on
the GPU to steady state reproduces the reference's mean absolute depth error
0.01873574206931199 within Julia's default isapprox tolerance (sqrt(eps)).

The land grid with its river (wf_li_domain_*, update_overland_flow_model!, :1153-1193) is held to
the same bar on a grid with a main river and a tributary, from a warm and a cold state.

The argument checks of wf_li_river_create and wf_li_domain_create run before any device call and
are tested on CPU.
"""

import numpy as np
import pytest

from li_cases import OracleLi, macdonald_case, random_river

FIELDS = ("h", "storage", "q", "q_cumulative", "q_average", "error", "abstraction_cumulative")
ORACLE_ATTR = {"h": "h", "storage": "storage", "q": "q", "q_cumulative": "q_cum", "q_average": "q_avg",
               "error": "error", "abstraction_cumulative": "abs_cum"}


def _river(net, **kw):
    from wflow_gb300.li_river import LiRiver
    return LiRiver(net["src"], net["dst"], net["zb"], net["flow_length"], net["flow_width"], net["h"], net["zb_e"],
                   net["w_e"], net["l_e"], net["nsq_e"], net["n_active"], **kw)


def _max_rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    if a.size == 0:
        return 0.0
    return float(np.max(np.abs(a - b) / np.maximum(np.maximum(np.abs(a), np.abs(b)), 1e-300)))


def _assert_same(gpu, orc, tag):
    for f in FIELDS:
        g, o = gpu.get(f), getattr(orc, ORACLE_ATTR[f])
        assert g.shape == o.shape, (tag, f)
        assert _max_rel(g, o) <= 1e-9, (tag, f, _max_rel(g, o))


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [0, 1])
def test_random_river_steps(gpu_lib, seed):
    """Three hourly model steps of a 3000-cell river tree with confluences, four outlets of
    fixed depth, wet, dry and near-threshold starting depths, lateral inflow, abstractions and
    positive and negative external inflows."""
    net = random_river(seed)
    gpu, orc = _river(net), OracleLi(net)
    for m in (gpu, orc):
        m.set_state(net["h"])
        m.set_inwater(net["inwater"])
        m.set_boundary(net["external_inflow"], net["abstraction"])
    for step in range(3):
        k_gpu, k_orc = gpu.step(3600.0), orc.step(3600.0)
        assert k_gpu == k_orc, (seed, step, k_gpu, k_orc)
        _assert_same(gpu, orc, (seed, step))
    gpu.close()


@pytest.mark.gpu
def test_substeps_and_warm_discharge(gpu_lib):
    """Explicit sub-steps from a warm state with discharge on the edges, and the stable time
    step of each, without lateral inflow (the network drains and cells fall dry)."""
    net = random_river(7, n_active=500, n_bound=2)
    rng = np.random.default_rng(7)
    q0 = rng.uniform(-2.0, 20.0, len(net["src"]))
    gpu, orc = _river(net, h_thresh=1e-3, froude_limit=False, alpha=0.5), OracleLi(net, froude=False, alpha=0.5)
    for m in (gpu, orc):
        m.set_state(net["h"], q0)
        m.set_inwater(np.zeros(net["n"]))
    for s in range(40):
        dt_g, dt_o = gpu.stable_timestep(), orc.stable_timestep()
        assert _max_rel(dt_g, dt_o) <= 1e-12, (s, dt_g, dt_o)
        gpu.substep(dt_o)
        orc.substep(dt_o)
    for f in ("h", "storage", "q", "q_cumulative"):
        assert _max_rel(gpu.get(f), getattr(orc, ORACLE_ATTR[f])) <= 1e-9, f
    gpu.close()


@pytest.mark.gpu
def test_time_step_over_real_cells(gpu_lib):
    """A Wflow model's river: the stable time step over the real cells only, the outlets' ghost
    cells (fixed depth) after them (stable_timestep loops over parameters.n)."""
    net = random_river(11, n_active=800, n_bound=3)
    gpu, orc = _river(net), OracleLi(net)
    for m in (gpu, orc):
        m.set_timestep_cells(net["n_active"])
        m.set_state(net["h"])
        m.set_inwater(net["inwater"])
    assert gpu.step(3600.0) == orc.step(3600.0)
    _assert_same(gpu, orc, "real cells")
    gpu.close()


@pytest.mark.gpu
def test_dry_network_time_step(gpu_lib):
    """Every cell dry: the stable time step is the 60 s default and a sub-step moves nothing."""
    net = random_river(3, n_active=300, n_bound=2)
    net = dict(net, h=np.zeros(net["n"]))
    gpu = _river(net)
    assert gpu.stable_timestep() == 60.0
    gpu.substep(60.0)
    for f in FIELDS[:4]:
        assert not np.any(gpu.get(f)), f
    gpu.close()


@pytest.mark.gpu
def test_macdonald_steady_state(gpu_lib):
    pytest.importorskip("scipy.integrate")
    a = dict(L=1000.0, dx=5.0, width=10.0, mannings_n=0.03, h_thresh=1e-3, alpha=0.7, epsilon=1e-12, inflow=20.0)
    net, h_a = macdonald_case(a)
    runs = {}
    for name, m in (("gpu", _river(net, h_thresh=a["h_thresh"], alpha=a["alpha"])),
                    ("oracle", OracleLi(net, h_thresh=a["h_thresh"], alpha=a["alpha"]))):
        inw = np.zeros(net["n"])
        inw[0] = a["inflow"]
        m.set_inwater(inw)
        h = np.array(net["h"], float)
        for it in range(1_000_000):
            h0 = h.mean()
            m.substep(m.stable_timestep())
            h = m.get("h") if name == "gpu" else m.h
            if abs(h0 - h.mean()) <= a["epsilon"]:
                break
        runs[name] = (it, float(np.mean(np.abs(h - h_a))))
    assert runs["gpu"][0] == runs["oracle"][0], runs
    assert _max_rel(runs["gpu"][1], runs["oracle"][1]) <= 1e-9, runs
    assert np.isclose(runs["gpu"][1], 0.01873574206931199, rtol=np.sqrt(np.finfo(float).eps), atol=0.0), runs


DOMAIN_FIELDS = ("h_land", "storage", "error", "qx", "qy", "qx_average", "qy_average", "h_river", "storage_river",
                 "q_river", "q_river_average", "abstraction_cumulative")


def _domain(land, river, h_river):
    from wflow_gb300.li_river import LiDomain
    return LiDomain(land, river, h_river)


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [0, 1])
def test_land_domain_steps(gpu_lib, seed):
    """Two hourly steps of the land grid with its river (update_overland_flow_model!,
    surface_staggered_scheme.jl:1153-1193): a 36 x 28 grid, main river and tributary, closed
    edges, an abstraction, a negative and a positive external inflow, a warm state with cells over
    bankfull. Every land and river field within relative 1e-9 of the oracle, equal sub-step
    counts, and the stable time step of the final state."""
    from li_cases import OracleLiDomain, random_land_domain
    land, river, h_river, state, inputs = random_land_domain(seed)
    gpu, orc = _domain(land, river, h_river), OracleLiDomain(land, river, h_river)
    for m in (gpu, orc):
        m.set_state(**state)
        m.set_inputs(**inputs)
    for step in range(2):
        k_gpu, k_orc = gpu.step(3600.0), orc.step(3600.0)
        assert k_gpu == k_orc, (seed, step, k_gpu, k_orc)
        for f in DOMAIN_FIELDS:
            assert _max_rel(gpu.get(f), orc.get(f)) <= 1e-9, (seed, step, f)
    assert _max_rel(gpu.stable_timestep(), orc.stable_timestep()) <= 1e-12
    gpu.close()


@pytest.mark.gpu
def test_land_domain_cold_start_substeps(gpu_lib):
    """A cold start (dry land and river but the ghost cell) under runoff, by explicit sub-steps."""
    from li_cases import OracleLiDomain, random_land_domain
    land, river, h_river, _, inputs = random_land_domain(4, nx=20, ny=16)
    gpu, orc = _domain(land, river, h_river), OracleLiDomain(land, river, h_river)
    for m in (gpu, orc):
        m.set_inputs(inputs["runoff"])
    for s in range(60):
        dt_g, dt_o = gpu.stable_timestep(), orc.stable_timestep()
        assert _max_rel(dt_g, dt_o) <= 1e-12, (s, dt_g, dt_o)
        gpu.substep(dt_o)
        orc.substep(dt_o)
    for f in ("h_land", "storage", "error", "qx", "qy", "h_river", "storage_river", "q_river"):
        assert _max_rel(gpu.get(f), orc.get(f)) <= 1e-9, f
    gpu.close()


def test_domain_create_rejects_bad_grids():
    """Argument checks of wf_li_domain_create (no device call is reached)."""
    from wflow_gb300 import build
    from li_cases import random_land_domain
    build.build_all()
    land, river, h_river, _, _ = random_land_domain(5, nx=10, ny=8)
    ri = land["river_index"]
    r0 = int(np.flatnonzero(ri == 0)[0])
    dup = ri.copy()
    dup[np.flatnonzero(ri < 0)[0]] = 0
    with pytest.raises(RuntimeError, match="two land cells hold one river cell"):
        _domain(dict(land, river_index=dup), river, h_river)
    gap = ri.copy()
    gap[r0] = -1
    with pytest.raises(RuntimeError, match="lies in no land cell"):
        _domain(dict(land, river_index=gap), river, h_river)
    bad = land["ind_x_down"].copy()
    bad[0] = len(bad) + 1
    with pytest.raises(RuntimeError, match="neighbour index out of range"):
        _domain(dict(land, ind_x_down=bad), river, h_river)
    ghost = ri.copy()
    ghost[r0] = river["n_active"]
    with pytest.raises(RuntimeError, match="active river cell"):
        _domain(dict(land, river_index=ghost), river, h_river)
    with pytest.raises(ValueError, match="h_river"):
        _domain(land, river, h_river[:-1])


def test_create_rejects_bad_networks():
    """Argument checks of wf_li_river_create (no device call is reached)."""
    from wflow_gb300 import abi, build
    from wflow_gb300.li_river import LiRiver
    build.build_all()
    net = random_river(1, n_active=20, n_bound=1)

    def make(**over):
        t = dict(net, **over)
        return LiRiver(t["src"], t["dst"], t["zb"], t["flow_length"], t["flow_width"], t["h"], t["zb_e"], t["w_e"],
                       t["l_e"], t["nsq_e"], t.get("n_active", net["n_active"]), alpha=t.get("alpha", 0.7))

    bad_dst = net["dst"].copy()
    bad_dst[3] = net["n"]
    with pytest.raises(RuntimeError, match=f"failed \\({abi.WF_ERR_INVALID}\\).*out of range"):
        make(dst=bad_dst)
    self_loop = net["dst"].copy()
    self_loop[2] = net["src"][2]
    with pytest.raises(RuntimeError, match="out of range"):
        make(dst=self_loop)
    fl = net["flow_length"].copy()
    fl[0] = 0.0
    with pytest.raises(RuntimeError, match="positive on active cells"):
        make(flow_length=fl)
    with pytest.raises(RuntimeError, match="sizes out of range"):
        make(n_active=net["n"] + 1)
    with pytest.raises(RuntimeError, match="alpha must be positive"):
        make(alpha=0.0)
    with pytest.raises(ValueError, match="zb_edge"):
        make(zb_e=net["zb_e"][:-1])


@pytest.mark.gpu
def test_device_and_host_sub_step_loops_agree(gpu_lib):
    """The device-side sub-step loop (one cooperative launch per model step, grid barriers) and
    the host-driven loop take the same sub-steps to the same states, bit for bit, for the river
    alone and for the land grid with its river."""
    from li_cases import random_land_domain
    net = random_river(2)
    a, b = _river(net), _river(net)
    b.set_host_loop(True)
    for m in (a, b):
        m.set_state(net["h"])
        m.set_inwater(net["inwater"])
        m.set_boundary(net["external_inflow"], net["abstraction"])
    for step in range(3):
        assert a.step(3600.0) == b.step(3600.0), step
        for f in FIELDS:
            assert np.array_equal(a.get(f), b.get(f)), (step, f)
    land, river, h_river, state, inputs = random_land_domain(3)
    c, d = _domain(land, river, h_river), _domain(land, river, h_river)
    d.set_host_loop(True)
    for m in (c, d):
        m.set_state(**state)
        m.set_inputs(**inputs)
    for step in range(3):
        assert c.step(3600.0) == d.step(3600.0), step
        for f in DOMAIN_FIELDS:
            assert np.array_equal(c.get(f), d.get(f)), (step, f)
    for m in (a, b, c, d):
        m.close()


# ---- local-inertial land and river routing inside the SBM step (wf_attach_local_inertial) ----

COUPLED_FIELDS = ["LAND_H", "LAND_STORAGE", "RIVER_H", "RIVER_STORAGE", "RIVER_Q", "TOTAL_STORAGE",
                  "SATURATED_WATER_DEPTH", "SSF_Q", "NET_RUNOFF", "BALANCE_LAND_ERROR", "BALANCE_OVERLAND_ERROR"]


def _coupled_pair(dom, dt, warm, seed):
    from wflow_gb300 import abi, synthetic
    from wflow_gb300.li_river import LiDomain
    from wflow_gb300.model import Model
    import oracle_py as O
    cfg = synthetic.make_config(dt, form=abi.WF_FORM_FP64)
    land, river, h_land, h_river = synthetic.li_coupling(dom, seed=seed, warm=warm)
    d = LiDomain(land, river, h_river)
    d.set_state(h_land, h_river)
    gpu = Model(cfg, dom)
    gpu.attach_local_inertial(d)
    orc = O.OracleModel(cfg, dom)
    orc.attach_li(land, river, h_land, h_river)
    return cfg, gpu, orc, d


@pytest.mark.gpu
@pytest.mark.parametrize("dt,warm,side", [(86400.0, True, 32), (3600.0, False, 48)])
def test_coupled_sbm_step_matches_oracle(gpu_lib, dt, warm, side):
    from wflow_gb300 import abi, synthetic
    import os
    dom = synthetic.make_domain(side, 250.0, seed=8)
    cfg, gpu, orc, d = _coupled_pair(dom, dt, warm, seed=8)
    threads = os.cpu_count() or 1
    total = 0
    for s in range(6):
        P, PET, T = synthetic.forcing(s, dt, dom.n_land, seed=8, precip_scale=4.0)
        gpu.run_timestep(P, PET, T)
        orc.set_forcing(P, PET, T)
        orc.step(threads)
        qo, qg = orc.outlets(0), gpu.outlets(0)
        assert _max_rel(qg, qo) <= 1e-9, (s, _max_rel(qg, qo))
        for f in COUPLED_FIELDS:
            g, o = gpu.get_value(f), orc.get(abi.FIELD[f])
            if "ERROR" in f:  # balance errors: absolute, against the step's fluxes
                assert np.max(np.abs(g - o)) <= 1e-9 * (np.max(np.abs(o)) + 1e-12), (s, f)
            else:
                assert _max_rel(g, o) <= 1e-9, (s, f, _max_rel(g, o))
        total += int(orc.li_get(-1)[0])
        assert gpu.metrics()["substeps_land"] == total, s  # the same sub-steps as the oracle
    for name, field in (("h_land", 0), ("storage", 1), ("qx_average", 5), ("h_river", 7), ("q_river", 9)):
        assert _max_rel(d.get(name), orc.li_get(field)[:len(d.get(name))]) <= 1e-9, name
    assert np.all(gpu.get_value("BALANCE_RIVER_ERROR") == 0.0)
    assert d.get("h_land").max() > 0.0


@pytest.mark.gpu
def test_coupling_refuses_what_it_cannot_take(gpu_lib):
    from wflow_gb300 import abi, synthetic
    from wflow_gb300.li_river import LiDomain
    from wflow_gb300.model import Model
    dom = synthetic.make_domain(16, 250.0, seed=9)
    land, river, h_land, h_river = synthetic.li_coupling(dom, seed=9)
    d = LiDomain(land, river, h_river)
    for kw in (dict(form=abi.WF_FORM_SPLIT), dict(n_members=2), dict(adaptive=True)):
        m = Model(synthetic.make_config(86400.0, **{"form": abi.WF_FORM_FP64, **kw}), dom)
        with pytest.raises(RuntimeError):
            m.attach_local_inertial(d)
    other = synthetic.make_domain(12, 250.0, seed=9)
    with pytest.raises(RuntimeError):
        Model(synthetic.make_config(86400.0, form=abi.WF_FORM_FP64), other).attach_local_inertial(d)


@pytest.mark.gpu
@pytest.mark.parametrize("host_loop", [False, True])
def test_manning_river_matches_oracle(gpu_lib, host_loop):
    # river_routing = "manning_staggered": Manning's equation at the edges (upstream depth,
    # discharge limited to the upstream storage), the edges' stable sub-step
    from li_cases import manning_edges
    net = random_river(7, n_active=2000)
    slope_e, n_e = manning_edges(net)
    gpu = _river(net)
    gpu.set_manning(slope_e, n_e)
    gpu.set_host_loop(host_loop)
    orc = OracleLi(net)
    orc.set_manning(slope_e, n_e)
    gpu.set_state(net["h"])
    orc.set_state(net["h"])
    gpu.set_inwater(net["inwater"])
    orc.set_inwater(net["inwater"])
    gpu.set_boundary(net["external_inflow"], net["abstraction"])
    orc.set_boundary(net["external_inflow"], net["abstraction"])
    for s in range(3):
        kg, ko = gpu.step(3600.0), orc.step(3600.0)
        assert kg == ko, (s, kg, ko)
        _assert_same(gpu, orc, f"manning step {s}")
    assert np.all(gpu.get("q") >= 0.0)
