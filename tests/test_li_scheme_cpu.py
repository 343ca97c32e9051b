"""The local-inertial river scheme's arithmetic (wflow.jl_gb300/csrc/li_scheme.cuh, the functions
the GPU kernels call) built for the host and compared with the oracle, bit for bit.

Random river trees with confluences, outlets of fixed depth, dry and near-threshold cells and
lateral inflow over hourly model steps (update_river_flow_model!, surface_staggered_scheme.jl:
800-826), and MacDonald's long channel (routing_process.jl:1189-1318) run to steady state with
the reference's mean depth error 0.01873574206931199 within Julia's isapprox tolerance.
"""

import ctypes as C
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from li_cases import OracleLi, _pd, _pl, macdonald_case, random_river

REPO = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def host_lib(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    out = tmp_path_factory.mktemp("li_host") / "li_host.so"
    subprocess.run([cxx, "-O2", "-ffp-contract=off", "-std=c++17", "-shared", "-fPIC",
                    "-I", str(REPO / "wflow.jl_gb300" / "csrc"), "-I", str(REPO / "include"),
                    str(REPO / "tests" / "li_host_driver.cpp"), "-o", str(out)], check=True)
    lib = C.CDLL(str(out))
    lib.host_li_stable_timestep.restype = C.c_double
    return lib


class HostLi(OracleLi):
    """OracleLi's driver over the host build of the product's scheme functions."""

    def __init__(self, lib, net, **kw):
        super().__init__(net, **kw)
        self.H = lib

    def stable_timestep(self):
        return self.H.host_li_stable_timestep(C.c_int64(self.n_dt), _pd(self.net["flow_length"]), _pd(self.h),
                                              C.c_double(self.alpha))

    def substep(self, dt):
        t = self.net
        self.H.host_li_substep(C.c_int64(self.n), C.c_int64(self.na), C.c_int64(self.ne), _pl(t["src"]), _pl(t["dst"]),
                               _pd(t["zb"]), _pd(t["flow_length"]), _pd(t["flow_width"]), _pd(self.inwater),
                               _pd(t["zb_e"]), _pd(t["w_e"]), _pd(t["l_e"]), _pd(t["nsq_e"]),
                               C.c_double(self.h_thresh), C.c_int32(int(self.froude)), C.c_double(dt), _pd(self.h),
                               _pd(self.storage), _pd(self.q), _pd(self.q_prev), _pd(self.q_cum),
                               _pd(self.abstraction), _pd(self.external_inflow), _pd(self.error), _pd(self.abs_cum))


@pytest.mark.parametrize("seed,froude,alpha", [(0, True, 0.7), (1, False, 0.5)])
def test_random_river_bit_identical(host_lib, seed, froude, alpha):
    net = random_river(seed, n_active=1500)
    a, b = OracleLi(net, froude=froude, alpha=alpha), HostLi(host_lib, net, froude=froude, alpha=alpha)
    for m in (a, b):
        m.set_state(net["h"])
        m.set_inwater(net["inwater"])
        m.set_boundary(net["external_inflow"], net["abstraction"])
    for step in range(2):
        assert a.step(3600.0) == b.step(3600.0)
        for f in ("h", "storage", "q", "q_prev", "q_cum", "q_avg", "error", "abs_cum"):
            assert np.array_equal(getattr(a, f), getattr(b, f)), (seed, step, f)
    assert a.abs_cum.sum() > 0.0
    assert (net["h"] == 0.0).any() and (np.abs(net["h"] - 1e-3) < 5e-4).any()  # dry and near-threshold starts
    assert np.abs(a.q).max() > 0.0


def test_macdonald_bit_identical(host_lib):
    pytest.importorskip("scipy.integrate")
    a = dict(L=1000.0, dx=5.0, width=10.0, mannings_n=0.03, h_thresh=1e-3, alpha=0.7, epsilon=1e-12, inflow=20.0)
    net, h_a = macdonald_case(a)
    runs = []
    for m in (OracleLi(net, alpha=a["alpha"]), HostLi(host_lib, net, alpha=a["alpha"])):
        inw = np.zeros(net["n"])
        inw[0] = a["inflow"]
        m.set_inwater(inw)
        for it in range(1_000_000):
            h0 = m.h.mean()
            m.substep(m.stable_timestep())
            if abs(h0 - m.h.mean()) <= a["epsilon"]:
                break
        runs.append((it, m.h.copy()))
    assert runs[0][0] == runs[1][0]
    assert np.array_equal(runs[0][1], runs[1][1])
    err = float(np.mean(np.abs(runs[1][1] - h_a)))
    assert np.isclose(err, 0.01873574206931199, rtol=np.sqrt(np.finfo(float).eps), atol=0.0), err


def test_dry_network_default_time_step(host_lib):
    net = random_river(3, n_active=200, n_bound=2)
    m = HostLi(host_lib, dict(net, h=np.zeros(net["n"])))
    assert m.stable_timestep() == 60.0


# ---- the land grid with its river -----------------------------------------------------------

DOMAIN_FIELDS = ("h_land", "storage", "error", "qx", "qy", "qx_average", "qy_average", "h_river", "storage_river",
                 "q_river", "q_river_average", "abstraction_cumulative")


def _host_domain_class(lib):
    from li_cases import OracleLiDomain, OrcLiState

    class HostLiDomain(OracleLiDomain):
        """OracleLiDomain's driver over the host build of the product's scheme functions, with
        the device's two swapped discharge buffers per direction."""

        def stable_timestep(self):
            return lib.host_li_domain_stable_timestep(C.byref(self.g), C.byref(self.r), C.byref(self.st))

        def substep(self, dt):
            a = self.a
            a["qx"], a["qx0"] = a["qx0"], a["qx"]
            a["qy"], a["qy0"] = a["qy0"], a["qy"]
            self.st = OrcLiState(**{k: _pd(v) for k, v in a.items()})
            lib.host_li_domain_substep(C.byref(self.g), C.byref(self.r), _pd(self.runoff), _pd(self.ext),
                                       _pd(self.abs), C.c_double(dt), C.byref(self.st))

    lib.host_li_domain_stable_timestep.restype = C.c_double
    return HostLiDomain


def test_struct_sizes_match_python(host_lib):
    from wflow_gb300.li_river import WfLiLandGrid, WfLiRiverNetwork
    out = np.zeros(2, np.int64)
    host_lib.host_li_struct_sizes(_pl(out))
    assert list(out) == [C.sizeof(WfLiLandGrid), C.sizeof(WfLiRiverNetwork)]


@pytest.mark.parametrize("seed,variant", [(0, None), (1, None), (2, "no_froude"), (3, "theta_1"), (4, "alpha_0.4")])
def test_land_domain_bit_identical(host_lib, seed, variant):
    """Two hourly steps of a 36 x 28 grid with a main river, a tributary, closed edges, an
    abstraction, a negative and a positive external inflow, from a warm state with cells over
    bankfull: every land and river field equal to the oracle's, with equal sub-step counts. The
    variants switch the Froude limit off (land and river), set theta to 1 (no neighbour
    weighting) and lower both stability coefficients."""
    from li_cases import OracleLiDomain, random_land_domain
    land, river, h_river, state, inputs = random_land_domain(seed)
    if variant == "no_froude":
        land, river = dict(land, froude_limit=False), dict(river, froude_limit=False)
    elif variant == "theta_1":
        land = dict(land, theta=1.0)
    elif variant == "alpha_0.4":
        land, river = dict(land, alpha=0.4), dict(river, alpha=0.4)
    a = OracleLiDomain(land, river, h_river)
    b = _host_domain_class(host_lib)(land, river, h_river)
    for m in (a, b):
        m.set_state(**state)
        m.set_inputs(**inputs)
    for step in range(2):
        assert a.step(3600.0) == b.step(3600.0)
        for f in DOMAIN_FIELDS:
            assert np.array_equal(a.get(f), b.get(f)), (seed, step, f)
    assert a.get("abstraction_cumulative").sum() > 0.0 and a.get("error").sum() > 0.0
    assert (state["h_land"][land["river_index"] >= 0] > 0.0).any()  # some river cells start over bankfull


def test_land_domain_dry_time_step(host_lib):
    """A dry grid whose river is dry but for its ghost cell: the ghost cells are outside the
    river's minimum (stable_timestep loops over parameters.n, the real river cells), so both
    minima are infinite and the step is the 60 s default; one wet river cell sets it."""
    from li_cases import random_land_domain
    land, river, h_river, _, _ = random_land_domain(2, nx=12, ny=10)
    H = _host_domain_class(host_lib)
    m = H(land, river, h_river)
    assert h_river[-1] > 0.0 and m.stable_timestep() == 60.0
    wet = h_river.copy()
    wet[3] = 0.4
    m = H(land, river, wet)
    g = 9.80665
    assert m.stable_timestep() == min(60.0, river["alpha"] * river["flow_length"][3] / np.sqrt(g * 0.4))


def test_bench_grid_is_valid_and_matches_oracle(host_lib):
    """The throughput grid of the local-inertial benchmark workload (synthetic.li_grid): every
    river cell in one land cell, edges in range, and its first sub-steps on the host build equal
    to the oracle's."""
    from li_cases import OracleLiDomain
    from wflow_gb300 import synthetic
    land, river, h_river, h_land, runoff = synthetic.li_grid(96, 100)
    ri, nra = land["river_index"], river["n_active"]
    assert sorted(ri[ri >= 0].tolist()) == list(range(nra))
    assert river["src"].max() < nra and river["dst"].max() < len(river["zb"])
    a = OracleLiDomain(land, river, h_river)
    b = _host_domain_class(host_lib)(land, river, h_river)
    for m in (a, b):
        m.set_state(h_land, h_river)
        m.set_inputs(runoff)
    for _ in range(5):
        dt = a.stable_timestep()
        assert dt == b.stable_timestep()
        a.substep(dt)
        b.substep(dt)
    for f in DOMAIN_FIELDS[:5] + DOMAIN_FIELDS[7:10]:
        assert np.array_equal(a.get(f), b.get(f)), f


def test_manning_river_oracle_conserves_water():
    # Manning's equation on the staggered grid (river_routing = "manning_staggered") in the oracle:
    # discharge flows downhill only, never takes more than the upstream storage over a sub-step,
    # and the water of the active cells changes by the inflows minus the outflow to the boundary
    from li_cases import OracleLi, manning_edges, random_river
    net = random_river(5, n_active=600)
    o = OracleLi(net, alpha=0.7)
    o.set_manning(*manning_edges(net))
    o.set_state(net["h"])
    o.set_inwater(net["inwater"])
    na = net["n_active"]
    before = o.storage[:na].sum()
    k = o.step(3600.0)
    assert k > 1
    assert np.all(o.q >= 0.0) and np.all(o.storage[:na] >= 0.0)
    to_boundary = o.q_cum[net["dst"] >= na].sum()
    change = o.storage[:na].sum() - before
    inflow = net["inwater"][:na].sum() * 3600.0
    assert abs(change - (inflow - to_boundary) - o.error[:na].sum()) <= 1e-9 * (before + inflow)
