"""Throughput of the SBM + kinematic-wave step on a GB300 (cell-timesteps per second).

Default workload: a 64-member ensemble on one 1024 x 1024 synthetic catchment (250 m cells,
67M cell-instances), hourly steps, SBM with snow, kinematic-wave subsurface/overland/river
routing with the reference's fixed sub-steps (land 3600 s, river 900 s, subsurface 86400 s
clamped to dt) and the water balance on, in the FP32/FP64 split form. The same line carries the
FP64 plain form on the same workload (`fp64_plain`, `split_over_fp64`) and the split form's
outlet-discharge and closure errors against it (`accuracy`).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--form fp64|split] [--workload NAME]
  python bench.py --impl reference ...   # the CPU restatement of the reference (the oracle)

`value` times K steps with the step's forcing already resident in HBM (CUDA events on the
library's stream). `e2e` times the same K steps through the public C ABI with host forcing
from pinned memory copied in (wf_set_forcing_async, FP32 arrays for the split form: the copy
of step k+1 overlaps step k) and
the outlet discharge copied out every step. Other workloads: `--workload
large_4096_adaptive_hourly` (4096 x 4096 at 100 m, Courant sub-steps, rain x3) and
`--workload ragged200_daily` (200 independent catchments of 10^3 - 10^6 cells), and
`--workload li_domain_2048_hourly` (local-inertial overland and river routing alone on a 2048 x
2048 grid, its own JSON line). The model state
(tens of GB for the ensemble, over 1 GB for one 1024^2 domain) is far larger than the 129 MB
L2, so no L2 flush is needed between steps.
"""

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "wflow.jl_gb300"))

WORKLOADS = {
    # name: (side, cell size [m], dt [s], members, default steps of the reference run)
    "single_1024_hourly": (1024, 250.0, 3600.0, 1, 720),
    "ensemble64_1024_hourly": (1024, 250.0, 3600.0, 64, 240),
    "single_64_daily": (64, 1000.0, 86400.0, 1, 365),
    # small case of the ensemble workload for multi-pass profiler captures (1/16 of the cells)
    "ensemble64_256_hourly": (256, 250.0, 3600.0, 64, 10),
    # one 4096 x 4096 domain at 100 m, hourly, adaptive (Courant) sub-steps, precipitation x3
    "large_4096_adaptive_hourly": (4096, 100.0, 3600.0, 1, 240),
    # uneven batch: 200 independent catchments of 10^3 - 10^6 cells (log-uniform), daily
    "ragged200_daily": (0, 1000.0, 86400.0, 1, 365),
}
# Local-inertial routing of the land grid with its river (include/wflow_gb300_li.h), measured by
# its own driver (run_li): side x side cells of 100 m, a river every 64th row, hourly model steps
# with the sub-step loop on the device.
LI_WORKLOADS = {"li_domain_2048_hourly": 2048}
LI_BYTES_PER_CELL_SUBSTEP = 224 + 96  # land fluxes + land depths per land cell and sub-step
WORKLOAD_OPTIONS = {
    "large_4096_adaptive_hourly": {"adaptive": True, "precip_scale": 3.0},
    "ragged200_daily": {"ragged": 200},
}

# Algorithmic bytes per cell (and member) of one launch of each kernel: the fields each kernel
# reads and writes once per cell. FP64 form: FP64 fields throughout. Split form (vertical): FP32
# forcing and member parameters (28 B), 11 FP64 states read (88 B), 20 FP64 states and fluxes
# written (160 B), 13 FP32 diagnostics and subsurface inputs written (52 B), static fields shared
# by the members of a cell (~8 B per member at 64 members).
ALGO_BYTES_FP64 = {"vertical": 729, "subsurface": 400, "overland": 136, "river": 160, "balance": 240}
ALGO_BYTES_SPLIT = {"vertical": 336, "subsurface": 200, "overland": 80, "river": 80, "balance": 200}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names[1:], parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def whole_job_rate(local_seconds, cells_per_rank, steps, device=None):
    """Replicas: every rank steps its own copy of the workload (members and catchments are
    independent, so the path has no exchange step); the job's time is the slowest rank's and its
    work the sum over ranks. Returns (cell-timesteps/s of the whole job, job seconds)."""
    import torch
    import torch.distributed as dist

    ws = dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1
    t = float(local_seconds)
    if ws > 1:
        x = torch.tensor([t], dtype=torch.float64, device=device)
        dist.all_reduce(x, op=dist.ReduceOp.MAX)
        t = float(x.item())
    return cells_per_rank * steps * ws / t, t


def build_workload(name, form, seed=1):
    from wflow_gb300 import abi, synthetic

    side, cell, dt, members, _ = WORKLOADS[name]
    opts = WORKLOAD_OPTIONS.get(name, {})
    t0 = time.time()
    if opts.get("ragged"):
        dom = synthetic.make_ragged(opts["ragged"], seed=seed, cell_size=cell, log10_min=3.0, log10_max=6.0)
    else:
        dom = synthetic.make_domain(side, cell, seed=seed)
    params = dom.params
    cfg = synthetic.make_config(dt, n_members=members, form=form, per_member_soil=members > 1,
                                adaptive=opts.get("adaptive", False))
    pfac = np.ones(members)
    if members > 1:
        kv0, f, pfac = synthetic.perturb_members(dom.params, members, seed=seed)
        params = dict(dom.params, kv_0=kv0, f=f)
    pfac = pfac * opts.get("precip_scale", 1.0)
    log(f"[bench] domain {name}: {dom.n_land} land cells, {dom.n_river} river cells, members {members}, "
        f"built in {time.time() - t0:.1f}s")
    return dom, params, cfg, pfac


def member_forcing(step, dt, n, members, pfac, seed=1):
    from wflow_gb300 import synthetic

    P, PET, T = synthetic.forcing(step, dt, n, seed=seed)
    if members == 1:
        return (P * pfac[0] if pfac[0] != 1.0 else P), PET, T
    return (np.concatenate([P * pfac[m] for m in range(members)]), np.tile(PET, members), np.tile(T, members))


def run_gpu(args):
    import torch

    from wflow_gb300 import abi, build, synthetic
    from wflow_gb300.model import Model

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    if rank == 0 or ws > 1:
        build.build_all()
    form = abi.WF_FORM_SPLIT if args.form == "split" else abi.WF_FORM_FP64
    dom, params, cfg, pfac = build_workload(args.workload, form, seed=args.seed)
    side, cell, dt, members, _ = WORKLOADS[args.workload]
    n = dom.n_land
    free0 = torch.cuda.mem_get_info(local)[0]
    model = Model(cfg, dom, params=params, device=local)
    state_gb = (free0 - torch.cuda.mem_get_info(local)[0]) / 1e9
    lib = model.lib
    # ---- forcing resident in HBM, in the library's slot order, for W + K steps
    slots = model.slot_order()
    valid = slots >= 0
    K, W = args.steps, args.warmup
    dev = torch.device(f"cuda:{local}")
    resident = []
    for s in range(W + K):
        P, PET, T = member_forcing(s, dt, n, members, pfac, seed=args.seed)
        bufs = []
        for arr in (P, PET, T):
            a2 = arr.reshape(members, n)
            slot_arr = np.zeros((len(slots), members))
            slot_arr[valid] = a2[:, slots[valid]].T
            bufs.append(torch.from_numpy(slot_arr.reshape(-1)).to(dev))
        resident.append(bufs)
    torch.cuda.synchronize()
    tuning = None
    if not args.no_autotune:
        from wflow_gb300 import autotune
        t0 = time.time()
        tuning, _ = autotune.tune(model, lambda s: member_forcing(10_000 + s, dt, n, members, pfac, seed=args.seed))
        log(f"[bench] autotune {tuning} in {time.time() - t0:.1f}s")
    stream = torch.cuda.ExternalStream(model.stream(), device=dev)
    m0 = model.metrics()
    for s in range(W):
        b = resident[s]
        model.set_forcing_device_slots(b[0].data_ptr(), b[1].data_ptr(), b[2].data_ptr())
        model.update_model()
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    mt0 = model.metrics()
    launches0 = mt0["kernel_launches"]
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    for s in range(W, W + K):
        b = resident[s]
        model.set_forcing_device_slots(b[0].data_ptr(), b[1].data_ptr(), b[2].data_ptr())
        model.step_async()
    ev1.record(stream)
    ev1.synchronize()
    model.synchronize()
    torch.cuda.synchronize()
    elapsed_ms = ev0.elapsed_time(ev1)
    mt1 = model.metrics()
    launches = mt1["kernel_launches"] - launches0
    substeps = {k: (mt1["substeps_" + k] - mt0["substeps_" + k]) / K for k in ("land", "river", "subsurface")}
    clk = clocks.stop()
    cells = n * members
    value, job_s = whole_job_rate(elapsed_ms / 1e3, cells, K, device=dev)
    elapsed_ms = job_s * 1e3
    # ---- end to end through the public API: pinned host forcing in, outlet discharge out
    # the split form computes with FP32 forcing, so it is handed FP32 arrays (wf_set_forcing_f32,
    # half the bytes to copy, the same state); the FP64 form takes FP64 arrays
    f32 = form == abi.WF_FORM_SPLIT
    fdt = np.float32 if f32 else np.float64
    # an ensemble perturbs the precipitation of every member; the potential evaporation and the
    # temperature are the same for all members, and the split form's FP32 upload takes them once
    shared = f32 and members > 1
    host = []
    for s in range(W, W + K):
        P, PET, T = member_forcing(s, dt, n, members, pfac, seed=args.seed)
        if shared:
            PET, T = PET[:n], T[:n]
        pin = [torch.from_numpy(np.ascontiguousarray(x, dtype=fdt)).pin_memory() for x in (P, PET, T)]
        host.append(pin)
    # The first device access to a freshly pinned host buffer maps its pages (about 30 GB/s
    # instead of 200 GB/s on this host); a model run reads its forcing into the same buffers
    # every step, so each buffer is touched once before the timed region.
    scratch = torch.empty(n * members, dtype=torch.float32 if f32 else torch.float64, device=dev)
    for pin in host:
        for x in pin:
            scratch[: x.numel()].copy_(x, non_blocking=True)
    torch.cuda.synchronize()
    del scratch
    n_out = max(1, len(dom.outlets) * members)
    out = torch.empty(n_out, dtype=torch.float64).pin_memory()
    import ctypes as C
    n_written = C.c_int64()
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ptr_t = abi._pf if f32 else abi._pd

    def set_forcing_async(s):
        P, PET, T = host[s]
        if f32:
            st = lib.wf_set_forcing_counts_async_f32(model.h, C.cast(P.data_ptr(), ptr_t), P.numel(),
                                                     C.cast(PET.data_ptr(), ptr_t), PET.numel(),
                                                     C.cast(T.data_ptr(), ptr_t), T.numel())
        else:
            st = lib.wf_set_forcing_async(model.h, C.cast(P.data_ptr(), ptr_t), C.cast(PET.data_ptr(), ptr_t),
                                          C.cast(T.data_ptr(), ptr_t), P.numel())
        if st:
            raise RuntimeError(f"wf_set_forcing_async failed {st}")

    # every step: its forcing copied in from pinned host memory (overlapping the previous step)
    # and its outlet discharge copied out
    t0 = time.perf_counter()
    set_forcing_async(0)
    for s in range(K):
        model.step_async()
        if s + 1 < K:
            set_forcing_async(s + 1)
        st = lib.wf_get_outlets(model.h, 0, C.cast(out.data_ptr(), abi._pd), n_out, C.byref(n_written))
        if st:
            raise RuntimeError(f"wf_get_outlets failed {st}")
    model.synchronize()
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e_value, e2e_s = whole_job_rate(e2e_s, cells, K, device=dev)
    # the forcing upload alone (copies and gathers, no step): what the step has to hide
    t1 = time.perf_counter()
    for s in range(K):
        set_forcing_async(s)
    model.synchronize()
    upload_ms = (time.perf_counter() - t1) / K * 1e3
    # the same loop with the forcing already on the device (no copies): the cost of the uploads
    # the step did not hide is e2e minus this
    t1 = time.perf_counter()
    for s in range(K):
        b = resident[W + s]
        model.set_forcing_device_slots(b[0].data_ptr(), b[1].data_ptr(), b[2].data_ptr())
        model.step_async()
        st = lib.wf_get_outlets(model.h, 0, C.cast(out.data_ptr(), abi._pd), n_out, C.byref(n_written))
        if st:
            raise RuntimeError(f"wf_get_outlets failed {st}")
    model.synchronize()
    loop_resident_ms = (time.perf_counter() - t1) / K * 1e3
    # ---- per-kernel times (eager launches with events between kernels) for the roofline; the
    # handle's counters also hold the autotuner's timed steps, so only this pass's share counts
    model.set_tuning(**(tuning or {}), use_graph=0, kernel_timing=1)
    kt0, calls0 = model.kernel_times()
    for s in range(min(K, 5)):
        b = resident[W + s]
        model.set_forcing_device_slots(b[0].data_ptr(), b[1].data_ptr(), b[2].data_ptr())
        model.update_model()
    kt, calls = model.kernel_times()
    kt = {k: (v - kt0[k]) / max(calls - calls0, 1) for k, v in kt.items()}
    mt = model.metrics()
    result = {
        "metric": "cell-timesteps/s",
        "value": value,
        "unit": "cell-timesteps/s",
        "n_gpus": ws,
        "steps": K,
        "warmup": W,
        "ms_per_step": elapsed_ms / K,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64" if form == abi.WF_FORM_FP64 else "f32+f64",
        "data": "synthetic (seeded fractal DEM, D8, SBM parameters and forcing of the benchmark configuration)",
        "config": {"workload": args.workload, "cells": n, "members": members, "river_cells": dom.n_river,
                   "dt_s": dt, "form": args.form,
                   "substeps_per_step": substeps,
                   "adaptive_substeps": bool(cfg.adaptive_timestep),
                   "catchments": len(dom.outlets),
                   "l2": f"model state {state_gb:.1f} GB on the device >> 129 MB L2, no flush needed",
                   "chains_land": mt["n_chains_land"], "max_chain_land": mt["max_chain_land"],
                   "max_chain_river": mt["max_chain_river"], "parallelism": f"replicas{ws}",
                   "tuning": tuning},
        "e2e": {"value": e2e_value, "unit": "cell-timesteps/s",
                "h2d_bytes_per_step": sum(x.numel() * x.element_size() for x in host[0]),
                "d2h_bytes_per_step": 8 * n_out, "forcing_dtype": np.dtype(fdt).name,
                "forcing_layout": ("precipitation per member, potential evaporation and temperature once for "
                                   "every member" if shared else "every array per member"),
                "upload_only_ms_per_step": upload_ms,
                "loop_with_resident_forcing_ms_per_step": loop_resident_ms},
        "gpu_launches": int(launches),
        "kernel_ms_per_step": kt,
        "clocks": clk,
    }
    # roofline of the dominant kernel: the vertical kernel is the largest single kernel of the
    # step (the routing phases are a sweep kernel plus a completion kernel each); every phase's
    # achieved bandwidth is reported beside it
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    algo = ALGO_BYTES_SPLIT if form == abi.WF_FORM_SPLIT else ALGO_BYTES_FP64

    def phase_bytes(k):
        if k == "river":
            return algo[k] * dom.n_river * members * substeps["river"]
        if k == "overland":
            return algo[k] * cells * substeps["land"]
        return algo[k] * cells

    def achieved_of(k):
        return phase_bytes(k) / (kt[k] / 1e3) / 1e9 if kt.get(k, 0) > 0 else 0.0

    dom_k = "vertical"
    achieved = achieved_of(dom_k)
    result["roofline"] = {"kernel": dom_k, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                          "frac": achieved / peak, "traffic": traffic_from_profiles(dom_k, args.workload),
                          "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback"}
    phases = {k: {"ms": kt[k], "achieved_gbs": achieved_of(k), "frac": achieved_of(k) / peak,
                  "algorithmic_bytes": phase_bytes(k)} for k in kt}
    # the split form's overland sweep and the river's first sub-steps share one launch (timed as
    # the overland phase; the river phase is then its completion kernel alone): one phase for both
    shared_launch = (form == abi.WF_FORM_SPLIT and not cfg.adaptive_timestep and dom.n_river > 0
                     and (tuning or {}).get("separate_overland_river", 0) == 0 and substeps["land"] <= 16)
    if shared_launch:
        b = phase_bytes("overland") + phase_bytes("river")
        ms = kt["overland"] + kt["river"]
        a = b / (ms / 1e3) / 1e9 if ms > 0 else 0.0
        phases.pop("overland")
        phases.pop("river")
        phases["overland+river"] = {"ms": ms, "achieved_gbs": a, "frac": a / peak, "algorithmic_bytes": b,
                                    "note": "overland sweep and the river sweep in one launch"}
        result["kernel_ms_note"] = ("overland: the shared overland-river launch and the overland completion; "
                                    "river: the river completion")
    result["roofline_phases"] = phases
    # ---- the FP64 plain form on the same workload and forcing: throughput ratio and the split
    # form's error against it (the FP64 form reproduces the FP64 oracle bit for bit)
    if form == abi.WF_FORM_SPLIT and not args.no_fp64_leg:
        result.update(fp64_leg(args, cfg, dom, params, resident, W, K, dt, members, n, dev))
        result["split_over_fp64"] = value / result["fp64_plain"]["value"]
    elif not args.no_fp64_leg:
        result["accuracy"] = accuracy_leg(args, cfg, dom, params, resident, W + K, dt, members, n, dev)
    model.close()
    if rank == 0:
        result["cpu_baseline"] = cpu_baseline(args) if not args.no_cpu_baseline else None
        print(json.dumps(result), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def fp64_leg(args, cfg, dom, params, resident, W, K, dt, members, n, dev):
    """Time the FP64 plain form on the same resident forcing (fewer steps: it is slower), then
    measure both forms against the oracle over the warm-up and timed steps (accuracy_leg)."""
    import copy

    import torch

    from wflow_gb300 import abi
    from wflow_gb300.model import Model

    cfg64 = copy.copy(cfg)
    cfg64.form = abi.WF_FORM_FP64
    m64 = Model(cfg64, dom, params=params, device=dev.index or 0)
    stream = torch.cuda.ExternalStream(m64.stream(), device=dev)
    k64 = max(2, min(K, 5))
    for s in range(W):
        b = resident[s]
        m64.set_forcing_device_slots(b[0].data_ptr(), b[1].data_ptr(), b[2].data_ptr())
        m64.update_model()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    for s in range(W, W + k64):
        b = resident[s]
        m64.set_forcing_device_slots(b[0].data_ptr(), b[1].data_ptr(), b[2].data_ptr())
        m64.step_async()
    ev1.record(stream)
    ev1.synchronize()
    m64.synchronize()
    ms64 = ev0.elapsed_time(ev1)
    m64.close()
    cells = n * members
    out = {"fp64_plain": {"value": cells * k64 / (ms64 / 1e3), "ms_per_step": ms64 / k64, "steps": k64,
                          "unit": "cell-timesteps/s"}}
    out["accuracy"] = accuracy_leg(args, cfg, dom, params, resident, W + K, dt, members, n, dev)
    return out


def closure_of(err, rel):
    """(max |relative error| as the reference defines it, error / mean of in- and outflow; max of
    |error| / max(local mean flux, median mean flux)), over the cells of one balance. The local mean
    flux is |error / relative error| where the relative error is non-zero."""
    err, rel = np.asarray(err), np.asarray(rel)
    nz = rel != 0.0
    flux = np.zeros_like(err)
    flux[nz] = np.abs(err[nz] / rel[nz])
    med = float(np.median(flux[nz])) if nz.any() else 1.0
    return float(np.max(np.abs(rel))), float(np.max(np.abs(err) / np.maximum(flux, med)))


def accuracy_leg(args, cfg, dom, params, resident, steps, dt, members, n, dev):
    """Both GPU forms and the FP64 oracle from the cold state over the warm-up and timed steps (the
    oracle on the first member of an ensemble, whose parameters and forcing it takes): outlet
    discharge and storage errors of each form against the oracle, and the land-balance closure of
    each form and of the oracle, by the reference's definition and against max(local, median) flux.
    The oracle's cost bounds the steps on the largest workloads (about a minute of host time)."""
    import copy

    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle_py

    from wflow_gb300 import abi, synthetic
    from wflow_gb300.model import Model

    steps = max(2, min(steps, int(60 * 1.5e6 / max(n, 1))))
    cfg64 = copy.copy(cfg)
    cfg64.form = abi.WF_FORM_FP64
    cfg_s = copy.copy(cfg)
    cfg_s.form = abi.WF_FORM_SPLIT
    cfg_o = synthetic.make_config(dt, n_members=1, form=abi.WF_FORM_FP64, adaptive=bool(cfg.adaptive_timestep))
    p0 = dict(params)
    for k in ("kv_0", "f"):
        p0[k] = np.ascontiguousarray(np.asarray(params[k])[:n])
    a = Model(cfg64, dom, params=params, device=dev.index or 0)
    b_ = Model(cfg_s, dom, params=params, device=dev.index or 0)
    orc = oracle_py.OracleModel(cfg_o, dom, params=p0)
    threads = os.cpu_count() or 1
    slots = a.slot_order()
    valid = slots >= 0
    n_out = len(dom.outlets)
    worst = {"fp64": {"outlet_q": 0.0, "soil_storage": 0.0}, "split": {"outlet_q": 0.0, "soil_storage": 0.0,
                                                                         "snow_storage": 0.0}}
    clos = {k: [0.0, 0.0] for k in ("split", "fp64", "oracle")}  # the member the oracle runs
    if members > 1:
        clos.update({k: [0.0, 0.0] for k in ("split_all_members", "fp64_all_members")})
    for s in range(steps):
        r = resident[s]
        for mdl in (a, b_):
            mdl.set_forcing_device_slots(r[0].data_ptr(), r[1].data_ptr(), r[2].data_ptr())
            mdl.update_model()
        # the oracle takes member 0's forcing in cell order (the resident arrays hold slot order)
        f0 = []
        for x in r:
            v = x.reshape(-1, members)[:, 0].cpu().numpy()
            c = np.zeros(n)
            c[slots[valid]] = v[valid]
            f0.append(c)
        orc.set_forcing(*f0)
        orc.step(threads)
        qo = orc.outlets(0)
        so = orc.get(abi.FIELD["TOTAL_SOIL_WATER_STORAGE"])
        wo = orc.get(abi.FIELD["SNOW_STORAGE"])
        for name, mdl in (("fp64", a), ("split", b_)):
            q = mdl.outlets(0)[:n_out]
            w = worst[name]
            w["outlet_q"] = max(w["outlet_q"], float(np.max(np.abs(q - qo) / np.maximum(np.abs(qo), 1e-12))))
            sg = mdl.get_value("TOTAL_SOIL_WATER_STORAGE", count=n)
            w["soil_storage"] = max(w["soil_storage"], float(np.max(np.abs(sg - so) / so)))
            if name == "split":
                wg = mdl.get_value("SNOW_STORAGE", count=n)
                big = wo > 1e-4
                if big.any():
                    w["snow_storage"] = max(w["snow_storage"], float(np.max(np.abs(wg - wo)[big] / wo[big])))
        for name, get in (("fp64", a.get_value), ("split", b_.get_value),
                          ("oracle", lambda f: orc.get(abi.FIELD[f]))):
            err, rel = get("BALANCE_LAND_ERROR"), get("BALANCE_LAND_RELATIVE_ERROR")
            for key, sl in ((name, slice(0, n)), (name + "_all_members", slice(None))):
                if key not in clos or (name == "oracle" and sl.stop is None):
                    continue
                rel_, flux_ = closure_of(err[sl], rel[sl])
                clos[key][0] = max(clos[key][0], rel_)
                clos[key][1] = max(clos[key][1], flux_)
    a.close()
    b_.close()
    return {"against": "FP64 oracle (CPU restatement of the reference)" +
                       (", first member of the ensemble" if members > 1 else ""),
            "steps": steps,
            "outlet_q_rel_err_max": worst["split"]["outlet_q"],
            "split": worst["split"], "fp64": worst["fp64"],
            "land_balance_closure_rel_max": {k: clos[k][0] for k in clos},
            "land_balance_closure_over_flux": {k: clos[k][1] for k in clos},
            "closure_note": "rel: error / mean of in- and outflow per cell (mass_balance.jl:84-93), which peaks "
                            "in cells whose fluxes are ~1e-12 m/s for the oracle as well; over_flux: error / "
                            "max(local mean flux, median mean flux over the cells), the closure bar of the "
                            "split form (<= 1e-7)"}


def traffic_from_profiles(kernel, workload):
    """DRAM bytes per launch of `kernel` from the committed ncu summary (profiles/traffic.txt)."""
    p = ROOT / "profiles" / "traffic.txt"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        parts = line.split()
        if len(parts) >= 3 and not line.startswith("#") and parts[0] == kernel and parts[1] == workload:
            return float(parts[2])
    return None


def cpu_baseline(args, steps=None):
    """The oracle (CPU restatement of the reference) on the same workload, a bounded sample."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle_py

    from wflow_gb300 import abi

    side, cell, dt, members, _ = WORKLOADS[args.workload]
    opts = WORKLOAD_OPTIONS.get(args.workload, {})
    sample_note = ""
    if opts.get("ragged") or side > 1024:
        # bounded sample of the largest workloads (the oracle's cost per cell-step does not depend
        # on the domain size): the first 10 catchments of the uneven batch, or a 1024 x 1024 domain
        # of the same generator, cell size, sub-stepping and rain scaling
        from wflow_gb300 import synthetic
        if opts.get("ragged"):
            dom = synthetic.make_ragged(10, seed=args.seed, cell_size=cell, log10_min=3.0, log10_max=6.0)
            sample_note = "the first 10 catchments of the uneven batch, "
        else:
            dom = synthetic.make_domain(1024, cell, seed=args.seed)
            sample_note = "a 1024 x 1024 domain of the same generator and settings, "
        params = dom.params
        cfg = synthetic.make_config(dt, form=abi.WF_FORM_FP64, adaptive=opts.get("adaptive", False))
        pfac = np.ones(1) * opts.get("precip_scale", 1.0)
    else:
        dom, params, cfg, pfac = build_workload(args.workload, abi.WF_FORM_FP64, seed=args.seed)
    if members > 1:  # bounded sample: the first member of the ensemble (cost is linear in members)
        from wflow_gb300 import synthetic
        cfg = synthetic.make_config(dt, n_members=1, form=abi.WF_FORM_FP64, adaptive=bool(cfg.adaptive_timestep))
        params = dom.params
        pfac = pfac[:1]
        members = 1
    threads = os.cpu_count() or 1
    orc = oracle_py.OracleModel(cfg, dom, params=params)
    n = dom.n_land
    budget_s = float(os.environ.get("WF_CPU_BASELINE_SECONDS", "20"))
    done = 0
    P, PET, T = member_forcing(0, dt, n, members, pfac, seed=args.seed)
    orc.set_forcing(P, PET, T)
    orc.step(threads)  # warm-up step
    t0 = time.perf_counter()
    max_steps = steps if steps is not None else 10**9
    while done < max_steps:
        P, PET, T = member_forcing(done + 1, dt, n, members, pfac, seed=args.seed)
        orc.set_forcing(P, PET, T)
        orc.step(threads)
        done += 1
        if steps is None and time.perf_counter() - t0 > budget_s:
            break
    el = time.perf_counter() - t0
    return {"value": n * members * done / el, "unit": "cell-timesteps/s", "cores": threads, "kind": "port",
            "cells": n * members,
            "sample": f"{done} steps of {n * members} cells of the {args.workload} workload "
                      f"({sample_note}{'first member of the ensemble, ' if WORKLOADS[args.workload][3] > 1 else ''}"
                      f"after 1 warm-up step), {el:.1f} s"}


def probe_julia():
    """Whether the reference's own runtime is on this host: `julia --version` on the PATH."""
    import shutil

    exe = shutil.which("julia")
    if exe is None:
        return "julia not found on PATH"
    try:
        out = subprocess.run([exe, "--version"], capture_output=True, text=True, timeout=60)
        return f"{exe}: {(out.stdout or out.stderr).strip()} (exit {out.returncode})"
    except Exception as e:  # a broken install counts as absent
        return f"{exe}: {type(e).__name__}: {e}"


def run_reference(args):
    ws, rank, local = dist_env()
    if rank != 0:
        return
    cb = cpu_baseline(args, steps=min(args.steps, 10))
    side, cell, dt, members, _ = WORKLOADS[args.workload]
    result = {
        "impl": "reference",
        "metric": "cell-timesteps/s",
        "value": cb["value"],
        "unit": "cell-timesteps/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": 1,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded), same workload as the GPU arm",
        "config": {"workload": args.workload, "sample_cells": cb["cells"], "members": members, "dt_s": dt,
                   "form": "fp64 (the reference's arithmetic)"},
        "cpu_baseline": cb,
        "e2e": {"value": cb["value"], "unit": "cell-timesteps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "julia_probe": probe_julia(),
        "note": "the reference arm is the C++ restatement of Wflow.jl's algorithm (oracle/) on all host "
                "threads: Wflow.jl needs Julia and its package depot, which this host lacks (julia_probe)",
    }
    print(json.dumps(result), flush=True)


def run_profile(args):
    """Profiler driver: build the workload, run --steps eager steps (one launch per kernel, no
    CUDA graph), print the per-kernel milliseconds to stderr and exit."""
    import torch

    from wflow_gb300 import abi, build
    from wflow_gb300.model import Model

    torch.cuda.set_device(0)
    build.build_all()
    form = abi.WF_FORM_SPLIT if args.form == "split" else abi.WF_FORM_FP64
    dom, params, cfg, pfac = build_workload(args.workload, form, seed=args.seed)
    side, cell, dt, members, _ = WORKLOADS[args.workload]
    model = Model(cfg, dom, params=params)
    model.set_tuning(vertical_block=128, routing_warps=args.routing_warps, routing_blocks_per_sm=args.routing_bps,
                     use_graph=0, kernel_timing=1, substep_lanes=args.sub_lanes, sweep_inputs=args.sweep_inputs,
                     separate_overland_river=args.separate_overland_river)
    for s in range(args.steps):
        P, PET, T = member_forcing(s, dt, dom.n_land, members, pfac, seed=args.seed)
        model.run_timestep(P, PET, T)
    kt, calls = model.kernel_times()
    log(f"[profile] {args.workload} {args.form}: ms per step {({k: round(v / max(calls, 1), 3) for k, v in kt.items()})}")
    model.close()


def run_li(args):
    """Local-inertial overland and river routing (wf_li_domain_step) on a synthetic grid: hourly
    model steps with the sub-step loop on the device (one cooperative launch and one read-back per
    step), then the same steps driven from the host (a time-step read-back per sub-step) for
    comparison; land cell-timesteps/s and the achieved bandwidth of the land kernels per
    sub-step."""
    import torch

    from wflow_gb300 import build, synthetic
    from wflow_gb300.li_river import LiDomain

    torch.cuda.set_device(0)
    build.build_all()
    side = LI_WORKLOADS[args.workload]
    land, river, h_river, h_land, runoff = synthetic.li_grid(side, side)
    n = len(h_land)
    dt = 3600.0
    d = LiDomain(land, river, h_river)
    d.set_state(h_land, h_river)
    d.set_inputs(runoff)
    for _ in range(args.warmup):
        d.step(dt)
    clocks = ClockSampler(0)
    clocks.start()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    k = sum(d.step(dt) for _ in range(args.steps))
    el = time.perf_counter() - t0
    clk = clocks.stop()
    d.set_host_loop(True)
    t1 = time.perf_counter()
    k_host = sum(d.step(dt) for _ in range(args.steps))
    el_host = time.perf_counter() - t1
    d.close()
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = n * LI_BYTES_PER_CELL_SUBSTEP * k / el / 1e9
    result = {
        "metric": "cell-timesteps/s", "value": n * args.steps / el, "unit": "cell-timesteps/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (square land grid with a river every 64th row, 5 mm/h runoff, warm state)",
        "config": {"workload": args.workload, "cells": n, "river_cells": int(river["n_active"]), "dt_s": dt,
                   "substeps_per_step": k / args.steps,
                   "l2": "the grid's state (~1 GB) exceeds the 129 MB L2; no flush"},
        "cell_substeps_per_s": n * k / el,
        "host_driven_loop": {"ms_per_step": el_host / args.steps * 1e3, "substeps": k_host,
                             "speedup_of_device_loop": el_host / el},
        "roofline": {"kernel": "land fluxes + land depths", "bound": "hbm", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "traffic": None,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback"},
        "clocks": clk,
    }
    print(json.dumps(result), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--form", default="split", choices=["fp64", "split"])
    ap.add_argument("--workload", default="ensemble64_1024_hourly", choices=list(WORKLOADS) + list(LI_WORKLOADS))
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-fp64-leg", action="store_true", help="skip the FP64 plain comparison leg")
    ap.add_argument("--sub-lanes", type=int, default=0,
                    help="profiler driver: cap of the routing sweeps' sub-step lanes (0: the library default)")
    ap.add_argument("--routing-warps", type=int, default=2, help="--profile: warps per block of the sweeps")
    ap.add_argument("--routing-bps", type=int, default=0, help="--profile: sweep blocks per SM (0: all resident)")
    ap.add_argument("--separate-overland-river", type=int, default=0, choices=[0, 1],
                    help="--profile: 1 runs the split form's overland and river sweeps in separate launches")
    ap.add_argument("--sweep-inputs", type=int, default=0,
                    help="profiler driver: bit k keeps the inputs of node-major sweep k (0 subsurface, 1 "
                         "overland, 2 river) in registers instead of staging them in shared memory")
    ap.add_argument("--profile", action="store_true",
                    help="profiler driver: run --steps eager steps of the workload and exit (no JSON line)")
    args = ap.parse_args()
    if args.warmup < 3 and not args.profile:
        args.warmup = 3
    if args.workload in LI_WORKLOADS:
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the local-inertial workload has no CPU arm"}))
        else:
            run_li(args)
    elif args.profile:
        run_profile(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
