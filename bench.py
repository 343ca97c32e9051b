"""Throughput of the SBM + kinematic-wave step on a GB300 (cell-timesteps per second).

Default workload: one 1024 x 1024 synthetic catchment (250 m cells), hourly steps, SBM with
snow, kinematic-wave subsurface/overland/river routing with the reference's fixed sub-steps
(land 3600 s, river 900 s, subsurface 86400 s clamped to dt) and the water balance on.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--form fp64|split] [--workload NAME]
  python bench.py --impl reference ...   # the CPU restatement of the reference (the oracle)

`value` times K steps with the step's forcing already resident in HBM (CUDA events on the
library's stream). `e2e` times the same K steps through the public C ABI with host forcing
from pinned memory copied in and the outlet discharge copied out every step. The state of a
1024^2 model (about 1.2 GB in FP64) is far larger than the 129 MB L2, so no L2 flush is
needed between steps.
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
}

# Algorithmic bytes per cell and launch of each kernel (FP64 form), from the fields each
# kernel reads and writes once per cell.
ALGO_BYTES_FP64 = {"vertical": 729, "subsurface": 400, "overland": 136, "river": 160, "balance": 240}


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


def build_workload(name, form, seed=1):
    from wflow_gb300 import abi, synthetic

    side, cell, dt, members, _ = WORKLOADS[name]
    t0 = time.time()
    dom = synthetic.make_domain(side, cell, seed=seed)
    params = dom.params
    cfg = synthetic.make_config(dt, n_members=members, form=form, per_member_soil=members > 1)
    pfac = np.ones(members)
    if members > 1:
        kv0, f, pfac = synthetic.perturb_members(dom.params, members, seed=seed)
        params = dict(dom.params, kv_0=kv0, f=f)
    log(f"[bench] domain {name}: {dom.n_land} land cells, {dom.n_river} river cells, members {members}, "
        f"built in {time.time() - t0:.1f}s")
    return dom, params, cfg, pfac


def member_forcing(step, dt, n, members, pfac, seed=1):
    from wflow_gb300 import synthetic

    P, PET, T = synthetic.forcing(step, dt, n, seed=seed)
    if members == 1:
        return P, PET, T
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
    model = Model(cfg, dom, params=params, device=local)
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
    launches0 = model.metrics()["kernel_launches"]
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
    launches = model.metrics()["kernel_launches"] - launches0
    clk = clocks.stop()
    if ws > 1:
        t = torch.tensor([elapsed_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        elapsed_ms = float(t.item())
    cells = n * members
    value = cells * K * ws / (elapsed_ms / 1e3)
    # ---- end to end through the public API: pinned host forcing in, outlet discharge out
    host = []
    for s in range(W, W + K):
        P, PET, T = member_forcing(s, dt, n, members, pfac, seed=args.seed)
        pin = [torch.from_numpy(x).pin_memory() for x in (P, PET, T)]
        host.append(pin)
    n_out = max(1, len(dom.outlets) * members)
    out = torch.empty(n_out, dtype=torch.float64).pin_memory()
    import ctypes as C
    n_written = C.c_int64()
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in range(K):
        P, PET, T = host[s]
        st = lib.wf_set_forcing(model.h, C.cast(P.data_ptr(), abi._pd), C.cast(PET.data_ptr(), abi._pd),
                                C.cast(T.data_ptr(), abi._pd), P.numel())
        if st:
            raise RuntimeError(f"wf_set_forcing failed {st}")
        model.update_model()
        st = lib.wf_get_outlets(model.h, 0, C.cast(out.data_ptr(), abi._pd), n_out, C.byref(n_written))
        if st:
            raise RuntimeError(f"wf_get_outlets failed {st}")
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    if ws > 1:
        t = torch.tensor([e2e_s], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_value = cells * K * ws / e2e_s
    # ---- per-kernel times (eager launches with events between kernels) for the roofline
    model.set_tuning(**(tuning or {}), use_graph=0, kernel_timing=1)
    for s in range(min(K, 5)):
        b = resident[W + s]
        model.set_forcing_device_slots(b[0].data_ptr(), b[1].data_ptr(), b[2].data_ptr())
        model.update_model()
    kt, calls = model.kernel_times()
    kt = {k: v / max(calls, 1) for k, v in kt.items()}
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
                   "dt_s": dt, "form": args.form, "substeps": {"land": int(round(dt / min(dt, 3600.0))),
                                                               "river": int(np.ceil(dt / 900.0)),
                                                               "subsurface": 1},
                   "l2": "state 1.2 GB per 1M cells >> 129 MB L2, no flush needed",
                   "chains_land": mt["n_chains_land"], "max_chain_land": mt["max_chain_land"],
                   "max_chain_river": mt["max_chain_river"], "parallelism": f"replicas{ws}",
                   "tuning": tuning},
        "e2e": {"value": e2e_value, "unit": "cell-timesteps/s", "h2d_bytes_per_step": 3 * 8 * cells,
                "d2h_bytes_per_step": 8 * n_out},
        "gpu_launches": int(launches),
        "kernel_ms_per_step": kt,
        "clocks": clk,
    }
    # roofline of the dominant kernel
    dom_k = max(kt, key=lambda k: kt[k])
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    bytes_launch = ALGO_BYTES_FP64[dom_k] * cells
    if dom_k == "river":
        bytes_launch = ALGO_BYTES_FP64[dom_k] * dom.n_river * members * int(np.ceil(dt / 900.0))
    achieved = bytes_launch / (kt[dom_k] / 1e3) / 1e9 if kt[dom_k] > 0 else 0.0
    result["roofline"] = {"kernel": dom_k, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                          "frac": achieved / peak, "traffic": traffic_from_profiles(dom_k, args.workload),
                          "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback"}
    model.close()
    if rank == 0:
        result["cpu_baseline"] = cpu_baseline(args) if not args.no_cpu_baseline else None
        print(json.dumps(result), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


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

    dom, params, cfg, pfac = build_workload(args.workload, abi.WF_FORM_FP64, seed=args.seed)
    side, cell, dt, members, _ = WORKLOADS[args.workload]
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
            "sample": f"{done} steps of the {args.workload} workload ({n * members} cells) after 1 warm-up step, "
                      f"{el:.1f} s"}


def run_reference(args):
    ws, rank, local = dist_env()
    if rank != 0:
        return
    cb = cpu_baseline(args, steps=args.steps)
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
        "config": {"workload": args.workload, "cells": side * side, "members": members, "dt_s": dt},
        "cpu_baseline": cb,
        "e2e": {"value": cb["value"], "unit": "cell-timesteps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "Julia (the reference's own runtime) is not installed on this host; the reference arm is the "
                "C++ restatement of Wflow.jl's algorithm (oracle/) on all host threads",
    }
    print(json.dumps(result), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--form", default="fp64", choices=["fp64", "split"])
    ap.add_argument("--workload", default="single_1024_hourly", choices=list(WORKLOADS))
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
