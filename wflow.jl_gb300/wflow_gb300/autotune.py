"""Launch-shape autotuner for a model handle.

The wavefront kernels are bound by the latency of the longest chain and by how many warps
share an SM's FP64 pipe while the short chains drain, so the best number of resident warps
depends on the graph (chain-length distribution) and the form; a sweep of several sub-steps also
depends on how many lanes share a chain-member pair on the diagonal schedule (more lanes: a
shorter critical path, fewer pairs per warp), and each node-major sweep on whether its inputs are
staged in shared memory or held in registers; the overland and river sweeps may share one launch
(the river walking behind the overland front) or run one after the other; the per-cell kernel
depends on its block size and on its grid, which sets how many elements each thread walks. The
tuner times a few steps of each candidate with per-kernel CUDA events and keeps the fastest for
each kernel family. Candidates only change the schedule, never the result: the wavefront
produces the same values for any dispatch order and any lane count.
"""

import itertools

from .model import Model


def _time_steps(model: Model, forcing, steps):
    model.set_tuning(**model._tune_state, use_graph=0, kernel_timing=1)
    before, calls0 = model.kernel_times()
    for s in range(steps):
        P, PET, T = forcing(s)
        model.run_timestep(P, PET, T)
    after, calls1 = model.kernel_times()
    n = max(calls1 - calls0, 1)
    return {k: (after[k] - before[k]) / n for k in after}


def _time_graph(model: Model, forcing, steps):
    """Device time per step of the replayed step graph (the first step captures it)."""
    model.set_tuning(**model._tune_state, use_graph=1)
    model.run_timestep(*forcing(0))
    m0 = model.metrics()["step_ms_total"]
    for s in range(steps):
        model.run_timestep(*forcing(s + 1))
    return (model.metrics()["step_ms_total"] - m0) / steps


def tune(model: Model, forcing, steps=1, verbose=False):
    """Pick routing warps/blocks per SM and the per-cell block size; returns the choice and the
    measured milliseconds per step of each candidate."""
    # the launch shapes of the separate sweeps first; whether the overland and river sweeps share a
    # launch is decided last
    model._tune_state = dict(vertical_block=0, routing_warps=0, routing_blocks_per_sm=0, substep_lanes=0,
                             separate_overland_river=1)
    _time_steps(model, forcing, 1)  # warm-up
    results = []
    best_route, best_route_t = None, float("inf")
    for warps, bps in itertools.product([2, 4], [1, 2, 4, 0]):
        model._tune_state = dict(vertical_block=0, routing_warps=warps, routing_blocks_per_sm=bps, substep_lanes=0,
                                 separate_overland_river=1)
        t = _time_steps(model, forcing, steps)
        route = t["subsurface"] + t["overland"] + t["river"]
        results.append(("routing", warps, bps, route))
        if verbose:
            print(f"routing warps={warps} blocks/SM={bps}: {route:.3f} ms")
        if route < best_route_t:
            best_route, best_route_t = (warps, bps), route
    # sub-step lanes of the sweeps with several sub-steps per launch (river 900 s in an hourly
    # step, daily overland and river)
    m = model.metrics()
    best_lanes = 0
    if m["steps"] > 0 and max(m["substeps_land"], m["substeps_river"]) > m["steps"]:
        best_lanes_t = best_route_t
        for lanes in [1, 2, 4, 16]:  # 0 (the default, 8) was measured above
            model._tune_state = dict(vertical_block=0, routing_warps=best_route[0],
                                     routing_blocks_per_sm=best_route[1], substep_lanes=lanes,
                                     separate_overland_river=1)
            t = _time_steps(model, forcing, steps)
            route = t["subsurface"] + t["overland"] + t["river"]
            results.append(("lanes", lanes, 0, route))
            if verbose:
                print(f"sub-step lanes={lanes}: {route:.3f} ms")
            if route < best_lanes_t:
                best_lanes, best_lanes_t = lanes, route
    # inputs of the node-major sweeps: staged in shared memory or held in registers, per sweep
    # (both runs time every sweep; each keeps its faster mode)
    base = dict(vertical_block=0, routing_warps=best_route[0], routing_blocks_per_sm=best_route[1],
                substep_lanes=best_lanes, separate_overland_river=1)
    model._tune_state = dict(base, sweep_inputs=0)
    staged = _time_steps(model, forcing, steps)
    model._tune_state = dict(base, sweep_inputs=7)
    regs = _time_steps(model, forcing, steps)
    best_inputs = sum(1 << k for k, name in enumerate(("subsurface", "overland", "river"))
                      if regs[name] < staged[name])
    results.append(("inputs", best_inputs, 0, 0.0))
    if verbose:
        print(f"sweep inputs held in registers (bit mask): {best_inputs}")
    # the overland sweep and the river's first sub-steps in one launch (the river walks behind
    # the overland front), against separate launches; both phases together, since the shared
    # launch is timed as the overland phase
    # (the shared launch runs the river's first-dispatched chains on the diagonal schedule when
    # the sub-step lanes allow it, so it is tried with the lanes chosen above and with none).
    # Timed as whole replayed step graphs, the way the steps run in production.
    best_sep = 1
    model._tune_state = dict(base, sweep_inputs=best_inputs)
    best_step_t = _time_graph(model, forcing, steps + 1)
    for lanes in dict.fromkeys([best_lanes, 1]):
        model._tune_state = dict(base, sweep_inputs=best_inputs, substep_lanes=lanes, separate_overland_river=0)
        t = _time_graph(model, forcing, steps + 1)
        results.append(("overland_river_shared_launch", lanes, 0, t))
        if verbose:
            print(f"step with overland and river in one launch (lanes={lanes}): {t:.3f} ms, "
                  f"separate {best_step_t:.3f} ms")
        if t < best_step_t:
            best_sep, best_lanes, best_step_t = 0, lanes, t
    # the per-cell kernel: block size and grid (the elements each thread walks in its grid-stride
    # loop: one wave of resident blocks, a few waves, or the default 16 blocks per SM)
    best_block, best_bps, best_block_t = 0, 0, float("inf")
    for block, vbps in itertools.product([128, 256], [0, 4, 8]):
        model._tune_state = dict(vertical_block=block, routing_warps=best_route[0],
                                 routing_blocks_per_sm=best_route[1], substep_lanes=best_lanes,
                                 sweep_inputs=best_inputs, vertical_blocks_per_sm=vbps,
                                 separate_overland_river=best_sep)
        t = _time_steps(model, forcing, steps)
        results.append(("vertical", block, vbps, t["vertical"]))
        if verbose:
            print(f"vertical block={block} blocks/SM={vbps}: {t['vertical']:.3f} ms")
        if t["vertical"] < best_block_t:
            best_block, best_bps, best_block_t = block, vbps, t["vertical"]
    choice = dict(vertical_block=best_block, routing_warps=best_route[0], routing_blocks_per_sm=best_route[1],
                  substep_lanes=best_lanes, sweep_inputs=best_inputs, vertical_blocks_per_sm=best_bps,
                  separate_overland_river=best_sep)
    model._tune_state = choice
    model.set_tuning(**choice, use_graph=1)
    return choice, results
