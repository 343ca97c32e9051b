"""The launch-shape autotuner's host logic (wflow_gb300.autotune) against a stand-in model (CPU).

The stand-in times each launch shape with a cost table instead of running kernels, so the test
checks what the tuner does with the timings: every shape it sets is one `Model.set_tuning`
accepts, each choice is the fastest candidate of its family, and the shared overland-river
launch is chosen on whole replayed steps.
"""

import inspect

from wflow_gb300 import autotune
from wflow_gb300.model import Model

PHASES = ("vertical", "subsurface", "overland", "river", "balance")


class StandIn:
    """Records tunings and charges each step by a cost function of the current tuning."""

    def __init__(self, cost):
        self.cost = cost
        self._tune_state = {}
        self.tuning = {}
        self.kt = dict.fromkeys(PHASES, 0.0)
        self.calls = 0
        self.steps = 0
        self.step_ms = 0.0
        self.accepted = set(inspect.signature(Model.set_tuning).parameters) - {"self"}

    def set_tuning(self, **kw):
        assert set(kw) <= self.accepted, set(kw) - self.accepted
        self.tuning = kw

    def run_timestep(self, P, PET, T):
        c = self.cost(self.tuning)
        self.steps += 1
        if self.tuning.get("kernel_timing"):
            self.calls += 1
            for k in PHASES:
                self.kt[k] += c[k]
        self.step_ms += sum(c.values()) + (c.get("graph_extra", 0.0) if self.tuning.get("use_graph") else 0.0)

    def kernel_times(self):
        return dict(self.kt), self.calls

    def metrics(self):
        return {"steps": self.steps, "substeps_land": self.steps, "substeps_river": 4 * self.steps,
                "step_ms_total": self.step_ms}


def cost_of(t):
    warps, bps = t.get("routing_warps", 0), t.get("routing_blocks_per_sm", 0)
    route = 10.0 - (2.0 if (warps, bps) == (4, 2) else 0.0)
    lanes = t.get("substep_lanes", 0)
    inputs = t.get("sweep_inputs", 0)
    shared = t.get("separate_overland_river", 0) == 0
    c = {"vertical": 5.0 - (1.0 if (t.get("vertical_block"), t.get("vertical_blocks_per_sm")) == (256, 8) else 0.0),
         "subsurface": route - (0.5 if inputs & 1 else 0.0),
         "overland": route / 2 - (0.3 if inputs & 2 else 0.0),
         "river": route / 2 - (0.7 if lanes == 4 else 0.0) - (0.2 if inputs & 4 else 0.0),
         "balance": 1.0}
    if shared:  # the shared launch: faster on replayed steps only with lanes 1
        c["overland"], c["river"] = c["overland"] + c["river"] - (1.5 if lanes == 1 else -1.0), 0.1
    return c


def test_tuner_picks_the_fastest_shapes():
    m = StandIn(cost_of)
    choice, results = autotune.tune(m, lambda s: (None, None, None))
    assert (choice["routing_warps"], choice["routing_blocks_per_sm"]) == (4, 2)
    assert (choice["vertical_block"], choice["vertical_blocks_per_sm"]) == (256, 8)
    assert choice["sweep_inputs"] == 7
    # separate launches are fastest with 4 lanes, the shared launch with 1 lane, and the shared
    # launch with 1 lane beats both on whole steps
    assert choice["separate_overland_river"] == 0 and choice["substep_lanes"] == 1, choice
    assert m.tuning.get("use_graph") == 1 and not m.tuning.get("kernel_timing")
    assert any(r[0] == "overland_river_shared_launch" for r in results)


def test_tuner_keeps_separate_launches_when_they_are_faster():
    def cost(t):
        c = cost_of(t)
        if t.get("separate_overland_river", 0) == 0:
            c["overland"] += 5.0
        return c

    m = StandIn(cost)
    choice, _ = autotune.tune(m, lambda s: (None, None, None))
    assert choice["separate_overland_river"] == 1 and choice["substep_lanes"] == 4, choice
