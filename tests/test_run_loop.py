"""The host side of run_oc's stopping rules (TopologyOptimizer.run and
objective_spread, src/topopt/TopologyOptimizer.cpp:124-130, 675-704) on a
scripted problem: no GPU is touched."""
import math
import types

import pytest

from sparlab_gb300.topopt import TopologyOptimizer, objective_spread


class Scripted:
    """iterate() returns the next (compliance, max change, final stage)."""

    def __init__(self, steps):
        self.steps = list(steps)
        self.calls = 0

    def iterate(self):
        c, dx, final = self.steps[self.calls]
        self.calls += 1
        return types.SimpleNamespace(
            compliance=c, volume_fraction=0.5, max_change=dx, lam=1.0, gray_level=0.1,
            linear_iterations=10, bisections=30, volume_converged=1, beta=1.0, final_stage=final,
            eroded_volume_fraction=0.0, dilated_volume_fraction=0.0, dilated_target_fraction=0.0)


def test_objective_spread():
    assert objective_spread([3.0, 2.0], 5) == math.inf          # fewer than window + 1 values
    assert objective_spread([9.0, 4.0, 5.0, 4.5], 2) == pytest.approx((5.0 - 4.0) / 4.5)
    assert objective_spread([1.0, 2.0], 0) == pytest.approx(0.5)  # a window below 1 counts as 1


def test_design_change_stops_first_and_only_at_the_final_stage():
    steps = [(10.0, 0.2, True), (9.0, 0.005, False), (8.0, 0.005, True), (7.0, 0.5, True)]
    opt = TopologyOptimizer(Scripted(steps), max_iterations=10, change_tolerance=0.01)
    hist = opt.run()
    assert len(hist) == 3 and opt.stop_reason == "design_change"


def test_objective_stall_stops_when_the_spread_settles():
    cs = [10.0, 6.0, 5.0, 5.001, 5.0002, 5.0001, 5.00015, 5.0001]
    # spreads of the last 3 values: 1, 0.2, 2.0e-4, 1.8e-4, then 2.0e-5 at iteration 7
    opt = TopologyOptimizer(Scripted([(c, 0.3, True) for c in cs]), max_iterations=10,
                            change_tolerance=0.01, objective_tolerance=1e-4, objective_window=2)
    hist = opt.run()
    assert len(hist) == 7 and opt.stop_reason == "objective_stall"
    assert opt.final_objective_change == pytest.approx(0.0001 / 5.00015)
    # before the projection's final stage a settled objective does not stop the run
    steps = [(c, 0.3, i >= 7) for i, c in enumerate(cs)]
    opt = TopologyOptimizer(Scripted(steps), max_iterations=10, change_tolerance=0.01,
                            objective_tolerance=1e-4, objective_window=2)
    assert len(opt.run()) == 8 and opt.stop_reason == "objective_stall"


def test_disabled_rules_run_to_the_cap():
    steps = [(5.0, 0.0, True)] * 4
    opt = TopologyOptimizer(Scripted(steps), max_iterations=4, change_tolerance=0)
    assert len(opt.run()) == 4 and opt.stop_reason == "iteration_cap"
