"""Solves advanced together in one CUDA graph (conditional nodes) compute
exactly what they compute one at a time.

block_pcg 2 advances a problem's load cases together; simp_iterate_batch
advances every load case of many independent problems together.  Each solve
keeps its own iterations, restarts and stopping test, so compliances,
iteration counts and OC multipliers must equal the one-at-a-time runs bit
for bit; the first history is also checked against the oracle, and a
failing problem (an iteration budget of one) reports its error while the
others iterate on unchanged."""
import numpy as np
import pytest

import oracle
from sparlab_gb300 import problems as P
from sparlab_gb300._lib import ConvergenceError
from sparlab_gb300.topopt import GpuSimpProblem, iterate_batch, run_batched

pytestmark = pytest.mark.gpu


def three_load_q4():
    spec = P.q4_cantilever_600x200()
    spec.nx, spec.ny, spec.lx, spec.ly = 60, 20, 60.0, 20.0
    spec.fixed = P.clamp_left(spec)
    loads = []
    for i, j in enumerate((5, 10, 15)):
        t = np.radians(P.SplitMix64(2, i).uniform(-90.0, 90.0))
        loads.append(P.point_load(spec, [spec.node_index(60, j)], (np.sin(t), -np.cos(t))))
    spec.loads = np.stack(loads)
    spec.rtol = 1e-10
    return spec


def rows(recs):
    return [(r.compliance, r.linear_iterations, r.lam, r.bisections) for r in recs]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_load_cases_in_one_graph_match_one_after_another(precision):
    spec = three_load_q4()
    out = {}
    for mode in (False, "graph"):
        gpu = GpuSimpProblem(spec, precision=precision, block_pcg=mode)
        out[mode] = rows([gpu.iterate() for _ in range(4)])
        gpu.close()
    assert out["graph"] == out[False]
    ref = oracle.Problem(spec)
    _, hist = ref.run(4)
    for k, r in enumerate(out["graph"]):
        assert abs(r[0] / hist[k, 0] - 1) < 1e-6


def test_five_load_cases_with_fused_operators_match_one_after_another():
    """Five load cases of one Hex8 problem in mixed precision whose K_ff
    (double-float value pairs) exceeds L2, so that in the graph the cases'
    CG products run as fused multi-RHS launches over the shared K_ff (four
    cases per launch, so two launches): every iteration's compliance,
    iteration count and OC multiplier equal the one-after-another solves bit
    for bit."""
    spec = P.hex8_cantilever(64, 36, 36, 0.3, "five_loads")   # K_ff 20.3 M values, 155 MiB
    loads = []
    for i in range(5):
        rng = P.SplitMix64(9, i)
        j, k = int(rng.uniform(0.0, 36.99)), int(rng.uniform(0.0, 36.99))
        t = np.radians(rng.uniform(-90.0, 90.0))
        loads.append(P.point_load(spec, [spec.node_index(64, j, k)], (0.0, np.sin(t), -np.cos(t))))
    spec.loads = np.stack(loads)
    spec.weights = np.full(5, 0.2)
    spec.rtol = 1e-10
    out = {}
    for mode in (False, "graph"):
        gpu = GpuSimpProblem(spec, precision="mixed", block_pcg=mode)
        assert gpu.nnz * 8 >= 128 * 1024 * 1024   # the fused launches apply from this size
        out[mode] = rows([gpu.iterate() for _ in range(3)])
        gpu.close()
    assert out["graph"] == out[False]


def test_batch_of_uneven_problems_matches_one_at_a_time():
    specs = P.batched_instances(seed=4, count_q4=4, count_hex=3)
    alone = []
    for spec in specs:
        prob = GpuSimpProblem(spec, precision="mixed")
        alone.append(rows([prob.iterate() for _ in range(3)]))
        prob.close()
    probs = [GpuSimpProblem(s, precision="mixed") for s in specs]
    recs = run_batched(probs, 3, together=True)
    for k in range(len(specs)):
        assert rows(recs[k]) == alone[k], specs[k].name
    for p in probs:
        p.close()


def test_batch_reports_a_failing_problem_and_iterates_the_others():
    specs = P.batched_instances(seed=4, count_q4=2, count_hex=1)
    specs[1].max_cg_iterations = 1
    specs[1].rtol = 1e-12
    alone = []
    for k in (0, 2):
        ref = GpuSimpProblem(specs[k], precision="fp64")
        ref.iterate()
        alone.append(ref.design())
        ref.close()
    probs = [GpuSimpProblem(s, precision="fp64") for s in specs]
    with pytest.raises(ConvergenceError) as e:
        iterate_batch(probs)
    assert "did not converge" in str(e.value)
    # the healthy problems took exactly the step they take alone
    np.testing.assert_array_equal(probs[0].design(), alone[0])
    np.testing.assert_array_equal(probs[2].design(), alone[1])
    for p in probs:
        p.close()
