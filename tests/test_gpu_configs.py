"""GPU parity at the workload configurations themselves, each against the
oracle (the CPU restatement of the reference's algorithms):

1. Q4 120x40 cantilever, 50 OC iterations in FP64 at rtol 1e-8: the
   compliance history within 1e-6, volume fractions within 1e-8, CG
   iteration counts within one.
2. Q4 600x200 with its three seeded point loads (weights 1/3), mixed
   precision, three iterations: weighted compliance within 1e-6 of the
   oracle's FP64 run.
3. Hex8 96x48x48 at the seeded i.i.d. U[0.01, 1] density (seed 3, filtered):
   one solve in FP64 and in mixed precision with the assembled and the
   matrix-free level-0 operators, against the oracle's FP64 AMG-PCG driven to
   rtol 1e-13 with a true-residual check (no sparse direct solver reaches
   691,488 unknowns here): compliance and displacements within 1e-6.
4. The 64 seeded uneven instances, two mixed-precision iterations run
   concurrently: every 8th instance's compliance history within 1e-6 of the
   oracle's.
5. Hex8 192x96x96 (5,419,584 free DOFs), the benchmark's own workload: two
   SIMP iterations with the learned start in mixed precision (an untrained
   network: the answer must not depend on the prediction) against the
   oracle's FP64 iterations (previous-displacement start), compliance within
   1e-6, CG iterations at most two above the oracle's.

Tolerances follow the reference's solver tests (tests/test_multigrid.cpp:
257-360: AMG against direct 1e-8 in the solution, SIMP contrast 1e-7 in the
compliance) loosened to the 1e-6 compliance bar of the benchmark metric."""
import numpy as np
import pytest

import oracle
from sparlab_gb300 import problems as P
from sparlab_gb300.topopt import GpuSimpProblem, TopologyOptimizer, run_batched

pytestmark = pytest.mark.gpu


def test_config1_q4_120x40_fifty_iterations_fp64():
    spec = P.q4_cantilever_120x40()
    ref = oracle.Problem(spec)
    _, hist = ref.run(50)
    gpu = GpuSimpProblem(spec, element_matrix=ref.element_matrix(), precision="fp64")
    recs = TopologyOptimizer(gpu, max_iterations=50, change_tolerance=0).run()
    assert len(recs) == 50 and len(hist) == 50
    for k, r in enumerate(recs):
        assert abs(r.compliance / hist[k, 0] - 1) < 1e-6, (k, r.compliance, hist[k, 0])
        assert abs(r.volume_fraction - hist[k, 1]) < 1e-8, k
        assert abs(r.linear_iterations - hist[k, 4]) <= 1, k
    assert recs[-1].compliance < 0.5 * recs[0].compliance


def test_config2_q4_600x200_three_loads_mixed():
    spec = P.q4_cantilever_600x200()
    ref = oracle.Problem(spec)
    _, hist = ref.run(3)
    gpu = GpuSimpProblem(spec, element_matrix=ref.element_matrix(), precision="mixed")
    recs = TopologyOptimizer(gpu, max_iterations=3, change_tolerance=0).run()
    for k, r in enumerate(recs):
        assert abs(r.compliance / hist[k, 0] - 1) < 1e-6, (k, r.compliance, hist[k, 0])
        assert abs(r.volume_fraction - hist[k, 1]) < 1e-8, k


@pytest.fixture(scope="module")
def config3():
    spec = P.hex8_96x48x48()
    x = P.seeded_density(spec, seed=3)
    tight = P.hex8_96x48x48()
    tight.rtol = 1e-13
    ref = oracle.Problem(tight)
    er = ref.evaluate(x, displacements=True)
    return spec, x, ref.element_matrix(), er


@pytest.mark.parametrize("precision,matrix_free", [("fp64", False), ("mixed", False), ("mixed", True)])
def test_config3_hex8_96x48x48_seeded_single_solve(config3, precision, matrix_free):
    spec, x, ke, er = config3
    spec.rtol = 1e-10
    gpu = GpuSimpProblem(spec, element_matrix=ke, precision=precision,
                         **({} if precision == "fp64" else {"matrix_free": int(matrix_free)}))
    gpu.set_design(x)
    ev = gpu.evaluate(displacements=True)
    assert abs(ev.compliance / er["compliance"] - 1) < 1e-6
    u, ur = ev.displacements[0], er["u"][0]
    assert np.linalg.norm(u - ur) <= 1e-6 * np.linalg.norm(ur)
    np.testing.assert_array_equal(ev.physical_density, er["rho"])
    scale = np.abs(er["dc_dx"]).max()
    assert np.abs(ev.dc_dx - er["dc_dx"]).max() <= 1e-6 * scale
    gpu.close()


def test_config4_batched_64_every_eighth_against_oracle():
    specs = P.batched_instances(seed=4)
    assert len(specs) == 64
    probs = [GpuSimpProblem(s, precision="mixed") for s in specs]
    recs = run_batched(probs, 2)
    for q in range(0, 64, 8):
        ref = oracle.Problem(specs[q])
        _, hist = ref.run(2)
        for k in range(2):
            assert abs(recs[q][k].compliance / hist[k, 0] - 1) < 1e-6, (q, k)
            assert abs(recs[q][k].volume_fraction - hist[k, 1]) < 1e-8, (q, k)
    for p in probs:
        p.close()


def test_config5_hex8_192x96x96_learned_mixed_against_the_oracle():
    from sparlab_gb300.surrogate import Surrogate
    spec = P.hex8_192x96x96()
    ref = oracle.Problem(spec)
    _, hist = ref.run(2)
    spec.warm_start = 3
    sur = Surrogate(seed=7)
    gpu = GpuSimpProblem(spec, element_matrix=ref.element_matrix(), precision="mixed")
    gpu.set_surrogate(sur)
    recs = [gpu.iterate() for _ in range(2)]
    for k, r in enumerate(recs):
        assert abs(r.compliance / hist[k, 0] - 1) < 1e-6, (k, r.compliance, hist[k, 0])
        assert abs(r.volume_fraction - hist[k, 1]) < 1e-8, k
        # the learned start may save iterations, never add many
        assert r.linear_iterations <= hist[k, 4] + 2, (k, r.linear_iterations, hist[k, 4])
    assert gpu.learned_seconds() > 0.0
    gpu.close()
