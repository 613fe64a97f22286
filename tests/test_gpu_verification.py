"""The GPU analysis against SparLab's own cross-validation results
(docs/results/cross_validation.csv, fixture tests/golden/verification.json;
the oracle meets the same numbers in tests/test_oracle_verification.py): the
largest displacement component of each static load case of
configs/verification/{cantilever_analysis, block_3d_analysis}.json at full
density, and the four smallest buckling load factors of
column_hex_buckling_analysis.json (3,000 free DOFs: the subspace iteration
on the GPU AMG), in FP64 within 1e-9 and 1e-8 relative."""
import numpy as np
import pytest

import oracle
from sparlab_gb300 import problems as P
from sparlab_gb300.topopt import GpuSimpProblem
from test_oracle_verification import STATIC, golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", sorted(STATIC))
def test_static_displacements(name):
    g = golden()["max_abs_displacement"]
    make, cases = STATIC[name]
    spec = make()
    prob = GpuSimpProblem(spec, element_matrix=oracle.Problem(spec).element_matrix(), precision="fp64")
    prob.set_design(np.ones(spec.num_elements))
    ev = prob.evaluate(displacements=True)
    prob.close()
    for l, case in enumerate(cases):
        got = float(np.abs(ev.displacements[l]).max())
        want = g[f"{name}/{case}"]
        assert abs(got / want - 1.0) <= 1e-9, (name, case, got, want)


def test_hex_column_buckling_load_factors():
    want = np.array(golden()["buckling_load_factors"]["column_hex_buckling_analysis"])
    spec = P.column_hex_buckling_analysis()
    prob = GpuSimpProblem(spec, element_matrix=oracle.Problem(spec).element_matrix(), precision="fp64")
    assert prob.nfree > 400
    b = prob.buckling(num_modes=4, tolerance=1e-10, residual_tolerance=1e-8)
    prob.close()
    assert b.converged and not b.transformed and b.iterations > 0
    np.testing.assert_allclose(b.load_factors, want, rtol=1e-8)
