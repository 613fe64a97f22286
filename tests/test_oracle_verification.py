"""The oracle against SparLab's own cross-validation results
(docs/results/cross_validation.csv, fixture tests/golden/verification.json):
the structured-grid models of configs/verification/{cantilever_analysis,
block_3d_analysis, column_hex_buckling_analysis}.json rebuilt by
sparlab_gb300.problems -- the largest displacement component of each static
load case (a total point load over a box of nodes; a uniform face traction
as consistent nodal forces) within 1e-9 relative, and the four smallest
buckling load factors of the Hex8 column within 1e-9 relative."""
import json
import os

import numpy as np

import oracle
from oracle import buckling as OB
from sparlab_gb300 import problems as P

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "verification.json")
STATIC = {"cantilever_analysis": (P.cantilever_analysis, ["tip_load"]),
          "block_3d_analysis": (P.block_3d_analysis, ["tip_load", "top_pressure"])}


def golden():
    with open(GOLDEN) as f:
        return json.load(f)


def test_static_displacements():
    g = golden()["max_abs_displacement"]
    for name, (make, cases) in STATIC.items():
        spec = make()
        ev = oracle.Problem(spec).evaluate(np.ones(spec.num_elements), displacements=True)
        for l, case in enumerate(cases):
            got = float(np.abs(ev["u"][l]).max())
            want = g[f"{name}/{case}"]
            assert abs(got / want - 1.0) <= 1e-9, (name, case, got, want)


def test_hex_column_buckling_load_factors():
    want = np.array(golden()["buckling_load_factors"]["column_hex_buckling_analysis"])
    spec = P.column_hex_buckling_analysis()
    r = OB.analyse_buckling(oracle.Problem(spec), spec, num_modes=4, tolerance=1e-10, residual_tolerance=1e-8)
    assert r.converged and not r.transformed
    np.testing.assert_allclose(r.load_factors, want, rtol=1e-9)
