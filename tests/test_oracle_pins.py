"""More pins of the CPU oracle against the reference's own tests.

* structured numbering: node(i, j) = j (nx + 1) + i, node-major DOFs, the
  free DOFs ascending without the clamped face, and K's block pattern (one
  dim x dim block per node pair sharing an element) -- tests/test_mesh.cpp:
  20-62, src/fem/Assembler.cpp:111-155;
* multi-load-case compliance is the weighted sum with the weights
  normalised to one, and its gradient passes the finite-difference check --
  tests/test_topopt.cpp:487-548;
* the multigrid solve is bitwise identical for one thread and several --
  tests/test_multigrid.cpp:379-391;
* a hierarchy set up with reused aggregates equals a fresh one bit for bit
  -- tests/test_multigrid.cpp:513-542;
* MMA with one constraint row reaches the known optima of the reference's
  analytic problems -- tests/test_mma.cpp:90-167 (the two-row case of
  :118-146 needs a second constraint row, which the compliance problem never
  has).
"""
import os
import subprocess
import sys

import numpy as np

import oracle
from sparlab_gb300 import problems as P

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _q4(nx, ny, lx, ly):
    spec = P.ProblemSpec(dim=2, nx=nx, ny=ny, nz=0, lx=lx, ly=ly, lz=0.0, young=70.0e9,
                         poisson=0.3, thickness=0.01, filter_radius=0.0, name=f"q4_{nx}x{ny}")
    spec.fixed = P.clamp_left(spec)
    return spec


def _block_pattern(ptr, col, free, dim):
    """Set of (node_a, node_b) pairs with a stored entry in K_ff."""
    pairs = set()
    for r in range(len(ptr) - 1):
        a = int(free[r]) // dim
        for c in col[ptr[r]:ptr[r + 1]]:
            pairs.add((a, int(free[c]) // dim))
    return pairs


def test_structured_numbering_coordinates_and_free_dofs():
    """test_mesh.cpp:20-62: 3 x 2 cells on [0,3] x [0,2]; node(i, j) =
    j (nx + 1) + i; node 4 is (0, 1); node 11 is (3, 2)."""
    spec = _q4(3, 2, 3.0, 2.0)
    spec.loads = P.point_load(spec, [spec.node_index(3, 0)], (0.0, -1.0))[None, :]
    spec.weights = np.ones(1)
    pr = oracle.Problem(spec)
    c = pr.coords().reshape(-1, 2)
    assert pr.nn == 12 and pr.ne == 6
    np.testing.assert_array_equal(c[0], [0.0, 0.0])
    np.testing.assert_array_equal(c[3], [3.0, 0.0])
    np.testing.assert_array_equal(c[4], [0.0, 1.0])
    np.testing.assert_array_equal(c[11], [3.0, 2.0])
    assert spec.node_index(2, 1) == 6
    np.testing.assert_array_equal(c, spec.node_coords())
    # free DOFs ascending, node-major (node * 2 + k), nodes 0, 4, 8 clamped
    expect = [n * 2 + k for n in range(12) if n % 4 != 0 for k in range(2)]
    np.testing.assert_array_equal(pr.free_dofs(), expect)


def test_hex8_numbering_and_block_pattern():
    """Hex8 node(i, j, k) = (k (ny + 1) + j)(nx + 1) + i, and K_ff holds one
    3 x 3 block for every pair of free nodes that share an element: nodes
    whose grid indices differ by at most one in each direction."""
    spec = P.ProblemSpec(dim=3, nx=3, ny=2, nz=2, lx=3.0, ly=2.0, lz=2.0, filter_radius=0.0)
    spec.fixed = P.clamp_left(spec)
    spec.loads = P.point_load(spec, [spec.node_index(3, 0, 0)], (0.0, 0.0, -1.0))[None, :]
    spec.weights = np.ones(1)
    pr = oracle.Problem(spec)
    c = pr.coords().reshape(-1, 3)
    assert spec.node_index(1, 2, 1) == (1 * 3 + 2) * 4 + 1
    np.testing.assert_array_equal(c[spec.node_index(1, 2, 1)], [1.0, 2.0, 1.0])
    free = pr.free_dofs()
    ptr, col, _ = pr.kff()
    got = _block_pattern(ptr, col, free, 3)
    nnx, nny, _ = spec.nodes_per_axis

    def ijk(n):
        return n % nnx, (n // nnx) % nny, n // (nnx * nny)

    free_nodes = sorted({int(d) // 3 for d in free})
    want = {(a, b) for a in free_nodes for b in free_nodes
            if all(abs(p - q) <= 1 for p, q in zip(ijk(a), ijk(b)))}
    assert got == want
    # every stored block is full: 9 entries per node pair
    assert len(col) == 9 * len(want)


def _two_case_spec(w0=3.0, w1=1.0, cases=(0, 1)):
    """test_topopt.cpp:487-548: Q4 10 x 5 on 0.5 x 0.25 (t = 0.01, E = 70e9,
    nu = 0.3), root clamped; case "down" (0, -500) at the node nearest
    (lx, 0) with weight 3, case "sideways" (300, 0) at the node nearest
    (lx, ly) with weight 1; density filter of radius 1.5 cells; x = 0.5."""
    spec = _q4(10, 5, 0.5, 0.25)
    spec.filter_radius = 1.5 * 0.05
    spec.volume_fraction = spec.initial_density = 0.5
    spec.rtol = 1e-13
    loads = [P.point_load(spec, [P.nearest_node(spec, (0.5, 0.0, 0.0))], (0.0, -500.0)),
             P.point_load(spec, [P.nearest_node(spec, (0.5, 0.25, 0.0))], (300.0, 0.0))]
    weights = [w0, w1]
    spec.loads = np.stack([loads[i] for i in cases])
    spec.weights = np.array([weights[i] for i in cases])
    return spec


def test_weighted_compliance_is_the_normalised_weighted_sum():
    x = np.full(50, 0.5)
    both = oracle.Problem(_two_case_spec(), amg=dict(coarse_size=40)).evaluate(x)
    c0 = oracle.Problem(_two_case_spec(cases=(0,)), amg=dict(coarse_size=40)).evaluate(x)
    c1 = oracle.Problem(_two_case_spec(cases=(1,)), amg=dict(coarse_size=40)).evaluate(x)
    want = 0.75 * c0["compliance"] + 0.25 * c1["compliance"]
    assert abs(both["compliance"] - want) <= 1e-12 * want
    np.testing.assert_allclose(both["dc_dx"], 0.75 * c0["dc_dx"] + 0.25 * c1["dc_dx"],
                               rtol=1e-12, atol=1e-12 * np.abs(both["dc_dx"]).max())
    # scaling every weight changes nothing (weights are normalised to one)
    scaled = oracle.Problem(_two_case_spec(30.0, 10.0), amg=dict(coarse_size=40)).evaluate(x)
    assert scaled["compliance"] == both["compliance"]


def test_weighted_gradient_passes_the_finite_difference_check():
    """verify_sensitivities at step 1e-4 and tolerance 1e-5 on the two-case
    objective, at a non-uniform design so that the filter matters."""
    pr = oracle.Problem(_two_case_spec(), amg=dict(coarse_size=40))
    x = 0.45 + 0.2 * np.sin(np.arange(pr.ne) * 0.9)
    ev = pr.evaluate(x)
    h = 1e-4
    for e in (0, 9, 23, 41, 49):
        xp, xm = x.copy(), x.copy()
        xp[e] += h
        xm[e] -= h
        fd = (pr.evaluate(xp)["compliance"] - pr.evaluate(xm)["compliance"]) / (2 * h)
        assert abs(fd - ev["dc_dx"][e]) <= 1e-5 * abs(ev["compliance"])


_SOLVE = r"""
import hashlib, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import oracle
from sparlab_gb300 import problems as P
spec = P.ProblemSpec(dim=3, nx=40, ny=12, nz=12, lx=1.6, ly=0.48, lz=0.48, young=70.0e9,
                     poisson=0.3, filter_radius=0.0)
spec.fixed = P.clamp_left(spec)
spec.loads = P.point_load(spec, [P.nearest_node(spec, (1.6, 0.0, 0.0))], (0.0, -1000.0, 0.0))[None, :]
spec.weights = np.ones(1)
pr = oracle.Problem(spec)
ptr, col, val = pr.kff()
sol = oracle.Solver(rtol=1e-10)
sol.factorize(ptr, col, val, 3, pr.coords(), pr.free_dofs())
x, it, _ = sol.solve(spec.loads[0][pr.free_dofs()])
print(len(ptr) - 1, it, hashlib.sha256(np.ascontiguousarray(x).tobytes()).hexdigest())
"""


def _solve_with_threads(n):
    env = dict(os.environ, OMP_NUM_THREADS=str(n))
    out = subprocess.run([sys.executable, "-c", _SOLVE, ROOT], env=env, capture_output=True,
                         text=True, timeout=600, check=True)
    return out.stdout.split()


def test_multigrid_solve_is_bitwise_identical_for_any_thread_count():
    """Hex8 40 x 12 x 12 beam (20,280 free DOFs, above the 16,384-row
    threshold at which the CSR kernels go parallel): one thread and four
    give the same iteration count and the same bits."""
    serial = _solve_with_threads(1)
    parallel = _solve_with_threads(4)
    assert int(serial[0]) > 16384
    assert serial == parallel


def test_reused_hierarchy_equals_a_fresh_one_bit_for_bit():
    """tests/test_multigrid.cpp:513-542: a uniformly scaled matrix (every
    element factor 2.5) aggregates like the first one, so the hierarchy set up
    on it with the first matrix's aggregates reused and a fresh hierarchy give
    the same V-cycle bits (coarse_size 50)."""
    spec = P.ProblemSpec(dim=3, nx=10, ny=4, nz=4, lx=1.0, ly=0.4, lz=0.4, young=70.0e9,
                         poisson=0.3, filter_radius=0.0)
    spec.fixed = P.clamp_left(spec)
    spec.loads = P.point_load(spec, [P.nearest_node(spec, (1.0, 0.0, 0.0))], (0.0, -1000.0, 0.0))[None, :]
    spec.weights = np.ones(1)
    pr = oracle.Problem(spec)
    first = pr.kff()
    second = pr.kff(np.full(pr.ne, 2.5))
    coords, free = pr.coords(), pr.free_dofs()
    reused = oracle.Solver(coarse_size=50)
    reused.factorize(*first, 3, coords, free)
    reused.factorize(*second, 3, coords, free)
    assert reused.stats()["reused_aggregates"]
    fresh = oracle.Solver(coarse_size=50)
    fresh.factorize(*second, 3, coords, free)
    assert not fresh.stats()["reused_aggregates"]
    assert reused.num_levels() == fresh.num_levels() > 1
    x = P.SplitMix64(11).uniform_array(len(free), -1.0, 1.0)
    np.testing.assert_array_equal(reused.apply(x), fresh.apply(x))


def test_mma_solves_the_separable_problem_with_a_known_optimum():
    """tests/test_mma.cpp:90-116: min sum x_i^2 s.t. 1 - sum x_i <= 0 on
    [0, 1]^12 from x = 0.9: x_i = 1/12, multiplier 2/12, row untouched."""
    n = 12
    mma = oracle.Mma(n)
    x = np.full(n, 0.9)
    for _ in range(60):
        x, step = mma.update(x, 2.0 * x, 1.0 - x.sum(), np.full(n, -1.0))
        assert step["lam"] >= 0.0
        if step["max_change"] < 1e-9:
            break
    assert np.abs(x - 1.0 / n).max() < 1e-6
    assert abs(x.sum() - 1.0) <= 1e-6
    assert step["constraint_scale"] == 1.0
    assert abs(step["lam"] / (2.0 / n) - 1.0) <= 1e-3
    assert step["iteration"] > 2


def test_mma_scales_a_badly_violated_constraint_down():
    """tests/test_mma.cpp:148-167: min x1 + x2 s.t. 1e5 (1 - x1 - x2) <= 0
    on [0, 1]^2: the row is scaled down for the subproblem and the answer
    keeps x1 + x2 = 1 with multiplier 1e-5."""
    mma = oracle.Mma(2)
    x = np.full(2, 0.9)
    for _ in range(80):
        x, step = mma.update(x, np.ones(2), 1.0e5 * (1.0 - x.sum()), np.full(2, -1.0e5))
        if step["max_change"] < 1e-10:
            break
    assert step["constraint_scale"] < 1.0
    assert abs(x.sum() - 1.0) <= 1e-6
    assert abs(step["lam"] / 1.0e-5 - 1.0) <= 0.05
