"""GPU parity of the LinearSolver boundary (C ABI) against the CPU oracle.

Integer work is compared bit for bit (aggregates of every level); values
within the stated tolerances: displacements 1e-9 relative at rtol 1e-12,
Galerkin level operators 1e-12 relative, compliance of the reference's
bench model within 1e-9 of its published value."""
import json
import os

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import oracle
from sparlab_gb300 import problems as P
from sparlab_gb300.linear_solver import ConvergenceError, GpuAmgCgSolver, SolverError

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "solver_scaling.json")


def system(spec, scale=None):
    pr = oracle.Problem(spec)
    ptr, col, val = pr.kff(scale)
    return pr, ptr, col, val


def both(spec, scale=None, rtol=1e-12, **amg):
    pr, ptr, col, val = system(spec, scale)
    ref = oracle.Solver(rtol=rtol, **amg)
    ref.factorize(ptr, col, val, spec.dim, pr.coords(), pr.free_dofs())
    gpu = GpuAmgCgSolver(iterative_tolerance=rtol, **amg)
    gpu.set_layout(spec.dim, pr.coords(), pr.free_dofs())
    gpu.factorize(ptr, col, val)
    return pr, (ptr, col, val), ref, gpu


@pytest.mark.parametrize("dim,nx,ny,nz", [(3, 8, 4, 2), (3, 16, 8, 4), (2, 40, 20, 0),
                                          (3, 48, 24, 12), (2, 160, 80, 0)])
def test_bench_model_matches_published_compliance(dim, nx, ny, nz):
    with open(GOLDEN) as f:
        rows = [r for r in json.load(f)["rows"] if r["solver"] == "amg" and r["nx"] == nx
                and r["ny"] == ny and r["element"] == ("Hex8" if dim == 3 else "Quad4")]
    gold = rows[0]
    spec = P.bench_model(dim, nx, ny, nz)
    pr, _, ref, gpu = both(spec, rtol=1e-10)
    f = spec.loads[0][pr.free_dofs()]
    x = gpu.solve(f)
    assert abs(f @ x / gold["compliance"] - 1) < 1e-9
    st = gpu.amg_stats()
    assert st["num_levels"] == gold["levels"]
    assert st["operator_complexity"] == gold["operator_complexity"]
    assert abs(gpu.last_iterations() - gold["iterations"]) <= 1


def test_aggregates_bit_exact_and_levels_match_oracle():
    spec = P.bench_model(3, 24, 12, 8)
    rng = P.SplitMix64(7)
    rho = rng.uniform_array(spec.num_elements, 0.01, 1.0)
    scale = 1e-9 + (1 - 1e-9) * rho ** 3
    pr, (ptr, col, val), ref, gpu = both(spec, scale, coarse_size=60)
    assert gpu.amg_stats()["num_levels"] == ref.num_levels()
    for lvl in range(ref.num_levels() - 1):
        np.testing.assert_array_equal(gpu.aggregates(lvl), ref.aggregates(lvl))
    for lvl in range(1, ref.num_levels()):
        gp, gc, gv = gpu.level_matrix(lvl)
        rp, rc, rv = ref.level_matrix(lvl)
        np.testing.assert_array_equal(gp, rp)
        np.testing.assert_array_equal(gc, rc)
        assert np.abs(gv - rv).max() <= 1e-12 * np.abs(rv).max()


def test_solution_matches_oracle_and_direct():
    spec = P.bench_model(3, 20, 10, 6)
    pr, (ptr, col, val), ref, gpu = both(spec, coarse_size=60)
    f = spec.loads[0][pr.free_dofs()]
    xg = gpu.solve(f)
    xr, itr, _ = ref.solve(f)
    n = len(ptr) - 1
    u = spla.spsolve(sp.csr_matrix((val, col, ptr), shape=(n, n)).tocsc(), f)
    assert np.linalg.norm(xg - xr) <= 1e-9 * np.linalg.norm(xr)
    assert np.linalg.norm(xg - u) <= 1e-8 * np.linalg.norm(u)
    assert abs(gpu.last_iterations() - itr) <= 1
    assert gpu.last_error() <= 1e-12


def test_vcycle_symmetric_and_matches_oracle():
    spec = P.bench_model(3, 12, 6, 4)
    pr, (ptr, col, val), ref, gpu = both(spec, coarse_size=60)
    n = len(ptr) - 1
    i = np.arange(n)
    x = np.sin(0.37 * i + 0.1) + 0.2
    y = np.sin(0.37 * i + 1.3) + 0.2
    mx, my = gpu.apply_preconditioner(x), gpu.apply_preconditioner(y)
    assert abs(x @ my - y @ mx) <= 1e-11 * abs(x @ my)
    rx = ref.apply(x)
    assert np.linalg.norm(mx - rx) <= 1e-10 * np.linalg.norm(rx)


def test_simp_contrast_reuse_and_warm_start():
    spec = P.bench_model(3, 16, 8, 4)
    rng = P.SplitMix64(11)
    rho = rng.uniform_array(spec.num_elements, 0.0, 1.0)
    rho[rho < 0.4] = 0.001
    scale = 1e-9 + (1 - 1e-9) * rho ** 3
    pr, (ptr, col, val), ref, gpu = both(spec, scale, rtol=1e-10, coarse_size=60)
    f = spec.loads[0][pr.free_dofs()]
    x = gpu.solve(f)
    xr, _, _ = ref.solve(f)
    assert abs((f @ x) / (f @ xr) - 1) < 1e-8
    gpu.factorize(ptr, col, val)
    assert gpu.amg_stats()["reused_aggregates"]
    x2 = gpu.solve_from(f, x)
    assert gpu.last_iterations() == 0
    assert np.array_equal(x2, x)


def test_deterministic_runs():
    spec = P.bench_model(3, 16, 8, 4)
    pr, (ptr, col, val), ref, gpu = both(spec, coarse_size=60)
    f = spec.loads[0][pr.free_dofs()]
    a = gpu.solve(f)
    b = gpu.solve(f)
    assert np.array_equal(a, b)


def test_errors_are_reported_and_context_survives():
    spec = P.bench_model(3, 8, 4, 2)
    spec.fixed = np.zeros_like(spec.fixed)
    pr, ptr, col, val = system(spec)
    gpu = GpuAmgCgSolver(coarse_size=60)
    gpu.set_layout(3, pr.coords(), pr.free_dofs())
    with pytest.raises(SolverError) as e:
        gpu.factorize(ptr, col, val)
    assert "under-constrained" in str(e.value)
    # not symmetric
    spec = P.bench_model(3, 8, 4, 2)
    pr, ptr, col, val = system(spec)
    bad = val.copy()
    bad[5] *= 1.5
    gpu = GpuAmgCgSolver(coarse_size=60)
    gpu.set_layout(3, pr.coords(), pr.free_dofs())
    with pytest.raises(SolverError) as e:
        gpu.factorize(ptr, col, bad)
    assert "not symmetric" in str(e.value)
    nan = val.copy()
    nan[3] = np.nan
    with pytest.raises(SolverError):
        gpu.factorize(ptr, col, nan)
    # iteration budget
    gpu = GpuAmgCgSolver(iterative_tolerance=1e-14, max_iterations=1, coarse_size=60)
    spec = P.bench_model(3, 16, 8, 4)
    pr, ptr, col, val = system(spec)
    gpu.set_layout(3, pr.coords(), pr.free_dofs())
    gpu.factorize(ptr, col, val)
    with pytest.raises(ConvergenceError) as e:
        gpu.solve(spec.loads[0][pr.free_dofs()])
    assert "did not converge" in str(e.value)
    # the context is still usable
    gpu2 = GpuAmgCgSolver(iterative_tolerance=1e-10, coarse_size=60)
    gpu2.set_layout(3, pr.coords(), pr.free_dofs())
    gpu2.factorize(ptr, col, val)
    gpu2.solve(spec.loads[0][pr.free_dofs()])


def _entry(ptr, col, i, j):
    return [k for k in range(ptr[i], ptr[i + 1]) if col[k] == j][0]


def test_zero_stiffness_node_is_reported_as_the_reference_does():
    """A node whose rows and columns are zero (an unconnected node) fails the
    positive-diagonal check of the setup (src/fem/Multigrid.cpp:727-733) in
    the oracle and on the GPU, with the same diagnosis and the entry's index;
    the context stays usable."""
    spec = P.bench_model(3, 16, 8, 4)
    pr, ptr, col, val = system(spec)
    z = val.copy()
    node = {90, 91, 92}
    rows = np.repeat(np.arange(len(ptr) - 1), np.diff(ptr))
    z[np.isin(rows, list(node)) | np.isin(col, list(node))] = 0.0
    ref = oracle.Solver(rtol=1e-10, coarse_size=60)
    with pytest.raises(oracle.OracleError) as eo:
        ref.factorize(ptr, col, z, 3, pr.coords(), pr.free_dofs())
    gpu = GpuAmgCgSolver(iterative_tolerance=1e-10, coarse_size=60)
    gpu.set_layout(3, pr.coords(), pr.free_dofs())
    with pytest.raises(SolverError) as eg:
        gpu.factorize(ptr, col, z)
    for msg in (str(eo.value), str(eg.value)):
        assert "diagonal entry 90" in msg and "positive diagonal" in msg
    gpu.factorize(ptr, col, val)
    x = gpu.solve(spec.loads[0][pr.free_dofs()])
    assert np.all(np.isfinite(x))


def test_pcg_breakdown_is_reported_as_the_reference_does():
    """p^T A p <= 0 (src/fem/Multigrid.cpp:1187-1193): the x-y coupling of one
    node raised 2 % above sqrt(d_xx d_yy) makes the stiffness indefinite in a
    mode the coarse level does not see; the oracle's PCG breaks down at its
    first iteration and so does the GPU's, with SIMP_BREAKDOWN and the
    reference's wording; the context stays usable."""
    from sparlab_gb300._lib import SIMP_BREAKDOWN
    spec = P.bench_model(3, 16, 8, 4)
    pr, ptr, col, val = system(spec)
    b = val.copy()
    i, j = 3 * 50, 3 * 50 + 1
    c = 1.02 * np.sqrt(val[_entry(ptr, col, i, i)] * val[_entry(ptr, col, j, j)])
    b[_entry(ptr, col, i, j)] = c
    b[_entry(ptr, col, j, i)] = c
    f = spec.loads[0][pr.free_dofs()]
    ref = oracle.Solver(rtol=1e-10)
    ref.factorize(ptr, col, b, 3, pr.coords(), pr.free_dofs())
    with pytest.raises(oracle.OracleError) as eo:
        ref.solve(f)
    assert "broke down at iteration 1" in str(eo.value)
    gpu = GpuAmgCgSolver(iterative_tolerance=1e-10)
    gpu.set_layout(3, pr.coords(), pr.free_dofs())
    gpu.factorize(ptr, col, b)
    with pytest.raises(SolverError) as eg:
        gpu.solve(f)
    assert eg.value.code == SIMP_BREAKDOWN
    assert "broke down at iteration 1" in str(eg.value)
    gpu.factorize(ptr, col, val)
    x = gpu.solve(f)
    assert np.all(np.isfinite(x))


def test_mixed_precision_matches_fp64_solution():
    """FP32 operator / V-cycle with FP64 refinement reaches the same
    tolerance on the FP64 residual: solution within 1e-6 of the FP64 one."""
    spec = P.bench_model(3, 24, 12, 8)
    rng = P.SplitMix64(5)
    rho = rng.uniform_array(spec.num_elements, 0.01, 1.0)
    scale = 1e-9 + (1 - 1e-9) * rho ** 3
    pr, ptr, col, val = system(spec, scale)
    f = spec.loads[0][pr.free_dofs()]
    out = {}
    for prec in ("fp64", "mixed"):
        s = GpuAmgCgSolver(iterative_tolerance=1e-8, precision=prec, coarse_size=60)
        s.set_layout(3, pr.coords(), pr.free_dofs())
        s.factorize(ptr, col, val)
        x = s.solve(f)
        assert s.last_error() <= 1e-8
        out[prec] = (x, s.last_iterations())
        s.factorize(ptr, col, val)          # reused structure: FP32 setup products
        x2 = s.solve(f)
        assert s.amg_stats()["reused_aggregates"]
        assert np.linalg.norm(x2 - x) <= 1e-6 * np.linalg.norm(x)
    xa, xb = out["fp64"][0], out["mixed"][0]
    assert np.linalg.norm(xa - xb) <= 1e-6 * np.linalg.norm(xa)
    assert abs((f @ xa) / (f @ xb) - 1) <= 1e-7


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_stepwise_setup_with_host_and_device_values(precision):
    """simp_set_pattern + simp_set_values(_device) + simp_setup is the same
    factorization as simp_factorize: identical solutions, aggregate reuse on
    the second value set."""
    import torch
    spec = P.bench_model(3, 16, 8, 4)
    pr, (ptr, col, val), ref, gpu = both(spec, coarse_size=60)
    f = spec.loads[0][pr.free_dofs()]
    x_fact = gpu.solve(f)
    step = GpuAmgCgSolver(iterative_tolerance=1e-12, precision=precision, coarse_size=60)
    step.set_layout(3, pr.coords(), pr.free_dofs())
    step.set_pattern(ptr, col)
    if precision == "fp64":
        step.set_values(val)
        step.setup()
        np.testing.assert_array_equal(step.solve(f), x_fact)
    dev = torch.tensor(val * 0.5, dtype=torch.float64, device="cuda")
    step.set_values_device(dev.data_ptr())
    step.setup()
    assert step.amg_stats()["reused_aggregates"] or precision == "mixed"
    x_half = step.solve(f)
    assert np.linalg.norm(x_half - 2.0 * x_fact) <= 1e-8 * np.linalg.norm(x_fact)
