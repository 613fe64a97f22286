"""Pin the CPU oracle before trusting it as the checker of the CUDA path.

Known answers: the reference's published bench-model compliances, CG
iteration counts, AMG level counts and operator complexities
(docs/results/solver_scaling.csv, fixture tests/golden/solver_scaling.json).
Identities: the ones the reference's tests assert for the hierarchy, the
V-cycle, the filter and the OC update (tests/test_multigrid.cpp:162-256,
tests/test_topopt.cpp:162-251, 550-586)."""
import json
import os

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import oracle
from sparlab_gb300 import problems as P

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "solver_scaling.json")


def golden_rows(solver, max_dofs):
    with open(GOLDEN) as f:
        rows = json.load(f)["rows"]
    return [r for r in rows if r["solver"] == solver and r["num_dofs"] <= max_dofs
            and r["element"] in ("Quad4", "Hex8")]


def bench_problem(r):
    dim = 3 if r["element"] == "Hex8" else 2
    return P.bench_model(dim, r["nx"], r["ny"], r["nz"]), dim


@pytest.mark.parametrize("row", golden_rows("amg", 60000),
                         ids=lambda r: f"{r['element']}-{r['nx']}x{r['ny']}x{r['nz']}")
def test_amg_matches_published_bench_model(row):
    spec, dim = bench_problem(row)
    pr = oracle.Problem(spec)
    assert pr.ndof == row["num_dofs"]
    ptr, col, val = pr.kff()
    sol = oracle.Solver(rtol=1e-10)
    sol.factorize(ptr, col, val, dim, pr.coords(), pr.free_dofs())
    f = spec.loads[0][pr.free_dofs()]
    x, it, rr = sol.solve(f)
    c = float(f @ x)
    assert abs(c / row["compliance"] - 1.0) < 1e-9
    assert it == row["iterations"]
    assert sol.num_levels() == row["levels"]
    # operator complexity is a ratio of integer counts: exact when the
    # hierarchy (aggregates, ranks, patterns) is the reference's
    assert sol.stats()["operator_complexity"] == pytest.approx(row["operator_complexity"],
                                                                rel=1e-15, abs=0)


@pytest.mark.parametrize("row", golden_rows("ldlt", 8000),
                         ids=lambda r: f"{r['element']}-{r['nx']}x{r['ny']}x{r['nz']}")
def test_direct_solution_matches_published_compliance(row):
    spec, dim = bench_problem(row)
    pr = oracle.Problem(spec)
    ptr, col, val = pr.kff()
    n = len(ptr) - 1
    k = sp.csr_matrix((val, col, ptr), shape=(n, n))
    f = spec.loads[0][pr.free_dofs()]
    u = spla.spsolve(k.tocsc(), f)
    assert abs(float(f @ u) / row["compliance"] - 1.0) < 1e-10


def test_free_free_pattern_size_matches_published_nonzeros():
    """The published stiffness_nonzeros is nnz(K_ff) of the reduced system."""
    with open(GOLDEN) as f:
        rows = json.load(f)["rows"]
    seen = 0
    for r in rows:
        if r["solver"] != "ldlt" or r["element"] not in ("Quad4", "Hex8"):
            continue
        spec, _ = bench_problem(r)
        pr = oracle.Problem(spec)
        assert pr.ndof == r["num_dofs"]
        assert pr.nnz == r["stiffness_nonzeros"]
        seen += 1
    assert seen >= 10


def small_hex(nx=12, ny=6, nz=4, scale=None):
    spec = P.bench_model(3, nx, ny, nz)
    pr = oracle.Problem(spec)
    ptr, col, val = pr.kff(scale)
    return spec, pr, ptr, col, val


def test_hierarchy_identities():
    spec, pr, ptr, col, val = small_hex()
    sol = oracle.Solver(rtol=1e-12, coarse_size=60)
    sol.factorize(ptr, col, val, 3, pr.coords(), pr.free_dofs())
    assert sol.num_levels() >= 3
    for lvl in range(sol.num_levels() - 1):
        rows, cols, pp, pc, pv = sol.prolongator(lvl, tentative=True)
        pt = sp.csr_matrix((pv, pc, pp), shape=(rows, cols))
        b = sol.nullspace(lvl)
        bc = sol.nullspace(lvl + 1)
        assert np.abs(pt @ bc - b).max() < 1e-12            # P-hat B_c = B
        g = (pt.T @ pt).toarray()
        assert np.abs(g - np.eye(cols)).max() < 1e-12       # orthonormal columns
        rows, cols, qp, qc, qv = sol.prolongator(lvl)
        p = sp.csr_matrix((qv, qc, qp), shape=(rows, cols))
        ap, ac, av = sol.level_matrix(lvl)
        a = sp.csr_matrix((av, ac, ap), shape=(rows, rows))
        cp, cc, cv = sol.level_matrix(lvl + 1)
        acoarse = sp.csr_matrix((cv, cc, cp), shape=(cols, cols))
        gal = (p.T @ a @ p)
        assert abs(acoarse - gal).max() <= 1e-12 * abs(gal).max()
        assert cols < rows
    oc = sol.stats()["operator_complexity"]
    assert 1.0 < oc < 3.0


def test_vcycle_is_symmetric_and_contracting():
    spec, pr, ptr, col, val = small_hex()
    sol = oracle.Solver(rtol=1e-12, coarse_size=60)
    sol.factorize(ptr, col, val, 3, pr.coords(), pr.free_dofs())
    n = len(ptr) - 1
    i = np.arange(n)
    x = np.sin(0.37 * i + 0.1) + 0.2
    y = np.sin(0.37 * i + 1.3) + 0.2
    mx, my = sol.apply(x), sol.apply(y)
    assert abs(x @ my - y @ mx) <= 1e-11 * abs(x @ my)
    assert x @ mx > 0
    a = sp.csr_matrix((val, col, ptr), shape=(n, n))
    ustar = spla.spsolve(a.tocsc(), x)
    e1 = ustar - sol.apply(x)
    assert np.sqrt(e1 @ (a @ e1)) < 0.9 * np.sqrt(ustar @ (a @ ustar))


def test_simp_contrast_matches_direct_and_reuses_aggregates():
    spec = P.bench_model(3, 16, 8, 4)
    pr = oracle.Problem(spec)
    rng = P.SplitMix64(11)
    rho = rng.uniform_array(pr.ne, 0.0, 1.0)
    rho[rho < 0.4] = 0.001
    scale = 1e-9 + (1 - 1e-9) * rho ** 3
    ptr, col, val = pr.kff(scale)
    n = len(ptr) - 1
    sol = oracle.Solver(rtol=1e-10, coarse_size=60)
    sol.factorize(ptr, col, val, 3, pr.coords(), pr.free_dofs())
    f = spec.loads[0][pr.free_dofs()]
    x, it, _ = sol.solve(f)
    assert it < 200
    u = spla.spsolve(sp.csr_matrix((val, col, ptr), shape=(n, n)).tocsc(), f)
    assert abs((f @ x) / (f @ u) - 1) < 1e-7
    sol.factorize(ptr, col, val, 3, pr.coords(), pr.free_dofs())
    assert sol.stats()["reused_aggregates"]


def test_warm_start_from_solution_takes_no_iterations():
    spec, pr, ptr, col, val = small_hex(8, 4, 2)
    sol = oracle.Solver(rtol=1e-10, coarse_size=60)
    sol.factorize(ptr, col, val, 3, pr.coords(), pr.free_dofs())
    f = spec.loads[0][pr.free_dofs()]
    x, it, _ = sol.solve(f)
    x2, it2, _ = sol.solve(f, x0=x)
    assert it2 == 0


def test_under_constrained_is_reported():
    spec = P.bench_model(3, 8, 4, 2)
    spec.fixed = np.zeros_like(spec.fixed)   # no supports at all
    pr = oracle.Problem(spec)
    ptr, col, val = pr.kff()
    sol = oracle.Solver(rtol=1e-10, coarse_size=60)
    with pytest.raises(oracle.OracleError) as e:
        sol.factorize(ptr, col, val, 3, pr.coords(), pr.free_dofs())
    assert "under-constrained" in str(e.value)


def test_filter_rows_and_adjoint():
    for spec in (P.q4_cantilever_120x40(), P.hex8_cantilever(12, 6, 6, 0.3, "t")):
        pr = oracle.Problem(spec)
        ones = np.ones(pr.ne)
        assert np.abs(pr.filter_forward(ones) - 1).max() < 1e-12
        rng = P.SplitMix64(5)
        x = rng.uniform_array(pr.ne, 0, 1)
        v = rng.uniform_array(pr.ne, 0, 1)
        lhs = pr.filter_forward(x) @ v
        rhs = x @ pr.filter_adjoint(v)
        assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
        hx = pr.filter_forward(x)
        assert hx.min() >= x.min() - 1e-15 and hx.max() <= x.max() + 1e-15


def test_gradients_signs_and_strain_energy_sum():
    spec = P.q4_cantilever_120x40()
    spec.nx, spec.ny, spec.lx, spec.ly = 30, 10, 30.0, 10.0
    spec.fixed = P.clamp_left(spec)
    spec.loads = P.point_load(spec, [spec.node_index(30, 5)], (0.0, -1.0))[None, :]
    pr = oracle.Problem(spec)
    x = 0.4 + 0.25 * np.sin(np.arange(pr.ne) * 0.3)
    ev = pr.evaluate(x)
    assert ev["dc_dx"].max() <= 0 and ev["dv_dx"].min() > 0
    assert abs(ev["se"].sum() - 0.5 * ev["compliance"]) <= 1e-10 * ev["compliance"]


def test_finite_difference_sensitivities():
    spec = P.q4_cantilever_120x40()
    spec.nx, spec.ny, spec.lx, spec.ly = 12, 6, 12.0, 6.0
    spec.fixed = P.clamp_left(spec)
    spec.loads = P.point_load(spec, [spec.node_index(12, 3)], (0.0, -1.0))[None, :]
    spec.rtol = 1e-13
    pr = oracle.Problem(spec, amg=dict(coarse_size=60))
    x = 0.4 + 0.25 * np.sin(np.arange(pr.ne) * 0.7)
    ev = pr.evaluate(x)
    h = 1e-4
    for e in (0, 7, 33, 60):
        xp, xm = x.copy(), x.copy()
        xp[e] += h
        xm[e] -= h
        fd = (pr.evaluate(xp)["compliance"] - pr.evaluate(xm)["compliance"]) / (2 * h)
        assert abs(fd - ev["dc_dx"][e]) <= 1e-5 * abs(ev["compliance"])


def test_mma_reaches_the_oc_optimum():
    """tests/test_mma.cpp:419 of the reference: MMA and OC end at the same
    design quality on the compliance problem; MMA keeps V <= V* at the end."""
    spec = P.q4_cantilever_120x40()
    spec.nx, spec.ny, spec.lx, spec.ly = 30, 15, 30.0, 15.0
    spec.fixed = P.clamp_left(spec)
    spec.loads = P.point_load(spec, [spec.node_index(30, 7)], (0.0, -1.0))[None, :]
    spec.volume_fraction = 0.4
    spec.initial_density = 0.4
    pr = oracle.Problem(spec)
    _, hm = pr.run_mma(40)
    _, ho = pr.run(40)
    assert abs(hm[-1, 0] / ho[-1, 0] - 1) < 0.03
    assert hm[-1, 1] <= 0.4 + 1e-3
    assert np.all(hm[:, 5] > 0)


def test_oc_meets_volume_and_end_to_end_run_improves():
    spec = P.q4_cantilever_120x40()
    spec.nx, spec.ny, spec.lx, spec.ly = 30, 15, 30.0, 15.0
    spec.fixed = P.clamp_left(spec)
    spec.loads = P.point_load(spec, [spec.node_index(30, 7)], (0.0, -1.0))[None, :]
    spec.volume_fraction = 0.4
    spec.initial_density = 0.4
    pr = oracle.Problem(spec)
    x, hist = pr.run(30)
    assert np.all(np.abs(hist[:, 1] - 0.4) < 1e-6)
    assert hist[0, 0] / hist[-1, 0] > 1.5


def _projected_q4(nx=12, ny=6, beta=4.0):
    spec = P.q4_cantilever_120x40()
    spec.nx, spec.ny, spec.lx, spec.ly = nx, ny, float(nx), float(ny)
    spec.fixed = P.clamp_left(spec)
    spec.loads = P.point_load(spec, [spec.node_index(nx, ny // 2)], (0.0, -1.0))[None, :]
    spec.rtol = 1e-13
    spec.projection, spec.beta_start, spec.beta_max = True, beta, 64.0
    return spec


def test_projection_matches_the_reference_formula():
    """rho_bar = (tanh(b e) + tanh(b (rho - e))) / (tanh(b e) + tanh(b (1 - e)))
    (src/topopt/Projection.cpp:56-60) on the clamped filtered density."""
    spec = _projected_q4()
    pr = oracle.Problem(spec, amg=dict(coarse_size=60))
    x = 0.4 + 0.25 * np.sin(np.arange(pr.ne) * 0.7)
    rt = np.clip(pr.filter_forward(x), 0.0, 1.0)
    b, e = 4.0, 0.5
    want = (np.tanh(b * e) + np.tanh(b * (rt - e))) / (np.tanh(b * e) + np.tanh(b * (1 - e)))
    np.testing.assert_allclose(pr.evaluate(x)["rho"], want, rtol=0, atol=1e-15)


def test_projected_finite_difference_sensitivities():
    """dc/dx and dv/dx through the projection's chain rule (Sensitivity.cpp:
    100-108) against central differences."""
    spec = _projected_q4()
    pr = oracle.Problem(spec, amg=dict(coarse_size=60))
    x = 0.4 + 0.25 * np.sin(np.arange(pr.ne) * 0.7)
    ev = pr.evaluate(x)
    h = 1e-5
    for e in (0, 7, 33, 60):
        xp, xm = x.copy(), x.copy()
        xp[e] += h
        xm[e] -= h
        ep, em = pr.evaluate(xp), pr.evaluate(xm)
        fd = (ep["compliance"] - em["compliance"]) / (2 * h)
        assert abs(fd - ev["dc_dx"][e]) <= 1e-5 * abs(ev["compliance"])
        fv = (ep["volume"] - em["volume"]) / (2 * h)
        assert abs(fv - ev["dv_dx"][e]) <= 1e-6 * abs(ev["dv_dx"]).max()


def test_beta_continuation_schedule():
    """BetaSchedule (TopologyOptimizer.cpp:17-46): beta_start * factor^k,
    capped, a stage ends after beta_interval iterations."""
    spec = _projected_q4(20, 10, beta=1.0)
    spec.beta_max, spec.beta_interval, spec.advance_on_convergence = 4.0, 2, False
    spec.volume_fraction = 0.45
    _, hist = oracle.Problem(spec, amg=dict(coarse_size=100)).run(7)
    assert list(hist[:, 6]) == [1.0, 1.0, 2.0, 2.0, 4.0, 4.0, 4.0]


def _block_q4(nx=30, ny=15):
    """make_block of the reference's manufacturing tests (tests/
    test_manufacturing.cpp:55-82): 0.6 x 0.3 plate, E = 70e9, nu = 0.3,
    t = 0.01, root clamped, -1000 N at the node nearest (0.6, 0)."""
    spec = P.ProblemSpec(dim=2, nx=nx, ny=ny, nz=0, lx=0.6, ly=0.3, lz=0.0, young=70e9, poisson=0.3,
                         thickness=0.01, filter_radius=2.0 * 0.6 / nx, volume_fraction=0.4,
                         rtol=1e-12, name="block")
    spec.fixed = P.clamp_left(spec)
    spec.loads = P.point_load(spec, [P.nearest_node(spec, (0.6, 0.0, 0.0))], (0.0, -1000.0))[None, :]
    spec.weights = np.ones(1)
    return spec


def test_robust_thresholds_order_and_gradients():
    """test_manufacturing.cpp:246-306 (no overhang filter): eroded <=
    blueprint <= dilated, the objective on the eroded design, the dilated
    volume gradient against central differences."""
    spec = _block_q4(12, 6)
    spec.filter_radius = 1.5 * 0.05
    spec.projection, spec.robust, spec.robust_delta = True, True, 0.1
    spec.beta_start = spec.beta_max = 6.0
    pr = oracle.Problem(spec, amg=dict(coarse_size=60))
    x = P.SplitMix64(5).uniform_array(pr.ne, 0.0, 1.0)
    rt = np.clip(pr.filter_forward(x), 0.0, 1.0)

    def proj(eta):
        return oracle_project(rt, 6.0, eta)

    eroded, blueprint, dilated = proj(0.6), proj(0.5), proj(0.4)
    assert np.all(blueprint - eroded >= 0) and np.all(dilated - blueprint >= 0)
    ev = pr.evaluate(x)
    assert np.abs(ev["rho"] - eroded).max() <= 1e-15  # the objective's design is the eroded one
    v = np.full(pr.ne, 0.6 * 0.3 * 0.01 / pr.ne)
    grad = pr.filter_adjoint(v * oracle_project_derivative(rt, 6.0, 0.4))

    def vol_d(xx):
        return v @ oracle_project(np.clip(pr.filter_forward(xx), 0.0, 1.0), 6.0, 0.4)

    worst = 0.0
    for e in range(0, pr.ne, 3):
        xp, xm = x.copy(), x.copy()
        xp[e] += 1e-6
        xm[e] -= 1e-6
        fd = (vol_d(xp) - vol_d(xm)) / 2e-6
        worst = max(worst, abs(fd - grad[e]) / max(abs(fd), abs(grad[e]), 1e-3 * np.abs(grad).max()))
    assert worst < 1e-6
    c_worst = 0.0
    for e in range(0, pr.ne, 5):
        xp, xm = x.copy(), x.copy()
        xp[e] += 1e-4
        xm[e] -= 1e-4
        fd = (pr.evaluate(xp)["compliance"] - pr.evaluate(xm)["compliance"]) / 2e-4
        g = ev["dc_dx"][e]
        c_worst = max(c_worst, abs(fd - g) / max(abs(fd), abs(g), 1e-3 * np.abs(ev["dc_dx"]).max()))
    assert c_worst < 3e-5


def oracle_project(r, beta, eta):
    return (np.tanh(beta * eta) + np.tanh(beta * (r - eta))) / (np.tanh(beta * eta) + np.tanh(beta * (1 - eta)))


def oracle_project_derivative(r, beta, eta):
    return beta * (1 - np.tanh(beta * (r - eta)) ** 2) / (np.tanh(beta * eta) + np.tanh(beta * (1 - eta)))


@pytest.mark.parametrize("method", ["oc", "mma"])
def test_robust_run_reports_the_blueprint(method):
    """test_manufacturing.cpp:308-347 (OC and MMA, no overhang filter): the
    blueprint meets the volume fraction up to the target's lag, eroded <
    blueprint < dilated volumes, and the eroded design is the softest."""
    spec = _block_q4()
    spec.projection, spec.robust, spec.robust_delta = True, True, 0.1
    spec.beta_start, spec.beta_max, spec.beta_interval = 2.0, 8.0, 15
    pr = oracle.Problem(spec)
    x, hist = pr.run(60, change_tol=1e-3) if method == "oc" else pr.run_mma(60)
    last = hist[-1]
    assert abs(last[1] - 0.4) < 0.02
    assert last[7] < last[1] < last[8]
    comp = {}
    for name, eta in (("eroded", 0.6), ("intermediate", 0.5), ("dilated", 0.4)):
        s2 = _block_q4()
        s2.projection, s2.eta, s2.beta_start, s2.beta_max = True, eta, 8.0, 8.0
        comp[name] = oracle.Problem(s2).evaluate(x)["compliance"]
    assert comp["eroded"] > comp["intermediate"] > comp["dilated"]
