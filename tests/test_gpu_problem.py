"""GPU parity of the whole-iteration boundary (structured problem) against
the oracle: assembly and filter bit for bit, objective / gradients / OC step
within tolerance, and a short OC run whose history matches."""
import numpy as np
import pytest

import oracle
from sparlab_gb300 import problems as P
from sparlab_gb300.topopt import GpuSimpProblem, TopologyOptimizer

pytestmark = pytest.mark.gpu


def small_q4(nx=30, ny=12, radius=1.5):
    spec = P.q4_cantilever_120x40()
    spec.nx, spec.ny, spec.lx, spec.ly = nx, ny, float(nx), float(ny)
    spec.filter_radius = radius
    spec.fixed = P.clamp_left(spec)
    spec.loads = P.point_load(spec, [spec.node_index(nx, ny // 2)], (0.0, -1.0))[None, :]
    spec.rtol = 1e-10
    return spec


def small_hex(nx=16, ny=8, nz=8):
    spec = P.hex8_cantilever(nx, ny, nz, 0.2, "t")
    spec.rtol = 1e-10
    return spec


def pair(spec, **kw):
    ref = oracle.Problem(spec)
    gpu = GpuSimpProblem(spec, element_matrix=ref.element_matrix(), **kw)
    return ref, gpu


@pytest.mark.parametrize("make", [small_q4, small_hex, lambda: small_q4(20, 10, 3.0)])
def test_assembly_and_filter_bit_exact(make):
    spec = make()
    ref, gpu = pair(spec)
    rng = P.SplitMix64(21)
    scale = 1e-9 + rng.uniform_array(ref.ne, 0.0, 1.0) ** 3
    rp, rc, rv = ref.kff(scale)
    gp, gc, gv = gpu.kff(scale)
    np.testing.assert_array_equal(gp, rp)
    np.testing.assert_array_equal(gc, rc)
    np.testing.assert_array_equal(gv, rv)
    x = rng.uniform_array(ref.ne, 0.0, 1.0)
    np.testing.assert_array_equal(gpu.filter_forward(x), ref.filter_forward(x))
    v = rng.uniform_array(ref.ne, -1.0, 1.0)
    np.testing.assert_array_equal(gpu.filter_adjoint(v), ref.filter_adjoint(v))


@pytest.mark.parametrize("make", [small_q4, small_hex])
def test_evaluate_and_oc_match_oracle(make):
    spec = make()
    # the seeded design has mean ~0.5: a target the move limit can reach
    spec.volume_fraction = 0.45
    ref, gpu = pair(spec)
    rng = P.SplitMix64(3)
    x = rng.uniform_array(ref.ne, 0.01, 1.0)
    gpu.set_design(x)
    ev = gpu.evaluate()
    er = ref.evaluate(x)
    assert abs(ev.compliance / er["compliance"] - 1) < 1e-8
    np.testing.assert_array_equal(ev.physical_density, er["rho"])
    scale = np.abs(er["dc_dx"]).max()
    assert np.abs(ev.dc_dx - er["dc_dx"]).max() <= 1e-7 * scale
    assert np.abs(ev.element_strain_energy.sum() - 0.5 * ev.compliance) <= 1e-8 * ev.compliance
    np.testing.assert_array_equal(ev.dv_dx, er["dv_dx"])
    assert abs(ev.volume_fraction - er["volume_fraction"]) < 1e-14
    step = gpu.oc_update(apply=False)
    xr, info = ref.oc_update(x, er["dc_dx"], er["dv_dx"])
    assert abs(step.lam / info["lam"] - 1) < 1e-6
    assert np.abs(step.x - xr).max() < 1e-6
    assert abs(step.achieved_volume / info["volume"] - 1) < 1e-9


def test_short_run_matches_oracle_history():
    spec = small_q4(40, 20)
    spec.initial_density = 0.5
    ref, gpu = pair(spec)
    _, hist = ref.run(8)
    recs = TopologyOptimizer(gpu, max_iterations=8, change_tolerance=0).run()
    for k, r in enumerate(recs):
        assert abs(r.compliance / hist[k, 0] - 1) < 1e-6, k
        assert abs(r.volume_fraction - hist[k, 1]) < 1e-9
    assert recs[-1].compliance < recs[0].compliance


def test_first_setup_aggregates_match_oracle_linear_solver():
    """The structured path assembles K_ff on the GPU; its level-0 aggregates
    must equal the oracle's on the oracle's assembly of the same factors."""
    from sparlab_gb300.linear_solver import GpuAmgCgSolver
    spec = small_hex(24, 12, 12)
    ref, gpu = pair(spec, coarse_size=200)
    gpu.evaluate()
    x = np.full(ref.ne, 0.2)
    rho = ref.filter_forward(x)
    sf = 1e-9 + (1 - 1e-9) * np.clip(rho, 0, 1) ** 3
    ptr, col, val = ref.kff(sf)
    solver = oracle.Solver(rtol=1e-10, coarse_size=200)
    solver.factorize(ptr, col, val, 3, ref.coords(), ref.free_dofs())
    st = gpu.amg_stats()
    assert st["num_levels"] == solver.num_levels()
    for lvl in range(solver.num_levels()):
        assert st["levels"][lvl]["unknowns"] == solver.level_info(lvl)[0]
        assert st["levels"][lvl]["nonzeros"] == solver.level_info(lvl)[1]


def test_mma_run_matches_oracle_history():
    """run_mma on the GPU against the oracle's restatement of the reference's
    MMA: same compliance and volume history, same subproblem iteration counts
    within one."""
    spec = small_q4(30, 15)
    spec.volume_fraction = 0.4
    spec.initial_density = 0.4
    ref, gpu = pair(spec, optimizer="mma")
    _, hist = ref.run_mma(10)
    recs = TopologyOptimizer(gpu, max_iterations=10, change_tolerance=0).run()
    for k, r in enumerate(recs):
        assert abs(r.compliance / hist[k, 0] - 1) < 1e-6, (k, r.compliance, hist[k, 0])
        assert abs(r.volume_fraction - hist[k, 1]) < 1e-8
        assert abs(r.lam / hist[k, 3] - 1) < 1e-5
        assert abs(r.bisections - hist[k, 5]) <= 1
    assert recs[-1].compliance < 0.6 * recs[0].compliance


def test_mixed_precision_iteration_matches_oracle():
    spec = small_hex(20, 10, 10)
    spec.rtol = 1e-8
    spec.initial_density = 0.2
    ref = oracle.Problem(spec)
    _, hist = ref.run(4)
    gpu = GpuSimpProblem(spec, element_matrix=ref.element_matrix(), precision="mixed")
    recs = TopologyOptimizer(gpu, max_iterations=4, change_tolerance=0).run()
    for k, r in enumerate(recs):
        assert abs(r.compliance / hist[k, 0] - 1) < 1e-6, (k, r.compliance, hist[k, 0])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_projected_warm_start_matches_oracle(precision):
    """warm_start 2 (energy-optimal start over the last three displacements)
    changes only the PCG's initial guess: the compliance history still matches
    the oracle's (which warm-starts from the previous displacement), and the
    solves need no more iterations in total than with warm_start 1."""
    spec = small_hex(20, 10, 10)
    spec.rtol = 1e-8
    spec.initial_density = 0.2
    ref = oracle.Problem(spec)
    _, hist = ref.run(8)
    its = {}
    for mode in (1, 2):
        spec.warm_start = mode
        gpu = GpuSimpProblem(spec, element_matrix=ref.element_matrix(), precision=precision)
        recs = TopologyOptimizer(gpu, max_iterations=8, change_tolerance=0).run()
        for k, r in enumerate(recs):
            assert abs(r.compliance / hist[k, 0] - 1) < 1e-6, (mode, k, r.compliance, hist[k, 0])
        its[mode] = sum(r.linear_iterations for r in recs)
    assert its[2] <= its[1], its


def test_mixed_cg_operator_matches_fp64_operator():
    """Mixed precision's CG operator (K_ff values split into float pairs,
    double-float products and sums) against the FP64 operator on the same
    design, after the exact first assembly and after a reuse assembly."""
    import torch
    spec = small_hex(20, 10, 10)
    spec.rtol = 1e-8
    ref = oracle.Problem(spec)
    rng = P.SplitMix64(17)
    probs = {p: GpuSimpProblem(spec, element_matrix=ref.element_matrix(), precision=p) for p in ("fp64", "mixed")}
    x = torch.tensor(rng.uniform_array(probs["fp64"].nfree, -1.0, 1.0), dtype=torch.float64, device="cuda")
    for design_seed in (5, 6):
        design = P.SplitMix64(design_seed).uniform_array(ref.ne, 0.05, 1.0)
        ys = {}
        for name, prob in probs.items():
            prob.set_design(design)
            prob.evaluate()
            y = torch.empty_like(x)
            prob.apply_operator(x.data_ptr(), y.data_ptr())
            torch.cuda.synchronize()
            ys[name] = y.cpu().numpy()
        scale = np.abs(ys["fp64"]).max()
        assert np.abs(ys["mixed"] - ys["fp64"]).max() <= 1e-11 * scale, design_seed


def test_batched_instances_match_sequential_and_oracle():
    """Independent instances driven concurrently from host threads (one CUDA
    stream each) compute exactly what they compute one at a time, and the
    first instance's history matches the oracle."""
    from sparlab_gb300.topopt import run_batched
    specs = P.batched_instances(seed=4, count_q4=3, count_hex=2)
    iters = 3
    seq = []
    for spec in specs:
        prob = GpuSimpProblem(spec, precision="mixed")
        seq.append([prob.iterate().compliance for _ in range(iters)])
        prob.close()
    probs = [GpuSimpProblem(spec, precision="mixed") for spec in specs]
    recs = run_batched(probs, iters, workers=4)
    for k, spec in enumerate(specs):
        assert [r.compliance for r in recs[k]] == seq[k], spec.name
    ref = oracle.Problem(specs[0])
    _, hist = ref.run(iters)
    for k in range(iters):
        assert abs(recs[0][k].compliance / hist[k, 0] - 1) < 1e-6


def test_run_writes_reference_history(tmp_path):
    """A GPU run's history.csv carries the records simp_iterate returned."""
    import csv
    from sparlab_gb300.results import OC_COLUMNS, write_results
    spec = small_q4(30, 12)
    gpu = GpuSimpProblem(spec)
    hist = TopologyOptimizer(gpu, max_iterations=4, change_tolerance=0).run()
    write_results(str(tmp_path), spec, hist, "oc", max_iterations=4, change_tolerance=0.0)
    rows = list(csv.reader(open(tmp_path / "history.csv")))
    assert rows[0] == OC_COLUMNS and len(rows) == 5
    for r, h in zip(rows[1:], hist):
        assert float(r[OC_COLUMNS.index("compliance[J]")]) == h.compliance
        assert int(float(r[OC_COLUMNS.index("oc_bisections[-]")])) == h.bisections
        assert r[OC_COLUMNS.index("volume_converged[-]")] in ("0", "1")


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_projected_run_matches_oracle(precision):
    """Heaviside projection with beta continuation (Projection.cpp,
    TopologyOptimizer.cpp:17-46): physical density, chain rule, projected OC
    volume and the beta schedule against the oracle."""
    spec = small_q4(40, 20)
    spec.rtol = 1e-10
    spec.initial_density = 0.5
    spec.projection, spec.beta_start, spec.beta_max = True, 1.0, 8.0
    spec.beta_interval, spec.advance_on_convergence = 2, False
    ref = oracle.Problem(spec)
    _, hist = ref.run(8)
    gpu = GpuSimpProblem(spec, element_matrix=ref.element_matrix(), precision=precision)
    recs = TopologyOptimizer(gpu, max_iterations=8, change_tolerance=0).run()
    assert [r.beta for r in recs] == list(hist[:, 6])
    for k, r in enumerate(recs):
        assert abs(r.compliance / hist[k, 0] - 1) < 1e-6, (k, r.compliance, hist[k, 0])
        assert abs(r.volume_fraction - hist[k, 1]) < 1e-8
    assert [r.final_stage for r in recs][-1]


def test_projected_evaluate_matches_oracle():
    spec = small_hex(12, 6, 6)
    spec.volume_fraction = 0.45
    spec.projection, spec.beta_start = True, 4.0
    ref, gpu = pair(spec)
    rng = P.SplitMix64(9)
    x = rng.uniform_array(ref.ne, 0.01, 1.0)
    gpu.set_design(x)
    ev = gpu.evaluate()
    er = ref.evaluate(x)
    assert abs(ev.compliance / er["compliance"] - 1) < 1e-8
    np.testing.assert_allclose(ev.physical_density, er["rho"], rtol=0, atol=1e-14)
    scale = np.abs(er["dc_dx"]).max()
    assert np.abs(ev.dc_dx - er["dc_dx"]).max() <= 1e-7 * scale
    np.testing.assert_allclose(ev.dv_dx, er["dv_dx"], rtol=1e-12, atol=0)
    step = gpu.oc_update(apply=False)
    xr, info = ref.oc_update(x, er["dc_dx"], er["dv_dx"])
    assert abs(step.lam / info["lam"] - 1) < 1e-6
    assert abs(step.achieved_volume / info["volume"] - 1) < 1e-9


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_concurrent_load_cases_match_sequential_and_oracle(precision):
    """Three load cases solved at the same time (block_pcg: one workspace and
    stream each) give exactly the sequential solves' results, and the
    weighted compliance history matches the oracle."""
    spec = P.q4_cantilever_600x200()
    spec.nx, spec.ny, spec.lx, spec.ly = 60, 20, 60.0, 20.0
    spec.fixed = P.clamp_left(spec)
    loads = []
    for i, j in enumerate((5, 10, 15)):
        t = np.radians(P.SplitMix64(2, i).uniform(-90.0, 90.0))
        loads.append(P.point_load(spec, [spec.node_index(60, j)], (np.sin(t), -np.cos(t))))
    spec.loads = np.stack(loads)
    spec.rtol = 1e-10
    ref = oracle.Problem(spec)
    _, hist = ref.run(4)
    recs = {}
    for together in (False, True):
        gpu = GpuSimpProblem(spec, element_matrix=ref.element_matrix(), precision=precision,
                             block_pcg=together)
        recs[together] = TopologyOptimizer(gpu, max_iterations=4, change_tolerance=0).run()
        gpu.close()
    assert [r.compliance for r in recs[True]] == [r.compliance for r in recs[False]]
    assert [r.linear_iterations for r in recs[True]] == [r.linear_iterations for r in recs[False]]
    for k, r in enumerate(recs[True]):
        assert abs(r.compliance / hist[k, 0] - 1) < 1e-6, (k, r.compliance, hist[k, 0])


@pytest.mark.parametrize("precision,optimizer", [("fp64", "oc"), ("mixed", "oc"), ("fp64", "mma")])
def test_robust_run_matches_oracle(precision, optimizer):
    """Robust formulation (Projection.hpp:44-60, run_oc at
    TopologyOptimizer.cpp:567-651): objective on the eroded design, OC on the
    dilated volume against the moved target, the blueprint's volume reported;
    every history column against the oracle."""
    spec = small_q4(40, 20)
    spec.rtol = 1e-10
    spec.initial_density = 0.5
    spec.projection, spec.beta_start, spec.beta_max = True, 2.0, 8.0
    spec.beta_interval, spec.advance_on_convergence = 3, False
    spec.robust, spec.robust_delta, spec.robust_volume_interval = True, 0.1, 2
    ref = oracle.Problem(spec)
    _, hist = ref.run(8) if optimizer == "oc" else ref.run_mma(8)
    gpu = GpuSimpProblem(spec, element_matrix=ref.element_matrix(), precision=precision, optimizer=optimizer)
    recs = TopologyOptimizer(gpu, max_iterations=8, change_tolerance=0).run()
    assert [r.beta for r in recs] == list(hist[:, 6])
    for k, r in enumerate(recs):
        assert abs(r.compliance / hist[k, 0] - 1) < 1e-6, (k, r.compliance, hist[k, 0])
        assert abs(r.volume_fraction - hist[k, 1]) < 1e-8
        assert abs(r.eroded_volume_fraction - hist[k, 7]) < 1e-8
        assert abs(r.dilated_volume_fraction - hist[k, 8]) < 1e-8
        assert abs(r.dilated_target_fraction - hist[k, 9]) < 1e-8
        assert r.eroded_volume_fraction < r.volume_fraction < r.dilated_volume_fraction
    gpu.close()


def test_projection_variants_match_oracle():
    """RobustRecord / erosion check (TopologyOptimizer.cpp:344-415): the
    current design's eroded, blueprint and dilated compliance and volume
    fraction against the oracle's evaluations at eta + delta, eta, eta - delta."""
    spec = small_q4(40, 20)
    spec.rtol = 1e-10
    spec.initial_density = 0.5
    spec.projection, spec.beta_start, spec.beta_max = True, 4.0, 4.0
    gpu = GpuSimpProblem(spec, precision="fp64")
    for _ in range(3):
        gpu.iterate()
    x = gpu.design()
    rec = gpu.projection_variants(0.15, densities=True)
    for key, eta in (("eroded", 0.65), ("intermediate", 0.5), ("dilated", 0.35)):
        s2 = small_q4(40, 20)
        s2.rtol = 1e-10
        s2.projection, s2.eta, s2.beta_start, s2.beta_max = True, eta, 4.0, 4.0
        ev = oracle.Problem(s2).evaluate(x)
        assert rec["eta_" + key] == pytest.approx(eta, abs=1e-15)
        assert rec["compliance_" + key] == pytest.approx(ev["compliance"], rel=1e-7)
        assert rec["volume_fraction_" + key] == pytest.approx(ev["volume_fraction"], abs=1e-12)
        if key != "intermediate":
            np.testing.assert_allclose(rec[key + "_density"], ev["rho"], atol=1e-14)
    assert rec["compliance_eroded"] > rec["compliance_intermediate"] > rec["compliance_dilated"]
    gpu.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cuda_graph_iterations_match_plain_launches(precision):
    """The PCG iterations replayed as a captured CUDA graph compute what the
    same kernels launched one by one compute, across setups (re-capture) and
    concurrent load cases (one graph per workspace)."""
    spec = P.q4_cantilever_600x200()
    spec.nx, spec.ny, spec.lx, spec.ly = 90, 30, 90.0, 30.0
    spec.fixed = P.clamp_left(spec)
    loads = []
    for i, j in enumerate((8, 15, 22)):
        loads.append(P.point_load(spec, [spec.node_index(90, j)], (0.3 * i, -1.0)))
    spec.loads = np.stack(loads)
    spec.rtol = 1e-10
    recs = {}
    for graphs in (0, 1):
        gpu = GpuSimpProblem(spec, precision=precision, cuda_graphs=graphs)
        recs[graphs] = [(r.compliance, r.linear_iterations) for r in
                        TopologyOptimizer(gpu, max_iterations=4, change_tolerance=0).run()]
        gpu.close()
    assert recs[0] == recs[1]


def test_matrix_free_transfers_match_stored_transfers():
    """Level 0's restriction and prolongation applied matrix-free in the FP32
    V-cycle, P^T (I - w A D^-1) and (I - w D^-1 A) P^, precondition as the
    stored R and P do: the same compliances (both solves reach rtol 1e-10) and
    CG iteration counts within one, across reuse setups."""
    spec = small_hex(24, 12, 12)
    side = [spec.node_index(24, j, 12) for j in range(13)]
    spec.loads = np.stack([spec.loads[0], P.point_load(spec, side, (0.0, 1.0, 0.0))])
    spec.weights = np.array([0.5, 0.5])
    recs = {}
    for mft in (0, 1):
        gpu = GpuSimpProblem(spec, precision="mixed", matrix_free_transfer=mft)
        recs[mft] = [(r.compliance, r.linear_iterations) for r in
                     TopologyOptimizer(gpu, max_iterations=5, change_tolerance=0).run()]
        gpu.close()
    for (c0, i0), (c1, i1) in zip(recs[0], recs[1]):
        assert abs(c1 / c0 - 1) < 1e-9, (c0, c1)
        assert abs(i1 - i0) <= max(1, i0 // 20), (i0, i1)
