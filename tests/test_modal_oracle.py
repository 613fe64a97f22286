"""The oracle's modal analysis (a restatement of src/fem/ModalAnalysis.cpp)
pinned against the known answers of the reference's own modal tests
(tests/test_modal.cpp): mass conservation, the dense cross-check of the
subspace iteration, Euler-Bernoulli bending and fixed-free rod frequencies,
thickness invariance, lumped below consistent and the rigid-body warning."""
import numpy as np
import pytest
import scipy.linalg as sla

import oracle
from oracle import modal as OM
from sparlab_gb300 import problems as P


def model(spec):
    return oracle.Problem(spec)


def test_mass_conserved_and_positive_definite():
    # test_modal.cpp:19-78 (structured instead of perturbed cells)
    spec = P.plane_cantilever(6, 4, length=1.2, height=0.5)
    free = P.plane_cantilever(6, 4, length=1.2, height=0.5)
    free.fixed = np.zeros_like(free.fixed)
    expected = spec.density * spec.lx * spec.ly * spec.thickness
    for kind in ("consistent", "lumped"):
        prob = model(free)
        m, total, _ = OM.mass_matrices(prob, free, free.density, kind)
        dense = m.toarray()
        assert np.abs(dense - dense.T).max() / np.abs(dense).max() <= 1e-15
        assert total == pytest.approx(2 * expected, rel=1e-11)
        assert dense.sum() == pytest.approx(2 * expected, rel=1e-11)
        tx = np.zeros(prob.ndof)
        tx[0::2] = 1.0
        assert tx @ dense @ tx == pytest.approx(expected, rel=1e-11)
        mff, _, _ = OM.mass_matrices(model(spec), spec, spec.density, kind)
        assert np.linalg.eigvalsh(mff.toarray()).min() > 0.0


def test_subspace_iteration_matches_dense_eigensolve():
    # test_modal.cpp:100-147
    spec = P.plane_cantilever(40, 8, poisson=0.3)
    prob = model(spec)
    r = OM.solve_modal(prob, spec, num_modes=5, tolerance=1e-12, density=spec.density)
    assert r.converged and prob.nfree > 400 and r.iterations > 0
    ptr, col, val = prob.kff()
    import scipy.sparse as sp
    k = sp.csr_matrix((val, col, ptr)).toarray()
    m = OM.mass_matrices(prob, spec, spec.density)[0].toarray()
    ref = sla.eigh(k, m, eigvals_only=True)
    np.testing.assert_allclose(r.eigenvalues, ref[:5], rtol=1e-8)
    assert np.all(np.diff(r.eigenvalues) >= 0)
    assert r.modal_residuals.max() < 1e-8
    phi = r.mode_shapes[prob.free_dofs()]
    np.testing.assert_allclose(np.einsum("ij,ik,kj->j", phi, m, phi), 1.0, rtol=1e-8)
    assert np.all(r.mode_shapes[spec.fixed.astype(bool)] == 0.0)


@pytest.mark.parametrize("linear", ["amg_cg", "direct"])
def test_bending_frequencies_match_euler_bernoulli(linear):
    # test_modal.cpp:149-194
    spec = P.plane_cantilever(120, 12, poisson=0.0)
    r = OM.solve_modal(model(spec), spec, num_modes=4, density=spec.density, linear=linear)
    f1t = OM.cantilever_bending_frequency(spec.young, spec.density, 1.0, 0.1, 0.01, 1)
    f2t = OM.cantilever_bending_frequency(spec.young, spec.density, 1.0, 0.1, 0.01, 2)
    f = r.frequencies_hz
    assert abs(f[0] - f1t) / f1t < 0.01 and f[0] < f1t
    f2 = f[1:][np.argmin(np.abs(f[1:] - f2t))]
    assert abs(f2 - f2t) / f2t < 0.06 and f2 < f2t
    assert f[0] > 0 and np.all(np.diff(f) >= 0) and not r.warnings


def test_first_axial_mode_matches_rod_theory():
    # test_modal.cpp:196-240
    spec = P.plane_cantilever(160, 16, poisson=0.0)
    r = OM.solve_modal(model(spec), spec, num_modes=8, density=spec.density)
    ux, uy = r.mode_shapes[0::2], r.mode_shapes[1::2]
    ratio = (ux ** 2).sum(0) / ((ux ** 2).sum(0) + (uy ** 2).sum(0))
    axial = int(np.argmax(ratio))
    assert ratio[axial] > 0.9
    expected = OM.rod_axial_frequency(spec.young, spec.density, 1.0, 1)
    assert abs(r.frequencies_hz[axial] - expected) / expected < 0.01


def test_frequencies_invariant_under_thickness_scaling():
    # test_modal.cpp:255-279
    a = P.plane_cantilever(30, 6, poisson=0.3)
    b = P.plane_cantilever(30, 6, poisson=0.3, thickness=0.01 * 0.37)
    ra = OM.solve_modal(model(a), a, num_modes=3, density=a.density)
    rb = OM.solve_modal(model(b), b, num_modes=3, density=b.density)
    np.testing.assert_allclose(rb.frequencies_hz, ra.frequencies_hz, rtol=1e-9)
    assert rb.total_mass == pytest.approx(0.37 * ra.total_mass, rel=1e-10)


def test_lumped_mass_lowers_frequencies():
    # test_modal.cpp:281-306
    spec = P.plane_cantilever(60, 6, poisson=0.0)
    mc = OM.solve_modal(model(spec), spec, num_modes=3, density=spec.density)
    ml = OM.solve_modal(model(spec), spec, num_modes=3, density=spec.density, mass_type="lumped")
    assert np.all(ml.frequencies_hz < mc.frequencies_hz)
    assert np.all(np.abs(ml.frequencies_hz - mc.frequencies_hz) / mc.frequencies_hz < 0.05)


def test_unconstrained_model_flags_rigid_body_modes():
    # test_modal.cpp:308-334
    spec = P.plane_cantilever(6, 6, length=0.5, height=0.5, young=70e9, poisson=0.3)
    spec.fixed = np.zeros_like(spec.fixed)
    r = OM.solve_modal(model(spec), spec, num_modes=4, density=spec.density)
    assert r.warnings
    assert r.eigenvalues[0] < 1e-6 * r.eigenvalues[3]


def test_frequency_helpers():
    # test_modal.cpp:242-253, 350-380
    base = OM.rod_axial_frequency(70e9, 2700.0, 1.0, 1)
    assert base == pytest.approx(np.sqrt(70e9 / 2700.0) / 4.0)
    assert OM.rod_axial_frequency(70e9, 2700.0, 1.0, 3) == pytest.approx(5 * base)
    b1 = OM.cantilever_bending_frequency(70e9, 2700.0, 1.0, 0.1, 0.01, 1)
    assert OM.cantilever_bending_frequency(70e9, 2700.0, 2.0, 0.1, 0.01, 1) == pytest.approx(0.25 * b1)
    b2 = OM.cantilever_bending_frequency(70e9, 2700.0, 1.0, 0.1, 0.01, 2)
    assert b2 / b1 == pytest.approx((4.69409113 / 1.87510407) ** 2, rel=1e-9)
    with pytest.raises(ValueError):
        OM.cantilever_bending_frequency(70e9, 2700.0, 1.0, 0.1, 0.01, 6)


@pytest.mark.parametrize("dim", [2, 3])
def test_library_element_mass_equals_oracle(dim):
    """The library's element mass (host code, no GPU) is the oracle's bit for bit."""
    from sparlab_gb300.topopt import element_mass
    args = (dim, 0.5, 0.25, 0.125 if dim == 3 else 0.0, 2700.0, 0.01 if dim == 2 else 1.0)
    np.testing.assert_array_equal(element_mass(*args), OM.element_mass(*args))
