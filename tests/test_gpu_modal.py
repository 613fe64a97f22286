"""GPU modal analysis (simp_modal) against the oracle's restatement of
solve_modal (src/fem/ModalAnalysis.cpp) and the reference's known answers."""
import numpy as np
import pytest
import scipy.sparse as sp

import oracle
from oracle import modal as OM
from sparlab_gb300 import problems as P
from sparlab_gb300._lib import SolverError
from sparlab_gb300.topopt import GpuSimpProblem

pytestmark = pytest.mark.gpu


def pair(spec, precision="fp64"):
    ref = oracle.Problem(spec)
    gpu = GpuSimpProblem(spec, element_matrix=ref.element_matrix(), precision=precision)
    return ref, gpu


def check_shapes(g, o, rtol=1e-6):
    """Mode shapes equal up to sign."""
    for i in range(o.mode_shapes.shape[1]):
        a, b = g.mode_shapes[:, i], o.mode_shapes[:, i]
        sgn = np.sign(a @ b)
        assert np.abs(a - sgn * b).max() <= rtol * np.abs(b).max(), i


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_subspace_iteration_matches_oracle(precision):
    spec = P.plane_cantilever(40, 8, poisson=0.3)
    ref, gpu = pair(spec, precision)
    o = OM.solve_modal(ref, spec, num_modes=5, tolerance=1e-12, density=spec.density)
    g = gpu.modal(num_modes=5, tolerance=1e-12)
    assert g.converged and g.iterations > 0 and g.subspace_size == 13
    np.testing.assert_allclose(g.eigenvalues, o.eigenvalues, rtol=1e-9)
    assert g.modal_residuals.max() < 1e-8
    assert g.total_mass == pytest.approx(o.total_mass, rel=1e-13)
    m = OM.mass_matrices(ref, spec, spec.density)[0]
    phi = g.mode_shapes[ref.free_dofs()]
    np.testing.assert_allclose(np.einsum("ij,ij->j", phi, m @ phi), 1.0, rtol=1e-10)
    assert np.all(g.mode_shapes[spec.fixed.astype(bool)] == 0.0)
    check_shapes(g, o)
    gpu.close()


def test_bending_frequency_matches_euler_bernoulli():
    spec = P.plane_cantilever(120, 12, poisson=0.0)
    _, gpu = pair(spec, "mixed")
    g = gpu.modal(num_modes=4, mode_shapes=False)
    f1t = OM.cantilever_bending_frequency(spec.young, spec.density, 1.0, 0.1, 0.01, 1)
    assert abs(g.frequencies_hz[0] - f1t) / f1t < 0.01 and g.frequencies_hz[0] < f1t
    assert not g.warnings
    gpu.close()


@pytest.mark.parametrize("mass_type", ["consistent", "lumped"])
def test_hex8_simp_design_matches_oracle(mass_type):
    """Hex8 with SIMP stiffness and mass factors of a seeded density field,
    including the low-density kinetic-energy fractions."""
    spec = P.hex8_cantilever(16, 8, 8, 0.3, "modal_hex")
    spec.density = 7.8
    spec.rtol = 1e-12
    ref, gpu = pair(spec)
    rho = P.SplitMix64(8).uniform_array(ref.ne, 0.05, 1.0)
    ks = 1e-9 + (1 - 1e-9) * rho ** 3
    ms = rho.copy()
    o = OM.solve_modal(ref, spec, num_modes=4, density=spec.density, stiffness_scale=ks,
                       mass_scale=ms, mass_type=mass_type)
    g = gpu.modal(num_modes=4, stiffness_scale=ks, mass_scale=ms, mass_type=mass_type)
    np.testing.assert_allclose(g.eigenvalues, o.eigenvalues, rtol=1e-9)
    np.testing.assert_allclose(g.modal_mass_fraction, o.modal_mass_fraction, rtol=1e-7, atol=1e-12)
    assert g.total_mass == pytest.approx(o.total_mass, rel=1e-12)
    check_shapes(g, o, rtol=1e-5)
    gpu.close()


def test_negative_shift_gives_the_same_modes():
    """sigma = shift_factor * min k_ii / m_ii; min k_ii / m_ii is near the top
    of the spectrum, so a useful shift factor is small (here sigma is about
    -0.4 lambda_1)."""
    spec = P.plane_cantilever(60, 6, poisson=0.3)
    _, gpu = pair(spec)
    a = gpu.modal(num_modes=3, mode_shapes=False)
    b = gpu.modal(num_modes=3, mode_shapes=False, shift_factor=-1e-6)
    np.testing.assert_allclose(b.eigenvalues, a.eigenvalues, rtol=1e-9)
    with pytest.raises(SolverError, match="shift"):
        gpu.modal(num_modes=3, shift_factor=0.5)
    gpu.close()


def test_dense_path_flags_rigid_body_modes():
    spec = P.plane_cantilever(6, 6, length=0.5, height=0.5, poisson=0.3)
    spec.fixed = np.zeros_like(spec.fixed)
    ref, gpu = pair(spec)
    o = OM.solve_modal(ref, spec, num_modes=4, density=spec.density)
    g = gpu.modal(num_modes=4)
    assert g.iterations == 0 and g.warnings
    assert g.eigenvalues[0] < 1e-6 * g.eigenvalues[3]
    assert g.eigenvalues[3] == pytest.approx(o.eigenvalues[3], rel=1e-9)
    gpu.close()


def test_modal_leaves_the_simp_state_alone():
    """A modal analysis between iterations changes nothing the SIMP loop sees."""
    spec = P.hex8_cantilever(12, 6, 6, 0.3, "modal_simp")
    spec.rtol = 1e-10
    a = GpuSimpProblem(spec)
    b = GpuSimpProblem(spec)
    ra = [a.iterate().compliance for _ in range(2)]
    rb = [b.iterate().compliance for _ in range(2)]
    b.modal(num_modes=2, mode_shapes=False)
    ra.append(a.iterate().compliance)
    rb.append(b.iterate().compliance)
    assert ra == rb
    a.close()
    b.close()
