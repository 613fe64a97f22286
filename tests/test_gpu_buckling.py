"""GPU linear buckling (simp_buckling) against the oracle's restatement of
analyse_buckling / solve_buckling (src/fem/Buckling.cpp) and the
reference's known answers (Euler columns, tests/test_buckling.cpp)."""
import numpy as np
import pytest

import oracle
from oracle import buckling as OB
from sparlab_gb300 import problems as P
from sparlab_gb300._lib import SolverError
from sparlab_gb300.topopt import GpuSimpProblem

pytestmark = pytest.mark.gpu


def pair(spec, precision="fp64"):
    ref = oracle.Problem(spec)
    return ref, GpuSimpProblem(spec, element_matrix=ref.element_matrix(), precision=precision)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_q4_columns_match_oracle_and_engesser(precision):
    h, t = 0.05, 0.02
    theory = OB.engesser_cantilever_load(200e9, 0.3, t * h ** 3 / 12, h * t, 1.0)
    prev = 1.0
    for nx in (20, 40, 80):
        spec = P.column(2, nx, 4, height=h, thickness=t)
        ref, gpu = pair(spec, precision)
        o = OB.analyse_buckling(ref, spec, num_modes=3)
        b = gpu.buckling(num_modes=3)
        assert b.converged and len(b.load_factors) == 3
        np.testing.assert_allclose(b.load_factors, o.load_factors, rtol=1e-8)
        err = b.load_factors[0] / theory - 1.0
        assert 0.0 < err < prev
        prev = err
        assert b.residuals.max() < 1e-6
        gpu.close()
    assert prev < 0.04


def test_hex8_column_matches_oracle():
    spec = P.column(3, 20, 2, 2, height=0.05, width=0.05)
    ref, gpu = pair(spec)
    o = OB.analyse_buckling(ref, spec, num_modes=2)
    b = gpu.buckling(num_modes=2)
    np.testing.assert_allclose(b.load_factors, o.load_factors, rtol=1e-8)
    assert b.load_factors[1] == pytest.approx(b.load_factors[0], rel=0.002)
    gpu.close()


def test_modes_normalised_warm_started_and_scaled():
    spec = P.column(2, 60, 4, height=0.08, thickness=0.01, force=-1e3)
    ref, gpu = pair(spec)
    assert gpu.nfree > 400
    o = OB.analyse_buckling(ref, spec, num_modes=4)
    b = gpu.buckling(num_modes=4)
    assert b.converged and b.iterations > 0
    np.testing.assert_allclose(b.load_factors, o.load_factors, rtol=1e-8)
    ptr, col, val = ref.kff()
    import scipy.sparse as sp
    k = sp.csr_matrix((val, col, ptr))
    free = ref.free_dofs()
    for i in range(4):
        phi = b.mode_shapes[free, i]
        assert phi @ (k @ phi) == pytest.approx(1.0, rel=1e-10)
        oi = o.mode_shapes[free, i]
        sgn = np.sign(phi @ oi)
        assert np.abs(phi - sgn * oi).max() <= 1e-5 * np.abs(oi).max()
    assert np.all(b.mode_shapes[spec.fixed.astype(bool)] == 0.0)
    warm = gpu.buckling(num_modes=4, initial_subspace=b.subspace)
    assert warm.iterations < b.iterations
    assert warm.load_factors[0] == pytest.approx(b.load_factors[0], rel=1e-9)
    gpu.close()
    spec2 = P.column(2, 60, 4, height=0.08, thickness=0.01, force=-2e3)
    _, gpu2 = pair(spec2)
    half = gpu2.buckling(num_modes=4, mode_shapes=False)
    assert half.load_factors[0] == pytest.approx(0.5 * b.load_factors[0], rel=1e-8)
    gpu2.close()


def test_simp_factors_and_solid_fractions_match_oracle():
    spec = P.column(3, 24, 3, 3, height=0.06, width=0.06)
    ref, gpu = pair(spec)
    rho = P.SplitMix64(12).uniform_array(ref.ne, 0.3, 1.0)
    ks = 1e-9 + (1 - 1e-9) * rho ** 3
    ss = rho ** 3
    solid = (rho >= 0.5).astype(np.uint8)
    o = OB.analyse_buckling(ref, spec, num_modes=3, stiffness_scale=ks, stress_scale=ss, solid_mask=solid)
    b = gpu.buckling(num_modes=3, stiffness_scale=ks, stress_scale=ss, solid_mask=solid)
    np.testing.assert_allclose(b.load_factors, o.load_factors, rtol=1e-7)
    np.testing.assert_allclose(b.solid_energy_fraction, o.solid_energy_fraction, rtol=1e-6)
    gpu.close()


def test_tension_has_no_positive_load_factor():
    """400 free DOFs: the dense path, as in the reference's test."""
    spec = P.column(2, 40, 4, thickness=0.02, force=+1e3)
    _, gpu = pair(spec)
    b = gpu.buckling(num_modes=2)
    assert b.no_positive_load_factor and len(b.load_factors) == 0
    gpu.close()


def test_crowded_spectrum_takes_the_spectral_transformation():
    """Large axial tension plus a small transverse load (the reference's
    tests/test_buckling.cpp:301-381): the reversed-load factors crowd the
    subspace and the iteration switches to (K - sigma G)^-1 K with sigma
    below lambda_1, placed by the inertia of K - sigma G; without the axial
    tension the plain iteration runs.  Both reproduce the oracle and the
    dense eigensolve to 1e-7, as does the transformation from the start."""
    for tension in (0.0, 2.0e8):
        spec = P.column(2, 60, 6, height=0.1, thickness=0.002, force=tension * 0.1 * 0.002,
                        transverse=1.0e6 * 0.1 * 0.002)
        ref, gpu = pair(spec)
        assert gpu.nfree > 400
        o = OB.analyse_buckling(ref, spec, num_modes=3)
        b = gpu.buckling(num_modes=3)
        assert b.converged and o.converged
        assert b.transformed == o.transformed == (tension > 0)
        assert len(b.load_factors) == len(o.load_factors) >= 1
        np.testing.assert_allclose(b.load_factors, o.load_factors, rtol=1e-7)
        if tension > 0:
            assert 0.0 < b.sigma < b.load_factors[0] and b.factorizations >= 1
        else:
            assert b.factorizations == 0
        s = gpu.buckling(num_modes=3, transform="shift_invert")
        assert s.converged and s.transformed and 0.0 < s.sigma < s.load_factors[0]
        np.testing.assert_allclose(s.load_factors, o.load_factors, rtol=1e-7)
        h = gpu.buckling(num_modes=3, transform="shift_invert", shift_hint=o.load_factors[0])
        assert h.transformed and 0.0 < h.sigma < h.load_factors[0]
        np.testing.assert_allclose(h.load_factors, o.load_factors, rtol=1e-7)
        gpu.close()


def test_tension_shift_invert_finds_no_positive_load_factor():
    """Pure tension past the dense path's size: the shift search grows sigma
    by factors of 8 up to 1e15 without meeting a load factor."""
    spec = P.column(2, 60, 6, height=0.1, thickness=0.002, force=2.0e8 * 0.1 * 0.002)
    ref, gpu = pair(spec)
    assert gpu.nfree > 400
    o = OB.analyse_buckling(ref, spec, num_modes=2, transform="shift_invert")
    b = gpu.buckling(num_modes=2, transform="shift_invert")
    assert o.no_positive_load_factor and b.no_positive_load_factor
    assert len(b.load_factors) == 0 and b.converged and b.factorizations == o.factorizations
    gpu.close()


def test_dense_path_matches_oracle():
    spec = P.column(2, 20, 4)
    ref, gpu = pair(spec)
    assert gpu.nfree <= 400
    o = OB.analyse_buckling(ref, spec, num_modes=3)
    b = gpu.buckling(num_modes=3)
    assert b.iterations == 0
    np.testing.assert_allclose(b.load_factors, o.load_factors, rtol=1e-9)
    gpu.close()
