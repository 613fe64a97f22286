"""The oracle's linear buckling (a restatement of src/fem/Buckling.cpp and
the continuum geometric stiffness of src/elements/Element.cpp) pinned
against the reference's own buckling tests (tests/test_buckling.cpp):
element identities, Euler columns converging on the Engesser load, the
dense cross-check, load scaling, warm start and the tensile / crowded
spectra."""
import numpy as np
import pytest
import scipy.linalg as sla
import scipy.sparse as sp

import oracle
from oracle import buckling as OB
from sparlab_gb300 import problems as P


@pytest.mark.parametrize("dim", [2, 3])
def test_element_geometric_stiffness_identities(dim):
    # test_buckling.cpp:114-172 (box cells)
    hx, hy, hz = 0.3, 0.25, 0.2 if dim == 3 else 0.0
    d = OB.constitutive(dim, 1.0, 0.3)
    t = 0.01 if dim == 2 else 1.0
    ed = 8 if dim == 2 else 24
    ue = 1e-4 * P.SplitMix64(11).uniform_array(ed, -1.0, 1.0)
    kg = OB.element_geometric_stiffness(dim, hx, hy, hz, d, ue, 0.7, t)
    assert np.abs(kg - kg.T).max() <= 1e-12 * np.abs(kg).max()
    for k in range(dim):
        shift = np.zeros(ed)
        shift[k::dim] = 1.0
        assert np.abs(kg @ shift).max() <= 1e-10 * np.abs(kg).max()
    # uniaxial stress s0 = E eps contracted with phi_y = x gives s0 * measure * t
    corners = (np.array([[0, 0], [1, 0], [1, 1], [0, 1]]) if dim == 2 else
               np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]]))
    xyz = corners * np.array([hx, hy, hz][:dim])
    eps = 1e-3
    axial = np.zeros(ed)
    mode = np.zeros(ed)
    for a in range(len(corners)):
        axial[dim * a] = eps * xyz[a, 0]
        for k in range(1, dim):
            axial[dim * a + k] = -0.3 * eps * xyz[a, k]
        mode[dim * a + 1] = xyz[a, 0]
    kga = OB.element_geometric_stiffness(dim, hx, hy, hz, d, axial, 1.0, t)
    measure = hx * hy * (hz if dim == 3 else 1.0) * t
    assert mode @ kga @ mode == pytest.approx(1.0 * eps * measure, rel=1e-9)


def run(spec, **kw):
    return OB.analyse_buckling(oracle.Problem(spec), spec, **kw)


def test_q4_euler_columns_converge_on_engesser():
    # test_buckling.cpp:176-205
    h, t = 0.05, 0.02
    theory = OB.engesser_cantilever_load(200e9, 0.3, t * h ** 3 / 12, h * t, 1.0)
    prev = 1.0
    for nx in (20, 40, 80):
        r = run(P.column(2, nx, 4, height=h, thickness=t), num_modes=3)
        assert r.converged and len(r.load_factors) == 3
        err = r.load_factors[0] / theory - 1.0
        assert 0.0 < err < prev
        prev = err
        assert r.load_factors[1] / r.load_factors[0] == pytest.approx(9.0, rel=0.05)
        assert r.residuals.max() < 1e-6
    assert prev < 0.04


def test_hex8_euler_column():
    # test_buckling.cpp:206-241 (the Hex8 case)
    h = 0.05
    theory = OB.engesser_cantilever_load(200e9, 0.3, h ** 4 / 12, h * h, 1.0)
    r = run(P.column(3, 20, 2, 2, height=h, width=h), num_modes=2)
    err = r.load_factors[0] / theory - 1.0
    assert r.converged and 0.0 < err < 0.5
    assert r.load_factors[1] == pytest.approx(r.load_factors[0], rel=0.002)


def test_modes_match_dense_eigensolve_and_scale_with_the_load():
    # test_buckling.cpp:243-299
    spec = P.column(2, 60, 4, height=0.08, thickness=0.01, force=-1e3)
    prob = oracle.Problem(spec)
    assert prob.nfree > 400
    r = OB.analyse_buckling(prob, spec, num_modes=4)
    assert r.converged and r.iterations > 0 and len(r.load_factors) == 4
    ptr, col, val = prob.kff()
    k = sp.csr_matrix((val, col, ptr)).toarray()
    free = prob.free_dofs()
    u = np.zeros(prob.ndof)
    u[free] = np.linalg.solve(k, spec.loads[0][free])
    g = -OB.geometric_stiffness_ff(prob, spec, u).toarray()
    mu = sla.eigh(g, k, eigvals_only=True)[::-1]
    np.testing.assert_allclose(r.load_factors, 1.0 / mu[:4], rtol=1e-8)
    for i in range(4):
        phi = r.mode_shapes[free, i]
        assert phi @ k @ phi == pytest.approx(1.0, rel=1e-10)
        res = k @ phi - r.load_factors[i] * (g @ phi)
        assert np.linalg.norm(res) <= 1e-6 * np.linalg.norm(k @ phi)
    assert np.all(r.mode_shapes[spec.fixed.astype(bool)] == 0.0)
    half = run(P.column(2, 60, 4, height=0.08, thickness=0.01, force=-2e3), num_modes=4)
    assert half.load_factors[0] == pytest.approx(0.5 * r.load_factors[0], rel=1e-8)
    warm = OB.analyse_buckling(prob, spec, num_modes=4, initial_subspace=r.subspace)
    assert warm.iterations < r.iterations
    assert warm.load_factors[0] == pytest.approx(r.load_factors[0], rel=1e-9)


def test_tension_has_no_positive_load_factor_and_crowding_shifts():
    # test_buckling.cpp:301-381
    r = run(P.column(2, 40, 4, thickness=0.02, force=+1e3), num_modes=2)
    assert r.no_positive_load_factor and len(r.load_factors) == 0
    for tension in (0.0, 2.0e8):
        spec = P.column(2, 60, 6, height=0.1, thickness=0.002, force=tension * 0.1 * 0.002,
                        transverse=1.0e6 * 0.1 * 0.002)
        prob = oracle.Problem(spec)
        b = OB.analyse_buckling(prob, spec, num_modes=3)
        assert b.converged
        ptr, col, val = prob.kff()
        k = sp.csr_matrix((val, col, ptr)).toarray()
        free = prob.free_dofs()
        u = np.zeros(prob.ndof)
        u[free] = np.linalg.solve(k, spec.loads[0][free])
        g = -OB.geometric_stiffness_ff(prob, spec, u).toarray()
        mu = sla.eigh(g, k, eigvals_only=True)[::-1]
        assert mu[0] > 0 and mu[-1] < 0
        crowding = int(np.sum(mu < -mu[2]))
        if tension > 0:
            assert crowding > b.subspace_size and b.transformed
            assert 0.0 < b.sigma < b.load_factors[0]
        else:
            assert not b.transformed
        positive = 0
        while positive < 3 and mu[positive] > 1e-10 * np.abs(mu).max():
            positive += 1
        assert positive >= 1 and len(b.load_factors) == positive
        np.testing.assert_allclose(b.load_factors, 1.0 / mu[:positive], rtol=1e-7)


def test_column_helpers():
    # test_buckling.cpp:383-399
    assert OB.euler_cantilever_load(200e9, 1e-8, 1.0) == pytest.approx(np.pi ** 2 * 200e9 * 1e-8 / 4)
    assert OB.engesser_cantilever_load(200e9, 0.3, 1e-8, 1e-4, 1.0) < OB.euler_cantilever_load(200e9, 1e-8, 1.0)
