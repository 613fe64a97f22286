"""The blocked symmetric sweep of csrc/dense.cuh (k_sweep_pivot /
k_sweep_update), restated in numpy, as the inertia test of the buckling
spectral transformation.

The reference places its shift sigma by the number of negative pivots of a
sparse LDL^T of K - sigma G (src/fem/Buckling.cpp:190-201).  The device
inverts K - sigma G by Gauss-Jordan elimination without pivoting, block by
block (32 columns), and counts the negative scalar pivots it meets.  Those
pivots are the diagonal of the natural-order LDL^T (each is a Schur
complement's diagonal), so by Sylvester's law of inertia their negative
count equals the number of negative eigenvalues.  These tests check that
claim on the restated sweep: the count against numpy's eigenvalues and
scipy's Bunch-Kaufman LDL^T, the pivots against an unpivoted LDL^T, and the
swept matrix against the inverse -- on random symmetric indefinite matrices
and on the shifted pencil of the reference's crowded-spectrum beam.
tests/test_gpu_buckling.py runs the device kernels themselves."""
import numpy as np
import pytest
import scipy.linalg as sla

NB = 32  # pivot block width of the device sweep


def sweep(a):
    """-A^-1 and the scalar pivots, in the device sweep's order."""
    m = np.array(a, dtype=np.float64)
    n = m.shape[0]
    piv = np.zeros(n)
    for k0 in range(0, n, NB):
        kb = min(NB, n - k0)
        blk = slice(k0, k0 + kb)
        s = m[blk, blk].copy()
        for j in range(kb):
            d = s[j, j]
            piv[k0 + j] = d
            p = 1.0 / d
            u = s[j, :].copy()
            t = p * u
            s -= np.outer(u, t)  # rows and column j are then overwritten
            s[:, j] = t
            s[j, :] = t
            s[j, j] = -p
        # s = -S^-1; U = M[:, block], V = U S^-1 outside the block
        out = np.r_[0:k0, k0 + kb:n]
        uu = m[np.ix_(out, np.arange(k0, k0 + kb))]
        vv = -(uu @ s)
        m[np.ix_(out, out)] -= vv @ uu.T
        m[np.ix_(out, np.arange(k0, k0 + kb))] = vv
        m[np.ix_(np.arange(k0, k0 + kb), out)] = vv.T
        m[blk, blk] = s
    return m, piv


def ldl_unpivoted(a):
    a = np.array(a, dtype=np.float64)
    n = a.shape[0]
    d = np.zeros(n)
    l = np.eye(n)
    for j in range(n):
        d[j] = a[j, j] - (l[j, :j] ** 2) @ d[:j]
        for i in range(j + 1, n):
            l[i, j] = (a[i, j] - (l[i, :j] * l[j, :j]) @ d[:j]) / d[j]
    return d


@pytest.mark.parametrize("n,neg", [(40, 0), (75, 3), (96, 17), (130, 64)])
def test_sweep_inverse_and_inertia_on_random_matrices(n, neg):
    rng = np.random.default_rng(n)
    q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    ev = rng.uniform(0.5, 4.0, n)
    ev[rng.choice(n, neg, replace=False)] *= -1.0
    a = (q * ev) @ q.T
    a = 0.5 * (a + a.T)
    m, piv = sweep(a)
    np.testing.assert_allclose(-m, np.linalg.inv(a), rtol=0, atol=1e-8 * np.abs(np.linalg.inv(a)).max())
    assert int(np.sum(piv < 0)) == int(np.sum(np.linalg.eigvalsh(a) < 0)) == neg
    _, dd, _ = sla.ldl(a)
    assert int(np.sum(np.linalg.eigvalsh(dd) < 0)) == neg
    if n <= 96:
        np.testing.assert_allclose(piv, ldl_unpivoted(a), rtol=1e-8)


def test_sweep_inertia_counts_load_factors_below_the_shift():
    """K - s G on the reference's crowded beam (Q4 60 x 6, axial tension plus a
    small transverse load): the negative pivots count the load factors in
    (0, s), as the dense generalised eigenvalues do."""
    from sparlab_gb300 import problems as P
    import oracle
    from oracle import buckling as OB
    import scipy.sparse as sp
    spec = P.column(2, 60, 6, height=0.1, thickness=0.002, force=2.0e8 * 0.1 * 0.002,
                    transverse=1.0e6 * 0.1 * 0.002)
    prob = oracle.Problem(spec)
    ptr, col, val = prob.kff()
    k = sp.csr_matrix((val, col, ptr)).toarray()
    free = prob.free_dofs()
    u = np.zeros(prob.ndof)
    u[free] = np.linalg.solve(k, spec.loads[0][free])
    g = -OB.geometric_stiffness_ff(prob, spec, u).toarray()
    mu = sla.eigh(g, k, eigvals_only=True)
    lam = np.sort(1.0 / mu[mu > 1e-10 * np.abs(mu).max()])
    assert k.shape[0] == 840 and lam.size >= 2
    for s in (0.5 * lam[0], 0.5 * (lam[0] + lam[1]), 1.5 * lam[1]):
        _, piv = sweep(k - s * g)
        assert int(np.sum(piv < 0)) == int(np.sum(lam < s))
