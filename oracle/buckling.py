"""Linear buckling of a structured problem, restated from SparLab's
``analyse_buckling`` / ``solve_buckling`` (src/fem/Buckling.cpp:100-466) and
the continuum geometric stiffness (src/elements/Element.cpp:77-100) -- test
infrastructure only: the GPU buckling path is checked against it, nothing in
the product imports it.

(K_ff + lambda K_G,ff(u)) phi = 0 for the stress state of the static solution
u of one load case.  mu = 1 / lambda solves the definite pencil
(G, K), G = -K_G; subspace iteration X <- K^-1 G X with an orthonormal basis
(column-pivoted QR, rank threshold 1e-12) and a Rayleigh-Ritz projection
finds the largest mu.  When more reversed-load (negative) Ritz values than
the spare slots crowd the subspace, the reference switches to the buckling
spectral transformation (K - sigma G)^-1 K, with sigma placed below
lambda_1 by the inertia of LDL^T factorisations; this restatement does the
same with dense factorisations (scipy.linalg.ldl), which limits it to small
models.  Systems of at most 400 free DOFs take the dense path.

Deviation: the start subspace is filled from the project's SplitMix64
(seed 20240917) instead of std::mt19937; the start only affects the path of
the iteration, not the converged load factors.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np
import scipy.linalg as sla
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import Problem
from .modal import element_dofs

K_ZERO_FRACTION = 1e-10
K_DENSE_LIMIT = 400
SEED = 20240917


def euler_cantilever_load(e, second_moment, length):
    """pi^2 E I / (4 L^2) (Buckling.cpp:468-474)."""
    return np.pi ** 2 * e * second_moment / (4.0 * length * length)


def engesser_cantilever_load(e, poisson, second_moment, area, length):
    """Euler with the Engesser shear correction, kappa = 5/6 (Buckling.cpp:476-482)."""
    euler = euler_cantilever_load(e, second_moment, length)
    shear = (5.0 / 6.0) * e / (2.0 * (1.0 + poisson)) * area
    return euler / (1.0 + euler / shear)


def constitutive(dim, young, poisson):
    """Plane stress (2-D) or three-dimensional isotropic D
    (src/material/IsotropicMaterial.cpp:34-66)."""
    if dim == 2:
        f = young / (1.0 - poisson * poisson)
        return np.array([[f, f * poisson, 0.0], [f * poisson, f, 0.0], [0.0, 0.0, f * (1.0 - poisson) / 2.0]])
    lam = young * poisson / ((1.0 + poisson) * (1.0 - 2.0 * poisson))
    g = young / (2.0 * (1.0 + poisson))
    d = np.zeros((6, 6))
    d[:3, :3] = lam
    for i in range(3):
        d[i, i] = lam + 2.0 * g
        d[3 + i, 3 + i] = g
    return d


def gauss_points(dim, hx, hy, hz):
    """(weight * det J, dN/dx (nodes x dim)) at the 2 x 2 (x 2) stiffness
    points of a box cell, in the quadrature order (x fastest)."""
    g = 1.0 / np.sqrt(3.0)
    pts = []
    if dim == 2:
        for eta in (-g, g):
            for xi in (-g, g):
                dn = 0.25 * np.array([[-(1 - eta), -(1 - xi)], [1 - eta, -(1 + xi)],
                                      [1 + eta, 1 + xi], [-(1 + eta), 1 - xi]])
                pts.append((0.25 * hx * hy, dn * np.array([2.0 / hx, 2.0 / hy])))
        return pts
    corner = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                       [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], float)
    for zeta in (-g, g):
        for eta in (-g, g):
            for xi in (-g, g):
                f = 1 + np.array([xi, eta, zeta])[None, :] * corner
                dn = 0.125 * corner * np.stack([f[:, 1] * f[:, 2], f[:, 0] * f[:, 2], f[:, 0] * f[:, 1]], 1)
                pts.append((0.125 * hx * hy * hz, dn * np.array([2.0 / hx, 2.0 / hy, 2.0 / hz])))
    return pts


def strain_matrix(grad, dim):
    """Voigt strain operator: (xx, yy, xy) or (xx, yy, zz, xy, yz, zx)."""
    nn = grad.shape[0]
    if dim == 2:
        b = np.zeros((3, 2 * nn))
        b[0, 0::2] = grad[:, 0]
        b[1, 1::2] = grad[:, 1]
        b[2, 0::2] = grad[:, 1]
        b[2, 1::2] = grad[:, 0]
        return b
    b = np.zeros((6, 3 * nn))
    b[0, 0::3] = grad[:, 0]
    b[1, 1::3] = grad[:, 1]
    b[2, 2::3] = grad[:, 2]
    b[3, 0::3] = grad[:, 1]
    b[3, 1::3] = grad[:, 0]
    b[4, 1::3] = grad[:, 2]
    b[4, 2::3] = grad[:, 1]
    b[5, 0::3] = grad[:, 2]
    b[5, 2::3] = grad[:, 0]
    return b


def stress_tensor(s, dim):
    if dim == 2:
        return np.array([[s[0], s[2]], [s[2], s[1]]])
    return np.array([[s[0], s[3], s[5]], [s[3], s[1], s[4]], [s[5], s[4], s[2]]])


def element_geometric_stiffness(dim, hx, hy, hz, d, ue, scale=1.0, thickness=1.0):
    """s K_G,e(u_e): block = sum_g t w det G^T S G, symmetrised, one copy per
    displacement component (Element.cpp:77-100)."""
    pts = gauss_points(dim, hx, hy, hz)
    nn = pts[0][1].shape[0]
    t = thickness if dim == 2 else 1.0
    block = np.zeros((nn, nn))
    for wdet, grad in pts:
        sigma = scale * (d @ (strain_matrix(grad, dim) @ ue))
        block += (t * wdet) * (grad @ stress_tensor(sigma, dim) @ grad.T)
    sym = 0.5 * (block + block.T)
    return np.kron(sym, np.eye(dim))


def geometric_stiffness_ff(prob: Problem, spec, u_full, stress_scale=None):
    """Free-free K_G of the stress state of u (full length)."""
    dim = spec.dim
    hx, hy = spec.lx / spec.nx, spec.ly / spec.ny
    hz = spec.lz / spec.nz if dim == 3 else 0.0
    d = constitutive(dim, spec.young, spec.poisson)
    edofs = element_dofs(spec)
    ne, ed = edofs.shape
    pts = gauss_points(dim, hx, hy, hz)
    nn = ed // dim
    t = spec.thickness if dim == 2 else 1.0
    s = np.ones(ne) if stress_scale is None else np.asarray(stress_scale, float)
    ue = u_full[edofs]                                      # ne x ed
    blocks = np.zeros((ne, nn, nn))
    for wdet, grad in pts:
        b = strain_matrix(grad, dim)
        sig = s[:, None] * ((ue @ b.T) @ d.T)               # ne x nv
        if dim == 2:
            st = np.stack([np.stack([sig[:, 0], sig[:, 2]], -1), np.stack([sig[:, 2], sig[:, 1]], -1)], 1)
        else:
            st = np.stack([np.stack([sig[:, 0], sig[:, 3], sig[:, 5]], -1),
                           np.stack([sig[:, 3], sig[:, 1], sig[:, 4]], -1),
                           np.stack([sig[:, 5], sig[:, 4], sig[:, 2]], -1)], 1)
        blocks += (t * wdet) * np.einsum("ai,eij,bj->eab", grad, st, grad)
    sym = 0.5 * (blocks + blocks.transpose(0, 2, 1))
    kge = np.einsum("eab,kl->eakbl", sym, np.eye(dim)).reshape(ne, ed, ed)
    kge[s == 0.0] = 0.0
    rows = np.repeat(edofs, ed, axis=1).ravel()
    cols = np.tile(edofs, (1, ed)).ravel()
    full = sp.csr_matrix((kge.ravel(), (rows, cols)), shape=(prob.ndof, prob.ndof))
    free = prob.free_dofs()
    return full[free][:, free].tocsr()


def end_traction(spec, force):
    """Consistent nodal forces of a uniform axial traction on the face x = lx
    whose resultant is `force` (x direction), spread over the face cells."""
    f = np.zeros(spec.num_dofs)
    nx = spec.nx
    if spec.dim == 2:
        per = force / spec.ny / 2.0
        for j in range(spec.ny):
            for jj in (j, j + 1):
                f[spec.node_index(nx, jj) * 2] += per
        return f
    per = force / (spec.ny * spec.nz) / 4.0
    for k in range(spec.nz):
        for j in range(spec.ny):
            for jj, kk in ((j, k), (j + 1, k), (j + 1, k + 1), (j, k + 1)):
                f[spec.node_index(nx, jj, kk) * 3] += per
    return f


def _splitmix_columns(n, count, state):
    """`count` columns of U[-1, 1) numbers from a SplitMix64 stream."""
    from sparlab_gb300.problems import SplitMix64
    rng = state.setdefault("rng", SplitMix64(SEED))
    return np.stack([rng.uniform_array(n, -1.0, 1.0) for _ in range(count)], 1)


@dataclass
class BucklingResult:
    load_factors: np.ndarray
    mode_shapes: np.ndarray
    residuals: np.ndarray
    solid_energy_fraction: np.ndarray
    no_positive_load_factor: bool
    iterations: int
    subspace_size: int
    converged: bool
    transformed: bool
    sigma: float
    factorizations: int
    final_change: float
    subspace: Optional[np.ndarray]
    warnings: List[str] = field(default_factory=list)


def solve_buckling(prob: Problem, spec, k, g, num_modes=4, max_iterations=400, tolerance=1e-8,
                   residual_tolerance=1e-6, transform="auto", shift_hint=0.0, initial_subspace=None,
                   stiffness_scale=None, solid_mask=None, solve=None) -> BucklingResult:
    """``solve_buckling`` on free-free K and G = -K_G (scipy CSR)."""
    n = k.shape[0]
    g_norm = np.abs(g.data).max() if g.nnz else 0.0
    m_req = min(num_modes, n)
    q = min(n, max(2 * m_req, m_req + 8))
    res = dict(iterations=0, converged=False, no_pos=False, transformed=False, sigma=0.0, factorizations=0,
               final_change=0.0)
    warnings: List[str] = []
    mu_top = np.zeros(0)
    phi_top = np.zeros((n, 0))
    subspace = None
    if not g_norm > 0.0:
        res["converged"] = res["no_pos"] = True
    elif n <= K_DENSE_LIMIT or q >= n:
        mu, v = sla.eigh(g.toarray(), k.toarray())
        mu_top = mu[::-1][:m_req]
        phi_top = v[:, ::-1][:, :m_req]
        subspace = phi_top
        res["converged"] = True
    else:
        if solve is None:
            lu = spla.splu(k.tocsc())
            solve = lu.solve
        state = {}
        x = np.zeros((n, q))
        col = 0
        if initial_subspace is not None and initial_subspace.shape[0] == n:
            keep = min(initial_subspace.shape[1], q - 2)
            x[:, :keep] = initial_subspace[:, :keep]
            col = keep
        x[:, col:] = _splitmix_columns(n, q - col, state)
        shifted = {"lu": None}

        def inertia(s):
            a = (k - s * g).toarray()
            res["factorizations"] += 1
            _, dd, _ = sla.ldl(a)
            ev = np.linalg.eigvalsh(dd)
            if np.any(ev == 0.0) or not np.all(np.isfinite(ev)):
                return -1
            shifted["lu"] = spla.splu((k - s * g).tocsc())
            return int(np.sum(ev < 0.0))

        def choose_sigma(guess):
            s = guess if guess > 0.0 else 1.0
            neg = inertia(s)
            if neg != 0:
                halvings = 0
                while neg != 0:
                    halvings += 1
                    if halvings > 120:
                        raise RuntimeError("the buckling shift search found no shift below the smallest load factor")
                    s *= 0.5
                    neg = inertia(s)
            elif not guess > 0.0:
                clean = s
                while True:
                    if s > 1e15:
                        return False
                    nxt = 8.0 * s
                    if inertia(nxt) != 0:
                        break
                    s = nxt
                    clean = s
                s = clean
                if inertia(s) != 0:
                    raise RuntimeError("inconsistent inertia in the buckling shift search")
            res["sigma"] = s
            res["transformed"] = True
            return True

        refined = False
        if transform == "shift_invert":
            if not choose_sigma(0.8 * shift_hint if shift_hint > 0 else 0.0):
                res["no_pos"] = res["converged"] = True
        previous = np.full(m_req, np.nan)
        mu_desc = ritz = None
        it = 0
        while it < max_iterations and not res["no_pos"]:
            it += 1
            if res["transformed"]:
                y = k @ x
                z = np.stack([shifted["lu"].solve(y[:, c]) for c in range(q)], 1)
            else:
                y = g @ x
                z = np.stack([solve(y[:, c]) for c in range(q)], 1)
            if not np.all(np.isfinite(z)):
                raise RuntimeError("buckling subspace iteration produced a non-finite basis")
            qm, rm, _ = sla.qr(z, mode="economic", pivoting=True)
            dr = np.abs(np.diag(rm))
            r = int(np.sum(dr > 1e-12 * dr.max())) if dr.size else 0
            if r < m_req:
                raise RuntimeError(f"the buckling subspace collapsed to {r} independent vectors")
            basis = qm[:, :r]
            gr = basis.T @ (g @ basis)
            kr = basis.T @ (k @ basis)
            mu, v = sla.eigh(0.5 * (gr + gr.T), 0.5 * (kr + kr.T))
            mu_desc = mu[::-1]
            ritz = basis @ v[:, ::-1]
            x[:, :r] = ritz
            if r < q:
                x[:, r:] = _splitmix_columns(n, q - r, state)
            scale = np.abs(mu_desc).max()
            zero = K_ZERO_FRACTION * scale
            mu_m = mu_desc[m_req - 1] if mu_desc[m_req - 1] > zero else 0.0
            change = 0.0
            resid = 0.0
            for i in range(m_req):
                m_i = mu_desc[i]
                denom = m_i if m_i > zero else scale
                delta = np.inf if np.isnan(previous[i]) else abs(m_i - previous[i]) / denom
                change = max(change, delta)
                if m_i > zero:
                    kphi = k @ ritz[:, i]
                    rr = g @ ritz[:, i] - m_i * kphi
                    resid = max(resid, np.linalg.norm(rr) / max(m_i * np.linalg.norm(kphi), 1e-300))
            previous = mu_desc[:m_req].copy()
            res["iterations"], res["final_change"] = it, change
            if change < tolerance and resid < residual_tolerance:
                res["converged"] = True
                break
            if not res["transformed"] and transform == "auto":
                competing = int(np.sum(mu_desc < -mu_m))
                if competing + m_req > q - 2:
                    est = 0.8 / mu_desc[0] if mu_desc[0] > zero else 0.0
                    if not choose_sigma(0.8 * shift_hint if shift_hint > 0 else est):
                        res["no_pos"] = res["converged"] = True
                        break
                    previous[:] = np.nan
            elif res["transformed"] and not refined and mu_desc[0] > zero and change < 1e-3 \
                    and res["sigma"] < 0.5 / mu_desc[0]:
                refined = True
                if not choose_sigma(0.8 / mu_desc[0]):
                    raise RuntimeError("the refined buckling shift found no load factor")
        if not res["converged"]:
            raise RuntimeError(f"buckling subspace iteration did not converge in {max_iterations} iterations")
        if not res["no_pos"]:
            mu_top = mu_desc[:m_req]
            phi_top = ritz[:, :m_req]
            subspace = ritz
    keep = []
    if mu_top.size:
        zero = K_ZERO_FRACTION * np.abs(mu_top).max()
        keep = [i for i in range(len(mu_top)) if mu_top[i] > zero]
    found = len(keep)
    lf = np.zeros(found)
    resids = np.zeros(found)
    frac = np.ones(found)
    shapes = np.zeros((prob.ndof, found))
    free = prob.free_dofs()
    for j, i in enumerate(keep):
        phi = phi_top[:, i].copy()
        kn = np.sqrt(max(phi @ (k @ phi), 0.0))
        if not kn > 0.0:
            raise RuntimeError("a buckling mode has zero strain energy")
        phi /= kn
        lam = 1.0 / mu_top[i]
        lf[j] = lam
        kphi = k @ phi
        resids[j] = np.linalg.norm(kphi - lam * (g @ phi)) / max(np.linalg.norm(kphi), 1e-300)
        shapes[free, j] = phi
        if resids[j] > residual_tolerance:
            warnings.append(f"buckling mode {j + 1} has an eigenpair residual of {resids[j]}")
    if found == 0:
        res["no_pos"] = True
    elif found < m_req:
        warnings.append(f"only {found} of the {m_req} requested modes have a positive load factor")
    if solid_mask is not None and found:
        ke = prob.element_matrix()
        edofs = element_dofs(spec)
        s = np.ones(prob.ne) if stiffness_scale is None else np.asarray(stiffness_scale, float)
        mask = np.asarray(solid_mask, bool)
        for j in range(found):
            pe = shapes[edofs, j]
            energy = s * np.einsum("ei,ij,ej->e", pe, ke, pe)
            tot = energy.sum()
            frac[j] = energy[mask].sum() / tot if tot > 0 else 0.0
    return BucklingResult(lf, shapes, resids, frac, res["no_pos"], res["iterations"], q, res["converged"],
                          res["transformed"], res["sigma"], res["factorizations"], res["final_change"],
                          subspace, warnings)


def analyse_buckling(prob: Problem, spec, load_case=0, stiffness_scale=None, stress_scale=None,
                     linear="direct", rtol=1e-12, **options) -> BucklingResult:
    """``analyse_buckling`` (Buckling.cpp:438-466) with optional SIMP factors:
    static solve of the load case, K_G of its stress state, solve_buckling.
    ``linear``: "direct" (SuperLU) or "amg_cg" (the oracle's AMG-PCG, what
    the reference's Auto solver picks above 10,000 3-D unknowns)."""
    ptr, col, val = prob.kff(stiffness_scale)
    k = sp.csr_matrix((val, col, ptr), shape=(prob.nfree, prob.nfree))
    if linear == "direct":
        solve = spla.splu(k.tocsc()).solve
    else:
        from . import Solver
        solver = Solver(rtol=rtol)
        solver.factorize(k.indptr, k.indices, k.data, spec.dim, prob.coords(), prob.free_dofs())

        def solve(b):
            return solver.solve(b)[0]
    free = prob.free_dofs()
    f = np.atleast_2d(spec.loads)[load_case][free]
    u = np.zeros(prob.ndof)
    u[free] = solve(f)
    g = -geometric_stiffness_ff(prob, spec, u, stress_scale)
    return solve_buckling(prob, spec, k, g, solve=solve, stiffness_scale=stiffness_scale, **options)
