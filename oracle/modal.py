"""Modal analysis of a structured problem, restated from SparLab's
``solve_modal`` (src/fem/ModalAnalysis.cpp:120-418) -- test infrastructure
only: the GPU modal path is checked against it, nothing in the product
imports it.

Undamped free vibration on the free DOFs, K_ff phi = lambda M_ff phi, by
Bathe's subspace iteration with shift-invert (the reference's algorithm):
q = min(n, max(2m, m + 8)) trial vectors started from the mass diagonal and
unit vectors at the largest m_ii / k_ii; per iteration Xbar = A^-1 M X
(A = K - sigma M, each column warm-started from x_c / (mu_c - sigma)), the
projected pencil (Xbar^T K Xbar, Xbar^T M Xbar) solved densely, X = Xbar
times its eigenvectors; stop when the requested eigenvalues change by less
than ``tolerance`` and every requested eigenpair residual is below
``residual_tolerance``.  Systems with n <= 400 (or q >= n) take the dense
path.  The dense generalised eigensolves use LAPACK (scipy.linalg.eigh:
Cholesky of the mass, then the symmetric eigenproblem, the algorithm of
Eigen's GeneralizedSelfAdjointEigenSolver that the reference calls).

Pinning: the reference's own modal tests (tests/test_modal.cpp) -- the dense
cross-check at 1e-8, the Euler-Bernoulli bending and fixed-free rod
frequencies, thickness invariance, lumped below consistent, mass
conservation -- are restated in tests/test_modal_oracle.py.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np
import scipy.linalg as sla
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import Problem, Solver, _check, _p, lib

TWO_PI = 6.283185307179586476925286766559
_BETA_L = (1.87510407, 4.69409113, 7.85475744, 10.99554073, 14.13716839)


def element_mass(dim, hx, hy, hz, density, thickness=1.0):
    """Consistent mass of one box cell (3-point Gauss per direction)."""
    ed = 8 if dim == 2 else 24
    me = np.zeros((ed, ed))
    _check(lib().orc_element_mass(C.c_int(dim), C.c_double(hx), C.c_double(hy), C.c_double(hz),
                                  C.c_double(density), C.c_double(thickness), _p(me)))
    return me


def cantilever_bending_frequency(e, rho, length, height, thickness, mode_number=1):
    """Euler-Bernoulli cantilever frequency (ModalAnalysis.cpp:96-117)."""
    if mode_number < 1 or mode_number > 5:
        raise ValueError("cantilever_bending_frequency supports mode numbers 1..5")
    if not (e > 0 and rho > 0 and length > 0 and height > 0 and thickness > 0):
        raise ValueError("cantilever_bending_frequency requires positive E, rho, L, h, t")
    bl = _BETA_L[mode_number - 1]
    return (bl * bl) / (TWO_PI * length * length) * np.sqrt(e * height * height / (12.0 * rho))


def rod_axial_frequency(e, rho, length, mode_number=1):
    """Fixed-free rod frequency (ModalAnalysis.cpp:119-128)."""
    if mode_number < 1:
        raise ValueError("rod_axial_frequency requires mode_number >= 1")
    if not (e > 0 and rho > 0 and length > 0):
        raise ValueError("rod_axial_frequency requires positive E, rho and L")
    return (2 * mode_number - 1) * np.sqrt(e / rho) / (4.0 * length)


def lowest_pencil_pairs(k, m, count):
    """The ``count`` lowest pairs of (K, M), ascending, M-normalised; through
    the reversed pencil M y = mu K y when M is only semi-definite
    (ModalAnalysis.cpp:27-48).  None when neither form applies."""
    try:
        w, v = sla.eigh(k, m)
        return w[:count], v[:, :count]
    except (sla.LinAlgError, ValueError):
        pass
    try:
        w, v = sla.eigh(m, k)
    except (sla.LinAlgError, ValueError):
        return None
    n = len(w)
    lam = np.zeros(count)
    vec = np.zeros((k.shape[0], count))
    for i in range(count):
        mu = w[n - 1 - i]
        if not mu > 0.0:
            return None
        lam[i] = 1.0 / mu
        vec[:, i] = v[:, n - 1 - i]
    return lam, vec


def starting_subspace(kd, md, q):
    """Bathe's start (ModalAnalysis.cpp:55-88): the mass diagonal, then unit
    vectors at the DOFs of largest m_ii / k_ii (stable order)."""
    n = len(kd)
    x = np.zeros((n, q))
    x[:, 0] = md
    ratio = np.where(kd > 0.0, md / np.where(kd > 0.0, kd, 1.0), 0.0)
    order = np.argsort(-ratio, kind="stable")
    if n < q - 1:
        raise NotImplementedError("the seeded random fill needs q - 1 > n (never on the iterative path)")
    for c in range(1, q):
        x[order[c - 1], c] = 1.0
    return x


def connectivity(spec):
    """Element nodes of the structured mesh (n0, n0+1, n0+nnx+1, n0+nnx, then
    the same one layer up)."""
    nnx, nny = spec.nx + 1, spec.ny + 1
    if spec.dim == 2:
        iy, ix = np.meshgrid(np.arange(spec.ny), np.arange(spec.nx), indexing="ij")
        n0 = (iy * nnx + ix).ravel()
        return np.stack([n0, n0 + 1, n0 + nnx + 1, n0 + nnx], axis=1)
    iz, iy, ix = np.meshgrid(np.arange(spec.nz), np.arange(spec.ny), np.arange(spec.nx), indexing="ij")
    n0 = ((iz * nny + iy) * nnx + ix).ravel()
    lay = nnx * nny
    base = np.stack([n0, n0 + 1, n0 + nnx + 1, n0 + nnx], axis=1)
    return np.concatenate([base, base + lay], axis=1)


def element_dofs(spec):
    conn = connectivity(spec)
    d = spec.dim
    return (conn[:, :, None] * d + np.arange(d)[None, None, :]).reshape(conn.shape[0], -1)


@dataclass
class ModalResult:
    eigenvalues: np.ndarray
    angular_frequencies: np.ndarray
    frequencies_hz: np.ndarray
    mode_shapes: np.ndarray          # ndof x modes, M-orthonormal
    modal_residuals: np.ndarray
    modal_mass_fraction: np.ndarray
    total_mass: float
    iterations: int
    subspace_size: int
    converged: bool
    linear_iterations: int
    final_change: float
    warnings: List[str] = field(default_factory=list)


def mass_matrices(prob: Problem, spec, density, mass_type="consistent", mass_scale=None):
    """(M_ff as a scipy CSR or diagonal vector, full-matrix sum, M_e^0)."""
    hx, hy = spec.lx / spec.nx, spec.ly / spec.ny
    hz = spec.lz / spec.nz if spec.dim == 3 else 0.0
    me = element_mass(spec.dim, hx, hy, hz, density, spec.thickness if spec.dim == 2 else 1.0)
    scale = None if mass_scale is None else np.ascontiguousarray(mass_scale, np.float64)
    if mass_type == "consistent":
        ptr, col, _ = prob.kff()
        val = np.zeros(prob.nnz)
        total = C.c_double()
        _check(lib().orc_problem_assemble(prob._h, _p(np.ascontiguousarray(me)), _p(scale), _p(val),
                                          C.byref(total)))
        m = sp.csr_matrix((val, col, ptr), shape=(prob.nfree, prob.nfree))
        return m, total.value, me
    # row-sum lumping (Assembler.cpp:334-343): per element and DOF, the row
    # sum of M_e, summed in element order
    rows = np.array([sum(me[i, j] for j in range(me.shape[1])) for i in range(me.shape[0])])
    edofs = element_dofs(spec)
    s = np.ones(prob.ne) if scale is None else scale
    diag = np.zeros(prob.ndof)
    contrib = s[:, None] * rows[None, :]
    keep = s != 0.0
    np.add.at(diag, edofs[keep].ravel(), contrib[keep].ravel())
    total = 0.0
    for v in diag:
        total += v
    free = prob.free_dofs()
    return sp.diags(diag[free]).tocsr(), total, me


def solve_modal(prob: Problem, spec, num_modes=6, mass_type="consistent", max_iterations=200,
                tolerance=1e-10, shift_factor=0.0, rigid_body_ratio=1e-10, residual_tolerance=1e-6,
                density=1.0, stiffness_scale=None, mass_scale=None, rtol=1e-12, warm_start=True,
                linear="amg_cg", amg=None) -> ModalResult:
    """``solve_modal`` (ModalAnalysis.cpp:120-418) on the oracle's
    assembly.  ``linear``: "amg_cg" (the oracle's AMG-PCG, the GPU path's
    solver) or "direct" (SuperLU on K - sigma M)."""
    if num_modes < 1:
        raise ValueError("modal analysis requires num_modes >= 1")
    ptr, col, kval = prob.kff(stiffness_scale)
    n = prob.nfree
    k = sp.csr_matrix((kval, col, ptr), shape=(n, n))
    m, full_sum, me = mass_matrices(prob, spec, density, mass_type, mass_scale)
    warnings: List[str] = []
    total_mass = full_sum / spec.dim
    m_req = min(num_modes, n)
    if m_req < num_modes:
        warnings.append(f"requested {num_modes} modes but the model has only {n} free DOFs; "
                        f"returning {m_req}")
    q = min(n, max(2 * m_req, m_req + 8))
    iterations, converged, final_change, lin_its = 0, False, 0.0, 0
    if q >= n or n <= 400:
        pairs = lowest_pencil_pairs(k.toarray(), m.toarray(), m_req)
        if pairs is None:
            raise RuntimeError("dense generalised eigensolve failed")
        lam, phi = pairs
        converged = True
    else:
        sigma = 0.0
        kd, md = k.diagonal(), m.diagonal()
        if shift_factor != 0.0:
            pos = md > 0.0
            if pos.any():
                sigma = shift_factor * np.min(kd[pos] / md[pos])
        a = k if sigma == 0.0 else (k - sigma * m).tocsr()
        if linear == "direct":
            lu = spla.splu(a.tocsc())
            warm = False

            def solve(b, guess):
                return lu.solve(b), 0
        else:
            if sigma > 0.0:
                raise ValueError("a positive shift needs a direct solver")
            solver = Solver(rtol=rtol, **(amg or {}))
            solver.factorize(a.indptr, a.indices, a.data, spec.dim, prob.coords(), prob.free_dofs())
            warm = warm_start

            def solve(b, guess):
                x, its, _ = solver.solve(b, guess)
                return x, its
        x = starting_subspace(kd, md, q)
        prev = np.full(m_req, np.finfo(float).max)
        mu_prev = None
        for it in range(1, max_iterations + 1):
            y = m @ x
            xbar = np.zeros((n, q))
            for c in range(q):
                guess = None
                if warm and mu_prev is not None and mu_prev[c] - sigma > 0.0:
                    guess = x[:, c] / (mu_prev[c] - sigma)
                xbar[:, c], its = solve(y[:, c], guess)
                lin_its += its
            if not np.all(np.isfinite(xbar)):
                raise RuntimeError("subspace iteration produced a non-finite basis")
            kr = xbar.T @ (k @ xbar)
            mr = xbar.T @ (m @ xbar)
            pairs = lowest_pencil_pairs(0.5 * (kr + kr.T), 0.5 * (mr + mr.T), q)
            if pairs is None:
                raise RuntimeError(f"the projected {q} x {q} eigenproblem became numerically singular "
                                   f"at subspace iteration {it}")
            mu, ritz = pairs
            x = xbar @ ritz
            mu_prev = mu
            cur = mu[:m_req]
            with np.errstate(over="ignore"):
                change = float(np.max(np.abs(cur - prev) / np.maximum(np.abs(cur), 1e-300)))
            prev = cur
            iterations, final_change = it, change
            max_res = 0.0
            for i in range(m_req):
                mx = m @ x[:, i]
                r = k @ x[:, i] - cur[i] * mx
                ref = max(np.linalg.norm(cur[i] * mx), 1e-300)
                max_res = max(max_res, np.linalg.norm(r) / ref)
            if change < tolerance and max_res < residual_tolerance:
                converged = True
                break
        if not converged:
            raise RuntimeError(f"subspace iteration did not converge in {max_iterations} iterations")
        lam = prev
        phi = x[:, :m_req].copy()
    for i in range(m_req):
        mn = np.sqrt(max(phi[:, i] @ (m @ phi[:, i]), 0.0))
        if not mn > 0.0:
            raise RuntimeError("a computed mode shape has zero modal mass")
        phi[:, i] /= mn
    ks = np.abs(k.data).max() if k.nnz else 0.0
    ms = np.abs(m.data).max() if m.nnz else 1.0
    lam_scale = ks / ms if ms > 0 else 1.0
    res = np.zeros(m_req)
    for i in range(m_req):
        if not np.isfinite(lam[i]):
            raise RuntimeError(f"eigenvalue {i} is not finite")
        if lam[i] < -rigid_body_ratio * lam_scale:
            raise RuntimeError(f"eigenvalue {i} is negative ({lam[i]} 1/s^2)")
        if lam[i] < rigid_body_ratio * lam_scale:
            warnings.append(f"eigenvalue {i} is {lam[i]} 1/s^2, indistinguishable from zero")
        mx = m @ phi[:, i]
        res[i] = np.linalg.norm(k @ phi[:, i] - lam[i] * mx) / max(np.linalg.norm(lam[i] * mx), 1e-300)
        if res[i] > residual_tolerance:
            warnings.append(f"mode {i} has an eigenpair residual of {res[i]}")
    omega = np.sqrt(np.maximum(lam, 0.0))
    shapes = np.zeros((prob.ndof, m_req))
    shapes[prob.free_dofs()] = phi
    frac = np.zeros(m_req)
    if mass_scale is not None:
        edofs = element_dofs(spec)
        s = np.asarray(mass_scale, np.float64)
        for i in range(m_req):
            pe = shapes[edofs, i]
            ke = s * np.einsum("ei,ij,ej->e", pe, me, pe)
            total = ke.sum()
            frac[i] = ke[s < 0.3].sum() / total if total > 0 else 0.0
    return ModalResult(np.asarray(lam, float), omega, omega / TWO_PI, shapes, res, frac, total_mass,
                       iterations, q, converged, lin_its, final_change, warnings)
