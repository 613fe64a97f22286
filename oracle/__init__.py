"""CPU oracle of the SIMP inner loop (test infrastructure only).

A restatement of SparLab's algorithms in plain C++ (``simp_oracle.cpp``),
loaded through ctypes.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` use it, and only as the checker: the product
library in ``sparlab_gb300`` never imports it.

Pinning: the restatement is checked against the reference's published
known-answer compliances (``docs/results/solver_scaling.csv`` of the
reference) and against the identities the reference's tests assert
(``tests/test_multigrid.cpp``, ``tests/test_topopt.cpp``); see
``tests/test_oracle.py``.  The reference itself cannot be compiled here (it
needs Eigen), so there is no ``_ref`` build.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SRC = os.path.join(HERE, "simp_oracle.cpp")

_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with g++ (OpenMP where the reference uses it)."""
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "simp_oracle.h"))):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared",
           "-ffp-contract=off", SRC, "-o", tmp]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


class AmgOptions(C.Structure):
    _fields_ = [("strength_threshold", C.c_double), ("max_levels", C.c_int32),
                ("coarse_size", C.c_int32), ("smoother_degree", C.c_int32),
                ("chebyshev_ratio", C.c_double), ("prolongator_damping", C.c_double),
                ("lanczos_steps", C.c_int32), ("coarse_pivot_tolerance", C.c_double),
                ("reuse_aggregates", C.c_int32)]


class ProblemDesc(C.Structure):
    _fields_ = [("dim", C.c_int32), ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
                ("lx", C.c_double), ("ly", C.c_double), ("lz", C.c_double),
                ("young", C.c_double), ("poisson", C.c_double), ("thickness", C.c_double),
                ("fixed", C.POINTER(C.c_uint8)), ("num_loads", C.c_int32),
                ("loads", C.POINTER(C.c_double)), ("weights", C.POINTER(C.c_double)),
                ("filter_radius", C.c_double), ("volume_fraction", C.c_double),
                ("initial_density", C.c_double), ("penalty", C.c_double),
                ("emin_ratio", C.c_double), ("move_limit", C.c_double),
                ("damping", C.c_double), ("rtol", C.c_double),
                ("max_cg_iterations", C.c_int32), ("warm_start", C.c_int32),
                ("amg", AmgOptions), ("projection", C.c_int32), ("eta", C.c_double),
                ("beta_start", C.c_double), ("beta_max", C.c_double), ("beta_factor", C.c_double),
                ("beta_interval", C.c_int32), ("advance_on_convergence", C.c_int32),
                ("change_tolerance", C.c_double), ("robust", C.c_int32),
                ("robust_delta", C.c_double), ("robust_volume_interval", C.c_int32)]


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            _lib = C.CDLL(LIB)
            _lib.orc_last_error.restype = C.c_char_p
    return _lib


class OracleError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


def _check(code):
    if code != 0:
        raise OracleError(code, lib().orc_last_error().decode())


def _p(a, ctype=C.c_double):
    return a.ctypes.data_as(C.POINTER(ctype)) if a is not None else None


def amg_options(**kw) -> AmgOptions:
    o = AmgOptions()
    lib().orc_default_amg_options(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def element_stiffness(dim, hx, hy, hz, young, poisson, thickness=1.0):
    ed = 8 if dim == 2 else 24
    ke = np.zeros((ed, ed))
    _check(lib().orc_element_stiffness(C.c_int(dim), C.c_double(hx), C.c_double(hy),
                                       C.c_double(hz), C.c_double(young), C.c_double(poisson),
                                       C.c_double(thickness), _p(ke)))
    return ke


class Solver:
    """AMG-PCG on a caller's K_ff, the LinearSolver boundary of the oracle."""

    def __init__(self, rtol=1e-12, max_iterations=0, **amg):
        self._h = C.c_void_p()
        self._opts = amg_options(**amg)
        _check(lib().orc_solver_create(C.byref(self._opts), C.c_double(rtol),
                                       C.c_int32(max_iterations), C.byref(self._h)))
        self._keep = []

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.orc_solver_destroy(self._h)
            self._h = None

    def factorize(self, rowptr, col, val, dim, coords, unknowns, ndpn=None):
        rowptr = np.ascontiguousarray(rowptr, np.int32)
        col = np.ascontiguousarray(col, np.int32)
        val = np.ascontiguousarray(val, np.float64)
        coords = np.ascontiguousarray(coords, np.float64)
        unknowns = np.ascontiguousarray(unknowns, np.int32)
        self.n = len(rowptr) - 1
        self._keep = [unknowns]
        _check(lib().orc_solver_factorize(
            self._h, C.c_int32(self.n), _p(rowptr, C.c_int32), _p(col, C.c_int32), _p(val),
            C.c_int(dim), C.c_int(ndpn or dim), _p(coords), C.c_int32(coords.size // dim),
            _p(unknowns, C.c_int32)))

    def solve(self, b, x0=None):
        b = np.ascontiguousarray(b, np.float64)
        x = np.zeros(self.n)
        it = C.c_int32()
        rr = C.c_double()
        x0 = None if x0 is None else np.ascontiguousarray(x0, np.float64)
        _check(lib().orc_solver_solve(self._h, _p(b), _p(x0), _p(x), C.byref(it), C.byref(rr)))
        return x, it.value, rr.value

    def apply(self, r):
        r = np.ascontiguousarray(r, np.float64)
        z = np.zeros(self.n)
        _check(lib().orc_solver_apply(self._h, _p(r), _p(z)))
        return z

    def num_levels(self):
        return lib().orc_solver_num_levels(self._h)

    def level_info(self, level):
        info = np.zeros(3, np.int64)
        lam = C.c_double()
        _check(lib().orc_solver_level_info(self._h, C.c_int(level), _p(info, C.c_int64),
                                           C.byref(lam)))
        return int(info[0]), int(info[1]), int(info[2]), lam.value

    def level_matrix(self, level):
        rows, nnz, _, _ = self.level_info(level)
        ptr = np.zeros(rows + 1, np.int32)
        col = np.zeros(nnz, np.int32)
        val = np.zeros(nnz)
        _check(lib().orc_solver_level_matrix(self._h, C.c_int(level), _p(ptr, C.c_int32),
                                             _p(col, C.c_int32), _p(val)))
        return ptr, col, val

    def prolongator(self, level, tentative=False):
        sz = np.zeros(3, np.int64)
        _check(lib().orc_solver_prolongator_nnz(self._h, C.c_int(level), C.c_int(int(tentative)),
                                                _p(sz, C.c_int64)))
        ptr = np.zeros(sz[0] + 1, np.int32)
        col = np.zeros(sz[2], np.int32)
        val = np.zeros(sz[2])
        _check(lib().orc_solver_prolongator(self._h, C.c_int(level), C.c_int(int(tentative)),
                                            _p(ptr, C.c_int32), _p(col, C.c_int32), _p(val)))
        return int(sz[0]), int(sz[1]), ptr, col, val

    def aggregates(self, level):
        nn = C.c_int32()
        _check(lib().orc_solver_num_nodes(self._h, C.c_int(level), C.byref(nn)))
        agg = np.zeros(nn.value, np.int32)
        _check(lib().orc_solver_aggregates(self._h, C.c_int(level), _p(agg, C.c_int32)))
        return agg

    def nullspace(self, level):
        rows = self.level_info(level)[0]
        cols = C.c_int32()
        _check(lib().orc_solver_nullspace(self._h, C.c_int(level), C.byref(cols), None))
        b = np.zeros((rows, cols.value))
        _check(lib().orc_solver_nullspace(self._h, C.c_int(level), C.byref(cols), _p(b)))
        return b

    def stats(self):
        oc = C.c_double()
        pr = C.c_double()
        re = C.c_int32()
        _check(lib().orc_solver_stats(self._h, C.byref(oc), C.byref(pr), C.byref(re)))
        return {"operator_complexity": oc.value, "coarse_pivot_ratio": pr.value,
                "reused_aggregates": bool(re.value)}


class Mma:
    """MmaOptimizer(n, 1, 0, 1): n variables in [0, 1], one constraint row,
    one update per call with the asymptotes kept between calls."""

    def __init__(self, n):
        self.n = int(n)
        self._h = C.c_void_p()
        _check(lib().orc_mma_create(C.c_int32(self.n), C.byref(self._h)))

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.orc_mma_destroy(self._h)
            self._h = None

    def update(self, x, df0, fval, dfdx):
        x = np.ascontiguousarray(x, np.float64)
        df0 = np.ascontiguousarray(df0, np.float64)
        dfdx = np.ascontiguousarray(dfdx, np.float64)
        assert x.size == df0.size == dfdx.size == self.n
        xn = np.zeros(self.n)
        out = np.zeros(7)
        _check(lib().orc_mma_update(self._h, _p(x), _p(df0), C.c_double(fval), _p(dfdx), _p(xn),
                                    _p(out)))
        return xn, dict(lam=out[0], y=out[1], z=out[2], max_change=out[3],
                        constraint_scale=out[4], subproblem_iterations=int(out[5]),
                        iteration=int(out[6]))


class Problem:
    """Structured SIMP problem: the ComplianceObjective / OC boundary of the oracle.

    ``spec`` is a :class:`sparlab_gb300.problems.ProblemSpec`-like object with
    the attributes read below."""

    def __init__(self, spec, amg=None):
        self.spec = spec
        self._fixed = np.ascontiguousarray(spec.fixed, np.uint8)
        self._loads = np.ascontiguousarray(spec.loads, np.float64)
        self._weights = np.ascontiguousarray(spec.weights, np.float64)
        d = ProblemDesc()
        d.dim, d.nx, d.ny, d.nz = spec.dim, spec.nx, spec.ny, spec.nz
        d.lx, d.ly, d.lz = spec.lx, spec.ly, spec.lz
        d.young, d.poisson, d.thickness = spec.young, spec.poisson, spec.thickness
        d.fixed = _p(self._fixed, C.c_uint8)
        d.num_loads = self._loads.shape[0]
        d.loads = _p(self._loads)
        d.weights = _p(self._weights)
        d.filter_radius = spec.filter_radius
        d.volume_fraction = spec.volume_fraction
        d.initial_density = spec.initial_density
        d.penalty, d.emin_ratio = spec.penalty, spec.emin_ratio
        d.move_limit, d.damping = spec.move_limit, spec.damping
        d.rtol, d.max_cg_iterations = spec.rtol, spec.max_cg_iterations
        d.warm_start = int(spec.warm_start)
        d.amg = amg_options(**(amg or spec.amg))
        d.projection = int(getattr(spec, "projection", False))
        d.eta = getattr(spec, "eta", 0.5)
        d.beta_start = getattr(spec, "beta_start", 1.0)
        d.beta_max = getattr(spec, "beta_max", 32.0)
        d.beta_factor = getattr(spec, "beta_factor", 2.0)
        d.beta_interval = getattr(spec, "beta_interval", 50)
        d.advance_on_convergence = int(getattr(spec, "advance_on_convergence", True))
        d.change_tolerance = getattr(spec, "change_tolerance", 1e-3)
        d.robust = int(getattr(spec, "robust", False))
        d.robust_delta = getattr(spec, "robust_delta", 0.1)
        d.robust_volume_interval = getattr(spec, "robust_volume_interval", 1)
        self._desc = d
        self._h = C.c_void_p()
        _check(lib().orc_problem_create(C.byref(d), C.byref(self._h)))
        s = np.zeros(5, np.int64)
        lib().orc_problem_sizes(self._h, _p(s, C.c_int64))
        self.ne, self.nn, self.ndof, self.nfree, self.nnz = (int(v) for v in s)

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.orc_problem_destroy(self._h)
            self._h = None

    def free_dofs(self):
        f = np.zeros(self.nfree, np.int32)
        lib().orc_problem_free_dofs(self._h, _p(f, C.c_int32))
        return f

    def coords(self):
        c = np.zeros(self.nn * self.spec.dim)
        lib().orc_problem_coords(self._h, _p(c))
        return c

    def element_matrix(self):
        ed = 8 if self.spec.dim == 2 else 24
        ke = np.zeros((ed, ed))
        lib().orc_problem_element_matrix(self._h, _p(ke))
        return ke

    def kff(self, scale=None):
        ptr = np.zeros(self.nfree + 1, np.int32)
        col = np.zeros(self.nnz, np.int32)
        val = np.zeros(self.nnz)
        scale = None if scale is None else np.ascontiguousarray(scale, np.float64)
        _check(lib().orc_problem_kff(self._h, _p(scale), _p(ptr, C.c_int32),
                                     _p(col, C.c_int32), _p(val)))
        return ptr, col, val

    def filter_forward(self, x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros(self.ne)
        _check(lib().orc_filter_forward(self._h, _p(x), _p(y)))
        return y

    def filter_adjoint(self, v):
        v = np.ascontiguousarray(v, np.float64)
        g = np.zeros(self.ne)
        _check(lib().orc_filter_adjoint(self._h, _p(v), _p(g)))
        return g

    def filter_row_sums(self):
        s = np.zeros(self.ne)
        lib().orc_filter_row_sums(self._h, _p(s))
        return s

    def evaluate(self, x, displacements=False):
        x = np.ascontiguousarray(x, np.float64)
        out = np.zeros(4)
        arrs = {k: np.zeros(self.ne) for k in ("rho", "dc_dphys", "dc_dx", "dv_dx", "se")}
        u = np.zeros((self._loads.shape[0], self.ndof)) if displacements else None
        _check(lib().orc_evaluate(self._h, _p(x), _p(out), _p(arrs["rho"]), _p(arrs["dc_dphys"]),
                                  _p(arrs["dc_dx"]), _p(arrs["dv_dx"]), _p(arrs["se"]), _p(u)))
        res = dict(compliance=out[0], volume=out[1], volume_fraction=out[2],
                   linear_iterations=int(out[3]), **arrs)
        if displacements:
            res["u"] = u
        return res

    def oc_update(self, x, dc_dx, dv_dx):
        x = np.ascontiguousarray(x, np.float64)
        dc = np.ascontiguousarray(dc_dx, np.float64)
        dv = np.ascontiguousarray(dv_dx, np.float64)
        xn = np.zeros(self.ne)
        out = np.zeros(5)
        _check(lib().orc_oc_update(self._h, _p(x), _p(dc), _p(dv), _p(xn), _p(out)))
        return xn, dict(lam=out[0], volume=out[1], max_change=out[2], bisections=int(out[3]),
                        converged=bool(out[4]))

    def run_mma(self, iterations):
        """run_mma: final design and history rows in run()'s layout (the
        MMA subproblem iterations in the bisections column)."""
        x = np.zeros(self.ne)
        hist = np.zeros((iterations, 10))
        done = C.c_int32()
        _check(lib().orc_run_mma(self._h, C.c_int32(iterations), _p(x), _p(hist), C.byref(done)))
        return x, hist[: done.value]

    def run(self, iterations, change_tol=0.0):
        """run_oc: final design and history rows (compliance, volume
        fraction (the blueprint's in a robust run), max change, lambda, CG
        iterations, bisections, beta, and for a robust run the eroded and
        dilated volume fractions and the dilated target fraction)."""
        x = np.zeros(self.ne)
        hist = np.zeros((iterations, 10))
        done = C.c_int32()
        _check(lib().orc_run(self._h, C.c_int32(iterations), C.c_double(change_tol), _p(x),
                             _p(hist), C.byref(done)))
        return x, hist[: done.value]
