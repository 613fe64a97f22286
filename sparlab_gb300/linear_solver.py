"""``GpuAmgCgSolver``: the reference's LinearSolver interface over the C ABI.

Mirrors ``sparlab::LinearSolver`` (include/sparlab/fem/LinearSolver.hpp:64-109)
and its AMG-CG implementation ``AmgCgSolver`` (src/fem/LinearSolver.cpp:
219-290): ``set_layout`` then ``factorize`` (AMG setup; aggregates are reused
while the structure is unchanged) and ``solve`` / ``solve_from`` per load
case; the queries ``iterative``, ``last_iterations``, ``last_error``,
``amg_stats`` and ``storage_nonzeros``.  Failures raise ``SolverError`` /
``ConvergenceError`` with the reference's wording.  The solve runs entirely
on the GPU; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import ConvergenceError, SolverError, ptr  # noqa: F401  (re-exported)


def parse_linear_solver_type(text: str) -> str:
    """The solver key this library adds to ``parse_linear_solver_type``
    (src/fem/LinearSolver.cpp:406-422)."""
    lower = text.lower()
    if lower in ("gpu_amg_cg", "gpu_amg", "gpu"):
        return "gpu_amg_cg"
    raise ValueError(f"unknown linear solver '{text}' (this library provides gpu_amg_cg)")


class GpuAmgCgSolver:
    def __init__(self, iterative_tolerance=1e-12, max_iterations=0, precision="fp64", device=0,
                 **amg):
        self._lib = _lib.load()
        prec = {"fp64": _lib.PRECISION_FP64, "mixed": _lib.PRECISION_MIXED}[precision]
        self.options = _lib.default_options(iterative_tolerance=iterative_tolerance,
                                            max_iterations=max_iterations, precision=prec,
                                            device=device, **amg)
        self._h = C.c_void_p()
        code = self._lib.simp_ctx_create(C.byref(self.options), C.byref(self._h))
        if code:
            _lib.raise_for(code, self._lib.simp_last_error(None).decode())
        self._n = 0
        self._iterations = 0
        self._error = 0.0

    def close(self):
        if getattr(self, "_h", None):
            self._lib.simp_ctx_destroy(self._h)
            self._h = None

    __del__ = close

    def _check(self, code):
        if code:
            _lib.raise_for(code, self._lib.simp_last_error(self._h).decode())

    def name(self) -> str:
        return "AMG-CG(chebyshev, GPU)"

    def iterative(self) -> bool:
        return True

    def set_layout(self, dim, coordinates, unknowns, dofs_per_node=0):
        coords = np.ascontiguousarray(coordinates, np.float64)
        unknowns = np.ascontiguousarray(unknowns, np.int32)
        self._check(self._lib.simp_set_layout(self._h, C.c_int32(dim), C.c_int32(dofs_per_node),
                                              ptr(coords), C.c_int32(coords.size // dim),
                                              ptr(unknowns, C.c_int32), C.c_int32(len(unknowns))))

    def factorize(self, rowptr, colidx, values):
        rowptr = np.ascontiguousarray(rowptr, np.int32)
        colidx = np.ascontiguousarray(colidx, np.int32)
        values = np.ascontiguousarray(values, np.float64)
        self._n = len(rowptr) - 1
        self._check(self._lib.simp_factorize(self._h, C.c_int32(self._n), ptr(rowptr, C.c_int32),
                                             ptr(colidx, C.c_int32), ptr(values)))

    def set_pattern(self, rowptr, colidx):
        """The pattern once (copied); values and setup per factorization."""
        rowptr = np.ascontiguousarray(rowptr, np.int32)
        colidx = np.ascontiguousarray(colidx, np.int32)
        self._n = len(rowptr) - 1
        self._check(self._lib.simp_set_pattern(self._h, C.c_int32(self._n), ptr(rowptr, C.c_int32),
                                               ptr(colidx, C.c_int32)))

    def set_values(self, values):
        values = np.ascontiguousarray(values, np.float64)
        self._check(self._lib.simp_set_values(self._h, ptr(values)))

    def set_values_device(self, device_ptr: int):
        """FP64 values already on the device (e.g. ``tensor.data_ptr()``)."""
        self._check(self._lib.simp_set_values_device(self._h, C.c_void_p(device_ptr)))

    def setup(self):
        self._check(self._lib.simp_setup(self._h))

    def factorize_scipy(self, k):
        k = k.tocsr()
        k.sort_indices()
        self.factorize(k.indptr, k.indices, k.data)

    def solve_many(self, b, x0=None):
        b = np.ascontiguousarray(np.atleast_2d(b), np.float64)
        nrhs = b.shape[0]
        x = np.zeros_like(b)
        x0 = None if x0 is None else np.ascontiguousarray(np.atleast_2d(x0), np.float64)
        its = np.zeros(nrhs, np.int32)
        rel = np.zeros(nrhs)
        self._check(self._lib.simp_solve(self._h, C.c_int32(nrhs), ptr(b), ptr(x0), ptr(x),
                                         ptr(its, C.c_int32), ptr(rel)))
        self._iterations = int(its[-1])
        self._error = float(rel[-1])
        return x, its, rel

    def solve(self, b):
        x, _, _ = self.solve_many(b)
        return x[0]

    def solve_from(self, b, initial_guess):
        g = np.asarray(initial_guess)
        x0 = g if g.size == np.asarray(b).size else None
        x, _, _ = self.solve_many(b, x0)
        return x[0]

    def apply_preconditioner(self, r):
        r = np.ascontiguousarray(r, np.float64)
        z = np.zeros_like(r)
        self._check(self._lib.simp_apply_preconditioner(self._h, ptr(r), ptr(z)))
        return z

    def last_iterations(self) -> int:
        return self._iterations

    def last_error(self) -> float:
        return self._error

    def amg_stats(self) -> dict:
        s = _lib.AmgStats()
        self._check(self._lib.simp_stats(self._h, C.byref(s)))
        return s.as_dict()

    def storage_nonzeros(self) -> int:
        return self.amg_stats()["storage_nonzeros"]

    def aggregates(self, level: int) -> np.ndarray:
        cnt = C.c_int32()
        self._check(self._lib.simp_level_aggregates(self._h, C.c_int32(level), None, C.byref(cnt)))
        a = np.zeros(cnt.value, np.int32)
        self._check(self._lib.simp_level_aggregates(self._h, C.c_int32(level), ptr(a, C.c_int32),
                                                    C.byref(cnt)))
        return a

    def level_matrix(self, level: int):
        rows = C.c_int32()
        nnz = C.c_int64()
        self._check(self._lib.simp_level_matrix(self._h, C.c_int32(level), C.byref(rows),
                                                C.byref(nnz), None, None, None))
        p = np.zeros(rows.value + 1, np.int32)
        c = np.zeros(nnz.value, np.int32)
        v = np.zeros(nnz.value)
        self._check(self._lib.simp_level_matrix(self._h, C.c_int32(level), C.byref(rows),
                                                C.byref(nnz), ptr(p, C.c_int32),
                                                ptr(c, C.c_int32), ptr(v)))
        return p, c, v

    def prolongator(self, level: int):
        rows, cols, nnz = C.c_int32(), C.c_int32(), C.c_int64()
        self._check(self._lib.simp_level_prolongator(self._h, C.c_int32(level), C.byref(rows),
                                                     C.byref(cols), C.byref(nnz), None, None, None))
        p = np.zeros(rows.value + 1, np.int32)
        c = np.zeros(nnz.value, np.int32)
        v = np.zeros(nnz.value)
        self._check(self._lib.simp_level_prolongator(self._h, C.c_int32(level), C.byref(rows),
                                                     C.byref(cols), C.byref(nnz),
                                                     ptr(p, C.c_int32), ptr(c, C.c_int32), ptr(v)))
        return rows.value, cols.value, p, c, v


def make_linear_solver(type: str = "gpu_amg_cg", **options) -> GpuAmgCgSolver:
    """``make_linear_solver`` for this library's key (src/fem/LinearSolver.cpp:424-443)."""
    parse_linear_solver_type(type)
    return GpuAmgCgSolver(**options)
