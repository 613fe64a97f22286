"""The SIMP iteration over the C ABI, with the reference's interfaces.

``ComplianceObjective.evaluate`` mirrors ``sparlab::ComplianceObjective::
evaluate`` (src/topopt/Sensitivity.cpp:110-237), ``optimality_criteria_update``
mirrors src/topopt/OptimalityCriteria.cpp:40-149, and
``TopologyOptimizer.run`` drives them as ``TopologyOptimizer::run_oc``
(src/topopt/TopologyOptimizer.cpp:556-724).  The design, densities,
displacements and gradients live in GPU memory; arrays are copied to the host
only when asked for.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import math
import time
from typing import List, Optional, Sequence

import numpy as np

from . import _lib
from ._lib import ptr
from .problems import ProblemSpec


def element_stiffness(dim, hx, hy, hz, young, poisson, thickness=1.0) -> np.ndarray:
    ed = 8 if dim == 2 else 24
    ke = np.zeros((ed, ed))
    code = _lib.load().simp_element_stiffness(C.c_int32(dim), C.c_double(hx), C.c_double(hy),
                                              C.c_double(hz), C.c_double(young),
                                              C.c_double(poisson), C.c_double(thickness), ptr(ke))
    if code:
        _lib.raise_for(code, _lib.load().simp_last_error(None).decode())
    return ke


@dataclasses.dataclass
class ObjectiveEvaluation:
    compliance: float
    volume: float
    volume_fraction: float
    linear_iterations: int
    relres_max: float
    physical_density: Optional[np.ndarray] = None
    dc_dphysical: Optional[np.ndarray] = None
    dc_dx: Optional[np.ndarray] = None
    dv_dx: Optional[np.ndarray] = None
    element_strain_energy: Optional[np.ndarray] = None
    displacements: Optional[np.ndarray] = None


@dataclasses.dataclass
class OptimalityCriteriaStep:
    x: Optional[np.ndarray]
    lam: float
    achieved_volume: float
    max_change: float
    bisections: int
    volume_converged: bool


@dataclasses.dataclass
class TopologyIteration:
    iteration: int
    compliance: float
    volume_fraction: float
    max_change: float
    lam: float
    gray_level: float
    linear_iterations: int
    bisections: int
    seconds: float
    volume_converged: bool = False
    beta: float = 0.0          # projection sharpness (0: no projection)
    final_stage: bool = True   # no projection, or its last beta stage
    # robust runs (volume_fraction is then the blueprint's)
    eroded_volume_fraction: float = 0.0
    dilated_volume_fraction: float = 0.0
    dilated_target_fraction: float = 0.0


def element_mass(dim, hx, hy, hz, density, thickness=1.0) -> np.ndarray:
    """Consistent mass of a box cell (Quad4Element / Hex8Element::consistent_mass)."""
    ed = 8 if dim == 2 else 24
    me = np.zeros((ed, ed))
    lib = _lib.load()
    code = lib.simp_element_mass(C.c_int32(dim), C.c_double(hx), C.c_double(hy), C.c_double(hz),
                                 C.c_double(density), C.c_double(thickness), ptr(me))
    if code:
        _lib.raise_for(code, lib.simp_problem_last_error(None).decode())
    return me


@dataclasses.dataclass
class ModalResult:
    """``sparlab::ModalResult`` (include/sparlab/fem/ModalAnalysis.hpp:67-86)."""
    eigenvalues: np.ndarray
    angular_frequencies: np.ndarray
    frequencies_hz: np.ndarray
    mode_shapes: Optional[np.ndarray]   # num_dofs x num_modes
    modal_residuals: np.ndarray
    modal_mass_fraction: np.ndarray
    total_mass: float
    iterations: int
    subspace_size: int
    converged: bool
    linear_iterations: int
    final_change: float
    warnings: List[str]
    linear_solver: str = "AMG-CG(chebyshev, GPU)"


@dataclasses.dataclass
class BucklingResult:
    """``sparlab::BucklingResult`` (include/sparlab/fem/Buckling.hpp:111-140)."""
    load_factors: np.ndarray
    mode_shapes: Optional[np.ndarray]   # num_dofs x modes, phi^T K phi = 1
    residuals: np.ndarray
    solid_energy_fraction: np.ndarray
    no_positive_load_factor: bool
    iterations: int
    subspace_size: int
    converged: bool
    linear_iterations: int
    final_change: float
    subspace: Optional[np.ndarray]      # free DOFs x columns
    warnings: List[str]
    transformed: bool = False
    sigma: float = 0.0                  # the transformation's shift, below lambda_1
    factorizations: int = 0             # factorisations of K - sigma G
    linear_solver: str = "AMG-CG(chebyshev, GPU)"


class GpuSimpProblem:
    """A structured SIMP problem resident on the GPU (boundary 2 of the C ABI)."""

    def __init__(self, spec: ProblemSpec, precision="fp64", element_matrix=None, device=0,
                 block_pcg=True, optimizer="oc", **amg):
        self._lib = _lib.load()
        self.spec = spec
        hx, hy = spec.lx / spec.nx, spec.ly / spec.ny
        hz = spec.lz / spec.nz if spec.dim == 3 else 0.0
        if element_matrix is None:
            element_matrix = element_stiffness(spec.dim, hx, hy, hz, spec.young, spec.poisson,
                                               spec.thickness if spec.dim == 2 else 1.0)
        self._ke = np.ascontiguousarray(element_matrix, np.float64)
        self._fixed = np.ascontiguousarray(spec.fixed, np.uint8)
        self._loads = np.ascontiguousarray(np.atleast_2d(spec.loads), np.float64)
        self._weights = np.ascontiguousarray(spec.weights, np.float64)
        d = _lib.ProblemDesc()
        d.dim, d.nx, d.ny, d.nz = spec.dim, spec.nx, spec.ny, spec.nz
        d.lx, d.ly, d.lz = spec.lx, spec.ly, spec.lz
        d.thickness = spec.thickness if spec.dim == 2 else 1.0
        d.element_matrix = ptr(self._ke)
        d.fixed = ptr(self._fixed, C.c_uint8)
        d.num_loads = self._loads.shape[0]
        d.loads = ptr(self._loads)
        d.weights = ptr(self._weights)
        d.filter_radius = spec.filter_radius
        d.volume_fraction = spec.volume_fraction
        d.initial_density = spec.initial_density
        d.penalty, d.emin_ratio = spec.penalty, spec.emin_ratio
        d.move_limit, d.damping = spec.move_limit, spec.damping
        d.warm_start = int(spec.warm_start)
        # load cases: False / 0 one after another, True / 1 concurrent host
        # threads, "graph" / 2 advanced together in one CUDA graph
        d.block_pcg = 2 if block_pcg == "graph" else int(block_pcg)
        d.optimizer = {"oc": 0, "mma": 1}[optimizer]
        d.projection = int(spec.projection)
        d.eta, d.beta_start, d.beta_max = spec.eta, spec.beta_start, spec.beta_max
        d.beta_factor, d.beta_interval = spec.beta_factor, spec.beta_interval
        d.advance_on_convergence = int(spec.advance_on_convergence)
        d.change_tolerance = spec.change_tolerance
        d.robust = int(getattr(spec, "robust", False))
        d.robust_delta = getattr(spec, "robust_delta", 0.1)
        d.robust_volume_interval = getattr(spec, "robust_volume_interval", 1)
        d.warm_history = int(getattr(spec, "warm_history", 0))
        prec = {"fp64": _lib.PRECISION_FP64, "mixed": _lib.PRECISION_MIXED}[precision]
        opts = dict(spec.amg)
        opts.update(amg)
        self.options = _lib.default_options(iterative_tolerance=spec.rtol,
                                            max_iterations=spec.max_cg_iterations,
                                            precision=prec, device=device, **opts)
        self._h = C.c_void_p()
        code = self._lib.simp_problem_create(C.byref(d), C.byref(self.options), C.byref(self._h))
        if code:
            _lib.raise_for(code, self._lib.simp_problem_last_error(None).decode())
        s = np.zeros(5, np.int64)
        self._check(self._lib.simp_problem_sizes(self._h, ptr(s, C.c_int64)))
        self.ne, self.nn, self.ndof, self.nfree, self.nnz = (int(v) for v in s)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.simp_problem_destroy(self._h)
            self._h = None

    __del__ = close

    def _check(self, code):
        if code:
            _lib.raise_for(code, self._lib.simp_problem_last_error(self._h).decode())

    def set_surrogate(self, surrogate):
        """Attaches a displacement surrogate (sparlab_gb300.surrogate) for
        warm start 3; None detaches.  The problem keeps no ownership."""
        self._surrogate = surrogate
        self._check(self._lib.simp_problem_set_surrogate(self._h, surrogate.handle if surrogate else None))

    def learned_seconds(self) -> float:
        """Seconds this problem's solves spent in surrogate predictions."""
        v = C.c_double()
        self._check(self._lib.simp_problem_learned_seconds(self._h, C.byref(v)))
        return v.value

    def set_design(self, x):
        x = np.ascontiguousarray(x, np.float64)
        self._check(self._lib.simp_set_design(self._h, ptr(x)))

    def design(self, out: Optional[np.ndarray] = None) -> np.ndarray:
        """The device design copied to host memory (into ``out`` when given:
        a contiguous float64 array of ne values, e.g. pinned memory)."""
        x = np.zeros(self.ne) if out is None else out
        if x.dtype != np.float64 or x.size != self.ne or not x.flags.c_contiguous:
            raise ValueError("design(out=...) needs a contiguous float64 array of ne values")
        self._check(self._lib.simp_get_design(self._h, ptr(x)))
        return x

    def evaluate(self, arrays=True, displacements=False) -> ObjectiveEvaluation:
        ev = _lib.Evaluation()
        out = {k: (np.zeros(self.ne) if arrays else None)
               for k in ("rho", "dcp", "dcx", "dvx", "se")}
        u = np.zeros((self._loads.shape[0], self.ndof)) if displacements else None
        self._check(self._lib.simp_evaluate(self._h, C.byref(ev), ptr(out["rho"]), ptr(out["dcp"]),
                                            ptr(out["dcx"]), ptr(out["dvx"]), ptr(out["se"]),
                                            ptr(u)))
        return ObjectiveEvaluation(ev.compliance, ev.volume, ev.volume_fraction,
                                   ev.linear_iterations, ev.relres_max, out["rho"], out["dcp"],
                                   out["dcx"], out["dvx"], out["se"], u)

    def oc_update(self, apply=True, download=True) -> OptimalityCriteriaStep:
        st = _lib.OcStep()
        xn = np.zeros(self.ne) if download else None
        self._check(self._lib.simp_oc_update(self._h, C.c_int32(int(apply)), C.byref(st), ptr(xn)))
        return OptimalityCriteriaStep(xn, st.lam, st.achieved_volume, st.max_change, st.bisections,
                                      bool(st.volume_converged))

    def mma_update(self, apply=True, download=True) -> OptimalityCriteriaStep:
        """MMA step (``MmaOptimizer::update``) with the last evaluation's
        gradients; ``bisections`` holds the subproblem's Newton iterations."""
        st = _lib.OcStep()
        xn = np.zeros(self.ne) if download else None
        self._check(self._lib.simp_mma_update(self._h, C.c_int32(int(apply)), C.byref(st), ptr(xn)))
        return OptimalityCriteriaStep(xn, st.lam, st.achieved_volume, st.max_change, st.bisections,
                                      bool(st.volume_converged))

    def iterate(self) -> _lib.IterationRecord:
        rec = _lib.IterationRecord()
        self._check(self._lib.simp_iterate(self._h, C.byref(rec)))
        return rec

    def amg_stats(self) -> dict:
        s = _lib.AmgStats()
        self._check(self._lib.simp_problem_stats(self._h, C.byref(s)))
        return s.as_dict()

    def apply_operator(self, x_device_ptr: int, y_device_ptr: int):
        """y = K_ff x on device pointers (nfree doubles each)."""
        self._check(self._lib.simp_problem_apply_operator(self._h, C.c_void_p(x_device_ptr),
                                                          C.c_void_p(y_device_ptr)))

    def apply_level0(self, x_device_ptr: int, y_device_ptr: int):
        """y = K_ff x through the V-cycle's level-0 operator (FP32 in mixed
        precision: matrix-free, on the tensor cores with tensor_cores=1)."""
        self._check(self._lib.simp_problem_apply_level0(self._h, C.c_void_p(x_device_ptr),
                                                        C.c_void_p(y_device_ptr)))

    def time_operator(self, reps: int = 20):
        """(ms per launch, algorithmic bytes per launch) of the FP64 level-0
        operator application (the CG operator), timed with CUDA events."""
        ms, by = C.c_double(), C.c_double()
        self._check(self._lib.simp_problem_time_operator(self._h, C.c_int32(reps), C.byref(ms),
                                                         C.byref(by)))
        return ms.value, by.value

    def filter_volume_noalloc(self, x_device_ptr: int, rho_device_ptr: int,
                              volume_device_ptr: int):
        """Physical density rho = clamp(H x, 0, 1) (Heaviside-projected at the
        current beta when the projection is on) and its volume, written to
        device memory, without allocating any device memory.

        For callers that cannot call cudaMalloc where they evaluate volumes:
        an optimiser trying many designs per iteration that must not stall
        the device on allocation, or an application that owns all device
        memory through its own pool.  Partial sums go to a fixed 128 KiB
        array of the library (at most 67,108,864 elements); make the first
        call on a device before any stream capture (and no cudaDeviceReset
        after it), and do not let two calls overlap on the GPU: they share
        that array."""
        self._check(self._lib.simp_filter_volume_noalloc(
            self._h, C.c_void_p(x_device_ptr), C.c_void_p(rho_device_ptr),
            C.c_void_p(volume_device_ptr)))

    def filter_forward(self, x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros(self.ne)
        self._check(self._lib.simp_filter_forward(self._h, ptr(x), ptr(y)))
        return y

    def filter_adjoint(self, v):
        v = np.ascontiguousarray(v, np.float64)
        g = np.zeros(self.ne)
        self._check(self._lib.simp_filter_adjoint(self._h, ptr(v), ptr(g)))
        return g

    def modal(self, num_modes=6, mass_type="consistent", max_iterations=200, tolerance=1e-10,
              shift_factor=0.0, rigid_body_ratio=1e-10, residual_tolerance=1e-6, warm_start=True,
              density=None, element_mass=None, stiffness_scale=None, mass_scale=None,
              mode_shapes=True, concurrent_solves=4) -> ModalResult:
        """``solve_modal`` (src/fem/ModalAnalysis.cpp:120-418) on this
        problem's grid and supports, with the problem's AMG-PCG options for
        the shifted solves.  Scales: per-element stiffness / mass factors
        (None: ones).  ``density`` defaults to ``spec.density``."""
        o = _lib.ModalOptions()
        self._lib.simp_default_modal_options(C.byref(o))
        o.num_modes, o.max_iterations = num_modes, max_iterations
        o.mass_type = {"consistent": 0, "lumped": 1}[mass_type]
        o.tolerance, o.shift_factor = tolerance, shift_factor
        o.rigid_body_ratio, o.residual_tolerance = rigid_body_ratio, residual_tolerance
        o.warm_start = int(warm_start)
        o.density = self.spec.density if density is None else density
        o.concurrent_solves = concurrent_solves
        me = None
        if element_mass is not None:
            me = np.ascontiguousarray(element_mass, np.float64)
            o.element_mass = ptr(me)
        ks = None if stiffness_scale is None else np.ascontiguousarray(stiffness_scale, np.float64)
        ms = None if mass_scale is None else np.ascontiguousarray(mass_scale, np.float64)
        m = max(1, min(num_modes, self.nfree))
        lam, freq, res, frac = (np.zeros(m) for _ in range(4))
        shapes = np.zeros((m, self.ndof)) if mode_shapes else None
        info = _lib.ModalInfo()
        self._check(self._lib.simp_modal(self._h, C.byref(o), ptr(ks), ptr(ms), ptr(lam), ptr(freq),
                                         ptr(res), ptr(frac), ptr(shapes), C.byref(info)))
        warnings = [self._lib.simp_modal_warning(self._h, k).decode() for k in range(info.num_warnings)]
        return ModalResult(lam, np.sqrt(np.maximum(lam, 0.0)), freq,
                           None if shapes is None else shapes.T.copy(), res, frac, info.total_mass,
                           info.iterations, info.subspace_size, bool(info.converged),
                           info.linear_iterations, info.final_change, warnings)

    def projection_variants(self, delta=0.0, densities=False) -> dict:
        """``RobustRecord`` of the current design (eroded / blueprint /
        dilated compliance and volume fraction at the current beta); with
        ``densities`` also the eroded and dilated physical densities."""
        rec = _lib.RobustRecord()
        er = np.zeros(self.ne) if densities else None
        di = np.zeros(self.ne) if densities else None
        self._check(self._lib.simp_projection_variants(self._h, C.c_double(delta), C.byref(rec),
                                                       ptr(er), ptr(di)))
        out = rec.as_dict()
        if densities:
            out["eroded_density"], out["dilated_density"] = er, di
        return out

    def buckling(self, load_case=0, num_modes=4, max_iterations=400, tolerance=1e-8,
                 residual_tolerance=1e-6, transform="auto", stiffness_scale=None, stress_scale=None,
                 solid_mask=None, initial_subspace=None, mode_shapes=True,
                 concurrent_solves=4, shift_hint=0.0) -> BucklingResult:
        """``analyse_buckling`` (src/fem/Buckling.cpp:438-466) of one load case
        with the problem's AMG-PCG; the material is ``spec.young`` /
        ``spec.poisson``."""
        o = _lib.BucklingOptions()
        self._lib.simp_default_buckling_options(C.byref(o))
        o.num_modes, o.max_iterations = num_modes, max_iterations
        o.tolerance, o.residual_tolerance = tolerance, residual_tolerance
        o.young, o.poisson = self.spec.young, self.spec.poisson
        o.transform = {"auto": 0, "shift_invert": 1}[transform]
        o.concurrent_solves = concurrent_solves
        o.shift_hint = shift_hint
        ks = None if stiffness_scale is None else np.ascontiguousarray(stiffness_scale, np.float64)
        ss = None if stress_scale is None else np.ascontiguousarray(stress_scale, np.float64)
        mask = None if solid_mask is None else np.ascontiguousarray(solid_mask, np.uint8)
        start = None
        cols = 0
        if initial_subspace is not None:
            start = np.asfortranarray(initial_subspace, np.float64)
            cols = start.shape[1]
        m = max(1, min(num_modes, self.nfree))
        q = min(self.nfree, max(2 * m, m + 8))
        lf, res, frac = (np.zeros(m) for _ in range(3))
        shapes = np.zeros((m, self.ndof)) if mode_shapes else None
        sub = np.zeros((q, self.nfree))
        info = _lib.BucklingInfo()
        self._check(self._lib.simp_buckling(
            self._h, C.byref(o), C.c_int32(load_case), ptr(ks), ptr(ss), ptr(mask, C.c_uint8),
            None if start is None else start.ctypes.data_as(C.POINTER(C.c_double)), C.c_int32(cols),
            ptr(lf), ptr(res), ptr(frac), ptr(shapes), ptr(sub), C.byref(info)))
        k = info.num_modes
        warnings = [self._lib.simp_buckling_warning(self._h, i).decode() for i in range(info.num_warnings)]
        return BucklingResult(lf[:k].copy(), None if shapes is None else shapes[:k].T.copy(), res[:k].copy(),
                              frac[:k].copy(), bool(info.no_positive_load_factor), info.iterations,
                              info.subspace_size, bool(info.converged), info.linear_iterations,
                              info.final_change,
                              sub[:info.subspace_cols].T.copy() if info.subspace_cols else None, warnings,
                              bool(info.transformed), info.sigma, info.factorizations)

    def kff(self, scale=None):
        p = np.zeros(self.nfree + 1, np.int32)
        c = np.zeros(self.nnz, np.int32)
        v = None if scale is None else np.zeros(self.nnz)
        scale = None if scale is None else np.ascontiguousarray(scale, np.float64)
        self._check(self._lib.simp_problem_kff(self._h, ptr(scale), ptr(p, C.c_int32),
                                               ptr(c, C.c_int32), ptr(v)))
        return p, c, v


class ComplianceObjective:
    """``ComplianceObjective`` over a :class:`GpuSimpProblem`."""

    def __init__(self, problem: GpuSimpProblem):
        self.problem = problem

    def evaluate(self, x, need_gradients=True) -> ObjectiveEvaluation:
        self.problem.set_design(x)
        return self.problem.evaluate(arrays=True)


def optimality_criteria_update(problem: GpuSimpProblem) -> OptimalityCriteriaStep:
    """OC step with the gradients of the problem's last evaluation (the volume
    callback of the reference is the problem's own filter)."""
    return problem.oc_update(apply=False, download=True)


def objective_spread(compliances: Sequence[float], window: int) -> float:
    """Relative spread (max - min) / |c_k| of the last ``window`` + 1
    compliances, infinite while fewer are known
    (``objective_spread``, src/topopt/TopologyOptimizer.cpp:124-130)."""
    w = max(int(window), 1)
    if len(compliances) <= w:
        return math.inf
    last = compliances[-(w + 1):]
    return (max(last) - min(last)) / max(abs(compliances[-1]), 1e-30)


class TopologyOptimizer:
    """``run_oc`` with the evaluation, OC update and clamp on the GPU.

    The run stops (src/topopt/TopologyOptimizer.cpp:675-704), once the
    projection's beta schedule is at its final stage, when the design change
    is at most ``change_tolerance`` (stop reason "design_change") or, with a
    positive ``objective_tolerance``, when the compliance's relative spread
    over the last ``objective_window`` + 1 iterations is at most that
    ("objective_stall"); otherwise after ``max_iterations``
    ("iteration_cap").  ``change_tolerance`` <= 0 disables the first rule."""

    def __init__(self, problem: GpuSimpProblem, max_iterations=200, change_tolerance=1e-3,
                 objective_tolerance=0.0, objective_window=5):
        self.problem = problem
        self.max_iterations = max_iterations
        self.change_tolerance = change_tolerance
        self.objective_tolerance = objective_tolerance
        self.objective_window = objective_window
        self.stop_reason = ""
        self.final_objective_change = math.inf

    def run(self) -> List[TopologyIteration]:
        history = []
        compliances: List[float] = []
        self.stop_reason = "iteration_cap"
        for it in range(1, self.max_iterations + 1):
            t0 = time.perf_counter()
            r = self.problem.iterate()
            history.append(TopologyIteration(it, r.compliance, r.volume_fraction, r.max_change,
                                             r.lam, r.gray_level, r.linear_iterations,
                                             r.bisections, time.perf_counter() - t0,
                                             bool(r.volume_converged), r.beta, bool(r.final_stage),
                                             r.eroded_volume_fraction, r.dilated_volume_fraction,
                                             r.dilated_target_fraction))
            compliances.append(r.compliance)
            change_ok = self.change_tolerance > 0 and r.max_change <= self.change_tolerance
            self.final_objective_change = objective_spread(compliances, self.objective_window)
            objective_ok = (self.objective_tolerance > 0
                            and self.final_objective_change <= self.objective_tolerance)
            # during beta continuation only the final stage may stop the run
            if r.final_stage and (change_ok or objective_ok):
                self.stop_reason = "design_change" if change_ok else "objective_stall"
                break
        return history


def iterate_batch(problems: List[GpuSimpProblem]) -> List[_lib.IterationRecord]:
    """One SIMP iteration of every problem with their linear solves advanced
    together (``simp_iterate_batch``): one CUDA graph launch runs one PCG
    iteration of every load case of every problem still iterating.  Each
    problem computes what ``iterate()`` computes alone."""
    lib = _lib.load()
    n = len(problems)
    handles = (C.c_void_p * n)(*[p._h.value for p in problems])
    recs = (_lib.IterationRecord * n)()
    code = lib.simp_iterate_batch(handles, C.c_int32(n), recs)
    if code:
        for p in problems:
            msg = lib.simp_problem_last_error(p._h).decode()
            if msg:
                _lib.raise_for(code, msg)
        _lib.raise_for(code, lib.simp_problem_last_error(None).decode())
    return list(recs)


def run_batched(problems: List[GpuSimpProblem], iterations: int, workers: Optional[int] = None,
                tune: bool = False, report: Optional[dict] = None, together: bool = False):
    """Iterate independent problem instances concurrently.

    Each problem owns a CUDA stream and the library releases the GIL during
    a call, so ``workers`` host threads (default: one per host core, at most
    one per problem) each drive their share of the instances, round robin
    (largest instance first), and the instances' kernels overlap on the GPU.
    Every instance computes exactly what it computes alone, whatever the
    worker count.  With ``tune`` the iterations after a problem set's first
    (which builds the hierarchies) try worker counts n, n/2, n/4, ... (one
    iteration each, timed on the host) and the rest use the fastest; ``report`` (a dict) receives the counts tried, their
    seconds and the choice.  With ``together`` every iteration is one
    :func:`iterate_batch` over all problems instead.  Returns the
    per-problem iteration records (lists, in problem order)."""
    import concurrent.futures as cf
    import os
    n = len(problems)
    order = sorted(range(n), key=lambda i: -problems[i].nnz)
    out: List[List[_lib.IterationRecord]] = [[] for _ in range(n)]
    if together:
        for _ in range(iterations):
            for i, r in enumerate(iterate_batch(problems)):
                out[i].append(r)
        return out

    def step(count, its):
        count = max(1, min(count, n))
        shares = [order[w::count] for w in range(count)]

        def drive(share):
            for _ in range(its):
                for i in share:
                    out[i].append(problems[i].iterate())

        with cf.ThreadPoolExecutor(max_workers=count) as ex:
            for f in [ex.submit(drive, sh) for sh in shares]:
                f.result()

    chosen = max(1, min(workers or os.cpu_count() or 1, n))
    done = 0
    if tune:
        if iterations > 0 and not out[0]:
            step(chosen, 1)   # a first iteration builds every hierarchy: not a fair sample
            done = 1
        cands, c = [], chosen
        while c >= 1 and len(cands) < 4:
            cands.append(c)
            c //= 2
        tried = []
        for c in cands:
            if done >= iterations:
                break
            t0 = time.perf_counter()
            step(c, 1)
            tried.append((c, time.perf_counter() - t0))
            done += 1
        if tried:
            chosen = min(tried, key=lambda t: t[1])[0]
        if report is not None:
            report["workers_tried"] = [c for c, _ in tried]
            report["seconds"] = [round(t, 4) for _, t in tried]
            report["workers"] = chosen
    if iterations > done:
        step(chosen, iterations - done)
    return out
