"""``history.csv`` and ``summary.json`` of a GPU SIMP run in the reference's
formats, so its plotting package (``python/sparlab_viz``: ``load_csv`` of
``history.csv``, ``summary["optimization_setup"]`` and
``summary["optimization_result"]``) reads a GPU run unchanged.

* ``history.csv``: the columns of ``ResultWriter::write_history``
  (``src/io/ResultWriter.cpp:1428-1460``) for a run without stress, buckling
  or robust terms (``beta[-]`` when the projection is on), numbers as
  ``CsvWriter`` prints them (``std::setprecision(17)``,
  ``src/io/CsvWriter.cpp:58-97``).
* ``summary.json``: the ``optimization_setup`` / ``optimization_result`` /
  ``tolerances`` / ``provenance`` members of ``make_topology_summary``
  (``src/io/ResultWriter.cpp:2546-2883``) that this path determines; mesh,
  material and post-processing blocks of the reference's summary have no
  counterpart here and are left out.
"""
from __future__ import annotations

import json
import os
from typing import List, Optional, Sequence

from .problems import ProblemSpec

OC_COLUMNS = ["iteration", "penalty[-]", "compliance[J]", "volume[m3]", "volume_fraction[-]",
              "max_design_change[-]", "lagrange_multiplier[-]", "grey_level[-]", "oc_bisections[-]",
              "volume_converged[-]", "seconds[s]", "linear_iterations[-]"]
MMA_COLUMNS = ["iteration", "penalty[-]", "compliance[J]", "volume[m3]", "volume_fraction[-]",
               "max_design_change[-]", "lagrange_multiplier[-]", "grey_level[-]", "mma_iterations[-]",
               "volume_converged[-]", "seconds[s]", "max_stress_ratio[-]", "stress_constraint[-]",
               "constraint_violation[-]", "linear_iterations[-]"]


def _num(v) -> str:
    """A Scalar as std::ostream prints it at precision 17 (like printf %.17g)."""
    return format(float(v), ".17g")


def domain_volume(spec: ProblemSpec) -> float:
    if spec.dim == 2:
        return spec.lx * spec.ly * spec.thickness
    return spec.lx * spec.ly * spec.lz


def history_columns(method: str = "oc", projected: bool = False, robust: bool = False) -> List[str]:
    cols = list(MMA_COLUMNS if method == "mma" else OC_COLUMNS)
    if projected:
        cols.append("beta[-]")
    if robust:
        cols += ["eroded_volume_fraction[-]", "dilated_volume_fraction[-]", "dilated_target_fraction[-]"]
    return cols


def write_history_csv(path: str, history: Sequence, spec: ProblemSpec, method: str = "oc") -> None:
    """One row per :class:`~sparlab_gb300.topopt.TopologyIteration`."""
    mma = method == "mma"
    vol = domain_volume(spec)
    projected = bool(getattr(spec, "projection", False))
    robust = projected and bool(getattr(spec, "robust", False))
    with open(path, "w") as f:
        f.write(",".join(history_columns(method, projected, robust)) + "\n")
        for it in history:
            row = [spec.penalty, it.compliance, it.volume_fraction * vol, it.volume_fraction,
                   it.max_change, it.lam, it.gray_level, it.bisections,
                   1.0 if it.volume_converged else 0.0, it.seconds]
            if mma:
                # no stress constraint on this path; the volume constraint's violation
                row += [0.0, 0.0, max(0.0, it.volume_fraction / spec.volume_fraction - 1.0)]
            row.append(it.linear_iterations)
            if projected:
                row.append(it.beta)
            if robust:
                row += [it.eroded_volume_fraction, it.dilated_volume_fraction, it.dilated_target_fraction]
            f.write(str(int(it.iteration)) + "," + ",".join(_num(v) for v in row) + "\n")


def summary(spec: ProblemSpec, history: Sequence, method: str = "oc", max_iterations: int = 200,
            change_tolerance: float = 1e-3, stop_reason: Optional[str] = None,
            load_case_compliance: Optional[List[float]] = None, case: Optional[str] = None,
            solver: str = "gpu_amg_cg", robust_record: Optional[dict] = None) -> dict:
    """The summary members the plotting and result tables read.
    ``robust_record``: ``GpuSimpProblem.projection_variants()`` of the final
    design, written as the reference's ``robust`` (robust runs) or
    ``erosion_check`` block (src/io/ResultWriter.cpp:2766-2797); for a robust
    run the blueprint's compliance and volume fraction are the result's."""
    vol = domain_volume(spec)
    last = history[-1] if history else None
    converged = bool(last and change_tolerance > 0 and last.max_change <= change_tolerance)
    if stop_reason is None:
        stop_reason = "design_change" if converged else "iteration_cap"
    weights = [float(w) for w in spec.weights]
    wsum = sum(weights) or 1.0
    total_seconds = sum(it.seconds for it in history)
    lin = sum(it.linear_iterations for it in history)
    solves = len(history) * len(weights)
    setup = {
        "load_case_names": [f"load_{k}" for k in range(len(weights))],
        "load_case_weights": weights,
        "load_case_weights_normalised": [w / wsum for w in weights],
        "volume_fraction_target": spec.volume_fraction,
        "volume_target_m3": spec.volume_fraction * vol,
        "initial_density": spec.initial_density if spec.initial_density >= 0 else spec.volume_fraction,
        "domain_volume_m3": vol,
        "num_design_variables": spec.num_elements,
        "num_free_variables": spec.num_elements,
        "num_passive_solid": 0, "num_passive_void": 0,
        "passive_solid_volume_m3": 0.0, "passive_void_volume_m3": 0.0,
        "filter_type": "density", "filter_radius_m": spec.filter_radius,
        "simp_penalty": spec.penalty, "simp_emin_ratio": spec.emin_ratio,
        "move_limit": spec.move_limit, "damping": spec.damping,
        "max_iterations": max_iterations, "change_tolerance": change_tolerance,
        "method": method,
        "projection": ({"enabled": True, "eta": spec.eta, "beta_start": spec.beta_start,
                        "beta_max": spec.beta_max, "beta_factor": spec.beta_factor,
                        "beta_interval": spec.beta_interval,
                        "advance_on_convergence": bool(spec.advance_on_convergence),
                        "robust": bool(getattr(spec, "robust", False)),
                        **({"robust_delta": spec.robust_delta,
                            "robust_volume_interval": spec.robust_volume_interval}
                           if getattr(spec, "robust", False) else {})}
                       if getattr(spec, "projection", False) else {"enabled": False}),
    }
    if method == "mma":
        setup["constraint_tolerance"] = 1.0e-4
    result = {
        "converged": converged, "stop_reason": stop_reason,
        "final_design_change": last.max_change if last else 0.0,
        "iterations": len(history), "linear_solves": solves,
        "linear_solver": {"solver": solver, "iterative_iterations_total": lin,
                          "iterative_iterations_per_solve": lin / solves if solves else 0.0},
        "compliance_J": last.compliance if last else 0.0,
        "load_case_compliance_J": list(load_case_compliance or ([last.compliance] if last else [])),
        "volume_m3": last.volume_fraction * vol if last else 0.0,
        "volume_fraction": last.volume_fraction if last else 0.0,
        "volume_constraint_relative_violation":
            max(0.0, last.volume_fraction / spec.volume_fraction - 1.0) if last else 0.0,
        "grey_level": last.gray_level if last else 0.0,
        "total_seconds": total_seconds,
        "seconds_per_iteration": total_seconds / len(history) if history else 0.0,
        "warnings": [],
        "robust": bool(getattr(spec, "projection", False) and getattr(spec, "robust", False)),
    }
    result["volume_constraint_satisfied"] = result["volume_constraint_relative_violation"] <= 1.0e-6
    if getattr(spec, "projection", False) and last:
        result["projection"] = {"final_beta": last.beta, "eta": spec.eta}
    if robust_record is not None:
        rr = robust_record
        designs = [{"design": name, "eta": rr["eta_" + key], "compliance_J": rr["compliance_" + key],
                    "volume_fraction": rr["volume_fraction_" + key]}
                   for name, key in (("eroded", "eroded"), ("intermediate (blueprint)", "intermediate"),
                                     ("dilated", "dilated"))]
        if getattr(spec, "robust", False):
            result["robust"] = {
                "designs": designs, "dilated_target_fraction": rr["dilated_target_fraction"],
                "note": "compliance_J and volume_fraction below are the blueprint's; the optimiser "
                        "minimised the eroded design's compliance"}
            result["compliance_J"] = rr["compliance_intermediate"]
            result["volume_fraction"] = rr["volume_fraction_intermediate"]
            result["volume_m3"] = rr["volume_fraction_intermediate"] * vol
        else:
            result["erosion_check"] = {
                "designs": designs,
                "note": "a design optimised without the robust formulation, evaluated once at the "
                        "eroded and dilated thresholds eta +- robust_delta of the final beta"}
    if history:
        c0 = history[0].compliance
        result["initial_compliance_J"] = c0
        result["compliance_reduction_factor"] = c0 / last.compliance if last.compliance > 0 else 0.0
    return {
        "provenance": {"case": case or spec.name, "producer": "sparlab_gb300 (GPU SIMP loop)"},
        "tolerances": {"optimizer_change_tolerance": change_tolerance,
                       "optimizer_volume_tolerance": 1.0e-10},
        "optimization_setup": setup,
        "optimization_result": result,
    }


def write_results(out_dir: str, spec: ProblemSpec, history: Sequence, method: str = "oc",
                  **summary_kw) -> None:
    """``history.csv`` and ``summary.json`` into ``out_dir``."""
    os.makedirs(out_dir, exist_ok=True)
    write_history_csv(os.path.join(out_dir, "history.csv"), history, spec, method)
    with open(os.path.join(out_dir, "summary.json"), "w") as f:
        json.dump(summary(spec, history, method, **summary_kw), f, indent=2)
