"""Regenerate tests/golden/solver_scaling.json and tests/golden/benchmarks.json
from the reference checkout.

Reads the reference's published tables and keeps the columns the parity
tests pin:
* docs/results/solver_scaling.csv (the sparlab_bench model solved by LDL^T,
  AMG-CG and Jacobi-CG): mesh, solver, DOF count, stored non-zeros of K,
  compliance, CG iterations, AMG levels and operator complexity;
* docs/results/benchmarks.csv (the topology benchmarks of
  configs/benchmarks/), the rows on structured Q4/Hex8 grids with point
  loads: DOF count, volume fraction, the first iteration's compliance, the
  full-solid compliance and, where published, the full-solid design's first
  natural frequency (consistent mass) and mass, and (docs/results/buckling.csv)
  its smallest buckling load factor; and the optimisation's length, stop
  reason, final compliance and achieved volume fraction;
* docs/results/cross_validation.csv, the structured-grid models of
  configs/verification/ (cantilever_analysis, block_3d_analysis,
  column_hex_buckling_analysis): SparLab's largest displacement per load
  case and its buckling load factors.
Run from the repository root:

    python tests/golden/make_golden.py /path/to/reference
"""
import csv
import json
import os
import sys


def main(ref):
    rows = []
    with open(os.path.join(ref, "docs", "results", "solver_scaling.csv")) as f:
        for r in csv.DictReader(f):
            rows.append({
                "element": r["element"], "solver": r["solver"],
                "nx": int(float(r["nx"])), "ny": int(float(r["ny"])), "nz": int(float(r["nz"])),
                "num_dofs": int(float(r["num_dofs"])),
                "stiffness_nonzeros": int(float(r["stiffness_nonzeros"])),
                "compliance": float(r["compliance[J]"]),
                "iterations": int(float(r["iterations"])),
                "levels": int(float(r["levels"])),
                "operator_complexity": float(r["operator_complexity"]),
            })
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "solver_scaling.json")
    with open(out, "w") as f:
        json.dump({"source": "docs/results/solver_scaling.csv (sparlab_bench model, "
                             "tolerance 1e-10)", "rows": rows}, f, indent=1)
    print("wrote", out, len(rows), "rows")
    keep = {"cantilever_beam", "mbb_beam", "mbb_beam_projected", "mbb_beam_robust", "bracket_3d",
            "bracket_3d_projected", "bracket_3d_large", "column_buckling"}
    lam1 = {}
    with open(os.path.join(ref, "docs", "results", "buckling.csv")) as f:
        for r in csv.DictReader(f):
            if r["full_solid_lambda_1"]:
                lam1[r["case"]] = float(r["full_solid_lambda_1"])
    bench = []
    with open(os.path.join(ref, "docs", "results", "benchmarks.csv")) as f:
        for r in csv.DictReader(f):
            if r["case"] not in keep:
                continue
            bench.append({
                "case": r["case"], "dim": int(r["dim"]), "element_type": r["element_type"],
                "elements": int(r["elements"]), "dofs": int(r["dofs"]),
                "volume_fraction": float(r["volume_fraction_target"]),
                "initial_compliance": float(r["initial_compliance_J"]),
                "full_solid_compliance": float(r["full_solid_compliance_J"]),
                "linear_solver": r["linear_solver"],
                "f1_solid_hz": float(r["f1_solid_Hz"]) if r["f1_solid_Hz"] else None,
                "mass_solid_kg": float(r["mass_solid_kg"]) if r["mass_solid_kg"] else None,
                "full_solid_lambda_1": lam1.get(r["case"]),
                "iterations": int(r["iterations"]), "stop_reason": r["stop_reason"],
                "final_compliance": float(r["compliance_J"]),
                "volume_fraction_achieved": float(r["volume_fraction_achieved"]),
            })
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "benchmarks.json")
    with open(out, "w") as f:
        json.dump({"source": "docs/results/benchmarks.csv (configs/benchmarks/<case>.json)",
                   "rows": bench}, f, indent=1)
    print("wrote", out, len(bench), "rows")
    static, buckling = {}, {}
    with open(os.path.join(ref, "docs", "results", "cross_validation.csv")) as f:
        for r in csv.DictReader(f):
            if r["case"] in ("cantilever_analysis", "block_3d_analysis") and r["sparlab_max_abs_m"]:
                static[r["case"] + "/" + r["load_case"]] = float(r["sparlab_max_abs_m"])
            if r["case"] == "column_hex_buckling_analysis" and r["sparlab_load_factors"]:
                buckling[r["case"]] = json.loads(r["sparlab_load_factors"])
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "verification.json")
    with open(out, "w") as f:
        json.dump({"source": "docs/results/cross_validation.csv (configs/verification/<case>.json), "
                             "SparLab's own columns",
                   "max_abs_displacement": static, "buckling_load_factors": buckling}, f, indent=1)
    print("wrote", out, len(static) + len(buckling), "entries")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path to the reference checkout>")
    main(sys.argv[1])
