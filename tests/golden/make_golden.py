"""Regenerate tests/golden/solver_scaling.json from the reference checkout.

Reads the reference's published benchmark table
(docs/results/solver_scaling.csv: the sparlab_bench model solved by LDL^T,
AMG-CG and Jacobi-CG) and keeps the columns the parity tests pin: mesh,
solver, DOF count, stored non-zeros of K, compliance, CG iterations, AMG
levels and operator complexity.  Run from the repository root:

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


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path to the reference checkout>")
    main(sys.argv[1])
