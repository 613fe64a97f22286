"""history.csv / summary.json in the reference's formats (the columns of
ResultWriter::write_history, src/io/ResultWriter.cpp:1428-1460, and the
summary members its plotting reads), on synthetic iteration records."""
import csv
import json

from sparlab_gb300 import problems as P
from sparlab_gb300.results import MMA_COLUMNS, OC_COLUMNS, write_results
from sparlab_gb300.topopt import TopologyIteration


def _history(n=3):
    return [TopologyIteration(k + 1, 10.0 / (k + 1), 0.5, 0.2 / (k + 1), 1e-3 * (k + 1), 0.25, 20 + k, 35 + k,
                              0.1, True) for k in range(n)]


def test_history_columns_and_number_format(tmp_path):
    spec = P.q4_cantilever_120x40()
    write_results(str(tmp_path), spec, _history(), "oc", max_iterations=3)
    rows = list(csv.reader(open(tmp_path / "history.csv")))
    assert rows[0] == OC_COLUMNS
    assert OC_COLUMNS == ["iteration", "penalty[-]", "compliance[J]", "volume[m3]", "volume_fraction[-]",
                          "max_design_change[-]", "lagrange_multiplier[-]", "grey_level[-]",
                          "oc_bisections[-]", "volume_converged[-]", "seconds[s]", "linear_iterations[-]"]
    assert rows[1][0] == "1" and rows[3][0] == "3"
    # std::setprecision(17): 0.1 prints as 0.10000000000000001, 3 as 3
    assert rows[1][OC_COLUMNS.index("seconds[s]")] == "0.10000000000000001"
    assert rows[1][OC_COLUMNS.index("penalty[-]")] == "3"
    assert float(rows[2][OC_COLUMNS.index("compliance[J]")]) == 5.0
    assert float(rows[1][OC_COLUMNS.index("volume[m3]")]) == 0.5 * 120 * 40


def test_mma_history_columns(tmp_path):
    spec = P.q4_cantilever_120x40()
    write_results(str(tmp_path), spec, _history(2), "mma")
    header = next(csv.reader(open(tmp_path / "history.csv")))
    assert header == MMA_COLUMNS
    assert header[8] == "mma_iterations[-]" and header[-1] == "linear_iterations[-]"


def test_summary_members_the_plots_read(tmp_path):
    spec = P.q4_cantilever_120x40()
    write_results(str(tmp_path), spec, _history(), "oc", max_iterations=3, change_tolerance=0.0)
    s = json.load(open(tmp_path / "summary.json"))
    setup, res = s["optimization_setup"], s["optimization_result"]
    assert setup["method"] == "oc" and setup["volume_fraction_target"] == 0.5
    assert res["iterations"] == 3 and res["stop_reason"] == "iteration_cap"
    assert res["compliance_J"] == 10.0 / 3
    assert res["initial_compliance_J"] == 10.0
    assert res["linear_solver"]["iterative_iterations_total"] == 20 + 21 + 22
    assert "optimizer_volume_tolerance" in s["tolerances"]
    assert s["provenance"]["case"] == spec.name


def test_robust_history_columns():
    """ResultWriter::write_history appends the eroded / dilated / target
    fractions for a robust run (src/io/ResultWriter.cpp:1445-1448)."""
    import os
    import tempfile
    from sparlab_gb300 import problems as P
    from sparlab_gb300.results import write_history_csv
    from sparlab_gb300.topopt import TopologyIteration
    spec = P.q4_cantilever_120x40()
    spec.projection, spec.robust = True, True
    hist = [TopologyIteration(1, 2.0, 0.5, 0.1, 1.0, 0.3, 20, 30, 0.01, True, 2.0, False, 0.45, 0.55, 0.56)]
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "history.csv")
        write_history_csv(path, hist, spec)
        head, row = open(path).read().splitlines()
    cols = head.split(",")
    assert cols[-4:] == ["beta[-]", "eroded_volume_fraction[-]", "dilated_volume_fraction[-]",
                         "dilated_target_fraction[-]"]
    assert [float(v) for v in row.split(",")[-3:]] == [0.45, 0.55, 0.56]


def test_summary_robust_and_erosion_blocks():
    from sparlab_gb300 import problems as P
    from sparlab_gb300.results import summary
    from sparlab_gb300.topopt import TopologyIteration
    spec = P.q4_cantilever_120x40()
    spec.projection = True
    hist = [TopologyIteration(1, 2.0, 0.5, 0.1, 1.0, 0.3, 20, 30, 0.01, True, 2.0, True)]
    rr = {"eta_eroded": 0.6, "eta_intermediate": 0.5, "eta_dilated": 0.4, "compliance_eroded": 3.0,
          "compliance_intermediate": 2.0, "compliance_dilated": 1.5, "volume_fraction_eroded": 0.45,
          "volume_fraction_intermediate": 0.5, "volume_fraction_dilated": 0.55, "dilated_target_fraction": 0.56}
    s = summary(spec, hist, robust_record=rr)["optimization_result"]
    assert [d["design"] for d in s["erosion_check"]["designs"]] == ["eroded", "intermediate (blueprint)", "dilated"]
    spec.robust = True
    s = summary(spec, hist, robust_record=rr)["optimization_result"]
    assert s["robust"]["dilated_target_fraction"] == 0.56
    assert s["compliance_J"] == 2.0 and s["volume_fraction"] == 0.5
