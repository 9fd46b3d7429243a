"""CPU-only checks of the result-line format of the reference's driver
(main.cu:54-61) and of the log parser / CSV writer that replaces process.js."""
import csv

import pytest


@pytest.fixture(scope="module")
def pg():
    import pagerank_gb300
    pagerank_gb300.load()
    return pagerank_gb300


def reference_format(d, i, b, t, r, err, tech):
    # the printf of main.cu:56-59, restated with Python's % operator
    return ("{-%.3e/+%.3e batchf, %03d batchi, %03d threads} -> {%09.1fms, %09.1fms init, %09.1fms mark, "
            "%09.1fms comp, %03d iter, %.2e err} %s" % (d, i, b, t, r["time_ms"], r["initialization_time_ms"],
                                                         r["marking_time_ms"], r["computation_time_ms"],
                                                         r["iterations"], err, tech))


RESULTS = [
    {"iterations": 57, "time_ms": 12.25, "initialization_time_ms": 0.5, "marking_time_ms": 0.0,
     "computation_time_ms": 11.75},
    {"iterations": 3, "time_ms": 1234567.5, "initialization_time_ms": 0.125, "marking_time_ms": 7.5,
     "computation_time_ms": 0.0625},
    {"iterations": 1000, "time_ms": 0.0, "initialization_time_ms": 0.0, "marking_time_ms": 0.0,
     "computation_time_ms": 0.0},
]


@pytest.mark.parametrize("k", range(len(RESULTS)))
def test_glog_line_matches_main_cu_format(pg, k):
    from pagerank_gb300.report import glog_line
    r = RESULTS[k]
    got = glog_line(r, "pagerankDynamicFrontierCuda", 3.14159e-11, batch_index=k * 7, threads=152,
                    deletions_fraction=0.0, insertions_fraction=1e-4)
    want = reference_format(0.0, 1e-4, k * 7, 152, r, 3.14159e-11, "pagerankDynamicFrontierCuda")
    assert got == want


def test_parse_log_and_csv(pg, tmp_path):
    from pagerank_gb300 import report
    lines = ["2024-05-01 10:00:00 OMP_NUM_THREADS=64",
             "2024-05-01 10:00:00 Loading graph /data/sx-mathoverflow.txt ...",
             "2024-05-01 10:00:01 order: 24818 size: 187986 [directed] {} (90%)"]
    for b in range(2):
        lines.append(f"2024-05-01 10:00:02 order: 24818 size: {215000 + b} [directed] {{}} (insertions=50)")
        for k, tech in enumerate(("pagerankStaticCuda", "pagerankPruneDynamicFrontierCuda")):
            lines.append(report.glog_line(RESULTS[k], tech, 1e-9 * (b + 1), b, 64, 0.0, 1e-3))
    lines.append("{-0.000e+00/+1.000e-03 batchf, 064 threads} -> {0000012.5ms, 010 iter, 1.00e-10 err} "
                 "pagerankStaticOmp")   # the older line that process.js's pattern was written for
    rows = report.parse_log("\n".join(lines) + "\n")
    assert len(rows) == 5
    assert rows[0]["graph"] == "sx-mathoverflow" and rows[0]["omp_num_threads"] == 64.0
    assert rows[0]["size"] == 215000 and rows[2]["size"] == 215001
    assert rows[1]["technique"] == "pagerankPruneDynamicFrontierCuda"
    assert rows[1]["iterations"] == 3 and rows[1]["marking_time"] == 7.5 and rows[3]["batch_index"] == 1
    assert rows[3]["error"] == pytest.approx(2e-9) and rows[3]["insertions_fraction"] == pytest.approx(1e-3)
    assert rows[4]["technique"] == "pagerankStaticOmp" and rows[4]["time"] == 12.5
    out = tmp_path / "all.csv"
    report.write_csv(str(out), rows)
    got = list(csv.DictReader(open(out)))
    assert len(got) == 5 and got[1]["technique"] == "pagerankPruneDynamicFrontierCuda"
    report.write_csv_dir(str(tmp_path / "bygraph"), rows)
    assert (tmp_path / "bygraph" / "sx-mathoverflow.csv").exists()
    log = tmp_path / "log.txt"
    log.write_text("\n".join(lines) + "\n")
    report.main(["json", str(log), str(tmp_path / "r.json")])
    assert (tmp_path / "r.json").read_text().count("technique") == 5
