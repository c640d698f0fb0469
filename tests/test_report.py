"""The CSV report (phj-bench_gb300/report.py): the reference's 27 columns in
its order with its per-scheme blanks, then the GPU columns."""
import csv
from types import SimpleNamespace as NS

import report as R


def phase(ms, rows):
    return NS(wall_ms=ms, ns_per_row=ms * 1e6 / rows)


def result(scheme):
    r = NS(build=phase(1.0, 100), probe=phase(2.0, 800), build_shuffle=phase(0.5, 100), probe_shuffle=phase(0.7, 800),
           eviction_overhead=phase(0.1, 800), e2e_wall_ms=4.5, peak_mem_bytes=3 * 1024 * 1024)
    if scheme == "phj":
        r.bep_budget_mib, r.bep_evictions, r.bep_refinements = 32, 100, 7
        r.bep_peak_bytes, r.bep_build_skip_retries = 2 * 1024 * 1024, 0
    return r


def test_header_and_blanks(tmp_path):
    path = str(tmp_path / "r.csv")
    rows = [R.result_row(s, 0, result(s), threads=16, build_rows=100, probe_rows=800, build_types=[3, 2], probe_types=[],
                         partitions=256, gpu_device="GB300", tuples_per_s=1e9) for s in ("chj", "phj-pure", "phj")]
    R.write_csv(path, rows)
    R.write_csv(path, rows[:1])  # appended without a second header
    got = list(csv.reader(open(path)))
    assert got[0][:27] == R.REFERENCE_COLUMNS and len(got[0]) == 35
    assert len(got) == 5
    chj, pure, bep = (dict(zip(got[0], r)) for r in got[1:4])
    assert chj["scheme"] == "CHJ" and chj["build_shuffle_wall_ms"] == "" and chj["bep_budget_mib"] == ""
    assert pure["scheme"] == "PHJ-PURE" and pure["probe_shuffle_wall_ms"] == "0.700000" and pure["eviction_overhead_wall_ms"] == ""
    assert bep["scheme"] == "PHJ" and bep["bep_evictions"] == "100" and bep["bep_peak_mib"] == "2.000000"
    assert chj["build_payload_schema"] == "u64,u32" and chj["probe_payload_schema"] == "<none>"
    assert chj["peak_mem_mib"] == "3.000000" and chj["gpu_tuples_per_s"] == "1000000000.000000" and chj["p99_ms"] == ""
