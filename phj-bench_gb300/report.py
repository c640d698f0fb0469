"""CSV report in the reference's column order, plus GPU columns.

The first 27 columns are the reference's (src/Report.cpp:364-483: scheme,
rep, threads, sizes, payload schemas, partitions, distribution, match rate,
the phase timings as wall ms and ns per row, e2e, peak memory, the BEP
counters), with the same blanks per scheme: CHJ leaves the shuffle,
eviction and BEP columns empty, PHJ-PURE the eviction and BEP columns.  The
header is written when the file is new and rows are appended, as the
reference does.  The GPU columns that follow are empty where they do not
apply: device, tuples per second, the dominant kernel and its roofline
fraction, achieved DRAM GB/s of the join, and serving latency percentiles.
"""
from __future__ import annotations

import os
from typing import Iterable, List, Optional, Sequence

REFERENCE_COLUMNS = [
    "scheme", "rep", "threads", "build_rows", "probe_rows", "build_payload_schema", "probe_payload_schema", "partitions",
    "distribution", "match_rate",
    "build_wall_ms", "build_ns_per_row", "probe_wall_ms", "probe_ns_per_row",
    "build_shuffle_wall_ms", "build_shuffle_ns_per_row", "probe_shuffle_wall_ms", "probe_shuffle_ns_per_row",
    "eviction_overhead_wall_ms", "eviction_overhead_ns_per_row",
    "e2e_wall_ms", "peak_mem_mib",
    "bep_budget_mib", "bep_evictions", "bep_refinements", "bep_peak_mib", "bep_build_skip_retries",
]
GPU_COLUMNS = ["gpu_device", "gpu_tuples_per_s", "gpu_dominant_kernel", "roofline_frac", "dram_gbps", "p50_ms", "p99_ms", "p999_ms"]
COLUMNS = REFERENCE_COLUMNS + GPU_COLUMNS

TYPE_NAMES = {0: "u8", 1: "u16", 2: "u32", 3: "u64", 4: "u128"}
SCHEME_NAMES = {"chj": "CHJ", "phj-pure": "PHJ-PURE", "phj": "PHJ"}
MIB = 1024.0 * 1024.0


def schema_string(types: Sequence[int]) -> str:
    """schemaToString (src/CLI.cpp:361-373): comma-separated names, '<none>'."""
    return ",".join(TYPE_NAMES[t] for t in types) if types else "<none>"


def _num(v) -> str:
    return "" if v is None else f"{float(v):.6f}"


def _int(v) -> str:
    return "" if v is None else str(int(v))


def result_row(scheme: str, rep: int, result, *, threads: int, build_rows: int, probe_rows: int, build_types: Sequence[int],
               probe_types: Sequence[int], partitions: int, distribution: str = "uniform", match_rate: float = 1.0,
               gpu_device: str = "", tuples_per_s: Optional[float] = None, dominant_kernel: str = "",
               roofline_frac: Optional[float] = None, dram_gbps: Optional[float] = None,
               latency_ms: Optional[Sequence[float]] = None) -> List[str]:
    """One CSV row from a scheme result (the ctypes result struct of the C
    ABI: ChjResultC, PhjResultC or BepResultC)."""
    phase = lambda name: getattr(result, name, None)  # noqa: E731
    row = [SCHEME_NAMES.get(scheme, scheme), str(rep), str(threads), str(build_rows), str(probe_rows),
           f'"{schema_string(build_types)}"', f'"{schema_string(probe_types)}"', str(partitions), distribution, f"{match_rate:.1f}"]
    b, p = phase("build"), phase("probe")
    row += [_num(b.wall_ms), _num(b.ns_per_row), _num(p.wall_ms), _num(p.ns_per_row)]
    if scheme == "chj":
        row += [""] * 6
    else:
        bs, ps = phase("build_shuffle"), phase("probe_shuffle")
        row += [_num(bs.wall_ms), _num(bs.ns_per_row), _num(ps.wall_ms), _num(ps.ns_per_row)]
        if scheme == "phj":
            ev = phase("eviction_overhead")
            row += [_num(ev.wall_ms), _num(ev.ns_per_row)]
        else:
            row += ["", ""]
    row += [_num(result.e2e_wall_ms), _num(result.peak_mem_bytes / MIB)]
    if scheme == "phj":
        row += [_int(result.bep_budget_mib), _int(result.bep_evictions), _int(result.bep_refinements),
                _num(result.bep_peak_bytes / MIB), _int(result.bep_build_skip_retries)]
    else:
        row += [""] * 5
    lat = list(latency_ms) if latency_ms else [None, None, None]
    row += [gpu_device, _num(tuples_per_s), dominant_kernel, _num(roofline_frac), _num(dram_gbps), _num(lat[0]), _num(lat[1]),
            _num(lat[2])]
    return row


def write_csv(path: str, rows: Iterable[Sequence[str]]) -> None:
    """Appends rows; writes the header first when the file is new."""
    need_header = not os.path.exists(path)
    with open(path, "a") as f:
        if need_header:
            f.write(",".join(COLUMNS) + "\n")
        for r in rows:
            if len(r) != len(COLUMNS):
                raise ValueError(f"row has {len(r)} columns, the report {len(COLUMNS)}")
            f.write(",".join(r) + "\n")
