"""Writes tests/golden/fullsize.json: the oracle's answer for each benchmark
workload at its full size.

For every workload of bench.py (the 1M x 8M, 16M x 256M, 32M x 128M
multi-match and 64M x 512M Zipf joins) the inputs are made by the host form
of the library's seeded generator (phj_datagen: the same integers the device
generator phj_table_generate produces, which tests/test_device_gpu.py checks),
and the oracle (oracle/oracle.c, the CPU restatement of the reference's
referenceOutput, src/Reference.cpp:48-76) computes the join's
order-independent fingerprint: output row count and two sums of per-row
hashes over the serialised rows.  For the 1M x 8M join, whose 8M output rows
fit the sorted-multiset compare, it also records the sha256 of the sorted
serialised rows (compareOutputs' multiset, src/Reference.cpp:113-133).

    python tests/golden/gen_fullsize.py [workload ...]     (minutes; ~20 GB RAM)
"""
import hashlib
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "phj-bench_gb300"), os.path.join(ROOT, "oracle")]

import bench  # noqa: E402  (workload specifications and the host generator calls)
import oracle as O  # noqa: E402

PATH = os.path.join(HERE, "fullsize.json")
SORTED_DIGEST_MAX_ROWS = 16 << 20


def main(names):
    out = json.load(open(PATH)) if os.path.exists(PATH) else {}
    for wl in names:
        t = time.time()
        b, p = bench.host_tables(wl)
        fp = O.join_fingerprint(b, p)
        e = {"build_rows": len(b.keys), "probe_rows": len(p.keys), "rows": int(fp[0]),
             "fingerprint": [str(v) for v in fp], "workload": bench.WORKLOADS[wl][0]}
        if fp[0] <= SORTED_DIGEST_MAX_ROWS:
            rows = O.sort_rows(O.join_rows(b, p))
            e["sha256_sorted_rows"] = hashlib.sha256(rows.tobytes()).hexdigest()
        out[wl] = e
        print(wl, e["rows"], f"{time.time() - t:.1f} s", flush=True)
        del b, p
        with open(PATH, "w") as f:
            json.dump(out, f, indent=1, sort_keys=True)
            f.write("\n")


if __name__ == "__main__":
    main(sys.argv[1:] or ["c1", "c2", "c3", "c4"])
