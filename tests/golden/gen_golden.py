"""Writes tests/golden/golden.json from the reference itself.

Runs the reference's referenceOutput and its three schemes (runCHJ, runPHJ,
runPhjBep), compiled from its own sources into oracle/_ref/libphjref.so by
oracle/Makefile, on the seeded cases of cases.py, and records per case the
output row count, the sha256 of the sorted serialised rows (compareOutputs'
multiset, src/Reference.cpp:113-133) and the oracle fingerprint of those
rows.  Also records known answers: intHash64 values, the reference DataGen's
first keys, and radixShuffle's per-partition row counts.

    python tests/golden/gen_golden.py      (needs the reference sources)
"""
import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "phj-bench_gb300"), os.path.join(ROOT, "oracle"), HERE]

import numpy as np  # noqa: E402

import cases  # noqa: E402
import oracle as O  # noqa: E402


def main():
    if not O.ref_available():
        raise SystemExit("oracle/_ref/libphjref.so is missing: run `make -C oracle` where the reference sources exist")
    R = O.ref()
    out = {"cases": {}, "kat": {}}
    for name in cases.NAMES:
        b, p = cases.make(name)
        ref_rows = O.ref_reference_rows(b, p)
        dig = hashlib.sha256(O.sort_rows(ref_rows.copy()).tobytes()).hexdigest()
        for scheme in (0, 1, 2):
            rows, _ = O.ref_run_scheme(scheme, b, p, cases.BITS[name], threads=3, budget_mib=1)
            assert O.compare_outputs(ref_rows, rows) == "", (name, scheme)
        out["cases"][name] = {
            "rows": int(len(ref_rows)),
            "sha256_sorted_rows": dig,
            "fingerprint": [str(v) for v in O.rows_fingerprint(ref_rows, b.types, p.types)],
            "bits": cases.BITS[name],
        }
        print(name, len(ref_rows), dig[:16])
    xs = [0, 1, 42, 0xFFFFFFFFFFFFFFFF, 0x123456789ABCDEF0]
    out["kat"]["int_hash64"] = {str(x): hex(R.ref_int_hash64(x)) for x in xs}
    bk = np.zeros(16, dtype=np.uint64)
    pk = np.zeros(16, dtype=np.uint64)
    R.ref_generate_keys(16, 16, 42, 10000, bk.ctypes.data, pk.ctypes.data)
    out["kat"]["datagen_seed42"] = {"build": [hex(int(v)) for v in bk[:4]], "probe": [hex(int(v)) for v in pk[:4]]}
    b, _ = cases.make("c2_mini")
    for bits in ([4], [3, 3], [2, 2, 2]):
        parts = 1 << sum(bits)
        prow = np.zeros(parts, dtype=np.uint64)
        keys = np.zeros(len(b.keys), dtype=np.uint64)
        arr = (O.C.c_uint8 * len(bits))(*bits)
        n = R.ref_radix_shuffle_keys(O.C.byref(O.ostream(b)), 10000, arr, len(bits), 3, prow.ctypes.data, keys.ctypes.data)
        assert n == len(b.keys)
        out["kat"]["radix_partition_rows_c2_mini_" + "_".join(map(str, bits))] = [int(v) for v in prow]
        # the keys of each partition as a multiset: sorted inside each
        # partition, partitions in order (the order inside a partition
        # depends on the reference's threads)
        offs = np.concatenate([[0], np.cumsum(prow)]).astype(np.int64)
        per_part = np.concatenate([np.sort(keys[offs[i]:offs[i + 1]]) for i in range(parts)])
        out["kat"]["radix_partition_keys_sha256_c2_mini_" + "_".join(map(str, bits))] = hashlib.sha256(per_part.tobytes()).hexdigest()
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print("wrote", os.path.join(HERE, "golden.json"))


if __name__ == "__main__":
    main()
