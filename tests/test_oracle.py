"""The oracle (oracle/oracle.c, a CPU restatement of the reference's
Reference.cpp check) pinned against the reference's own outputs.

tests/golden/golden.json was produced by tests/golden/gen_golden.py from the
reference compiled from its sources; these tests need no GPU."""
import json
import os

import numpy as np
import pytest

import oracle as O
from golden import cases

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))


def test_int_hash64_known_answers():
    # src/Hash.h:18-25, values from the reference build
    for x, v in GOLDEN["kat"]["int_hash64"].items():
        assert O.int_hash64(int(x)) == int(v, 16)
    assert O.int_hash64(0) == 0x28BFAA0AFBB6AA0B
    assert O.int_hash64(0xFFFFFFFFFFFFFFFF) == 0x36137209C4D8F428


@pytest.mark.parametrize("name", cases.NAMES)
def test_oracle_reproduces_reference_output(name):
    b, p = cases.make(name)
    g = GOLDEN["cases"][name]
    rows = O.join_rows(b, p)
    assert len(rows) == g["rows"] == O.join_count(b, p)
    assert O.digest(rows) == g["sha256_sorted_rows"]
    assert [str(v) for v in O.rows_fingerprint(rows, b.types, p.types)] == g["fingerprint"]
    assert [str(v) for v in O.join_fingerprint(b, p, threads=3)] == g["fingerprint"]


@pytest.mark.parametrize("bits", [[4], [3, 3], [2, 2, 2]])
def test_leaf_ids_match_reference_radix_shuffle(bits):
    b, _ = cases.make("c2_mini")
    want = GOLDEN["kat"]["radix_partition_rows_c2_mini_" + "_".join(map(str, bits))]
    got = np.bincount(O.leaf_ids(b.keys, sum(bits)), minlength=1 << sum(bits))
    assert got.tolist() == want


def partition_key_digest(keys, leaf, parts):
    """sha256 of the keys grouped by partition, sorted inside each one."""
    import hashlib
    order = np.lexsort((keys, leaf))
    assert np.all(np.diff(leaf[order].astype(np.int64)) >= 0) and leaf.max(initial=0) < parts
    return hashlib.sha256(np.ascontiguousarray(keys[order]).tobytes()).hexdigest()


@pytest.mark.parametrize("bits", [[4], [3, 3], [2, 2, 2]])
def test_leaf_ids_place_every_key_where_radix_shuffle_does(bits):
    b, _ = cases.make("c2_mini")
    want = GOLDEN["kat"]["radix_partition_keys_sha256_c2_mini_" + "_".join(map(str, bits))]
    leaf = O.leaf_ids(b.keys, sum(bits))
    assert partition_key_digest(b.keys, leaf, 1 << sum(bits)) == want


def test_compare_detects_a_planted_mistake():
    b, p = cases.make("c2_mini")
    rows = O.join_rows(b, p)
    bad = rows.copy()
    bad[len(bad) // 2, -1] ^= 1  # one payload bit of one row
    assert O.compare_outputs(rows, rows.copy()) == ""
    assert "mismatch" in O.compare_outputs(rows, bad)
    assert O.rows_fingerprint(rows, b.types, p.types) != O.rows_fingerprint(bad, b.types, p.types)
    assert "row count" in O.compare_outputs(rows, rows[:-1])


def test_columns_fingerprint_equals_rows_fingerprint():
    b, p = cases.make("edge")
    rows = O.join_rows(b, p)
    # split the serialised rows back into columns
    import phj_gpu as P
    w = [8] + [P.TYPE_WIDTH[t] for t in b.types] + [P.TYPE_WIDTH[t] for t in p.types]
    offs = np.cumsum([0] + w)
    def col(i, t):
        raw = np.ascontiguousarray(rows[:, offs[i]:offs[i + 1]])
        return raw.view(np.uint64).reshape(-1, 2) if t == P.U128 else raw.view(P.TYPE_DTYPE[t]).reshape(-1)
    keys = np.ascontiguousarray(rows[:, :8]).view(np.uint64).reshape(-1)
    left = [col(1 + i, t) for i, t in enumerate(b.types)]
    right = [col(1 + len(b.types) + i, t) for i, t in enumerate(p.types)]
    out = P.JoinOutput(b.types, p.types, keys, left, right)
    assert O.columns_fingerprint(out) == O.rows_fingerprint(rows, b.types, p.types)
    assert np.array_equal(O.serialize_output(out), rows)


@pytest.mark.skipif(not O.ref_available(), reason="reference sources not compiled here")
@pytest.mark.parametrize("scheme,bits", [(0, [8]), (1, [5, 3]), (2, [3, 3])])
def test_reference_schemes_agree_with_oracle(scheme, bits):
    b, p = cases.make("c3_mini")
    rows, _ = O.ref_run_scheme(scheme, b, p, bits, threads=4, budget_mib=1)
    assert O.compare_outputs(O.join_rows(b, p), rows) == ""
