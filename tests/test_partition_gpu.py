"""The device radix shuffle (phj_radix_shuffle) against the reference's
radixShuffle (src/RadixPartition.cpp:546-586): per-partition row counts and
per-partition key multisets equal to the golden values the reference itself
produced (tests/golden/gen_golden.py), and every row -- key and payloads --
in the partition the oracle computes from its hash, at 1, 2 and 3 passes
and at the benchmark's 2 x 8 bits."""
import hashlib

import numpy as np
import pytest

import oracle as O
import phj_datagen as G
import phj_gpu as P
from golden import cases
from test_oracle import GOLDEN

pytestmark = pytest.mark.gpu


def rows_by_partition(s, leaf):
    """Rows (key, payload bytes) ordered by (partition, row bytes)."""
    parts = [s.keys.view(np.uint8).reshape(-1, 8)]
    for c in s.payloads:
        c = np.ascontiguousarray(c)
        parts.append(c.view(np.uint8).reshape(len(s.keys), c.itemsize * (c.shape[1] if c.ndim == 2 else 1)))
    rows = np.concatenate(parts, axis=1)
    order = np.lexsort(tuple(rows[:, j] for j in reversed(range(rows.shape[1]))) + (leaf,))
    return rows[order], leaf[order]


@pytest.mark.parametrize("bits", [[4], [3, 3], [2, 2, 2]])
def test_radix_shuffle_matches_the_reference(ctx, bits):
    b, _ = cases.make("c2_mini")
    t = ctx.upload(b)
    try:
        part, counts = ctx.radix_shuffle(t, bits)
        try:
            got = part.download()
        finally:
            part.free()
    finally:
        t.free()
    tag = "_".join(map(str, bits))
    assert counts.tolist() == GOLDEN["kat"]["radix_partition_rows_c2_mini_" + tag]
    offs = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    per_part = np.concatenate([np.sort(got.keys[offs[i]:offs[i + 1]]) for i in range(len(counts))])
    assert hashlib.sha256(per_part.tobytes()).hexdigest() == GOLDEN["kat"]["radix_partition_keys_sha256_c2_mini_" + tag]


@pytest.mark.parametrize("types,rows,bits", [
    ([P.U64, P.U32], 1 << 20, [8, 8]),                       # the benchmark's build side shape, 65,536 partitions
    ([P.U8, P.U16, P.U128], 300_001, [6, 6, 6]),             # 3 passes, every odd payload width, a ragged tail
    ([], 5_000, [11]),                                       # keys only, more partitions than rows
    ([P.U32], 0, [4]),                                       # empty input
])
def test_radix_shuffle_rows_land_in_their_partition(ctx, types, rows, bits):
    keys = G.gen_keys(0, rows, 41, 42)
    if rows > 10:
        keys[:3] = [0, 0xFFFFFFFFFFFFFFFF, 0]  # key 0 twice, UINT64_MAX
    s = P.BlockStream(types, keys, G.payload_columns(43, types, rows))
    t = ctx.upload(s)
    try:
        part, counts = ctx.radix_shuffle(t, bits)
        try:
            got = part.download()
        finally:
            part.free()
    finally:
        t.free()
    total = sum(bits)
    leaf_in = O.leaf_ids(s.keys, total)
    assert counts.tolist() == np.bincount(leaf_in, minlength=1 << total).tolist()
    leaf_out = np.repeat(np.arange(1 << total, dtype=np.uint32), counts.astype(np.int64))
    assert np.array_equal(O.leaf_ids(got.keys, total), leaf_out)
    want_rows, _ = rows_by_partition(s, leaf_in)
    got_rows, _ = rows_by_partition(got, leaf_out)
    assert np.array_equal(want_rows, got_rows)
