"""The no-allocation join (phj_run_chj_noalloc) against the allocating CHJ
entry point (phj_run_chj) and against the oracle (the CPU restatement of
the reference's referenceOutput): the same rows, as sorted multisets, on
two calls in a row (the second call must start from cleared scratch)."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
import phj_datagen as G
import phj_gpu as P
from golden import cases

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


class DeviceColumns:
    """Caller-owned output columns on cuda:0 (allocated here, by the caller)."""

    def __init__(self, left_types, right_types, cap):
        self.left_types, self.right_types, self.cap = list(left_types), list(right_types), cap
        n = max(cap, 1)
        self.keys = torch.empty(n * 8, dtype=torch.uint8, device="cuda:0")
        self.left = [torch.empty(n * P.TYPE_WIDTH[t], dtype=torch.uint8, device="cuda:0") for t in self.left_types]
        self.right = [torch.empty(n * P.TYPE_WIDTH[t], dtype=torch.uint8, device="cuda:0") for t in self.right_types]

    def pointers(self):
        return self.keys.data_ptr(), [c.data_ptr() for c in self.left], [c.data_ptr() for c in self.right]

    def to_output(self, rows):
        def col(buf, t):
            a = buf[: rows * P.TYPE_WIDTH[t]].cpu().numpy()
            return a.view(np.uint64).reshape(rows, 2) if t == P.U128 else a.view(P.TYPE_DTYPE[t])
        keys = self.keys[: rows * 8].cpu().numpy().view(np.uint64)
        return P.JoinOutput(self.left_types, self.right_types, keys,
                            [col(c, t) for c, t in zip(self.left, self.left_types)],
                            [col(c, t) for c, t in zip(self.right, self.right_types)])


def allocating_rows(ctx, tb, tp):
    out, _ = ctx.run_chj(tb, tp)
    rows = O.serialize_output(out.download())
    out.free()
    return rows


def noalloc_rows(ctx, tb, tp, b, p, cap):
    cols = DeviceColumns(b.types, p.types, cap)
    keys, left, right = cols.pointers()
    n = ctx.run_chj_noalloc(tb, tp, cap, keys, left, right)
    torch.cuda.synchronize()
    return O.serialize_output(cols.to_output(n)), n


@pytest.mark.parametrize("name", ["c2_mini", "c3_mini", "edge", "no_match", "empty_probe", "empty_build"])
def test_no_alloc_matches_allocating_entry_point_twice(ctx, name):
    b, p = cases.make(name)
    tb, tp = ctx.upload(b), ctx.upload(p)
    try:
        expected = allocating_rows(ctx, tb, tp)
        assert O.compare_outputs(O.join_rows(b, p), expected) == ""
        for _ in range(2):
            got, n = noalloc_rows(ctx, tb, tp, b, p, len(expected) + 17)
            assert n == len(expected)
            assert O.compare_outputs(expected, got) == ""
    finally:
        tb.free(), tp.free()


def test_no_alloc_largest_build_side(ctx):
    # 65,536 build rows (the scratch's maximum), multi-match keys
    bk, used = G.gen_multi_match_keys(65536, 201, 21)
    pk = G.gen_keys(4, 200000, 202, 21, domain=used, match_permille=700)
    b = P.BlockStream([P.U8, P.U128], bk, G.payload_columns(203, [P.U8, P.U128], 65536))
    p = P.BlockStream([P.U32], pk, G.payload_columns(204, [P.U32], 200000))
    tb, tp = ctx.upload(b), ctx.upload(p)
    try:
        expected = allocating_rows(ctx, tb, tp)
        assert O.compare_outputs(O.join_rows(b, p), expected) == ""
        for _ in range(2):
            got, n = noalloc_rows(ctx, tb, tp, b, p, len(expected))
            assert n == len(expected)
            assert O.compare_outputs(expected, got) == ""
    finally:
        tb.free(), tp.free()


def test_no_alloc_rejects_oversized_build_and_reports_short_capacity(ctx):
    b = P.BlockStream([P.U32], G.gen_keys(0, 65537, 211, 22), G.payload_columns(212, [P.U32], 65537))
    p = P.BlockStream([P.U32], G.gen_keys(4, 1000, 213, 22, domain=65537, match_permille=900), G.payload_columns(214, [P.U32], 1000))
    tb, tp = ctx.upload(b), ctx.upload(p)
    try:
        with pytest.raises(P.PhjError) as e:
            ctx.run_chj_noalloc(tb, tp, 0, 0, [], [])
        assert e.value.status == P.ERR_INVALID_ARGUMENT and "65536" in str(e.value)
    finally:
        tb.free(), tp.free()
    b, p = cases.make("c2_mini")
    tb, tp = ctx.upload(b), ctx.upload(p)
    try:
        expected = allocating_rows(ctx, tb, tp)
        cols = DeviceColumns(b.types, p.types, 100)
        keys, left, right = cols.pointers()
        with pytest.raises(P.PhjError) as e:
            ctx.run_chj_noalloc(tb, tp, 100, keys, left, right)
        assert e.value.status == 7 and e.value.rows == len(expected)
        got, n = noalloc_rows(ctx, tb, tp, b, p, len(expected))
        assert O.compare_outputs(expected, got) == ""
    finally:
        tb.free(), tp.free()


def test_no_alloc_counts_only_with_null_columns(ctx):
    # capacity 0 and no column arrays at all: the call counts the rows,
    # writes nothing and reports PHJ_ERR_CAPACITY with the count set
    b, p = cases.make("c2_mini")
    tb, tp = ctx.upload(b), ctx.upload(p)
    try:
        rows = C.c_uint64(0)
        st = ctx.lib.phj_run_chj_noalloc(ctx.ptr, tb.handle, tp.handle, 0, None, None, None, C.byref(rows))
        assert st == P.ERR_CAPACITY
        assert rows.value == len(O.join_rows(b, p)) > 0
        got, n = noalloc_rows(ctx, tb, tp, b, p, rows.value)
        assert O.compare_outputs(O.join_rows(b, p), got) == ""
    finally:
        tb.free(), tp.free()
