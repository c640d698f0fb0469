"""Bit-exact parity of the device schemes with the oracle (the restated
reference check, src/Reference.cpp:48-133) through the C ABI."""
import json
import os

import numpy as np
import pytest

import oracle as O
import phj_datagen as G
import phj_gpu as P
from golden import cases

pytestmark = pytest.mark.gpu
GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))


def run(ctx, scheme, b, p, bits=None, materialize=-1):
    ctx.set_int("probe_materialize", materialize)
    tb, tp = ctx.upload(b), ctx.upload(p)
    try:
        if scheme == "chj":
            out, res = ctx.run_chj(tb, tp)
        else:
            out, res = ctx.run_phj_pure(tb, tp, bits)
        jo = out.download()
        fp = out.fingerprint()
        out.free()
        return jo, fp, res
    finally:
        tb.free(), tp.free()
        ctx.set_int("probe_materialize", -1)


def check(b, p, jo, fp=None):
    expected = O.join_rows(b, p)
    assert jo.totalRows() == len(expected)
    err = O.compare_outputs(expected, O.serialize_output(jo))
    assert err == "", err
    if fp is not None:
        assert fp == O.rows_fingerprint(expected, b.types, p.types)


@pytest.mark.parametrize("name", cases.NAMES)
@pytest.mark.parametrize("scheme", ["chj", "phj-pure"])
def test_golden_cases(ctx, name, scheme):
    b, p = cases.make(name)
    jo, fp, _ = run(ctx, scheme, b, p, cases.BITS[name])
    rows = O.serialize_output(jo)
    g = GOLDEN["cases"][name]
    assert len(rows) == g["rows"]
    assert O.digest(rows) == g["sha256_sorted_rows"]
    assert [str(v) for v in fp] == g["fingerprint"]


@pytest.mark.parametrize("bits", [[1], [8], [4, 4], [3, 3, 3], [12], [16], [8, 8], [11, 2], [6, 6, 6], [13, 11]])
@pytest.mark.parametrize("materialize", [0, 1])
def test_phj_pure_radix_configs(ctx, bits, materialize):
    b, p = cases.make("c2_mini")
    jo, fp, _ = run(ctx, "phj-pure", b, p, bits, materialize)
    check(b, p, jo, fp)


@pytest.mark.parametrize("materialize", [0, 1])
def test_multi_match_and_edges(ctx, materialize):
    for name in ("c3_mini", "edge"):
        b, p = cases.make(name)
        for bits in ([2], [5, 5]):
            jo, fp, _ = run(ctx, "phj-pure", b, p, bits, materialize)
            check(b, p, jo, fp)
        jo, fp, _ = run(ctx, "chj", b, p)
        check(b, p, jo, fp)


def test_no_payload_columns(ctx):
    bk = G.gen_keys(0, 5000, 1, 2)
    pk = G.gen_keys(4, 20000, 3, 2, domain=5000, match_permille=800)
    b, p = P.BlockStream([], bk, []), P.BlockStream([], pk, [])
    for scheme in ("chj", "phj-pure"):
        jo, fp, _ = run(ctx, scheme, b, p, [6])
        check(b, p, jo, fp)


def test_irregular_blocks_for_chj(ctx):
    # CHJ's RowRefCell is (input block, row): blocks of uneven size.
    bk = G.gen_keys(0, 3000, 1, 4)
    sizes = np.array([7, 1000, 3, 990, 1000], dtype=np.uint32)
    b = P.BlockStream([P.U64, P.U16], bk, G.payload_columns(5, [P.U64, P.U16], 3000), block_rows=sizes)
    p = P.BlockStream([P.U32], G.gen_keys(4, 9000, 6, 4, domain=3000, match_permille=950), G.payload_columns(7, [P.U32], 9000))
    jo, fp, _ = run(ctx, "chj", b, p)
    check(b, p, jo, fp)


def test_heavy_duplicates_single_key(ctx):
    # every build row has the same key: one chain of 2000 rows
    bk = np.full(2000, 12345, dtype=np.uint64)
    pk = np.array([12345, 1, 12345, 7], dtype=np.uint64)
    b = P.BlockStream([P.U32], bk, G.payload_columns(8, [P.U32], 2000))
    p = P.BlockStream([P.U8], pk, G.payload_columns(9, [P.U8], 4))
    for scheme, bits in (("chj", None), ("phj-pure", [4]), ("phj-pure", [2, 2])):
        jo, fp, _ = run(ctx, scheme, b, p, bits)
        check(b, p, jo, fp)


def test_large_leaf_uses_global_table(ctx):
    # 1 partition bit over 40K unique keys: leaves of ~20K rows exceed the
    # shared-memory table and are built in global memory.
    b, p = cases.make("c2_mini")
    bk = G.gen_keys(0, 40000, 1, 5)
    b = P.BlockStream([P.U64], bk, G.payload_columns(2, [P.U64], 40000))
    p = P.BlockStream([P.U32], G.gen_keys(4, 80000, 3, 5, domain=40000, match_permille=600), G.payload_columns(4, [P.U32], 80000))
    jo, fp, _ = run(ctx, "phj-pure", b, p, [1])
    check(b, p, jo, fp)


def test_invalid_arguments_raise(ctx):
    b, p = cases.make("c2_mini")
    tb, tp = ctx.upload(b), ctx.upload(p)
    with pytest.raises(P.PhjError):
        ctx.run_phj_pure(tb, tp, [])
    with pytest.raises(P.PhjError):
        ctx.run_phj_pure(tb, tp, [17])
    with pytest.raises(P.PhjError):
        ctx.run_phj_pure(tb, tp, [16, 16, 1])  # > 32 total bits, the reference rejects it too
    tb.free(), tp.free()


def test_reference_shaped_entry_points(ctx):
    b, p = cases.make("c2_mini")
    r = P.runPHJ(b, p, [4, 4], ctx=ctx)
    assert r.build_shuffle.wall_ms >= 0 and r.e2e_wall_ms > 0 and r.peak_mem_bytes > 0
    check(b, p, r.output)
    r = P.runCHJ(b, p, ctx=ctx)
    assert r.build.wall_ms >= 0 and r.probe.wall_ms >= 0
    check(b, p, r.output)
