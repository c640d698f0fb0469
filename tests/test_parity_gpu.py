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


def run(ctx, scheme, b, p, bits=None, materialize=-1, budget_mib=1):
    ctx.set_int("probe_materialize", materialize)
    tb, tp = ctx.upload(b), ctx.upload(p)
    try:
        if scheme == "chj":
            out, res = ctx.run_chj(tb, tp)
        elif scheme == "phj":
            out, res = ctx.run_phj_bep(tb, tp, bits, budget_mib)
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
@pytest.mark.parametrize("scheme", ["chj", "phj-pure", "phj"])
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
    for scheme in ("chj", "phj-pure", "phj"):
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
    for scheme, bits in (("chj", None), ("phj-pure", [4]), ("phj-pure", [2, 2]), ("phj", [4]), ("phj", [2, 2])):
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
    jo, fp, _ = run(ctx, "phj", b, p, [1])
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


# ---- PHJ (BEP) -------------------------------------------------------------
def bep_inputs(n_build, n_probe, seed, types_b=(P.U64,), types_p=(P.U32,), match=900):
    bk = G.gen_keys(0, n_build, seed, seed + 1)
    pk = G.gen_keys(4, n_probe, seed + 2, seed + 1, domain=n_build, match_permille=match)
    return (P.BlockStream(list(types_b), bk, G.payload_columns(seed + 3, list(types_b), n_build)),
            P.BlockStream(list(types_p), pk, G.payload_columns(seed + 4, list(types_p), n_probe)))


@pytest.mark.parametrize("bits", [[1], [4], [3, 3], [6, 6, 6], [12], [13, 2], [4, 4, 4, 4]])
def test_bep_radix_configs(ctx, bits):
    b, p = cases.make("c2_mini")
    jo, fp, res = run(ctx, "phj", b, p, bits)
    check(b, p, jo, fp)
    assert res.bep_budget_mib == 1


@pytest.mark.parametrize("budget", [1, 2, 64])
def test_bep_budget_batches_and_counters(ctx, budget):
    # The batch form ("bep_engine" 1): 600K probe rows of 12 bytes (7.2 MB);
    # a 1 MiB budget gives 8 batches.
    b, p = bep_inputs(50000, 600000, 101)
    bits = [3, 5]
    ctx.set_int("bep_engine", 1)
    try:
        jo, fp, res = run(ctx, "phj", b, p, bits, budget_mib=budget)
    finally:
        ctx.set_int("bep_engine", 0)
    check(b, p, jo, fp)
    row_bytes = 8 + 4
    batch_rows = min(600000, max(4096, ((budget << 20) // row_bytes) & ~255))
    batches = -(-600000 // batch_rows)
    assert res.bep_peak_bytes == batch_rows * row_bytes
    assert res.bep_peak_bytes <= max(budget << 20, 4096 * row_bytes)
    # every batch touches (nearly) every one of the 8 first-pass buckets and
    # 256 leaves; each touched leaf is one eviction per batch
    assert batches * 8 >= res.bep_refinements >= batches * 7
    assert batches * 256 >= res.bep_evictions >= batches * 200
    assert res.probe.wall_ms > 0 and res.e2e_wall_ms >= res.probe.wall_ms


def test_bep_multi_match_edges_and_wide_payloads(ctx):
    for name in ("c3_mini", "edge", "c4_mini", "no_match", "empty_build", "empty_probe"):
        b, p = cases.make(name)
        for bits in ([2], [5, 5], [3, 3, 3]):
            jo, fp, _ = run(ctx, "phj", b, p, bits)
            check(b, p, jo, fp)


def test_bep_small_batches_multi_match(ctx):
    # 16K build rows over ~4K keys, 300K probe rows with u128 payloads
    # (24 bytes a row): 4096-row batches at the smallest budget.
    bk, used = G.gen_multi_match_keys(16000, 131, 16)
    pk = G.gen_keys(4, 300000, 133, 16, domain=used, match_permille=500)
    b = P.BlockStream([P.U16, P.U128], bk, G.payload_columns(134, [P.U16, P.U128], 16000))
    p = P.BlockStream([P.U128], pk, G.payload_columns(135, [P.U128], 300000))
    ctx.set_int("bep_engine", 1)
    try:
        jo, fp, res = run(ctx, "phj", b, p, [2, 4], budget_mib=1)
    finally:
        ctx.set_int("bep_engine", 0)
    check(b, p, jo, fp)
    assert res.bep_peak_bytes == (((1 << 20) // 24) & ~255) * 24
    # the device budget engine on the same inputs
    jo, fp, res = run(ctx, "phj", b, p, [2, 4], budget_mib=1)
    check(b, p, jo, fp)
    assert res.bep_evictions > 64 and res.bep_refinements >= 4


@pytest.mark.parametrize("budget", [1, 2, 64])
def test_bep_device_budget_counters(ctx, budget):
    """The device budget engine (default): 600K probe rows of 12 bytes
    (7.2 MB) through per-group unrefined chains.  At 64 MiB the leaf high
    water (40 MiB) is never reached: every row is refined before any
    eviction, the peak is the whole probe side and each of the 256 leaves
    is evicted once, in the final drain.  At 1-2 MiB the high water is
    crossed mid-stream: leaves are evicted more than once and the peak stays
    near the budget."""
    b, p = bep_inputs(50000, 600000, 101)
    bits = [3, 5]
    jo, fp, res = run(ctx, "phj", b, p, bits, budget_mib=budget)
    check(b, p, jo, fp)
    row_bytes = 12
    groups = ctx.get_int("num_sms")
    assert res.bep_refinements >= 8
    if budget == 64:
        assert res.bep_peak_bytes == 600000 * row_bytes
        assert res.bep_evictions == 256
    else:
        assert res.bep_evictions > 256
        # the leaf high water (5/8 of the budget) plus one wave of refines,
        # each group's at most half its share plus a tile of 256 rows
        wave = groups * ((budget << 20) // groups // 2 + 256 * row_bytes)
        assert (budget << 20) * 5 // 8 <= res.bep_peak_bytes <= (budget << 20) * 5 // 8 + wave
    assert res.bep_build_skip_retries == 0
    assert res.probe.wall_ms > 0 and res.e2e_wall_ms >= res.probe.wall_ms


@pytest.mark.parametrize("bits", [[2, 4], [6, 6, 6], [8], [1, 12]])
def test_bep_engine_and_batches_agree(ctx, bits):
    """Both PHJ (BEP) forms give the oracle's rows, on unique keys with a
    tight budget (evictions mid-stream) and on repeated build keys (more
    output rows than probe rows: the engine runs again into an output of
    the exact size)."""
    for name in ("c3_mini", "c4_mini", "c2_mini"):
        b, p = cases.make(name)
        for engine in (0, 1):
            ctx.set_int("bep_engine", engine)
            try:
                jo, fp, _ = run(ctx, "phj", b, p, bits, budget_mib=1)
            finally:
                ctx.set_int("bep_engine", 0)
            check(b, p, jo, fp)


def test_bep_repeated_runs_identical(ctx):
    b, p = bep_inputs(30000, 200000, 141)
    fps = [run(ctx, "phj", b, p, [4, 4])[1] for _ in range(3)]
    assert fps[0] == fps[1] == fps[2]
    assert fps[0] == run(ctx, "phj-pure", b, p, [4, 4])[1]


def test_bep_stuck_leaf_times_out_and_context_recovers(ctx):
    # A leaf left BUILDING (a hook that writes the state before the probe):
    # the warps that need it give up after the wait limit, the run fails
    # with PHJ_ERR_DEVICE_TIMEOUT, and the context runs the next join.
    b, p = cases.make("c2_mini")
    ctx.set_int("wait_limit_ms", 100)
    ctx.set_int("test_stuck_leaf", 3)
    try:
        with pytest.raises(P.PhjError) as e:
            run(ctx, "phj", b, p, [4])
        assert e.value.status == P.ERR_DEVICE_TIMEOUT
    finally:
        ctx.set_int("test_stuck_leaf", -1)
        ctx.set_int("wait_limit_ms", 1000)
    jo, fp, _ = run(ctx, "phj", b, p, [4])
    check(b, p, jo, fp)


def test_bep_engine_barrier_wait_runs_out_and_context_recovers(ctx):
    """One CTA group of the budget engine holds back from the first wave's
    grid barrier (a host-set hook, no fault): the other groups' bounded
    wait runs out, the grid ends, the run fails with PHJ_ERR_DEVICE_TIMEOUT,
    and the context runs the next join bit-exactly."""
    b, p = cases.make("c2_mini")
    ctx.set_int("wait_limit_ms", 50)
    ctx.set_int("test_engine_stall_wave", 0)
    try:
        with pytest.raises(P.PhjError) as e:
            run(ctx, "phj", b, p, [4, 4])
        assert e.value.status == P.ERR_DEVICE_TIMEOUT
    finally:
        ctx.set_int("test_engine_stall_wave", -1)
        ctx.set_int("wait_limit_ms", 1000)
    jo, fp, _ = run(ctx, "phj", b, p, [4, 4])
    check(b, p, jo, fp)


def test_bep_invalid_budget_and_too_many_leaves(ctx):
    b, p = cases.make("c2_mini")
    tb, tp = ctx.upload(b), ctx.upload(p)
    with pytest.raises(P.PhjError):
        ctx.run_phj_bep(tb, tp, [4], 0)
    with pytest.raises(P.PhjError) as e:
        ctx.run_phj_bep(tb, tp, [11, 10], 1)
    assert e.value.status == 4  # PHJ_ERR_UNSUPPORTED
    tb.free(), tp.free()


def test_bep_reference_shaped_entry_point(ctx):
    b, p = cases.make("c2_mini")
    r = P.runPhjBep(b, p, [4, 4], threads=4, bep_budget_mib=1, ctx=ctx)
    check(b, p, r.output)
    assert r.counters["bep_budget_mib"] == 1 and r.counters["bep_evictions"] > 0


@pytest.mark.parametrize("bits", [[1], [3], [6], [4, 4]])
def test_multi_match_grouped_and_chained_leaves(ctx, bits):
    # [1]: leaves of ~12K rows, too large to group (chain walk); the others
    # group each key's rows into a contiguous range.
    bk, used = G.gen_multi_match_keys(24000, 151, 40)
    b = P.BlockStream([P.U16, P.U128, P.U64], bk, G.payload_columns(152, [P.U16, P.U128, P.U64], 24000))
    p = P.BlockStream([P.U32, P.U8], G.gen_keys(4, 70000, 153, 40, domain=used, match_permille=800),
                      G.payload_columns(154, [P.U32, P.U8], 70000))
    for materialize in (0, 1):
        jo, fp, _ = run(ctx, "phj-pure", b, p, bits, materialize)
        check(b, p, jo, fp)


# ---- PHJ-PURE with host buffers (streamed probe chunks) ----------------------
def host_out(ctx, b, p, cap, pinned=True):
    def alloc(shape, dt):
        return ctx.pinned(shape, dt) if pinned else np.empty(shape, dtype=dt)
    keys = alloc((cap,), np.uint64)
    left = [alloc((cap, 2), np.uint64) if t == P.U128 else alloc((cap,), P.TYPE_DTYPE[t]) for t in b.types]
    right = [alloc((cap, 2), np.uint64) if t == P.U128 else alloc((cap,), P.TYPE_DTYPE[t]) for t in p.types]
    return keys, left, right


@pytest.mark.parametrize("name", ["c2_mini", "c3_mini", "edge", "empty_probe", "empty_build", "no_match"])
@pytest.mark.parametrize("chunk", [4096, 1 << 24])
def test_host_buffer_phj_pure(ctx, name, chunk):
    b, p = cases.make(name)
    expected = O.join_rows(b, p)
    ctx.set_int("host_chunk_rows", chunk)
    try:
        keys, left, right = host_out(ctx, b, p, len(expected) + 5, pinned=(chunk == 4096))
        rows, res = ctx.run_phj_pure_host(b, p, cases.BITS[name], keys, left, right)
    finally:
        ctx.set_int("host_chunk_rows", 16 << 20)
    assert rows == len(expected)
    jo = P.JoinOutput(b.types, p.types, keys[:rows], [c[:rows] for c in left], [c[:rows] for c in right])
    assert O.compare_outputs(expected, O.serialize_output(jo)) == ""
    assert res.e2e_wall_ms > 0


def test_host_buffer_short_capacity(ctx):
    b, p = cases.make("c2_mini")
    expected = O.join_rows(b, p)
    ctx.set_int("host_chunk_rows", 8192)
    try:
        keys, left, right = host_out(ctx, b, p, 1000)
        with pytest.raises(P.PhjError) as e:
            ctx.run_phj_pure_host(b, p, [4, 4], keys, left, right)
        assert e.value.status == 7
    finally:
        ctx.set_int("host_chunk_rows", 16 << 20)
    # the context keeps working
    keys, left, right = host_out(ctx, b, p, len(expected))
    rows, _ = ctx.run_phj_pure_host(b, p, [4, 4], keys, left, right)
    assert rows == len(expected)


@pytest.mark.parametrize("pack", [1, 0])
@pytest.mark.parametrize("build_types", [[P.U64, P.U32], [P.U8, P.U16, P.U32], [P.U32, P.U64, P.U32], [P.U64, P.U64],
                                         [P.U64, P.U64, P.U8], [P.U16]])
def test_packed_build_payloads(ctx, pack, build_types):
    # With unique build keys and 2+ build payload columns of at most 16 bytes
    # in all, the build payloads are packed row-major and the projection
    # gathers one 16-byte value per output row (pack 1); otherwise (and with
    # pack 0) it gathers each column.  Offsets follow the widest-first
    # packing; 17 bytes or one column stay unpacked.
    bk = G.gen_keys(0, 7000, 31, 9)
    b = P.BlockStream(build_types, bk, G.payload_columns(32, build_types, 7000))
    rows = 256 * 50 + 19
    p = P.BlockStream([P.U32], G.gen_keys(4, rows, 33, 9, domain=7000, match_permille=800), G.payload_columns(34, [P.U32], rows))
    ctx.set_int("pack_build", pack)
    try:
        for scheme, bits in (("phj-pure", [4, 3]), ("chj", None)):
            for materialize in (0, 1):
                jo, fp, _ = run(ctx, scheme, b, p, bits, materialize)
                check(b, p, jo, fp)
        # host-buffer PHJ-PURE, probe side in 4096-row chunks
        expected = O.join_rows(b, p)
        ctx.set_int("host_chunk_rows", 4096)
        try:
            keys, left, right = host_out(ctx, b, p, len(expected))
            n, _ = ctx.run_phj_pure_host(b, p, [4, 3], keys, left, right)
        finally:
            ctx.set_int("host_chunk_rows", 16 << 20)
        assert n == len(expected)
        jo = P.JoinOutput(b.types, p.types, keys[:n], [c[:n] for c in left], [c[:n] for c in right])
        assert O.compare_outputs(expected, O.serialize_output(jo)) == ""
    finally:
        ctx.set_int("pack_build", 1)


@pytest.mark.parametrize("bt,probe_types", [([P.U64, P.U32], [P.U32]), ([P.U64, P.U32], [P.U64, P.U16]), ([P.U64, P.U32], []),
                                            ([P.U64, P.U32], [P.U128, P.U8]), ([P.U64], [P.U32]), ([P.U32], [P.U64]),
                                            ([], [P.U32]), ([P.U16], [P.U32]), ([P.U64, P.U64, P.U32], [P.U32])])
def test_fused_probe_equals_split_and_oracle(ctx, bt, probe_types):
    # Unique build keys whose payloads are packed, one 4- or 8-byte column,
    # or none: the probe looks up and projects in one kernel (probe_fused 1,
    # output rows in reservation order) or in two (0); both give the
    # oracle's rows.  A 16-byte probe column, a 1- or 2-byte build column
    # alone, or build columns that do not pack keep the two-kernel form.
    bk = G.gen_keys(0, 9000, 41, 11)
    b = P.BlockStream(bt, bk, G.payload_columns(42, bt, 9000))
    rows = 256 * 37 + 5
    p = P.BlockStream(probe_types, G.gen_keys(4, rows, 43, 11, domain=9000, match_permille=700),
                      G.payload_columns(44, probe_types, rows))
    expected = O.join_rows(b, p)
    widths = [P.TYPE_WIDTH[t] for t in bt]
    gathers = (len(bt) >= 2 and sum(widths) <= 16) or bt == [] or widths in ([4], [8])
    fused_ok = gathers and all(t != P.U128 for t in probe_types)
    try:
        for fused in (1, 0):
            ctx.set_int("probe_fused", fused)
            for scheme, bits, mat in (("phj-pure", [4, 3], 1), ("phj-pure", [5], 0), ("chj", None, -1)):
                jo, fp, _ = run(ctx, scheme, b, p, bits, mat)
                check(b, p, jo, fp)
                names = {k["name"] for k in ctx.kernel_times()}
                assert ("probe_fused" in names) == (fused == 1 and fused_ok), names
    finally:
        ctx.set_int("probe_fused", 1)


@pytest.mark.parametrize("rows,match", [(1, 1000), (255, 1000), (256, 0), (257, 500), (512 * 3 + 1, 1000)])
def test_fused_probe_chunk_edges(ctx, rows, match):
    # The one-pass probe at warp-chunk edges (256 rows a chunk): a single
    # row, a chunk short by one, exactly one chunk with no match, one row
    # past a chunk, all rows matching; with and without the probe side's
    # written pass.
    bt = [P.U64, P.U32]
    b = P.BlockStream(bt, G.gen_keys(0, 3000, 71, 13), G.payload_columns(72, bt, 3000))
    p = P.BlockStream([P.U64], G.gen_keys(4, rows, 73, 13, domain=3000, match_permille=match), G.payload_columns(74, [P.U64], rows))
    for scheme, bits, mat in (("phj-pure", [3, 3], 1), ("phj-pure", [6], 0), ("chj", None, -1)):
        jo, fp, _ = run(ctx, scheme, b, p, bits, mat)
        check(b, p, jo, fp)
        assert "probe_fused" in {k["name"] for k in ctx.kernel_times()}


@pytest.mark.parametrize("name", ["c2_mini", "c3_mini", "edge", "empty_probe", "empty_build", "no_match"])
@pytest.mark.parametrize("chunk,budget", [(4096, 1), (1 << 24, 1), (1 << 24, 512)])
def test_host_buffer_phj_bep(ctx, name, chunk, budget):
    # runPhjBep with host inputs and outputs: batches of at most the budget
    # and at most host_chunk_rows rows, uploads / joins / downloads
    # overlapped; the rows must equal the oracle's
    b, p = cases.make(name)
    expected = O.join_rows(b, p)
    bits = cases.BITS[name]
    ctx.set_int("host_chunk_rows", chunk)
    try:
        keys, left, right = host_out(ctx, b, p, len(expected) + 5, pinned=(chunk == 4096))
        rows, res = ctx.run_phj_bep_host(b, p, bits, budget, keys, left, right)
    finally:
        ctx.set_int("host_chunk_rows", 16 << 20)
    assert rows == len(expected)
    jo = P.JoinOutput(b.types, p.types, keys[:rows], [c[:rows] for c in left], [c[:rows] for c in right])
    assert O.compare_outputs(expected, O.serialize_output(jo)) == ""
    assert res.e2e_wall_ms > 0 and res.bep_budget_mib == budget
    if p.total_rows and b.total_rows:
        assert res.bep_evictions > 0 and res.bep_refinements > 0


def test_host_buffer_phj_bep_short_capacity(ctx):
    b, p = cases.make("c2_mini")
    expected = O.join_rows(b, p)
    ctx.set_int("host_chunk_rows", 8192)
    try:
        keys, left, right = host_out(ctx, b, p, 1000)
        with pytest.raises(P.PhjError) as e:
            ctx.run_phj_bep_host(b, p, [4, 4], 1, keys, left, right)
        assert e.value.status == 7
    finally:
        ctx.set_int("host_chunk_rows", 16 << 20)
    keys, left, right = host_out(ctx, b, p, len(expected))
    rows, _ = ctx.run_phj_bep_host(b, p, [4, 4], 1, keys, left, right)
    assert rows == len(expected)


def test_host_buffer_bep_stuck_leaf_times_out_and_context_recovers(ctx):
    # The same bounded-wait failure through the host-buffer entry point:
    # the error comes back with the upload / download streams drained, and
    # the context runs the next host-buffer join.
    b, p = cases.make("c2_mini")
    expected = O.join_rows(b, p)
    keys, left, right = host_out(ctx, b, p, len(expected))
    ctx.set_int("wait_limit_ms", 100)
    ctx.set_int("test_stuck_leaf", 3)
    ctx.set_int("host_chunk_rows", 8192)
    try:
        with pytest.raises(P.PhjError) as e:
            ctx.run_phj_bep_host(b, p, [4], 1, keys, left, right)
        assert e.value.status == P.ERR_DEVICE_TIMEOUT
    finally:
        ctx.set_int("test_stuck_leaf", -1)
        ctx.set_int("wait_limit_ms", 1000)
    try:
        rows, _ = ctx.run_phj_bep_host(b, p, [4], 1, keys, left, right)
    finally:
        ctx.set_int("host_chunk_rows", 16 << 20)
    assert rows == len(expected)
    jo = P.JoinOutput(b.types, p.types, keys[:rows], [c[:rows] for c in left], [c[:rows] for c in right])
    assert O.compare_outputs(expected, O.serialize_output(jo)) == ""


@pytest.mark.parametrize("pb", [1, 6, 11])
def test_probe_pass_width_override(ctx, pb):
    # The probe side's written pass width is a performance choice: any
    # width gives the same rows (the lookup takes the leaf from the whole
    # hash), including one wider than the configuration's first pass.
    b, p = cases.make("c2_mini")
    ctx.set_int("probe_pass_bits", pb)
    try:
        for bits in ([4, 4], [3], [6, 5]):
            jo, fp, _ = run(ctx, "phj-pure", b, p, bits, 1)
            check(b, p, jo, fp)
            jo, fp, _ = run(ctx, "phj", b, p, bits)
            check(b, p, jo, fp)
    finally:
        ctx.set_int("probe_pass_bits", 0)


def test_chj_irregular_blocks_with_packed_payloads(ctx):
    # CHJ's build rows are (input block, row); the packed payload rows are
    # indexed by the global row the block offsets give.
    bk = G.gen_keys(0, 3000, 41, 4)
    sizes = np.array([5, 1200, 1, 794, 1000], dtype=np.uint32)
    b = P.BlockStream([P.U32, P.U16, P.U8], bk, G.payload_columns(42, [P.U32, P.U16, P.U8], 3000), block_rows=sizes)
    p = P.BlockStream([P.U64], G.gen_keys(4, 9000, 43, 4, domain=3000, match_permille=900), G.payload_columns(44, [P.U64], 9000))
    for pack in (1, 0):
        ctx.set_int("pack_build", pack)
        try:
            jo, fp, _ = run(ctx, "chj", b, p)
            check(b, p, jo, fp)
        finally:
            ctx.set_int("pack_build", 1)


def test_contexts_used_from_other_host_threads(ctx):
    # Every call makes its context's device current for the call: two host
    # threads, each with its own context, join at the same time and match
    # the oracle and the same join run on the test's own thread.
    import threading

    b, p = cases.make("c2_mini")
    want = run(ctx, "phj-pure", b, p, [4, 4])[1]
    results, errors = {}, []

    def worker(k):
        try:
            c = P.Context(0)
            try:
                for scheme in ("phj-pure", "phj", "chj"):
                    jo, fp, _ = run(c, scheme, b, p, [4, 4])
                    results[(k, scheme)] = (jo, fp)
            finally:
                c.close()
        except Exception as e:  # reported on the test's thread
            errors.append(repr(e))

    threads = [threading.Thread(target=worker, args=(k,)) for k in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=300)
    assert not errors, errors
    assert len(results) == 6
    for (k, scheme), (jo, fp) in results.items():
        assert fp == want, (k, scheme)
    check(b, p, results[(0, "phj")][0], want)


@pytest.mark.parametrize("scheme", ["phj-pure", "phj"])
def test_host_buffer_failure_after_build_shuffle_leaves_context_usable(ctx, scheme):
    # A host-side failure while the probe chunks' uploads are still queued:
    # the call returns the error after draining its copy streams, and the
    # next host-buffer join on the same context (reusing the pooled memory
    # those copies wrote) is bit-exact.
    b, p = cases.make("c2_mini")
    expected = O.join_rows(b, p)
    keys, left, right = host_out(ctx, b, p, len(expected))

    def join():
        if scheme == "phj":
            return ctx.run_phj_bep_host(b, p, [4, 4], 1, keys, left, right)[0]
        return ctx.run_phj_pure_host(b, p, [4, 4], keys, left, right)[0]

    ctx.set_int("host_chunk_rows", 8192)
    try:
        for _ in range(2):
            ctx.set_int("test_fail_build", 1)
            try:
                with pytest.raises(P.PhjError) as e:
                    join()
                assert e.value.status == P.ERR_CUDA and "test_fail_build" in str(e.value)
            finally:
                ctx.set_int("test_fail_build", 0)
            rows = join()
            assert rows == len(expected)
            jo = P.JoinOutput(b.types, p.types, keys[:rows], [c[:rows] for c in left], [c[:rows] for c in right])
            assert O.compare_outputs(expected, O.serialize_output(jo)) == ""
    finally:
        ctx.set_int("host_chunk_rows", 16 << 20)


@pytest.mark.parametrize("windows", [2, 16, 256])
def test_chj_sub_table_windows(ctx, windows):
    """The windowed CHJ probe (one sweep per group of sub-tables) gives the
    oracle's rows on unique keys, repeated keys on both sides and the edge
    keys, with packed and column-wise build payloads."""
    ctx.set_int("chj_windows", windows)
    try:
        for name in ("c2_mini", "c3_mini", "edge"):
            b, p = cases.make(name)
            jo, fp, _ = run(ctx, "chj", b, p)
            check(b, p, jo, fp)
        ctx.set_int("pack_build", 0)
        b, p = cases.make("c2_mini")
        jo, fp, _ = run(ctx, "chj", b, p)
        check(b, p, jo, fp)
    finally:
        ctx.set_int("pack_build", 1)
        ctx.set_int("chj_windows", 0)
