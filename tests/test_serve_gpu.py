"""Batched joins (phj_batch_run) and the request loop (phj_serve_*): every
join's output is the same alone, in a batch and in the served mix, and
matches the oracle."""
import numpy as np
import pytest

import oracle as O
import phj_datagen as G
import phj_gpu as P

pytestmark = pytest.mark.gpu


def host_sides(spec_b, spec_p):
    """The host form of a (build, probe) generator pair (kinds 0 and 4)."""
    tb = [spec_b.schema.types[i] for i in range(spec_b.schema.n_payloads)]
    tp = [spec_p.schema.types[i] for i in range(spec_p.schema.n_payloads)]
    bk = G.gen_keys(spec_b.kind, spec_b.rows, spec_b.seed, spec_b.key_seed)
    pk = G.gen_keys(spec_p.kind, spec_p.rows, spec_p.seed, spec_p.key_seed, domain=spec_p.domain,
                    match_permille=spec_p.match_permille)
    return (P.BlockStream(tb, bk, G.payload_columns(spec_b.seed, tb, spec_b.rows)),
            P.BlockStream(tp, pk, G.payload_columns(spec_p.seed, tp, spec_p.rows)))


def request(i, build_rows, probe_rows, match, tb, tp):
    b = P.gen_spec(0, build_rows, 1000 + i, 7000 + i, tb)
    p = P.gen_spec(4, probe_rows, 2000 + i, 7000 + i, tp, domain=max(build_rows, 1), match_permille=match)
    return b, p


def mix():
    rng = np.random.default_rng(5)
    reqs = []
    for i in range(24):
        big = i % 6 == 5
        B = int(rng.integers(200_000, 600_000)) if big else int(rng.integers(1, 40_000))
        Pn = B * int(rng.integers(4, 12))
        tb = [P.U32, P.U64][: 1 + i % 2]
        tp = [P.U64, P.U32, P.U64][: 1 + i % 3]
        reqs.append(request(i, B, Pn, int(rng.integers(100, 1000)), tb, tp))
    return reqs


def alone_fingerprint(ctx, b, p, bits=(8, 8)):
    tb = ctx.generate(b.kind, b.rows, b.seed, b.key_seed, [b.schema.types[i] for i in range(b.schema.n_payloads)])
    tp = ctx.generate(p.kind, p.rows, p.seed, p.key_seed, [p.schema.types[i] for i in range(p.schema.n_payloads)],
                      domain=p.domain, match_permille=p.match_permille)
    out, _ = ctx.run_phj_pure(tb, tp, list(bits))
    fp = out.fingerprint()
    out.free(), tb.free(), tp.free()
    return fp


def test_batch_matches_oracle_with_uneven_sizes(ctx):
    sizes = [(5000, 40000, 900), (1, 1000, 1000), (0, 500, 500), (3000, 0, 500), (70000, 300000, 300), (257, 9000, 1000)]
    specs = [request(i, B, Pn, m, [P.U64, P.U16], [P.U32]) for i, (B, Pn, m) in enumerate(sizes)]
    hosts = [host_sides(b, p) for b, p in specs]
    tbs = [ctx.upload(hb) for hb, _ in hosts]
    tps = [ctx.upload(hp) for _, hp in hosts]
    outs, res = ctx.run_batch(tbs, tps)
    assert res.n_joins == len(sizes)
    for (hb, hp), o in zip(hosts, outs):
        expected = O.join_rows(hb, hp)
        assert o.rows == len(expected)
        assert O.compare_outputs(expected, O.serialize_output(o.download())) == ""
        o.free()
    for t in tbs + tps:
        t.free()


def test_batch_multi_match_and_wide_payloads(ctx):
    bk, used = G.gen_multi_match_keys(20000, 61, 62)
    b1 = P.BlockStream([P.U8, P.U128], bk, G.payload_columns(63, [P.U8, P.U128], 20000))
    p1 = P.BlockStream([P.U128], G.gen_keys(4, 60000, 64, 62, domain=used, match_permille=600), G.payload_columns(65, [P.U128], 60000))
    bk2 = np.full(300, 42, dtype=np.uint64)
    b2 = P.BlockStream([P.U32], bk2, G.payload_columns(66, [P.U32], 300))
    p2 = P.BlockStream([P.U8], np.array([42, 1, 42], dtype=np.uint64), G.payload_columns(67, [P.U8], 3))
    tb = [ctx.upload(b1), ctx.upload(b2)]
    tp = [ctx.upload(p1), ctx.upload(p2)]
    outs, _ = ctx.run_batch(tb, tp)
    for (hb, hp), o in zip([(b1, p1), (b2, p2)], outs):
        assert O.compare_outputs(O.join_rows(hb, hp), O.serialize_output(o.download())) == ""
        o.free()
    for t in tb + tp:
        t.free()


def test_batch_of_medium_joins_equals_the_oracle(ctx):
    """Medium joins in one batch: 5M build rows (partitions of about 2,400
    rows, built and probed in two pieces each), 2M and 300K build rows, each
    equal to the oracle's fingerprint."""
    sizes = [(5_000_000, 20_000_000, 900), (2_000_000, 8_000_000, 500), (300_000, 9_000_000, 100)]
    specs = [request(50 + i, B, Pn, m, [P.U64, P.U32], [P.U32, P.U64]) for i, (B, Pn, m) in enumerate(sizes)]
    hosts = [host_sides(b, p) for b, p in specs]
    tbs = [ctx.upload(hb) for hb, _ in hosts]
    tps = [ctx.upload(hp) for _, hp in hosts]
    try:
        outs, res = ctx.run_batch(tbs, tps)
        assert res.n_joins == 3
        for (hb, hp), o in zip(hosts, outs):
            assert tuple(o.fingerprint()) == O.join_fingerprint(hb, hp)
            o.free()
    finally:
        for t in tbs + tps:
            t.free()


def test_batch_graph_replays_equal_the_launched_chain(ctx):
    """phj_batch_run replays its chain as a CUDA graph captured at the
    workspace's capacity.  Batches of changing shape -- past the first
    workspace's 16 joins and 4096 partitions (a new capture), then smaller
    again (a replay with stale entries past the batch's own) -- give every
    join the same rows as the chain launched at the batch's own sizes and
    as the join alone."""
    rng = np.random.default_rng(11)
    shapes = [(3, 1_000, 30_000), (40, 50_000, 100_000), (5, 1, 20_000), (1, 0, 1), (2, 200_000, 400_000)]
    for bi, (nj, lo, hi) in enumerate(shapes):
        specs = [request(400 + 64 * bi + i, int(rng.integers(lo, hi)), 0, int(rng.integers(100, 1000)),
                         [P.U64, P.U32][: 1 + i % 2], [P.U32, P.U16][: 1 + (i + 1) % 2]) for i in range(nj)]
        specs = [(b, P.gen_spec(4, max(1, b.rows * int(rng.integers(2, 6))), p.seed, p.key_seed,
                                [p.schema.types[k] for k in range(p.schema.n_payloads)], domain=max(b.rows, 1),
                                match_permille=p.match_permille)) for b, p in specs]
        tbs = [ctx.generate(b.kind, b.rows, b.seed, b.key_seed, [b.schema.types[k] for k in range(b.schema.n_payloads)])
               for b, _ in specs]
        tps = [ctx.generate(p.kind, p.rows, p.seed, p.key_seed, [p.schema.types[k] for k in range(p.schema.n_payloads)],
                            domain=p.domain, match_permille=p.match_permille) for _, p in specs]
        try:
            fps = {}
            for graph in (1, 0):
                ctx.set_int("batch_graph", graph)
                outs, res = ctx.run_batch(tbs, tps)
                names = {k["name"] for k in ctx.kernel_times()}
                assert ("batch_graph" in names) == bool(graph) and ("batch_join" in names) == (not graph)
                fps[graph] = [tuple(o.fingerprint()) for o in outs]
                for o in outs:
                    o.free()
            assert fps[1] == fps[0]
            for (b, p), fp in zip(specs, fps[1]):
                assert fp == tuple(alone_fingerprint(ctx, b, p))
        finally:
            ctx.set_int("batch_graph", 1)
            for t in tbs + tps:
                t.free()


@pytest.mark.parametrize("mode", ["plain", "batched"])
def test_served_results_equal_alone(ctx, mode):
    reqs = mix()
    if mode == "plain":
        srv = P.Server(workers=1)
    else:
        srv = P.Server(workers=3, batch_max_build_rows=65536, batch_max_joins=16, hbm_budget_bytes=2 << 30)
    rng = np.random.default_rng(9)
    t = 0.0
    for b, p in reqs:
        srv.submit(b, p, t)
        t += float(rng.exponential(0.002))
    recs = srv.run(timeout_s=300)
    srv.close()
    assert all(r["status"] == 0 for r in recs)
    for (b, p), r in zip(reqs, recs):
        assert r["fingerprint"] == alone_fingerprint(ctx, b, p), r
        assert r["done_s"] >= r["start_s"] >= r["admit_s"] >= r["arrival_s"] - 1e-6
    if mode == "batched":
        assert max(r["batch_size"] for r in recs) > 1
        assert len({r["slot"] for r in recs}) > 1
    else:
        assert all(r["batch_size"] == 1 for r in recs)
        # the admission estimate bounds the measured device footprint of a
        # join run alone (inputs, partitions, tables, output)
        for r in recs:
            assert 0 < r["job_peak_bytes"] <= r["footprint_bytes"] * 1.05 + (8 << 20), r


def test_served_small_requests_match_oracle():
    srv = P.Server(workers=2, batch_max_build_rows=1 << 20, batch_max_joins=8)
    specs = [request(i, 2000 + 500 * i, 10000 + 3000 * i, 500 + 50 * i, [P.U64], [P.U32, P.U8][: 1 + i % 2]) for i in range(6)]
    for b, p in specs:
        srv.submit(b, p, 0.0)
    recs = srv.run(timeout_s=120)
    srv.close()
    for (b, p), r in zip(specs, recs):
        hb, hp = host_sides(b, p)
        rows = O.join_rows(hb, hp)
        assert r["output_rows"] == len(rows)
        assert r["fingerprint"] == O.rows_fingerprint(rows, hb.types, hp.types)


def test_admission_budget_serialises_large_requests():
    # each request's footprint is above half the budget: never two in flight
    b, p = request(0, 100_000, 1_000_000, 900, [P.U64], [P.U32])
    fp = P.serve_footprint(b, p, batched=False)
    srv = P.Server(workers=4, hbm_budget_bytes=int(fp * 1.5))
    for i in range(6):
        bi, pi = request(i, 100_000, 1_000_000, 900, [P.U64], [P.U32])
        srv.submit(bi, pi, 0.0)
    recs = srv.run(timeout_s=120)
    srv.close()
    spans = sorted((r["start_s"], r["done_s"]) for r in recs)
    for (s0, d0), (s1, d1) in zip(spans, spans[1:]):
        assert s1 >= d0 - 1e-6
