"""Parity at the benchmark sizes, through properties that do not depend on
size: on the same generated inputs, CHJ (one unpartitioned table), PHJ-PURE
(both sides partitioned to leaf depth) and PHJ/BEP (budget-sized probe
batches, leaf tables built on first use) must produce the same output
multiset -- the same row count and the same two independent sums of row
hashes (the order-independent fingerprint) -- and, where every build key is
unique, at most one output row per probe row.  The oracle checks the same
kernels row by row at sizes it finishes in seconds."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
import bench  # noqa: E402  (the benchmark's workload definitions and generator calls)

pytestmark = pytest.mark.gpu


def fingerprint(ctx, scheme, b, p, bits, budget_mib=0):
    out, _ = bench.run_scheme(ctx, scheme, b, p, bits, budget_mib)
    try:
        return out.fingerprint()
    finally:
        out.free()


@pytest.mark.parametrize("wl,bits,unique", [
    ("c2", [8, 8], True),      # 16M x 256M, 10% of the probe keys match nothing
    ("c4", [6, 6, 6], True),   # 64M x 512M, Zipf(1.0) probe keys
    ("c3", [8, 8], False),     # 32M (8M distinct keys) x 128M, multi-match
])
def test_schemes_agree_at_full_size(ctx, wl, bits, unique):
    b, p = bench.make_tables(ctx, wl)
    try:
        budget = bench.BEP_BUDGET_PER_GROUP.get(wl, 32) * ctx.get_int("num_sms")
        fps = {s: fingerprint(ctx, s, b, p, bits, budget) for s in ("phj-pure", "phj", "chj")}
        assert fps["phj-pure"] == fps["phj"] == fps["chj"], fps
        rows = fps["chj"][0]
        assert rows > 0
        if unique:
            assert rows <= p.rows
        else:
            assert rows > p.rows // 2  # half of the probe keys match, ~4 build rows each
    finally:
        b.free(), p.free()


@pytest.mark.parametrize("scheme", ["phj-pure", "phj"])
def test_host_buffer_join_at_full_size_matches_device_join(ctx, scheme):
    # 16M x 256M through the host-buffer entry points (upload, join and
    # download overlapped in chunks or budget-sized batches): the rows that
    # land in host memory have the device join's fingerprint.
    import numpy as np

    import oracle as O
    import phj_gpu as P

    c = P.Context(0)  # its own context: the pinned output columns go with it
    try:
        b, p = bench.make_tables(c, "c2")
        try:
            budget = bench.BEP_BUDGET_PER_GROUP.get("c4", 32) * c.get_int("num_sms")
            want = fingerprint(c, scheme, b, p, [8, 8], budget)
            hb, hp = b.download(), p.download()
        finally:
            b.free(), p.free()
        cap = want[0]
        keys = c.pinned((cap,), np.uint64)
        left = [c.pinned((cap,), P.TYPE_DTYPE[t]) for t in hb.types]
        right = [c.pinned((cap,), P.TYPE_DTYPE[t]) for t in hp.types]
        if scheme == "phj":
            rows, _ = c.run_phj_bep_host(hb, hp, [8, 8], budget, keys, left, right)
        else:
            rows, _ = c.run_phj_pure_host(hb, hp, [8, 8], keys, left, right)
        assert rows == cap
        assert O.columns_fingerprint(P.JoinOutput(hb.types, hp.types, keys, left, right)) == want
    finally:
        c.close()
