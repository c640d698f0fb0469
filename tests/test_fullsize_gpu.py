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
