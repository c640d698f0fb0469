"""Parity with the oracle at the benchmark sizes.

Each benchmark workload (1M x 8M, 16M x 256M, 32M x 128M multi-match, 64M x
512M Zipf) is generated on the device exactly as bench.py generates it.  The
inputs are then downloaded and the oracle -- the CPU restatement of the
reference's referenceOutput / compareOutputs (src/Reference.cpp:48-133, the
check `--check` runs, src/Main.cpp:112-156) -- computes the join on the host.
Every scheme's device output must equal it:

  * 1M x 8M: the sorted multiset of serialised rows, row for row (the
    reference's own compare), and its sha256 in tests/golden/fullsize.json;
  * the larger joins: the order-independent fingerprint (row count and two
    sums of per-row hashes over the serialised rows), equal to the oracle's
    on the downloaded inputs and to the committed golden value that
    tests/golden/gen_fullsize.py computed from the host generator.

The host-buffer entry points are checked the same way on 16M x 256M."""
import hashlib
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
import bench  # noqa: E402  (the benchmark's workload definitions and generator calls)
import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu

GOLDEN = json.load(open(os.path.join(ROOT, "tests", "golden", "fullsize.json")))


def golden_fp(wl):
    return tuple(int(v) for v in GOLDEN[wl]["fingerprint"])


def device_inputs(ctx, wl):
    b, p = bench.make_tables(ctx, wl)
    assert (b.rows, p.rows) == (GOLDEN[wl]["build_rows"], GOLDEN[wl]["probe_rows"])
    return b, p


def budget_of(ctx, wl):
    return bench.BEP_BUDGET_PER_GROUP.get(wl, 32) * ctx.get_int("num_sms")


def bits_of(wl):
    bits = bench.WORKLOADS[wl][4]
    return bits if bits is not None else [8, 8]


def test_1m_x_8m_rows_equal_the_oracle(ctx):
    b, p = device_inputs(ctx, "c1")
    try:
        hb, hp = b.download(), p.download()
        expected = O.join_rows(hb, hp)
        expected_sorted = O.sort_rows(expected.copy())
        assert hashlib.sha256(expected_sorted.tobytes()).hexdigest() == GOLDEN["c1"]["sha256_sorted_rows"]
        for scheme in ("phj-pure", "chj", "phj"):
            out, _ = bench.run_scheme(ctx, scheme, b, p, bits_of("c1"), budget_of(ctx, "c1"))
            try:
                got = O.serialize_output(out.download())
            finally:
                out.free()
            assert O.compare_outputs(expected, got) == "", scheme
    finally:
        b.free(), p.free()


@pytest.mark.parametrize("wl,schemes", [
    ("c2", ("phj-pure", "chj", "phj")),   # 16M x 256M, 10% of the probe keys match nothing
    ("c3", ("phj-pure", "chj", "phj")),   # 32M (8M distinct keys) x 128M, multi-match, u128 gather
    ("c4", ("phj", "phj-pure", "chj")),   # 64M x 512M, Zipf(1.0) probe keys, BEP budget 32 MiB a CTA group
])
def test_full_size_fingerprint_equals_the_oracle(ctx, wl, schemes):
    b, p = device_inputs(ctx, wl)
    try:
        hb, hp = b.download(), p.download()
        want = O.join_fingerprint(hb, hp)
        del hb, hp
        assert want == golden_fp(wl)
        for scheme in schemes:
            out, _ = bench.run_scheme(ctx, scheme, b, p, bits_of(wl), budget_of(ctx, wl))
            try:
                assert out.fingerprint() == want, scheme
            finally:
                out.free()
    finally:
        b.free(), p.free()


@pytest.mark.parametrize("scheme", ["phj-pure", "phj"])
def test_host_buffer_join_at_full_size_equals_the_oracle(ctx, scheme):
    # 16M x 256M through the host-buffer entry points (upload, join and
    # download overlapped in chunks or budget-sized batches): the rows that
    # land in host memory have the oracle's fingerprint.
    import phj_gpu as P

    c = P.Context(0)  # its own context: the pinned output columns go with it
    try:
        b, p = device_inputs(c, "c2")
        try:
            hb, hp = b.download(), p.download()
        finally:
            b.free(), p.free()
        want = golden_fp("c2")
        cap = want[0]
        keys = c.pinned((cap,), np.uint64)
        left = [c.pinned((cap,), P.TYPE_DTYPE[t]) for t in hb.types]
        right = [c.pinned((cap,), P.TYPE_DTYPE[t]) for t in hp.types]
        if scheme == "phj":
            rows, _ = c.run_phj_bep_host(hb, hp, [8, 8], budget_of(c, "c4"), keys, left, right)
        else:
            rows, _ = c.run_phj_pure_host(hb, hp, [8, 8], keys, left, right)
        assert rows == cap
        assert O.columns_fingerprint(P.JoinOutput(hb.types, hp.types, keys, left, right)) == want
    finally:
        c.close()
