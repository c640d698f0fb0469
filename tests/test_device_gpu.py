"""Device generator and fingerprint against their host forms, and the
kernel-timing hooks."""
import numpy as np
import pytest

import oracle as O
import phj_datagen as G
import phj_gpu as P

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind,kw", [(0, {}), (1, {}), (3, {"domain": 777}), (4, {"domain": 5000, "match_permille": 900})])
def test_device_generator_matches_host(ctx, kind, kw):
    rows = 50_000
    types = [P.U8, P.U16, P.U32, P.U64, P.U128]
    t = ctx.generate(kind, rows, seed=123, key_seed=456, types=types, **kw)
    s = t.download()
    assert np.array_equal(s.keys, G.gen_keys(kind, rows, 123, 456, **kw))
    for got, want in zip(s.payloads, G.payload_columns(123, types, rows)):
        assert np.array_equal(got, want)
    t.free()


def test_device_multi_match_generator_matches_host(ctx):
    t = ctx.generate(2, 40_000, seed=5, key_seed=6, types=[P.U32])
    keys, used = G.gen_multi_match_keys(40_000, 5, 6)
    assert t.gen_distinct == used
    assert np.array_equal(t.download().keys, keys)
    t.free()


def test_device_zipf_generator_close_to_host(ctx):
    t = ctx.generate(5, 100_000, seed=8, key_seed=9, types=[P.U32], domain=20_000, theta=1.0)
    dev = t.download().keys
    host = G.gen_zipf_keys(100_000, 8, 9, 20_000, 1.0)
    assert np.mean(dev == host) > 0.999  # libm ulp differences may move a rare rank
    t.free()


def test_kernel_times_and_launch_count(ctx):
    b = ctx.generate(0, 100_000, 1, 2, [P.U64])
    p = ctx.generate(4, 400_000, 3, 2, [P.U32], domain=100_000, match_permille=900)
    n0 = ctx.launch_count()
    hb, hp = b.download(), p.download()
    # unique build keys with one 8-byte payload: the one-pass probe by
    # default, the lookup and projection kernels with probe_fused 0
    for fused, probe_kernels in ((1, ["probe_fused"]), (0, ["probe_lookup", "probe_project"])):
        ctx.set_int("probe_fused", fused)
        try:
            out, res = ctx.run_phj_pure(b, p, [6, 6])
        finally:
            ctx.set_int("probe_fused", 1)
        assert ctx.launch_count() > n0
        names = [k["name"] for k in ctx.kernel_times()]
        assert all(k in names for k in probe_kernels + ["build_scatter"]), names
        assert all(k["ms"] >= 0 for k in ctx.kernel_times())
        assert out.fingerprint() == O.join_fingerprint(hb, hp)
        out.free()
    b.free(), p.free()
