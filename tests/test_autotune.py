"""The measuring autotuner (phj-bench_gb300/autotune.py): candidate
generation and cache keys on the CPU; on the GPU, a tuned configuration
joins bit-exactly and a second call is served from the cache."""
import pytest

import autotune as A
import oracle as O
import phj_gpu as P
from golden import cases


def test_split_bits_follows_the_cli():
    assert A.split_bits(16, 2) == [8, 8]
    assert A.split_bits(17, 2) == [9, 8]
    assert A.split_bits(10, 3) == [4, 3, 3]


def test_radix_candidates_surround_the_heuristic():
    cands = A.radix_candidates(16 << 20)
    assert [8, 8] in cands and [16] in cands and [6, 6, 6] in cands
    assert all(1 <= sum(c) <= 24 and max(c) <= 16 for c in cands)
    assert all(abs(sum(c) - 16) <= 2 for c in cands)


def test_shape_key_buckets_sizes_and_widths():
    k1 = A.shape_key("phj-pure", 1 << 20, 1 << 24, [P.U64], [P.U32])
    k2 = A.shape_key("phj-pure", (1 << 20) + 5, (1 << 24) + 9, [P.U64], [P.U32])
    k3 = A.shape_key("phj-pure", 1 << 20, 1 << 24, [P.U64, P.U32], [P.U32])
    assert k1 == k2 != k3


@pytest.mark.gpu
@pytest.mark.parametrize("scheme", ["phj-pure", "phj"])
def test_tuned_join_is_bit_exact_and_cached(ctx, tmp_path, scheme):
    b, p = cases.make("c3_mini")
    tb, tp = ctx.upload(b), ctx.upload(p)
    cache = str(tmp_path / "tune.json")
    try:
        cfg = A.tune(ctx, tb, tp, scheme=scheme, reps=1, budget_mib=1, cache_path=cache)
        assert cfg["trials"] > 5 and cfg["ms"] > 0
        if scheme == "phj":
            out, _ = ctx.run_phj_bep(tb, tp, cfg["pass_bits"], 1)
        else:
            out, _ = ctx.run_phj_pure(tb, tp, cfg["pass_bits"])
        assert O.compare_outputs(O.join_rows(b, p), O.serialize_output(out.download())) == ""
        out.free()
        again = A.tune(ctx, tb, tp, scheme=scheme, cache_path=cache)
        assert again["cached"] and again["pass_bits"] == cfg["pass_bits"]
    finally:
        A.reset(ctx)
        tb.free(), tp.free()
