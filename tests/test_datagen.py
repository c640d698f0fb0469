"""Properties of the seeded workload generator (host form; the device form
is checked against it in test_device_gpu.py)."""
import numpy as np

import phj_datagen as G


def test_unique_keys_and_non_matching_tail():
    k = G.gen_keys(0, 200_000, 1, 5)
    assert len(np.unique(k)) == len(k)
    tail = G.key_of(5, np.arange(200_000, 300_000, dtype=np.uint64))
    assert not np.isin(tail, k).any()


def test_permutation_keys_are_1_to_n():
    k = G.gen_keys(1, 100_003, 9, 0)
    assert np.array_equal(np.sort(k), np.arange(1, 100_004, dtype=np.uint64))


def test_match_rate_and_uniform_domain():
    build = G.gen_keys(0, 10_000, 1, 3)
    probe = G.gen_keys(4, 200_000, 2, 3, domain=10_000, match_permille=900)
    rate = np.isin(probe, build).mean()
    assert 0.89 < rate < 0.91
    u = G.gen_keys(3, 100_000, 4, 0, domain=1000)
    assert u.min() >= 1 and u.max() <= 1000


def test_multi_match_multiplicities():
    keys, used = G.gen_multi_match_keys(100_000, 7, 11)
    _, counts = np.unique(keys, return_counts=True)
    assert len(counts) == used
    assert counts.max() <= 16
    assert 3.7 < counts[:-1].mean() < 4.2


def test_zipf_head_frequency():
    r = G.zipf_ranks(10_000, 1.0, 3, 400_000)
    h = np.sum(1.0 / np.arange(1, 10_001))
    f1 = np.mean(r == 1)
    assert abs(f1 - 1.0 / h) < 0.005
    assert r.min() >= 1 and r.max() <= 10_000
