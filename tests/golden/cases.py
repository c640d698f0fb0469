"""Seeded input cases shared by the golden-fixture generator and the tests.

Each case is a build/probe pair produced by phj_datagen (the host form of the
library's generator), small enough for the reference's std::string oracle.
"""
import numpy as np

import phj_datagen as G
from phj_gpu import BlockStream, U8, U16, U32, U64, U128

UINT64_MAX = np.uint64(0xFFFFFFFFFFFFFFFF)


def _stream(types, keys, seed):
    return BlockStream(list(types), keys, G.payload_columns(seed, types, len(keys)))


def edge_case():
    """Keys 0 and UINT64_MAX, duplicates on both sides, probe keys absent from
    the build, every payload width."""
    bk = np.concatenate([np.array([0, 0, UINT64_MAX, 5, 5, 5], dtype=np.uint64), G.gen_keys(0, 3000, 1, 77)])
    pk = np.concatenate([np.array([0, UINT64_MAX, 5, 6, 0], dtype=np.uint64), G.gen_keys(4, 9000, 2, 77, domain=3000, match_permille=700)])
    return _stream([U8, U16, U32, U64, U128], bk, 31), _stream([U128, U8, U16], pk, 32)


def make(name):
    if name == "c1_mini":  # permutation build keys, every probe row matches once
        n = 4096
        return _stream([U64], G.gen_keys(1, n, 11, 0), 12), _stream([U32], G.gen_keys(3, 8 * n, 13, 0, domain=n), 14)
    if name == "c2_mini":  # unique build keys, 90% match
        n = 20000
        return (_stream([U64, U32], G.gen_keys(0, n, 21, 5), 22),
                _stream([U64], G.gen_keys(4, 5 * n, 23, 5, domain=n, match_permille=900), 24))
    if name == "c3_mini":  # multi-match build, 50% match
        n = 16000
        bk, used = G.gen_multi_match_keys(n, 31, 6)
        return (_stream([U8, U16, U128], bk, 32),
                _stream([U32], G.gen_keys(4, 40000, 33, 6, domain=used, match_permille=500), 34))
    if name == "c4_mini":  # unique build keys, Zipf(1.0) probe
        n = 8192
        return _stream([U64], G.gen_keys(0, n, 41, 8), 42), _stream([U32], G.gen_zipf_keys(60000, 43, 8, n, 1.0), 44)
    if name == "edge":
        return edge_case()
    if name == "empty_probe":
        return _stream([U64], G.gen_keys(0, 1000, 51, 9), 52), _stream([U32], np.zeros(0, dtype=np.uint64), 53)
    if name == "empty_build":
        return _stream([U64], np.zeros(0, dtype=np.uint64), 61), _stream([U32], G.gen_keys(3, 1000, 62, 0, domain=50), 63)
    if name == "no_match":
        return (_stream([U32], G.gen_keys(0, 2000, 71, 10), 72),
                _stream([U64], G.gen_keys(4, 5000, 73, 10, domain=2000, match_permille=0), 74))
    raise KeyError(name)


NAMES = ["c1_mini", "c2_mini", "c3_mini", "c4_mini", "edge", "empty_probe", "empty_build", "no_match"]
# Radix configurations run for every case (RadixConfig::pass_bits).
BITS = {"c1_mini": [8], "c2_mini": [4, 4], "c3_mini": [3, 3], "c4_mini": [2, 2, 2], "edge": [5],
        "empty_probe": [4], "empty_build": [4], "no_match": [6, 2]}
