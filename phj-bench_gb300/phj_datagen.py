"""Host-side (numpy) form of the library's seeded workload generator.

Produces the same integers as the device generator (phj_table_generate,
csrc/gen.cu) for the integer-only kinds 0-4, so small test workloads can be
built on the host and large ones on the device from one specification.

    rand64(seed, stream, i) = splitmix64_mix((seed ^ stream*M) + (i+1)*GAMMA)
    K(i) = rand64(key_seed, 0, i)     -- a bijection of i: unique keys, and
                                          K(n + j) never equals K(0..n-1)
    uniform(r, n) = ((r >> 32) * n) >> 32
    payload column c of row i: low bytes of rand64(seed, 16 + c, i)
                               (u128: high word rand64(seed, 32 + c, i))
"""
from __future__ import annotations

from typing import List, Sequence

import numpy as np

GAMMA = np.uint64(0x9E3779B97F4A7C15)
STREAM_MUL = 0xD1B54A32D192ED03
M1 = np.uint64(0xBF58476D1CE4E5B9)
M2 = np.uint64(0x94D049BB133111EB)
MASK64 = (1 << 64) - 1

U8, U16, U32, U64, U128 = 0, 1, 2, 3, 4
_DT = {U8: np.uint8, U16: np.uint16, U32: np.uint32, U64: np.uint64}


def _mix(z: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * M1
        z = (z ^ (z >> np.uint64(27))) * M2
        return z ^ (z >> np.uint64(31))


def rand64(seed: int, stream: int, idx: np.ndarray) -> np.ndarray:
    base = np.uint64((seed ^ ((stream * STREAM_MUL) & MASK64)) & MASK64)
    with np.errstate(over="ignore"):
        z = base + (np.asarray(idx, dtype=np.uint64) + np.uint64(1)) * GAMMA
    return _mix(z)


def key_of(key_seed: int, idx: np.ndarray) -> np.ndarray:
    return rand64(key_seed, 0, idx)


def uniform_below(r: np.ndarray, n: int) -> np.ndarray:
    assert 0 < n <= (1 << 32)
    return ((r >> np.uint64(32)) * np.uint64(n)) >> np.uint64(32)


class Perm:
    """Seeded permutation of [0, n): cycle-walking over an invertible mix."""

    def __init__(self, n: int, seed: int):
        k = 1
        while k < 63 and (1 << k) < n:
            k += 1
        self.n = n
        self.mask = np.uint64((1 << k) - 1)
        one = np.array([0], dtype=np.uint64)
        self.a1 = rand64(seed, 48, one)[0] | np.uint64(1)
        self.c1 = rand64(seed, 49, one)[0]
        self.a2 = rand64(seed, 50, one)[0] | np.uint64(1)
        self.c2 = rand64(seed, 51, one)[0]
        self.s = np.uint64((k + 1) // 2)

    def _step(self, x: np.ndarray) -> np.ndarray:
        with np.errstate(over="ignore"):
            x = (x * self.a1 + self.c1) & self.mask
            x ^= x >> self.s
            x = (x * self.a2 + self.c2) & self.mask
            x ^= x >> self.s
            x = (x * self.a1 + self.c2) & self.mask
        return x

    def __call__(self, i: np.ndarray) -> np.ndarray:
        y = self._step(np.asarray(i, dtype=np.uint64).copy())
        bad = y >= np.uint64(self.n)
        while bad.any():
            y[bad] = self._step(y[bad])
            bad = y >= np.uint64(self.n)
        return y


def payload_columns(seed: int, types: Sequence[int], rows: int, start: int = 0) -> List[np.ndarray]:
    """Payload columns of rows [start, start + rows)."""
    idx = np.arange(start, start + rows, dtype=np.uint64)
    cols = []
    for c, t in enumerate(types):
        lo = rand64(seed, 16 + c, idx)
        if t == U128:
            hi = rand64(seed, 32 + c, idx)
            cols.append(np.stack([lo, hi], axis=1))
        else:
            cols.append(lo.astype(_DT[t]))
    return cols


def gen_keys(kind: int, rows: int, seed: int, key_seed: int, domain: int = 0, match_permille: int = 1000, start: int = 0,
             total: int = 0):
    """Keys of generator kinds 0, 1, 3, 4 (see include/phj_gpu.h, phj_gen_spec)
    for rows [start, start + rows) of a side of `total` rows (default: rows)."""
    idx = np.arange(start, start + rows, dtype=np.uint64)
    if kind == 0:
        return key_of(key_seed, idx)
    if kind == 1:
        return Perm(total or rows, seed)(idx) + np.uint64(1)
    if kind == 3:
        return uniform_below(rand64(seed, 1, idx), domain) + np.uint64(1)
    if kind == 4:
        sel = uniform_below(rand64(seed, 2, idx), 1000) < np.uint64(match_permille)
        hit = key_of(key_seed, uniform_below(rand64(seed, 3, idx), domain))
        miss = key_of(key_seed, np.uint64(domain) + idx)
        return np.where(sel, hit, miss)
    raise ValueError(f"kind {kind} has no host form here")


def gen_multi_match_keys(rows: int, seed: int, key_seed: int):
    """Kind 2: distinct key d has multiplicity 1 + #consecutive successes of
    p = 3/4 (cap 16); rows are the expansion truncated to `rows`, shuffled by
    a seeded permutation.  Returns (keys, distinct_keys_used)."""
    d = np.arange(rows, dtype=np.uint64)
    mult = np.ones(rows, dtype=np.uint64)
    alive = np.ones(rows, dtype=bool)
    for j in range(15):
        ok = uniform_below(rand64(seed, 52, d * np.uint64(16) + np.uint64(j)), 4) != 0
        alive &= ok
        mult += alive.astype(np.uint64)
    cum = np.concatenate([[0], np.cumsum(mult)]).astype(np.uint64)
    used = int(np.searchsorted(cum, rows, side="left"))  # first d+1 with cum[d+1] >= rows
    perm = Perm(rows, seed ^ 0x5BD1E9955BD1E995)
    e = perm(np.arange(rows, dtype=np.uint64))
    dist = np.searchsorted(cum[: used + 1], e, side="right") - 1
    return key_of(key_seed, dist.astype(np.uint64)), used


def _zh_integral(s, x):
    lx = np.log(x)
    t = (1.0 - s) * lx
    with np.errstate(divide="ignore", invalid="ignore"):
        h2 = np.where(np.abs(t) > 1e-8, np.expm1(t) / np.where(t == 0, 1.0, t), 1.0 + t * 0.5 * (1.0 + t * (1.0 / 3.0) * (1.0 + 0.25 * t)))
    return h2 * lx


def _zh(s, x):
    return np.exp(-s * np.log(x))


def _zh_integral_inv(s, x):
    t = np.maximum(x * (1.0 - s), -1.0)
    with np.errstate(divide="ignore", invalid="ignore"):
        h1 = np.where(np.abs(t) > 1e-8, np.log1p(t) / np.where(t == 0, 1.0, t), 1.0 - t * (0.5 - t * (1.0 / 3.0 - 0.25 * t)))
    return np.exp(h1 * x)


def zipf_ranks(n: int, theta: float, seed: int, rows: int, start: int = 0) -> np.ndarray:
    """Zipf(theta) ranks in [1, n] by rejection-inversion (Hoermann & Derflinger
    1996); attempt j of row i draws rand64(seed, 4, i*64 + j).  Rows
    [start, start + rows)."""
    s = float(theta)
    h_x1 = float(_zh_integral(s, np.array([1.5]))[0] - 1.0)
    h_n = float(_zh_integral(s, np.array([n + 0.5]))[0])
    s_const = float(2.0 - _zh_integral_inv(s, _zh_integral(s, np.array([2.5])) - _zh(s, np.array([2.0])))[0])
    idx = np.arange(start, start + rows, dtype=np.uint64)
    out = np.ones(rows, dtype=np.uint64)
    pending = np.ones(rows, dtype=bool)
    for attempt in range(64):
        if not pending.any():
            break
        ii = idx[pending]
        r = rand64(seed, 4, ii * np.uint64(64) + np.uint64(attempt))
        u01 = (r >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
        u = h_n + u01 * (h_x1 - h_n)
        x = _zh_integral_inv(s, u)
        kd = np.clip(np.floor(x + 0.5), 1.0, float(n))
        acc = (kd - x <= s_const) | (u >= _zh_integral(s, kd + 0.5) - _zh(s, kd))
        pos = (ii - np.uint64(start)).astype(np.int64)
        out[pos] = kd.astype(np.uint64)
        pending[pos[acc]] = False
    return out


def gen_zipf_keys(rows: int, seed: int, key_seed: int, domain: int, theta: float = 1.0, start: int = 0) -> np.ndarray:
    """Kind 5: Zipf ranks mapped through a seeded permutation onto K(0..domain-1)."""
    ranks = zipf_ranks(domain, theta, seed, rows, start)
    perm = Perm(domain, seed ^ 0x2545F4914F6CDD1D)
    return key_of(key_seed, perm(ranks - np.uint64(1)))


def parallel_rows(rows: int, make, dtype, width: int = 1, threads: int = 0) -> np.ndarray:
    """Fills an array of `rows` rows from make(start, n) -> rows [start,
    start + n), in chunks on a thread pool (numpy's arithmetic releases the
    interpreter lock): the same integers as one make(0, rows) call."""
    import os
    from concurrent.futures import ThreadPoolExecutor

    threads = threads or min(32, os.cpu_count() or 1)
    shape = (rows,) if width == 1 else (rows, width)
    out = np.empty(shape, dtype=dtype)
    step = max(1 << 20, -(-rows // (4 * threads)))

    def fill(lo):
        n = min(step, rows - lo)
        out[lo:lo + n] = make(lo, n)

    with ThreadPoolExecutor(threads) as ex:
        list(ex.map(fill, range(0, rows, step)))
    return out


def parallel_keys(kind: int, rows: int, seed: int, key_seed: int, domain: int = 0, match_permille: int = 1000,
                  theta: float = 1.0, threads: int = 0) -> np.ndarray:
    """gen_keys (kinds 0, 1, 3, 4) or gen_zipf_keys (kind 5) in parallel chunks."""
    if kind == 5:
        return parallel_rows(rows, lambda lo, n: gen_zipf_keys(n, seed, key_seed, domain, theta, start=lo), np.uint64, threads=threads)
    return parallel_rows(rows, lambda lo, n: gen_keys(kind, n, seed, key_seed, domain, match_permille, start=lo, total=rows),
                         np.uint64, threads=threads)


def parallel_payloads(seed: int, types: Sequence[int], rows: int, threads: int = 0) -> List[np.ndarray]:
    """payload_columns in parallel chunks."""
    cols = []
    for c, t in enumerate(types):
        def make(lo, n, c=c, t=t):
            return payload_columns(seed, [U8] * c + [t], n, start=lo)[c]
        cols.append(parallel_rows(rows, make, np.uint64 if t == U128 else _DT[t], width=2 if t == U128 else 1, threads=threads))
    return cols
