"""ctypes access to the oracle (liboracle.so) and, when it was built, to the
reference itself (_ref/libphjref.so).

TEST INFRASTRUCTURE ONLY: used by tests/, by bench.py's CPU-baseline leg and
by __graft_entry__.smoke() as the checker -- never by the product path.

Streams are any object with ``types`` (payload type codes), ``keys``
(uint64 array) and ``payloads`` (list of arrays; u128 as (rows, 2) uint64),
e.g. phj_gpu.BlockStream.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
WIDTH = {0: 1, 1: 2, 2: 4, 3: 8, 4: 16}


class OStream(C.Structure):
    _fields_ = [("rows", C.c_uint64), ("keys", C.c_void_p), ("n_payloads", C.c_uint32),
                ("types", C.c_uint8 * 8), ("cols", C.c_void_p * 8)]


_lib = None
_ref = None


def build():
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        P = C.c_void_p
        S = C.POINTER(OStream)
        U64P = C.POINTER(C.c_uint64)
        L.oracle_int_hash64.restype = C.c_uint64
        L.oracle_int_hash64.argtypes = [C.c_uint64]
        L.oracle_row_width.restype = C.c_uint64
        L.oracle_row_width.argtypes = [S, S]
        L.oracle_join_count.restype = C.c_int64
        L.oracle_join_count.argtypes = [S, S]
        L.oracle_join_rows.restype = C.c_int64
        L.oracle_join_rows.argtypes = [S, S, P, C.c_uint64]
        L.oracle_serialize_columns.restype = None
        L.oracle_serialize_columns.argtypes = [C.c_uint64, P, C.c_uint32, P, P, C.c_uint32, P, P, P]
        L.oracle_sort_rows.restype = None
        L.oracle_sort_rows.argtypes = [P, C.c_uint64, C.c_uint64]
        L.oracle_compare_rows.restype = C.c_int64
        L.oracle_compare_rows.argtypes = [P, C.c_uint64, P, C.c_uint64, C.c_uint64]
        L.oracle_join_fingerprint.restype = None
        L.oracle_join_fingerprint.argtypes = [S, S, C.c_uint32, U64P]
        L.oracle_columns_fingerprint.restype = None
        L.oracle_columns_fingerprint.argtypes = [C.c_uint64, P, C.c_uint32, P, P, C.c_uint32, P, P, U64P]
        L.oracle_rows_fingerprint.restype = None
        L.oracle_rows_fingerprint.argtypes = [P, C.c_uint64, C.c_uint32, P, C.c_uint32, P, U64P]
        L.oracle_leaf_ids.restype = None
        L.oracle_leaf_ids.argtypes = [P, C.c_uint64, C.c_uint32, P]
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(os.path.join(HERE, "_ref", "libphjref.so"))


def ref():
    """The reference compiled from its own sources (absent on a GPU machine)."""
    global _ref
    if _ref is None:
        R = C.CDLL(os.path.join(HERE, "_ref", "libphjref.so"))
        P = C.c_void_p
        S = C.POINTER(OStream)
        R.ref_int_hash64.restype = C.c_uint64
        R.ref_int_hash64.argtypes = [C.c_uint64]
        R.ref_generate_keys.restype = None
        R.ref_generate_keys.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64, C.c_uint64, P, P]
        R.ref_reference_rows.restype = C.c_int64
        R.ref_reference_rows.argtypes = [S, S, C.c_uint64, P, C.c_uint64, C.c_uint64]
        R.ref_run_scheme.restype = C.c_int64
        R.ref_run_scheme.argtypes = [C.c_int, S, S, C.c_uint64, P, C.c_uint32, C.c_uint64, C.c_uint64, P, C.c_uint64,
                                     C.c_uint64, C.POINTER(C.c_double)]
        R.ref_time_scheme.restype = C.c_double
        R.ref_time_scheme.argtypes = [C.c_int, S, S, C.c_uint64, P, C.c_uint32, C.c_uint64, C.c_uint64,
                                      C.POINTER(C.c_uint64)]
        R.ref_radix_shuffle_keys.restype = C.c_int64
        R.ref_radix_shuffle_keys.argtypes = [S, C.c_uint64, P, C.c_uint32, C.c_uint64, P, P]
        _ref = R
    return _ref


def ostream(s) -> OStream:
    o = OStream()
    o.rows = len(s.keys)
    o.keys = s.keys.ctypes.data if len(s.keys) else None
    o.n_payloads = len(s.types)
    for i, (t, p) in enumerate(zip(s.types, s.payloads)):
        o.types[i] = t
        o.cols[i] = p.ctypes.data if len(s.keys) else None
    o._keep = s  # keep arrays alive
    return o


def row_width(build, probe) -> int:
    return 8 + sum(WIDTH[t] for t in build.types) + sum(WIDTH[t] for t in probe.types)


def int_hash64(x: int) -> int:
    return lib().oracle_int_hash64(x)


def join_count(build, probe) -> int:
    return lib().oracle_join_count(C.byref(ostream(build)), C.byref(ostream(probe)))


def join_rows(build, probe) -> np.ndarray:
    """referenceOutput (src/Reference.cpp:48-76) as an (n, width) uint8 array."""
    b, p = ostream(build), ostream(probe)
    n = lib().oracle_join_count(C.byref(b), C.byref(p))
    w = row_width(build, probe)
    out = np.empty((max(n, 1), w), dtype=np.uint8)
    got = lib().oracle_join_rows(C.byref(b), C.byref(p), out.ctypes.data, n)
    assert got == n
    return out[:n]


def _ptrs(cols):
    arr = (C.c_void_p * 8)()
    for i, c in enumerate(cols):
        arr[i] = c.ctypes.data
    return arr


def _types(ts):
    return (C.c_uint8 * 8)(*ts)


def serialize_output(out) -> np.ndarray:
    """serializeOutput (src/Reference.cpp:79-110) of a columnar JoinOutput."""
    n = len(out.keys)
    w = 8 + sum(WIDTH[t] for t in out.left_types) + sum(WIDTH[t] for t in out.right_types)
    rows = np.empty((max(n, 1), w), dtype=np.uint8)
    if n:
        lib().oracle_serialize_columns(n, out.keys.ctypes.data, len(out.left_types), _types(out.left_types), _ptrs(out.left),
                                       len(out.right_types), _types(out.right_types), _ptrs(out.right), rows.ctypes.data)
    return rows[:n]


def sort_rows(rows: np.ndarray) -> np.ndarray:
    rows = np.ascontiguousarray(rows)
    if len(rows):
        lib().oracle_sort_rows(rows.ctypes.data, rows.shape[0], rows.shape[1])
    return rows


def compare_outputs(expected: np.ndarray, actual: np.ndarray) -> str:
    """compareOutputs (src/Reference.cpp:113-133): '' when equal."""
    if len(expected) != len(actual):
        return f"row count mismatch: expected {len(expected)}, actual {len(actual)}"
    if len(expected) == 0:
        return ""
    e, a = np.ascontiguousarray(expected).copy(), np.ascontiguousarray(actual).copy()
    r = lib().oracle_compare_rows(e.ctypes.data, len(e), a.ctypes.data, len(a), e.shape[1])
    if r == -1:
        return ""
    return f"row content mismatch at position {r}"


def digest(rows: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(sort_rows(rows.copy())).tobytes()).hexdigest()


def join_fingerprint(build, probe, threads: int = 0) -> tuple:
    fp = (C.c_uint64 * 3)()
    lib().oracle_join_fingerprint(C.byref(ostream(build)), C.byref(ostream(probe)), threads or (os.cpu_count() or 1), fp)
    return (fp[0], fp[1], fp[2])


def columns_fingerprint(out) -> tuple:
    fp = (C.c_uint64 * 3)()
    n = len(out.keys)
    lib().oracle_columns_fingerprint(n, out.keys.ctypes.data if n else None, len(out.left_types), _types(out.left_types),
                                     _ptrs(out.left), len(out.right_types), _types(out.right_types), _ptrs(out.right), fp)
    return (fp[0], fp[1], fp[2])


def rows_fingerprint(rows: np.ndarray, left_types, right_types) -> tuple:
    fp = (C.c_uint64 * 3)()
    rows = np.ascontiguousarray(rows)
    lib().oracle_rows_fingerprint(rows.ctypes.data if len(rows) else None, len(rows), len(left_types), _types(left_types),
                                  len(right_types), _types(right_types), fp)
    return (fp[0], fp[1], fp[2])


def leaf_ids(keys: np.ndarray, total_bits: int) -> np.ndarray:
    keys = np.ascontiguousarray(keys, dtype=np.uint64)
    out = np.empty(len(keys), dtype=np.uint32)
    if len(keys):
        lib().oracle_leaf_ids(keys.ctypes.data, len(keys), total_bits, out.ctypes.data)
    return out


# ---- the reference itself (only where its sources were compiled) ----------

def ref_reference_rows(build, probe, block_rows: int = 10_000) -> np.ndarray:
    b, p = ostream(build), ostream(probe)
    n = lib().oracle_join_count(C.byref(b), C.byref(p))
    w = row_width(build, probe)
    out = np.empty((max(n, 1), w), dtype=np.uint8)
    got = ref().ref_reference_rows(C.byref(b), C.byref(p), block_rows, out.ctypes.data, max(n, 1), w)
    assert got >= 0, got
    return out[:got]


def ref_run_scheme(scheme: int, build, probe, pass_bits, threads: int = 4, budget_mib: int = 512, block_rows: int = 10_000):
    """Runs reference runCHJ (0) / runPHJ (1) / runPhjBep (2); returns (sorted rows, stats)."""
    b, p = ostream(build), ostream(probe)
    n = lib().oracle_join_count(C.byref(b), C.byref(p))
    w = row_width(build, probe)
    out = np.empty((max(n, 1), w), dtype=np.uint8)
    bits = (C.c_uint8 * len(pass_bits))(*pass_bits)
    stats = (C.c_double * 5)()
    got = ref().ref_run_scheme(scheme, C.byref(b), C.byref(p), block_rows, bits, len(pass_bits), threads, budget_mib,
                               out.ctypes.data, max(n, 1), w, stats)
    assert got >= 0, got
    return out[:got], list(stats)


# ---- the CPU port of the reference's schemes (cpu_port.cpp) -----------------

class PortStream(C.Structure):
    _fields_ = [("rows", C.c_uint64), ("keys", C.c_void_p), ("n_payloads", C.c_uint32), ("types", C.c_uint8 * 8),
                ("cols", C.c_void_p * 8), ("block_rows", C.c_uint32)]


_port = None


def port():
    global _port
    if _port is None:
        path = os.path.join(HERE, "libcpuport.so")
        if not os.path.exists(path):
            subprocess.run(["make", "-s", "-C", HERE, "libcpuport.so"], check=True)
        L = C.CDLL(path)
        S = C.POINTER(PortStream)
        FP = C.POINTER(C.c_uint64)
        L.port_run_phj_pure.restype = C.c_int64
        L.port_run_phj_pure.argtypes = [S, S, C.POINTER(C.c_uint8), C.c_uint32, C.c_uint32, C.POINTER(C.c_double), FP]
        L.port_run_chj.restype = C.c_int64
        L.port_run_chj.argtypes = [S, S, C.c_uint32, C.POINTER(C.c_double), FP]
        L.port_run_phj_bep.restype = C.c_int64
        L.port_run_phj_bep.argtypes = [S, S, C.POINTER(C.c_uint8), C.c_uint32, C.c_uint32, C.c_uint64, C.POINTER(C.c_double),
                                       C.POINTER(C.c_uint64), FP]
        _port = L
    return _port


def port_stream(s, block_rows: int = 10_000) -> PortStream:
    o = PortStream()
    o.rows = len(s.keys)
    o.keys = s.keys.ctypes.data if len(s.keys) else None
    o.n_payloads = len(s.types)
    for i, (t, p) in enumerate(zip(s.types, s.payloads)):
        o.types[i] = t
        o.cols[i] = p.ctypes.data if len(s.keys) else None
    o.block_rows = block_rows
    o._keep = s
    return o


def port_run(scheme: str, build, probe, pass_bits=(8,), threads: int = 0, budget_mib: int = 512, fingerprint: bool = False):
    """Times the CPU port of the reference's runPHJ ('phj-pure'), runCHJ
    ('chj') or runPhjBep ('phj').  Returns (output rows, phase ms dict);
    for 'phj' the dict also holds the BEP counters.  With `fingerprint` the
    dict holds the oracle fingerprint of the rows the port materialised
    (computed after the timed region)."""
    threads = threads or (os.cpu_count() or 1)
    ms = (C.c_double * 6)()
    fp = (C.c_uint64 * 3)() if fingerprint else None
    b, p = port_stream(build), port_stream(probe)
    if scheme == "phj-pure":
        bits = (C.c_uint8 * len(pass_bits))(*pass_bits)
        n = port().port_run_phj_pure(C.byref(b), C.byref(p), bits, len(pass_bits), threads, ms, fp)
        d = {"build_shuffle": ms[0], "build": ms[1], "probe_shuffle": ms[2], "probe": ms[3], "e2e": ms[4]}
    elif scheme == "phj":
        bits = (C.c_uint8 * len(pass_bits))(*pass_bits)
        ctr = (C.c_uint64 * 4)()
        n = port().port_run_phj_bep(C.byref(b), C.byref(p), bits, len(pass_bits), threads, budget_mib, ms, ctr, fp)
        d = {"build_shuffle": ms[0], "build": ms[1], "probe_shuffle": ms[2], "probe": ms[3], "eviction_overhead": ms[4],
             "e2e": ms[5], "bep_evictions": ctr[0], "bep_refinements": ctr[1], "bep_peak_bytes": ctr[2],
             "bep_build_skip_retries": ctr[3]}
    else:
        n = port().port_run_chj(C.byref(b), C.byref(p), threads, ms, fp)
        d = {"build": ms[0], "probe": ms[1], "e2e": ms[2]}
    if fingerprint:
        d["fingerprint"] = (fp[0], fp[1], fp[2])
    return n, d


def ref_time(scheme: str, build, probe, pass_bits=(8,), threads: int = 0, budget_mib: int = 512):
    """Times the reference itself (only where it was compiled)."""
    threads = threads or (os.cpu_count() or 1)
    code = {"chj": 0, "phj-pure": 1, "phj": 2}[scheme]
    b, p = ostream(build), ostream(probe)
    bits = (C.c_uint8 * len(pass_bits))(*pass_bits)
    rows = C.c_uint64()
    ms = ref().ref_time_scheme(code, C.byref(b), C.byref(p), 10_000, bits, len(pass_bits), threads, budget_mib, C.byref(rows))
    return rows.value, ms
