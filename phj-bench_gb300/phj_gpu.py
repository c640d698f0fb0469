"""ctypes binding of include/phj_gpu.h, the C ABI of the GB300 hash-join path.

Python-side mirror of the reference's scheme interface for tests and the
benchmark: ``BlockStream`` stands for ``phj::BlockStream`` (src/Block.h:157-162)
with its blocks laid end to end, and ``runCHJ`` / ``runPHJ`` / ``runPhjBep``
take the same arguments as the reference's entry points (src/CHJ.h:31,
src/PHJ.h:31, src/PHJBep.h:97-98) and return result objects with the same
fields (``build``, ``probe``, ``e2e_wall_ms``, ``peak_mem_bytes``, ``output``
...).  Errors the reference throws (std::invalid_argument) raise
``PhjError`` here.  There is no fallback: every call goes through
libphj_gpu.so and fails loudly if the library or a GPU is missing.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("PHJ_GPU_LIB") or os.path.join(HERE, "libphj_gpu.so")
MAX_PAYLOADS = 8
ABI_VERSION = 3  # PHJ_GPU_ABI_VERSION of include/phj_gpu.h these structures follow

# PayloadType codes, src/Types.h:23-30
U8, U16, U32, U64, U128 = 0, 1, 2, 3, 4
TYPE_NAMES = {"u8": U8, "u16": U16, "u32": U32, "u64": U64, "u128": U128}
TYPE_WIDTH = {U8: 1, U16: 2, U32: 4, U64: 8, U128: 16}
TYPE_DTYPE = {U8: np.uint8, U16: np.uint16, U32: np.uint32, U64: np.uint64}
PIPELINE_BLOCK_ROWS = 10_000  # src/Types.h:107

STATUS = {
    0: "PHJ_OK", 1: "PHJ_ERR_INVALID_ARGUMENT", 2: "PHJ_ERR_CUDA", 3: "PHJ_ERR_OUT_OF_MEMORY",
    4: "PHJ_ERR_UNSUPPORTED", 5: "PHJ_ERR_DEVICE_TIMEOUT", 6: "PHJ_ERR_NO_DEVICE", 7: "PHJ_ERR_CAPACITY",
}
ERR_INVALID_ARGUMENT, ERR_CUDA, ERR_DEVICE_TIMEOUT, ERR_CAPACITY = 1, 2, 5, 7


class PhjError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


class Schema(C.Structure):
    _fields_ = [("n_payloads", C.c_uint32), ("types", C.c_uint8 * MAX_PAYLOADS)]


class BlockStreamDesc(C.Structure):
    _fields_ = [
        ("schema", Schema), ("total_rows", C.c_uint64), ("n_blocks", C.c_uint32),
        ("block_rows", C.POINTER(C.c_uint32)), ("keys", C.c_void_p),
        ("payloads", C.c_void_p * MAX_PAYLOADS), ("location", C.c_int32),
    ]


class PhaseTiming(C.Structure):
    _fields_ = [("wall_ms", C.c_double), ("ns_per_row", C.c_double)]

    def __repr__(self):
        return f"PhaseTiming(wall_ms={self.wall_ms:.4f}, ns_per_row={self.ns_per_row:.4f})"


class ChjResultC(C.Structure):
    _fields_ = [("build", PhaseTiming), ("probe", PhaseTiming), ("e2e_wall_ms", C.c_double), ("peak_mem_bytes", C.c_uint64)]


class PhjResultC(C.Structure):
    _fields_ = [("build_shuffle", PhaseTiming), ("build", PhaseTiming), ("probe_shuffle", PhaseTiming), ("probe", PhaseTiming),
                ("e2e_wall_ms", C.c_double), ("peak_mem_bytes", C.c_uint64)]


class BepResultC(C.Structure):
    _fields_ = [("build_shuffle", PhaseTiming), ("build", PhaseTiming), ("probe_shuffle", PhaseTiming), ("probe", PhaseTiming),
                ("eviction_overhead", PhaseTiming), ("e2e_wall_ms", C.c_double), ("peak_mem_bytes", C.c_uint64),
                ("bep_budget_mib", C.c_uint64), ("bep_evictions", C.c_uint64), ("bep_refinements", C.c_uint64),
                ("bep_peak_bytes", C.c_uint64), ("bep_build_skip_retries", C.c_uint64)]


class GenSpec(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("rows", C.c_uint64), ("seed", C.c_uint64), ("key_seed", C.c_uint64),
                ("domain", C.c_uint64), ("match_permille", C.c_uint32), ("theta", C.c_double), ("schema", Schema),
                ("block_rows", C.c_uint32)]


class KernelTime(C.Structure):
    _fields_ = [("name", C.c_char * 32), ("ms", C.c_double), ("rows", C.c_uint64), ("bytes", C.c_uint64), ("start_ms", C.c_double)]


class BatchResultC(C.Structure):
    _fields_ = [("e2e_wall_ms", C.c_double), ("n_joins", C.c_uint32), ("build_rows", C.c_uint64), ("probe_rows", C.c_uint64),
                ("output_rows", C.c_uint64), ("peak_mem_bytes", C.c_uint64)]


class ServeConfig(C.Structure):
    _fields_ = [("device", C.c_int), ("workers", C.c_uint32), ("hbm_budget_bytes", C.c_uint64),
                ("batch_max_build_rows", C.c_uint64), ("batch_max_joins", C.c_uint32), ("pass_bits", C.c_uint8 * 8),
                ("n_passes", C.c_uint32)]


class ServeRequest(C.Structure):
    _fields_ = [("build", GenSpec), ("probe", GenSpec), ("arrival_s", C.c_double)]


class ServeRecord(C.Structure):
    _fields_ = [("id", C.c_uint64), ("arrival_s", C.c_double), ("admit_s", C.c_double), ("start_s", C.c_double),
                ("done_s", C.c_double), ("build_rows", C.c_uint64), ("probe_rows", C.c_uint64), ("output_rows", C.c_uint64),
                ("footprint_bytes", C.c_uint64), ("fingerprint", C.c_uint64 * 3), ("batch_size", C.c_uint32), ("slot", C.c_uint32),
                ("status", C.c_int32), ("job_peak_bytes", C.c_uint64), ("gen_s", C.c_double), ("call_s", C.c_double),
                ("device_ms", C.c_double)]


_lib = None


def load() -> C.CDLL:
    """Loads libphj_gpu.so (built by __graft_entry__.build() / make)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with `make -C phj-bench_gb300` (no CPU fallback exists)")
    lib = C.CDLL(LIB_PATH)
    P = C.c_void_p
    sig = {
        "phj_abi_version": (C.c_uint32, []),
        "phj_ctx_create": (C.c_int, [C.c_int, C.POINTER(P)]),
        "phj_ctx_destroy": (None, [P]),
        "phj_last_error": (C.c_char_p, [P]),
        "phj_ctx_stream": (P, [P]),
        "phj_ctx_set_int": (C.c_int, [P, C.c_char_p, C.c_int64]),
        "phj_ctx_get_int": (C.c_int, [P, C.c_char_p, C.POINTER(C.c_int64)]),
        "phj_resolve_radix": (C.c_int, [C.c_uint64, C.c_uint32, C.POINTER(C.c_uint8), C.c_uint32, C.POINTER(C.c_uint8),
                                        C.POINTER(C.c_uint32)]),
        "phj_table_upload": (C.c_int, [P, C.POINTER(BlockStreamDesc), C.POINTER(P)]),
        "phj_table_wrap_device": (C.c_int, [P, C.POINTER(BlockStreamDesc), C.POINTER(P)]),
        "phj_table_generate": (C.c_int, [P, C.POINTER(GenSpec), C.POINTER(P)]),
        "phj_table_download": (C.c_int, [P, P, P, C.POINTER(C.c_void_p)]),
        "phj_radix_shuffle": (C.c_int, [P, P, C.POINTER(C.c_uint8), C.c_uint32, C.POINTER(P), P]),
        "phj_table_rows": (C.c_uint64, [P]),
        "phj_table_gen_distinct": (C.c_uint64, [P]),
        "phj_table_free": (None, [P, P]),
        "phj_run_chj": (C.c_int, [P, P, P, C.POINTER(P), C.POINTER(ChjResultC)]),
        "phj_run_phj_pure": (C.c_int, [P, P, P, C.POINTER(C.c_uint8), C.c_uint32, C.POINTER(P), C.POINTER(PhjResultC)]),
        "phj_run_phj_pure_host": (C.c_int, [P, C.POINTER(BlockStreamDesc), C.POINTER(BlockStreamDesc), C.POINTER(C.c_uint8), C.c_uint32,
                                            C.c_uint64, P, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.POINTER(C.c_uint64),
                                            C.POINTER(PhjResultC)]),
        "phj_run_phj_bep_host": (C.c_int, [P, C.POINTER(BlockStreamDesc), C.POINTER(BlockStreamDesc), C.POINTER(C.c_uint8), C.c_uint32,
                                           C.c_uint64, C.c_uint64, P, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.POINTER(C.c_uint64),
                                           C.POINTER(BepResultC)]),
        "phj_run_phj_bep": (C.c_int, [P, P, P, C.POINTER(C.c_uint8), C.c_uint32, C.c_uint64, C.c_uint32, C.POINTER(P),
                                      C.POINTER(BepResultC)]),
        "phj_autotune_radix": (C.c_int, [C.c_uint64, C.c_uint64, C.POINTER(C.c_uint8), C.POINTER(C.c_uint32)]),
        "phj_batch_run": (C.c_int, [P, C.c_uint32, C.POINTER(P), C.POINTER(P), C.POINTER(P), C.POINTER(BatchResultC)]),
        "phj_serve_create": (C.c_int, [C.POINTER(ServeConfig), C.POINTER(P)]),
        "phj_serve_submit": (C.c_int, [P, C.POINTER(ServeRequest), C.POINTER(C.c_uint64)]),
        "phj_serve_start": (C.c_int, [P]),
        "phj_serve_wait": (C.c_int, [P, C.c_double]),
        "phj_serve_records": (C.c_uint32, [P, C.POINTER(ServeRecord), C.c_uint32]),
        "phj_serve_error": (C.c_char_p, [P]),
        "phj_serve_destroy": (None, [P]),
        "phj_serve_footprint": (C.c_uint64, [C.POINTER(ServeRequest), C.c_int]),
        "phj_run_chj_noalloc": (C.c_int, [P, P, P, C.c_uint64, P, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                          C.POINTER(C.c_uint64)]),
        "phj_output_rows": (C.c_uint64, [P]),
        "phj_output_device_columns": (C.c_int, [P, C.POINTER(P), C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
        "phj_output_download": (C.c_int, [P, P, P, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
        "phj_output_fingerprint": (C.c_int, [P, P, C.POINTER(C.c_uint64)]),
        "phj_output_free": (None, [P, P]),
        "phj_last_kernel_times": (C.c_uint32, [P, C.POINTER(KernelTime), C.c_uint32]),
        "phj_launch_count": (C.c_uint64, [P]),
        "phj_host_alloc": (C.c_int, [P, C.c_size_t, C.POINTER(P)]),
        "phj_host_free": (None, [P, P]),
        "phj_flush_l2": (C.c_int, [P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.phj_abi_version() != ABI_VERSION:
        raise ImportError(f"{LIB_PATH} has ABI version {lib.phj_abi_version()}, these bindings need {ABI_VERSION}: rebuild it")
    _lib = lib
    return lib


def resolve_radix(partitions: int = 256, passes: int = 1, bits_per_pass: Optional[Sequence[int]] = None) -> List[int]:
    """--partitions / --passes / --partition-bits-per-pass resolution (src/CLI.cpp:330-355)."""
    lib = load()
    out = (C.c_uint8 * 32)()
    n = C.c_uint32()
    if bits_per_pass:
        arr = (C.c_uint8 * len(bits_per_pass))(*bits_per_pass)
        st = lib.phj_resolve_radix(0, 0, arr, len(bits_per_pass), out, C.byref(n))
    else:
        st = lib.phj_resolve_radix(partitions, passes, None, 0, out, C.byref(n))
    if st != 0:
        raise PhjError(st, "invalid radix configuration")
    return [out[i] for i in range(n.value)]


# ---------------------------------------------------------------------------
# Host-side streams
# ---------------------------------------------------------------------------
def column_view(arr: np.ndarray, t: int) -> np.ndarray:
    """Column storage: u8..u64 as their dtype, u128 as (rows, 2) uint64 (low, high)."""
    if t == U128:
        a = np.ascontiguousarray(arr, dtype=np.uint64)
        assert a.ndim == 2 and a.shape[1] == 2
        return a
    return np.ascontiguousarray(arr, dtype=TYPE_DTYPE[t])


@dataclass
class BlockStream:
    """phj::BlockStream (src/Block.h:157-162) with blocks laid end to end."""
    types: List[int]
    keys: np.ndarray
    payloads: List[np.ndarray]
    block_rows: Optional[np.ndarray] = None  # rows per block; None = PIPELINE_BLOCK_ROWS blocks

    def __post_init__(self):
        self.keys = np.ascontiguousarray(self.keys, dtype=np.uint64)
        if self.keys.ndim != 1:
            raise PhjError(ERR_INVALID_ARGUMENT, "the key column must be one-dimensional")
        if len(self.payloads) != len(self.types) or len(self.types) > MAX_PAYLOADS:
            raise PhjError(ERR_INVALID_ARGUMENT, f"{len(self.payloads)} payload columns for {len(self.types)} types")
        self.payloads = [column_view(p, t) for p, t in zip(self.payloads, self.types)]
        n = len(self.keys)
        for i, p in enumerate(self.payloads):
            if len(p) != n:
                raise PhjError(ERR_INVALID_ARGUMENT, f"payload column {i} has {len(p)} rows, the keys {n}")
        if self.block_rows is None:
            full, rem = divmod(n, PIPELINE_BLOCK_ROWS)
            self.block_rows = np.array([PIPELINE_BLOCK_ROWS] * full + ([rem] if rem else []), dtype=np.uint32)
        self.block_rows = np.ascontiguousarray(self.block_rows, dtype=np.uint32)
        if int(self.block_rows.sum(dtype=np.uint64)) != n:
            raise PhjError(ERR_INVALID_ARGUMENT, "block_rows do not add up to the rows of the stream")

    @property
    def total_rows(self) -> int:
        return len(self.keys)

    def schema(self) -> Schema:
        s = Schema()
        s.n_payloads = len(self.types)
        for i, t in enumerate(self.types):
            s.types[i] = t
        return s


def _schema_of(types: Sequence[int]) -> Schema:
    s = Schema()
    s.n_payloads = len(types)
    for i, t in enumerate(types):
        s.types[i] = t
    return s


@dataclass
class JoinOutput:
    """phj::JoinOutput (src/JoinOutput.h:55-70) as one block of columns."""
    left_types: List[int]
    right_types: List[int]
    keys: np.ndarray
    left: List[np.ndarray]
    right: List[np.ndarray]

    def totalRows(self) -> int:
        return len(self.keys)


@dataclass
class SchemeResult:
    output: Optional[JoinOutput]
    e2e_wall_ms: float
    peak_mem_bytes: int
    phases: dict = field(default_factory=dict)
    counters: dict = field(default_factory=dict)
    fingerprint: Optional[tuple] = None
    output_rows: int = 0

    def __getattr__(self, name):
        phases = self.__dict__.get("phases", {})
        if name in phases:
            return phases[name]
        counters = self.__dict__.get("counters", {})
        if name in counters:
            return counters[name]
        raise AttributeError(name)


class Table:
    """A device-resident stream (phj_table)."""

    def __init__(self, ctx: "Context", handle: C.c_void_p, types: Sequence[int]):
        self.ctx, self.handle, self.types = ctx, handle, list(types)

    @property
    def rows(self) -> int:
        return self.ctx.lib.phj_table_rows(self.handle)

    @property
    def gen_distinct(self) -> int:
        return self.ctx.lib.phj_table_gen_distinct(self.handle)

    def download(self) -> BlockStream:
        n = self.rows
        keys = np.empty(n, dtype=np.uint64)
        cols = [np.empty((n, 2), dtype=np.uint64) if t == U128 else np.empty(n, dtype=TYPE_DTYPE[t]) for t in self.types]
        ptrs = (C.c_void_p * MAX_PAYLOADS)(*[c.ctypes.data for c in cols])
        self.ctx._check(self.ctx.lib.phj_table_download(self.ctx.ptr, self.handle, keys.ctypes.data, ptrs))
        return BlockStream(self.types, keys, cols)

    def free(self):
        if self.handle:
            self.ctx.lib.phj_table_free(self.ctx.ptr, self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Output:
    def __init__(self, ctx: "Context", handle, left_types, right_types):
        self.ctx, self.handle, self.left_types, self.right_types = ctx, handle, list(left_types), list(right_types)

    @property
    def rows(self) -> int:
        return self.ctx.lib.phj_output_rows(self.handle)

    def download(self, host_buffers=None) -> JoinOutput:
        n = self.rows

        def alloc(t):
            return np.empty((n, 2), dtype=np.uint64) if t == U128 else np.empty(n, dtype=TYPE_DTYPE[t])
        if host_buffers is None:
            keys = np.empty(n, dtype=np.uint64)
            left = [alloc(t) for t in self.left_types]
            right = [alloc(t) for t in self.right_types]
        else:
            keys, left, right = host_buffers
        lp = (C.c_void_p * MAX_PAYLOADS)(*[c.ctypes.data for c in left])
        rp = (C.c_void_p * MAX_PAYLOADS)(*[c.ctypes.data for c in right])
        self.ctx._check(self.ctx.lib.phj_output_download(self.ctx.ptr, self.handle, keys.ctypes.data, lp, rp))
        if host_buffers is not None:
            keys, left, right = keys[:n], [c[:n] for c in left], [c[:n] for c in right]
        return JoinOutput(self.left_types, self.right_types, keys, left, right)

    def fingerprint(self) -> tuple:
        fp = (C.c_uint64 * 3)()
        self.ctx._check(self.ctx.lib.phj_output_fingerprint(self.ctx.ptr, self.handle, fp))
        return (fp[0], fp[1], fp[2])

    def free(self):
        if self.handle:
            self.ctx.lib.phj_output_free(self.ctx.ptr, self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Context:
    """One device, one stream (phj_ctx)."""

    def __init__(self, device: int = 0):
        self.lib = load()
        p = C.c_void_p()
        st = self.lib.phj_ctx_create(device, C.byref(p))
        if st != 0:
            raise PhjError(st, "phj_ctx_create failed (is a GB300 visible?)")
        self.ptr = p
        self._pinned = []  # phj_host_alloc blocks of pinned(), freed by close()

    def close(self):
        """Destroys the context and frees the pinned host memory that
        pinned() handed out (arrays over it must not be used afterwards)."""
        if self.ptr:
            for h in self._pinned:
                self.lib.phj_host_free(self.ptr, h)
            self._pinned = []
            self.lib.phj_ctx_destroy(self.ptr)
            self.ptr = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st: int):
        if st != 0:
            raise PhjError(st, self.lib.phj_last_error(self.ptr).decode())

    def set_int(self, name: str, value: int):
        self._check(self.lib.phj_ctx_set_int(self.ptr, name.encode(), int(value)))

    def get_int(self, name: str) -> int:
        v = C.c_int64()
        self._check(self.lib.phj_ctx_get_int(self.ptr, name.encode(), C.byref(v)))
        return v.value

    # ---- streams ----
    @staticmethod
    def _desc(s: BlockStream) -> "BlockStreamDesc":
        d = BlockStreamDesc()
        d.schema = s.schema()
        d.total_rows = s.total_rows
        d.n_blocks = len(s.block_rows)
        d.block_rows = s.block_rows.ctypes.data_as(C.POINTER(C.c_uint32)) if len(s.block_rows) else None
        d.keys = s.keys.ctypes.data if s.total_rows else None
        for i, p in enumerate(s.payloads):
            d.payloads[i] = p.ctypes.data if s.total_rows else None
        d.location = 0
        return d

    @staticmethod
    def _host_out(build: BlockStream, probe: BlockStream, out_keys: np.ndarray, out_left: Sequence[np.ndarray],
                  out_right: Sequence[np.ndarray]):
        """Column pointers of caller-owned host output columns, checked
        against the two schemas: the library writes up to len(out_keys) rows
        into every column, so each must be contiguous, of its type and at
        least that long."""
        def check(a, dtype, what, cols=None):
            if not isinstance(a, np.ndarray) or a.dtype != dtype or not a.flags.c_contiguous:
                raise PhjError(ERR_INVALID_ARGUMENT, f"{what}: a C-contiguous {np.dtype(dtype).name} array is required")
            if (a.ndim, a.shape[1:]) != ((2, (cols,)) if cols else (1, ())) or len(a) < len(out_keys):
                raise PhjError(ERR_INVALID_ARGUMENT, f"{what}: shape {a.shape} cannot hold {len(out_keys)} rows")

        check(out_keys, np.uint64, "output keys")
        ptrs = []
        for side, types, cols in (("left", build.types, out_left), ("right", probe.types, out_right)):
            if len(cols) != len(types):
                raise PhjError(ERR_INVALID_ARGUMENT, f"{len(cols)} {side} output columns for {len(types)} payload types")
            for i, (c, t) in enumerate(zip(cols, types)):
                check(c, np.uint64 if t == U128 else TYPE_DTYPE[t], f"{side} output column {i}", 2 if t == U128 else None)
            ptrs.append((C.c_void_p * MAX_PAYLOADS)(*[c.ctypes.data for c in cols]))
        return ptrs

    def run_phj_pure_host(self, build: BlockStream, probe: BlockStream, pass_bits: Sequence[int], out_keys: np.ndarray,
                          out_left: Sequence[np.ndarray], out_right: Sequence[np.ndarray]):
        """phj_run_phj_pure_host: host inputs, host output columns (pinned
        for full speed).  Returns (output rows, PhjResultC)."""
        db, dp = self._desc(build), self._desc(probe)
        bits = (C.c_uint8 * max(1, len(pass_bits)))(*pass_bits)
        lp, rp = self._host_out(build, probe, out_keys, out_left, out_right)
        rows = C.c_uint64()
        r = PhjResultC()
        self._check(self.lib.phj_run_phj_pure_host(self.ptr, C.byref(db), C.byref(dp), bits, len(pass_bits), len(out_keys),
                                                   out_keys.ctypes.data, lp, rp, C.byref(rows), C.byref(r)))
        return rows.value, r

    def run_phj_bep_host(self, build: BlockStream, probe: BlockStream, pass_bits: Sequence[int], budget_mib: int, out_keys: np.ndarray,
                         out_left: Sequence[np.ndarray], out_right: Sequence[np.ndarray]):
        """phj_run_phj_bep_host: host inputs, host output columns (pinned
        for full speed).  Returns (output rows, BepResultC)."""
        db, dp = self._desc(build), self._desc(probe)
        bits = (C.c_uint8 * max(1, len(pass_bits)))(*pass_bits)
        lp, rp = self._host_out(build, probe, out_keys, out_left, out_right)
        rows = C.c_uint64()
        r = BepResultC()
        self._check(self.lib.phj_run_phj_bep_host(self.ptr, C.byref(db), C.byref(dp), bits, len(pass_bits), budget_mib, len(out_keys),
                                                  out_keys.ctypes.data, lp, rp, C.byref(rows), C.byref(r)))
        return rows.value, r

    def upload(self, s: BlockStream) -> Table:
        d = BlockStreamDesc()
        d.schema = s.schema()
        d.total_rows = s.total_rows
        d.n_blocks = len(s.block_rows)
        d.block_rows = s.block_rows.ctypes.data_as(C.POINTER(C.c_uint32)) if len(s.block_rows) else None
        d.keys = s.keys.ctypes.data if s.total_rows else None
        for i, p in enumerate(s.payloads):
            d.payloads[i] = p.ctypes.data if s.total_rows else None
        d.location = 0
        h = C.c_void_p()
        self._check(self.lib.phj_table_upload(self.ptr, C.byref(d), C.byref(h)))
        return Table(self, h, s.types)

    def generate(self, kind: int, rows: int, seed: int, key_seed: int, types: Sequence[int], domain: int = 0,
                 match_permille: int = 1000, theta: float = 1.0, block_rows: int = PIPELINE_BLOCK_ROWS) -> Table:
        sp = GenSpec()
        sp.kind, sp.rows, sp.seed, sp.key_seed = kind, rows, seed, key_seed
        sp.domain, sp.match_permille, sp.theta = domain, match_permille, theta
        sp.schema = _schema_of(types)
        sp.block_rows = block_rows
        h = C.c_void_p()
        self._check(self.lib.phj_table_generate(self.ptr, C.byref(sp), C.byref(h)))
        return Table(self, h, types)

    # ---- the radix partition operator ----
    def radix_shuffle(self, table: Table, pass_bits: Sequence[int]):
        """radixShuffle (src/RadixPartition.cpp:546-586) on the device:
        returns (the partitioned Table, rows of every partition)."""
        bits = (C.c_uint8 * max(1, len(pass_bits)))(*pass_bits)
        counts = np.zeros(1 << min(24, sum(pass_bits)), dtype=np.uint64) if sum(pass_bits) <= 24 else None
        h = C.c_void_p()
        self._check(self.lib.phj_radix_shuffle(self.ptr, table.handle, bits, len(pass_bits), C.byref(h),
                                               counts.ctypes.data if counts is not None else None))
        return Table(self, h, table.types), counts

    # ---- schemes ----
    def run_chj(self, build: Table, probe: Table):
        r = ChjResultC()
        h = C.c_void_p()
        self._check(self.lib.phj_run_chj(self.ptr, build.handle, probe.handle, C.byref(h), C.byref(r)))
        return Output(self, h, build.types, probe.types), r

    def run_phj_pure(self, build: Table, probe: Table, pass_bits: Sequence[int]):
        r = PhjResultC()
        h = C.c_void_p()
        bits = (C.c_uint8 * max(1, len(pass_bits)))(*pass_bits)
        self._check(self.lib.phj_run_phj_pure(self.ptr, build.handle, probe.handle, bits, len(pass_bits), C.byref(h), C.byref(r)))
        return Output(self, h, build.types, probe.types), r

    def run_phj_bep(self, build: Table, probe: Table, pass_bits: Sequence[int], budget_mib: int, workers: int = 0):
        r = BepResultC()
        h = C.c_void_p()
        bits = (C.c_uint8 * max(1, len(pass_bits)))(*pass_bits)
        self._check(self.lib.phj_run_phj_bep(self.ptr, build.handle, probe.handle, bits, len(pass_bits), budget_mib, workers,
                                             C.byref(h), C.byref(r)))
        return Output(self, h, build.types, probe.types), r

    def run_chj_noalloc(self, build: Table, probe: Table, out_capacity: int, out_keys: int, out_left: Sequence[int],
                        out_right: Sequence[int]) -> int:
        """The no-allocation join into caller-owned device columns (raw
        device addresses).  Returns the join's row count; PhjError (with
        `.rows`) when it is above `out_capacity`."""
        rows = C.c_uint64(0)
        lp = (C.c_void_p * MAX_PAYLOADS)(*out_left)
        rp = (C.c_void_p * MAX_PAYLOADS)(*out_right)
        st = self.lib.phj_run_chj_noalloc(self.ptr, build.handle, probe.handle, out_capacity, out_keys, lp, rp, C.byref(rows))
        if st != 0:
            err = PhjError(st, self.lib.phj_last_error(self.ptr).decode())
            err.rows = rows.value
            raise err
        return rows.value

    def run_batch(self, builds: Sequence[Table], probes: Sequence[Table]):
        """phj_batch_run: n joins in one set of launches; returns ([Output], result)."""
        n = len(builds)
        bh = (C.c_void_p * max(n, 1))(*[b.handle for b in builds])
        ph = (C.c_void_p * max(n, 1))(*[p.handle for p in probes])
        oh = (C.c_void_p * max(n, 1))()
        r = BatchResultC()
        self._check(self.lib.phj_batch_run(self.ptr, n, bh, ph, oh, C.byref(r)))
        return [Output(self, C.c_void_p(oh[j]), builds[j].types, probes[j].types) for j in range(n)], r

    # ---- measurement ----
    def kernel_times(self) -> List[dict]:
        arr = (KernelTime * 256)()
        n = self.lib.phj_last_kernel_times(self.ptr, arr, 256)
        return [{"name": arr[i].name.decode(), "ms": arr[i].ms, "rows": arr[i].rows, "bytes": arr[i].bytes, "start_ms": arr[i].start_ms}
                for i in range(n)]

    def launch_count(self) -> int:
        return self.lib.phj_launch_count(self.ptr)

    def flush_l2(self):
        self._check(self.lib.phj_flush_l2(self.ptr))

    def pinned(self, shape, dtype) -> np.ndarray:
        """A numpy array over pinned host memory (freed with the context)."""
        nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        p = C.c_void_p()
        self._check(self.lib.phj_host_alloc(self.ptr, nbytes, C.byref(p)))
        self._pinned.append(p.value)
        buf = (C.c_uint8 * max(nbytes, 1)).from_address(p.value)
        arr = np.frombuffer(buf, dtype=np.uint8, count=nbytes).view(dtype).reshape(shape)
        return arr


# ---------------------------------------------------------------------------
# Reference-shaped entry points: runCHJ / runPHJ / runPhjBep
# ---------------------------------------------------------------------------
_default_ctx: Optional[Context] = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


def _phases(r, names):
    return {n: getattr(r, n) for n in names}


def runCHJ(build: BlockStream, probe: BlockStream, threads: int = 1, ctx: Optional[Context] = None) -> SchemeResult:
    """runCHJ (src/CHJ.h:31).  `threads` has no device meaning and is ignored."""
    ctx = ctx or default_context()
    b, p = ctx.upload(build), ctx.upload(probe)
    out, r = ctx.run_chj(b, p)
    jo = out.download()
    res = SchemeResult(jo, r.e2e_wall_ms, r.peak_mem_bytes, _phases(r, ["build", "probe"]), output_rows=out.rows)
    out.free(), b.free(), p.free()
    return res


def runPHJ(build: BlockStream, probe: BlockStream, pass_bits: Sequence[int], threads: int = 1,
           ctx: Optional[Context] = None) -> SchemeResult:
    """runPHJ (src/PHJ.h:31): `pass_bits` is RadixConfig::pass_bits."""
    ctx = ctx or default_context()
    b, p = ctx.upload(build), ctx.upload(probe)
    out, r = ctx.run_phj_pure(b, p, pass_bits)
    jo = out.download()
    res = SchemeResult(jo, r.e2e_wall_ms, r.peak_mem_bytes,
                       _phases(r, ["build_shuffle", "build", "probe_shuffle", "probe"]), output_rows=out.rows)
    out.free(), b.free(), p.free()
    return res


def runPhjBep(build: BlockStream, probe: BlockStream, pass_bits: Sequence[int], threads: int = 1, bep_budget_mib: int = 512,
              ctx: Optional[Context] = None, workers: int = 0) -> SchemeResult:
    """runPhjBep (src/PHJBep.h:97-98)."""
    ctx = ctx or default_context()
    b, p = ctx.upload(build), ctx.upload(probe)
    out, r = ctx.run_phj_bep(b, p, pass_bits, bep_budget_mib, workers)
    jo = out.download()
    res = SchemeResult(jo, r.e2e_wall_ms, r.peak_mem_bytes,
                       _phases(r, ["build_shuffle", "build", "probe_shuffle", "probe", "eviction_overhead"]),
                       counters={k: getattr(r, k) for k in ["bep_budget_mib", "bep_evictions", "bep_refinements",
                                                            "bep_peak_bytes", "bep_build_skip_retries"]},
                       output_rows=out.rows)
    out.free(), b.free(), p.free()
    return res


def gen_spec(kind: int, rows: int, seed: int, key_seed: int, types: Sequence[int], domain: int = 0, match_permille: int = 1000,
             theta: float = 1.0, block_rows: int = PIPELINE_BLOCK_ROWS) -> GenSpec:
    sp = GenSpec()
    sp.kind, sp.rows, sp.seed, sp.key_seed = kind, rows, seed, key_seed
    sp.domain, sp.match_permille, sp.theta = domain, match_permille, theta
    sp.schema = _schema_of(types)
    sp.block_rows = block_rows
    return sp


class Server:
    """The request loop (phj_serve_*): submit a trace of requests with
    arrival offsets, start, wait, read the per-request records."""

    def __init__(self, device: int = 0, workers: int = 1, hbm_budget_bytes: int = 150 << 30, batch_max_build_rows: int = 0,
                 batch_max_joins: int = 1, pass_bits: Sequence[int] = ()):
        self.lib = load()
        cfg = ServeConfig()
        cfg.device, cfg.workers, cfg.hbm_budget_bytes = device, workers, hbm_budget_bytes
        cfg.batch_max_build_rows, cfg.batch_max_joins = batch_max_build_rows, batch_max_joins
        for i, b in enumerate(pass_bits):
            cfg.pass_bits[i] = b
        cfg.n_passes = len(pass_bits)
        self.ptr = C.c_void_p()
        st = self.lib.phj_serve_create(C.byref(cfg), C.byref(self.ptr))
        if st != 0:
            raise PhjError(st, "phj_serve_create failed")

    def submit(self, build: GenSpec, probe: GenSpec, arrival_s: float) -> int:
        r = ServeRequest()
        r.build, r.probe, r.arrival_s = build, probe, arrival_s
        rid = C.c_uint64()
        st = self.lib.phj_serve_submit(self.ptr, C.byref(r), C.byref(rid))
        if st != 0:
            raise PhjError(st, "phj_serve_submit failed")
        return rid.value

    def run(self, timeout_s: float = 600.0) -> List[dict]:
        st = self.lib.phj_serve_start(self.ptr)
        if st != 0:
            raise PhjError(st, "phj_serve_start failed")
        st = self.lib.phj_serve_wait(self.ptr, timeout_s)
        if st != 0:
            raise PhjError(st, self.lib.phj_serve_error(self.ptr).decode())
        n = self.lib.phj_serve_records(self.ptr, None, 0)
        arr = (ServeRecord * max(n, 1))()
        self.lib.phj_serve_records(self.ptr, arr, n)
        return [{"id": r.id, "arrival_s": r.arrival_s, "admit_s": r.admit_s, "start_s": r.start_s, "done_s": r.done_s,
                 "build_rows": r.build_rows, "probe_rows": r.probe_rows, "output_rows": r.output_rows,
                 "footprint_bytes": r.footprint_bytes, "fingerprint": tuple(r.fingerprint), "batch_size": r.batch_size,
                 "slot": r.slot, "status": r.status, "job_peak_bytes": r.job_peak_bytes, "gen_s": r.gen_s, "call_s": r.call_s,
                 "device_ms": r.device_ms} for r in arr[:n]]

    def close(self):
        if self.ptr:
            self.lib.phj_serve_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune_radix(build_rows: int, probe_rows: int = 0) -> List[int]:
    bits = (C.c_uint8 * 8)()
    n = C.c_uint32()
    st = load().phj_autotune_radix(build_rows, probe_rows, bits, C.byref(n))
    if st != 0:
        raise PhjError(st, "phj_autotune_radix failed")
    return list(bits[: n.value])


def serve_footprint(build: GenSpec, probe: GenSpec, batched: bool) -> int:
    r = ServeRequest()
    r.build, r.probe = build, probe
    return load().phj_serve_footprint(C.byref(r), int(batched))
