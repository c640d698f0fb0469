"""Host-side checks of the C ABI that need no GPU: the library loads, it
exports every function include/phj_gpu.h declares, and the radix
configuration resolves as the reference CLI does (src/CLI.cpp:330-355)."""
import ctypes
import os
import re

import pytest

import phj_gpu as P

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            text = open(os.path.join(ROOT, "include", h)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names |= set(re.findall(r"\b(phj_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(P.LIB_PATH):
        import subprocess
        subprocess.run(["make", "-s", "-j4", "-C", os.path.join(ROOT, "phj-bench_gb300")], check=True)
    return P.load()


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_abi_version(lib):
    assert lib.phj_abi_version() == P.ABI_VERSION == 3


@pytest.mark.parametrize("parts,passes,want", [
    (256, 1, [8]), (65536, 2, [8, 8]), (262144, 3, [6, 6, 6]), (1024, 3, [4, 3, 3]), (2, 1, [1]), (1 << 32, 2, [16, 16]),
])
def test_resolve_radix_matches_cli(lib, parts, passes, want):
    assert P.resolve_radix(parts, passes) == want


def test_resolve_radix_bits_override(lib):
    assert P.resolve_radix(bits_per_pass=[6, 4]) == [6, 4]


@pytest.mark.parametrize("parts,passes,bits", [(100, 1, None), (256, 9, None), (0, 0, [0]), (0, 0, [17]), (0, 0, [16, 16, 1])])
def test_resolve_radix_rejects_what_the_cli_rejects(lib, parts, passes, bits):
    with pytest.raises(P.PhjError):
        P.resolve_radix(parts, passes, bits)


def test_context_without_a_device_reports_no_device(lib):
    try:
        import subprocess
        has_gpu = subprocess.run(["nvidia-smi", "-L"], capture_output=True).returncode == 0
    except FileNotFoundError:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    p = ctypes.c_void_p()
    assert lib.phj_ctx_create(0, ctypes.byref(p)) == 6  # PHJ_ERR_NO_DEVICE
    with pytest.raises(P.PhjError):
        P.Context(0)


def test_serve_footprint_estimate(lib):
    # 100K unique build keys (u64 payload), 1M probe rows (u32 payload)
    b = P.gen_spec(0, 100_000, 1, 2, [P.U64])
    p = P.gen_spec(4, 1_000_000, 3, 2, [P.U32], domain=100_000, match_permille=500)
    cells = 1 << 18  # bit_ceil(2 * 100K)
    inputs = 100_000 * 16 + 1_000_000 * 12
    table = cells * 16 + 100_000 * 8
    out = 1_000_000 * (16 + 12 - 8)
    assert P.serve_footprint(b, p, batched=True) == inputs + table + 100_000 * 16 + 1_000_000 * 12 + out
    assert P.serve_footprint(b, p, batched=False) == inputs + table + 2 * 100_000 * 16 + 1_000_000 * 12 + 1_000_000 * 4 + out


def test_serve_rejects_bad_config_and_needs_a_device(lib):
    with pytest.raises(P.PhjError):
        P.Server(workers=0)
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if not has_gpu:
        with pytest.raises(P.PhjError) as e:
            P.Server(workers=2)
        assert e.value.status == 6  # PHJ_ERR_NO_DEVICE


@pytest.mark.parametrize("rows,want", [(1, [1]), (4096, [4]), (1 << 19, [11]), (1 << 20, [6, 6]), (16 << 20, [8, 8]),
                                       (64 << 20, [9, 9]), (1 << 31, [8, 8, 7])])
def test_autotune_radix_leaf_target(lib, rows, want):
    assert P.autotune_radix(rows) == want


def test_entry_points_reject_a_null_context_without_a_device(lib):
    # Every join entry point checks its handles before any CUDA call, so a
    # missing context is PHJ_ERR_INVALID_ARGUMENT here as on a GPU machine.
    out = ctypes.c_void_p()
    desc = P.BlockStreamDesc()
    rows = ctypes.c_uint64()
    keys = (ctypes.c_uint64 * 1)()
    ptrs = (ctypes.c_void_p * 1)()
    calls = {
        "phj_run_chj": lambda: lib.phj_run_chj(None, None, None, ctypes.byref(out), None),
        "phj_run_phj_pure": lambda: lib.phj_run_phj_pure(None, None, None, None, 0, ctypes.byref(out), None),
        "phj_run_phj_bep": lambda: lib.phj_run_phj_bep(None, None, None, None, 0, 0, 0, ctypes.byref(out), None),
        "phj_run_phj_pure_host": lambda: lib.phj_run_phj_pure_host(None, ctypes.byref(desc), ctypes.byref(desc), None, 0, 1,
                                                                   keys, ptrs, ptrs, ctypes.byref(rows), None),
        "phj_run_phj_bep_host": lambda: lib.phj_run_phj_bep_host(None, ctypes.byref(desc), ctypes.byref(desc), None, 0, 0, 1,
                                                                 keys, ptrs, ptrs, ctypes.byref(rows), None),
        "phj_run_chj_noalloc": lambda: lib.phj_run_chj_noalloc(None, None, None, 0, None, None, None, ctypes.byref(rows)),
        "phj_batch_run": lambda: lib.phj_batch_run(None, 0, None, None, None, None),
        "phj_radix_shuffle": lambda: lib.phj_radix_shuffle(None, None, None, 0, ctypes.byref(out), None),
        "phj_table_generate": lambda: lib.phj_table_generate(None, None, ctypes.byref(out)),
        "phj_table_upload": lambda: lib.phj_table_upload(None, ctypes.byref(desc), ctypes.byref(out)),
        "phj_output_fingerprint": lambda: lib.phj_output_fingerprint(None, None, keys),
        "phj_flush_l2": lambda: lib.phj_flush_l2(None),
        "phj_host_alloc": lambda: lib.phj_host_alloc(None, 16, ctypes.byref(out)),
    }
    for name, call in calls.items():
        assert call() == 1, name  # PHJ_ERR_INVALID_ARGUMENT


@pytest.mark.parametrize("cmd", [["gcc", "-std=c99", "-x", "c"], ["g++", "-std=c++17", "-x", "c++"]])
def test_header_is_plain_c_and_cpp(cmd):
    # FFI users (ctypes, cgo, JNI shims) bind the header from C
    import subprocess
    r = subprocess.run(cmd + ["-Wall", "-Wextra", "-Werror", "-fsyntax-only", os.path.join(ROOT, "include", "phj_gpu.h")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_plain_c_caller_links_and_calls_the_library(lib, tmp_path):
    import subprocess
    so_dir = os.path.dirname(P.LIB_PATH)
    exe = str(tmp_path / "c_abi_main")
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "c_abi_main.c"), "-L", so_dir, "-lphj_gpu", f"-Wl,-rpath,{so_dir}", "-o", exe],
                   check=True)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    assert out[:7] == ["abi", "3", "radix", "0", "2", "8", "8"]
    assert out[7] == "ctx" and int(out[8]) in (0, 6)  # PHJ_OK on a GPU machine, PHJ_ERR_NO_DEVICE without one
