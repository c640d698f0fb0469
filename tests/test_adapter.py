"""The C++ adapter (phj-bench_gb300/host/phj_gpu.hpp): the reference's
runCHJ / runPHJ / runPhjBep signatures over BlockStreams of 10,000-row
blocks, on top of the C ABI."""
import os
import subprocess

import numpy as np
import pytest

import oracle as O
import phj_gpu as P
from golden import cases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def reference_src():
    """The reference's src/ directory: PHJ_REF_SRC, else the one the oracle's
    recipe builds from; None (tests skip) where neither exists."""
    d = os.environ.get("PHJ_REF_SRC")
    if not d:
        r = subprocess.run(["make", "-s", "--no-print-directory", "-C", os.path.join(ROOT, "oracle"), "ref-src"], capture_output=True, text=True)
        d = r.stdout.strip() if r.returncode == 0 else ""
    return d if d and os.path.isdir(d) else None


REF_SRC = reference_src()


@pytest.mark.skipif(REF_SRC is None, reason="reference headers not on this machine (set PHJ_REF_SRC)")
def test_adapter_compiles_against_the_reference_types():
    subprocess.run(["g++", "-std=c++23", "-fsyntax-only", "-I", REF_SRC, "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "ref_types_check.cpp")], check=True)


def test_adapter_compiles_standalone():
    subprocess.run(["g++", "-std=c++20", "-fsyntax-only", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "adapter_main.cpp")], check=True)


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    lib = os.path.join(ROOT, "phj-bench_gb300")
    exe = str(tmp_path_factory.mktemp("adapter") / "adapter_main")
    subprocess.run(["g++", "-std=c++20", "-O2", "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp", "adapter_main.cpp"),
                    "-L", lib, "-lphj_gpu", f"-Wl,-rpath,{lib}", "-o", exe], check=True)
    return exe


def write_side(d, side, s):
    with open(os.path.join(d, f"{side}.schema"), "w") as f:
        f.write(" ".join(str(t) for t in s.types))
    s.keys.tofile(os.path.join(d, f"{side}.keys"))
    for c, col in enumerate(s.payloads):
        col.tofile(os.path.join(d, f"{side}.col{c}"))


def read_output(d, b, p):
    keys = np.fromfile(os.path.join(d, "out.keys"), dtype=np.uint64)

    def col(name, t):
        raw = np.fromfile(os.path.join(d, name), dtype=np.uint8)
        return raw.view(np.uint64).reshape(-1, 2) if t == P.U128 else raw.view(P.TYPE_DTYPE[t])
    left = [col(f"out.left{c}", t) for c, t in enumerate(b.types)]
    right = [col(f"out.right{c}", t) for c, t in enumerate(p.types)]
    return P.JoinOutput(b.types, p.types, keys, left, right)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["c2_mini", "c3_mini", "edge"])
@pytest.mark.parametrize("scheme", ["chj", "phj-pure", "phj"])
def test_adapter_is_bit_exact(driver, tmp_path, name, scheme):
    b, p = cases.make(name)
    write_side(tmp_path, "build", b)
    write_side(tmp_path, "probe", p)
    bits = ",".join(str(x) for x in cases.BITS[name])
    out = subprocess.run([driver, str(tmp_path), scheme, bits, "32"], capture_output=True, text=True, check=True).stdout
    assert out.startswith("rows ")
    jo = read_output(tmp_path, b, p)
    assert O.compare_outputs(O.join_rows(b, p), O.serialize_output(jo)) == ""


@pytest.mark.gpu
def test_adapter_rejects_bad_radix_like_the_reference(driver, tmp_path):
    b, p = cases.make("c2_mini")
    write_side(tmp_path, "build", b)
    write_side(tmp_path, "probe", p)
    r = subprocess.run([driver, str(tmp_path), "phj-pure", "17", "32"], capture_output=True, text=True)
    assert r.returncode == 3 and "invalid_argument" in r.stdout
