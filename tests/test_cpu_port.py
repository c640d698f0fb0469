"""The CPU port of the reference's schemes (oracle/cpu_port.cpp), the timed
CPU baseline: its output rows equal the oracle's for every scheme (row
count and the order-independent fingerprint of the rows it materialised),
and PHJ (BEP) under a small budget refines, evicts and drains every row."""
import os
import subprocess

import pytest

import oracle as O
import phj_datagen as G
import phj_gpu as P
from golden import cases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module", autouse=True)
def built():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "libcpuport.so"], check=True)


@pytest.mark.parametrize("name", cases.NAMES)
@pytest.mark.parametrize("scheme", ["chj", "phj-pure", "phj"])
def test_port_rows_equal_the_oracle(name, scheme):
    b, p = cases.make(name)
    n, ms = O.port_run(scheme, b, p, cases.BITS[name], threads=4, budget_mib=1, fingerprint=True)
    rows = O.join_rows(b, p)
    assert n == len(rows)
    assert ms["fingerprint"] == O.rows_fingerprint(rows, b.types, p.types)
    assert ms["e2e"] >= 0


@pytest.mark.parametrize("budget", [1, 4, 512])
def test_port_bep_budget_counters(budget):
    bk = G.gen_keys(0, 40000, 301, 302)
    pk = G.gen_keys(4, 400000, 303, 302, domain=40000, match_permille=800)
    b = P.BlockStream([P.U64], bk, G.payload_columns(304, [P.U64], 40000))
    p = P.BlockStream([P.U32, P.U64], pk, G.payload_columns(305, [P.U32, P.U64], 400000))
    n, ms = O.port_run("phj", b, p, [3, 4], threads=4, budget_mib=budget, fingerprint=True)
    assert n == len(O.join_rows(b, p))
    assert ms["fingerprint"] == O.join_fingerprint(b, p, threads=4)
    assert ms["bep_refinements"] > 0 and ms["bep_evictions"] > 0
    if budget == 1:
        # 400K rows x 20 B = 8 MB through a 1 MiB budget: leaves are evicted
        # mid-stream, and the buffered peak stays near 5/8 of the budget
        assert ms["bep_peak_bytes"] <= (1 << 20)
