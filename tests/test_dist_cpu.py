"""The multi-process (N > 1) steps of bench.py, as two gloo ranks on the CPU.

Every box has one GPU, so `bench.py --gpus N` runs N independent replicas:
the only cross-rank steps are a barrier around the timed region, max and
sum reductions of the timings and counts, and the reference arm running on
rank 0 alone.  These tests run exactly those steps in two CPU processes
(gloo, rendezvous on 127.0.0.1), as the launcher would."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import json, sys
sys.path.insert(0, {root!r})
import bench
rank, world, local = bench.env_rank()
d = bench.Dist(world)
d.barrier()
mx = d.max(rank + 1.5)
sm = d.sum(rank + 1.0)
d.barrier()
print(json.dumps({{"rank": rank, "world": world, "local": local, "max": mx, "sum": sm}}), flush=True)
"""


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_dist_barrier_and_reductions_two_ranks():
    port = free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE="2", LOCAL_RANK=str(r), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD.format(root=ROOT)], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=300) for p in procs]
    for p, (_, err) in zip(procs, outs):
        assert p.returncode == 0, err[-2000:]
    res = sorted((json.loads(o.strip().splitlines()[-1]) for o, _ in outs), key=lambda x: x["rank"])
    assert [r["rank"] for r in res] == [0, 1]
    for r in res:
        assert r["world"] == 2 and r["local"] == r["rank"]
        assert r["max"] == 2.5  # the slowest rank's time is the job's
        assert r["sum"] == 3.0  # whole-job totals add over ranks


def test_reference_arm_two_ranks_prints_one_line():
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr", "127.0.0.1",
           "--master-port", str(port), os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "c1", "--steps", "1",
           "--warmup", "1", "--cpu-probe-frac", "0.01"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1  # rank 0 alone runs and prints; rank 1 exits 0
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["cores"] >= 1
