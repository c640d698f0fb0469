#!/usr/bin/env python3
"""Benchmark of the GB300 hash-join path (one JSON line on stdout).

Default workload (the 16M x 256M uint64 join the headline metric is quoted
on): build side 16M rows of unique splitmix64 keys with u64 and u32 payloads,
probe side 256M rows whose keys are drawn uniformly from the build keys with
10% replaced by non-matching keys, one u64 payload; radix 2 passes x 8 bits
(65,536 leaves); scheme PHJ-PURE (runPHJ).  Inputs are generated on the
device (seeded, synthetic) and are resident in HBM before timing.

  value  build+probe tuples/s of the join with inputs resident in HBM
         (CUDA events on the library's stream around each join);
  e2e    the same metric through the C ABI with HOST (pinned) inputs and
         outputs: upload, join, and download of the result inside the timing;
  roofline  the dominant kernel's algorithmic bytes per launch over its
         CUDA-event duration, against the measured HBM copy bandwidth;
  cpu_baseline  the reference's PHJ-PURE on the host cores (its C++ port in
         oracle/, since the reference sources are not on this machine) over a
         bounded sample of the same workload.

--impl reference runs only that CPU implementation, as the reference arm.
Multi-GPU: the join does not exchange data between GPUs here, so N ranks run
N independent replicas (weak scaling) with a barrier and max-over-ranks time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [os.path.join(ROOT, "phj-bench_gb300"), os.path.join(ROOT, "oracle")]

import numpy as np  # noqa: E402

M = 1 << 20
WIDTH = {0: 1, 1: 2, 2: 4, 3: 8, 4: 16}

WORKLOADS = {
    # name: (description, scheme, build spec, probe spec, radix bits)
    "c2": ("PHJ-PURE 16M x 256M: unique splitmix64 u64 build keys with u64,u32 payloads; probe keys uniform from the build "
           "keys with 10% non-matching, u64 payload; 2 passes x 8 bits (65,536 leaves)", "phj-pure",
           dict(kind=0, rows=16 * M, seed=0xB1, key_seed=0x5EED, types=[3, 2]),
           dict(kind=4, rows=256 * M, seed=0xB2, key_seed=0x5EED, types=[3], domain=16 * M, match_permille=900), [8, 8]),
    "c1": ("PHJ-PURE 1M x 8M: build keys a permutation of 1..1M with a u64 payload; probe keys uniform over 1..1M with a "
           "u32 payload; 1 pass x 8 bits", "phj-pure",
           dict(kind=1, rows=1 * M, seed=0xC1, key_seed=0, types=[3]),
           dict(kind=3, rows=8 * M, seed=0xC2, key_seed=0, types=[2], domain=1 * M), [8]),
    "c3": ("PHJ-PURE multi-match 32M x 128M: ~8M distinct build keys, geometric multiplicity (mean ~4, cap 16), u8,u16,u128 "
           "payloads; probe 50% from the distinct build keys, u32 payload; radix bits, table load and first-pass tiling from "
           "the autotuner", "phj-pure",
           dict(kind=2, rows=32 * M, seed=0xD1, key_seed=0x77, types=[0, 1, 4]),
           dict(kind=4, rows=128 * M, seed=0xD2, key_seed=0x77, types=[2], domain=None, match_permille=500), None),
    "c4": ("PHJ (BEP) under skew 64M x 512M: unique u64 build keys with a u64 payload; probe keys Zipf(1.0) ranks through a "
           "seeded permutation onto the build keys, u32 payload; 3 passes x 6 bits (262,144 leaves, partitioned on the device "
           "in 2 passes of 9 bits); 32 MiB probe budget per CTA group (one group per SM); lazy per-leaf build", "phj",
           dict(kind=0, rows=64 * M, seed=0xE1, key_seed=0x99, types=[3]),
           dict(kind=5, rows=512 * M, seed=0xE2, key_seed=0x99, types=[2], domain=64 * M, theta=1.0), [6, 6, 6]),
}
# PHJ (BEP) probe budget per CTA group, MiB (--bep-budget-mib)
BEP_BUDGET_PER_GROUP = {"c4": 32}


# ---- batched / served request stream ------------------------------------
def serve_trace(n, seed=0xC5):
    """n join requests: build rows log-uniform in 4K..8M with unique random
    u64 keys, probe rows = build rows x U(4,32), match rate U(0.1,1.0), 1 to 3
    payload columns per side drawn from {u32, u64}."""
    import phj_gpu as P
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n):
        B = int(np.exp(rng.uniform(np.log(4096), np.log(8 * M))))
        Pn = int(B * rng.uniform(4, 32))
        match = int(rng.uniform(100, 1000))
        tb = [int(t) for t in rng.choice([2, 3], size=int(rng.integers(1, 4)))]
        tp = [int(t) for t in rng.choice([2, 3], size=int(rng.integers(1, 4)))]
        b = P.gen_spec(0, B, seed * 7919 + 2 * i, seed * 104729 + i, tb)
        p = P.gen_spec(4, Pn, seed * 7919 + 2 * i + 1, seed * 104729 + i, tp, domain=B, match_permille=match)
        reqs.append((b, p, B + Pn))
    return reqs


def serve_once(reqs, arrivals, workers, batch_rows, batch_joins, budget):
    import phj_gpu as P
    srv = P.Server(workers=workers, hbm_budget_bytes=budget, batch_max_build_rows=batch_rows, batch_max_joins=batch_joins)
    for (b, p, _), t in zip(reqs, arrivals):
        srv.submit(b, p, float(t))
    recs = srv.run(timeout_s=1800)
    srv.close()
    lat = np.array([r["done_s"] - r["arrival_s"] for r in recs])
    span = max(r["done_s"] for r in recs) - min(r["arrival_s"] for r in recs)
    tuples = sum(t for _, _, t in reqs)
    # where a request's time goes: generating its inputs, the join call on
    # the host (launches, host round trips, allocations) and the join's
    # device time inside it
    dev_s = sum(r["device_ms"] for r in recs) / 1e3
    call_s = sum(r["call_s"] for r in recs)
    gen_s = sum(r["gen_s"] for r in recs)
    return {"tuples_per_s": tuples / span, "makespan_s": span, "p50_ms": float(np.percentile(lat, 50) * 1e3),
            "p99_ms": float(np.percentile(lat, 99) * 1e3), "p999_ms": float(np.percentile(lat, 99.9) * 1e3),
            "mean_batch": float(np.mean([r["batch_size"] for r in recs])), "requests": len(recs),
            "breakdown": {"join_device_s": dev_s, "join_call_s": call_s, "input_gen_s": gen_s,
                          "join_device_busy_frac_of_makespan": dev_s / span,
                          "call_overhead_ms_per_request": (call_s - dev_s) * 1e3 / len(recs),
                          "device_tuples_per_s": tuples / dev_s if dev_s > 0 else None}}, recs


def serving_benchmark(n_requests, workers=4, batch_rows=1 << 18, batch_joins=64, budget=150 << 30, seed=0xC5):
    """Closed-loop capacity of the plain form (one join per call, in order)
    and of the served form (slots + continuous batching); then Poisson
    arrivals at 80% of the plain capacity through both, with latencies."""
    reqs = serve_trace(n_requests, seed)
    tuples = np.array([t for _, _, t in reqs], dtype=np.float64)
    zero = np.zeros(len(reqs))
    plain_cap, plain_recs = serve_once(reqs, zero, 1, 0, 1, budget)
    served_cap, served_recs = serve_once(reqs, zero, workers, batch_rows, batch_joins, budget)
    rate = 0.8 * plain_cap["tuples_per_s"] / tuples.mean()  # requests per second
    rng = np.random.default_rng(seed + 1)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=len(reqs)))
    arrivals -= arrivals[0]
    plain_open, plain_open_recs = serve_once(reqs, arrivals, 1, 0, 1, budget)
    served_open, served_open_recs = serve_once(reqs, arrivals, workers, batch_rows, batch_joins, budget)
    fps = [r["fingerprint"] for r in plain_recs]
    identical = all(fps == [r["fingerprint"] for r in rr] for rr in (served_recs, plain_open_recs, served_open_recs))
    return {
        "requests": n_requests, "total_tuples": float(tuples.sum()),
        "trace": "build rows log-uniform 4K..8M (unique u64 keys), probe rows = build x U(4,32), match U(0.1,1.0), "
                 "1-3 payload columns per side from {u32,u64}; inputs generated on the device when a request starts",
        "plain": {"closed_loop": plain_cap, "poisson_80pct": plain_open},
        "served": {"closed_loop": served_cap, "poisson_80pct": served_open, "slots": workers,
                   "batch_max_build_rows": batch_rows, "batch_max_joins": batch_joins, "hbm_budget_bytes": budget},
        "arrival_rate_req_per_s": rate,
        "capacity_ratio_served_over_plain": served_cap["tuples_per_s"] / plain_cap["tuples_per_s"],
        "outputs_identical_across_forms": identical,
    }


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


class Dist:
    """Barrier and max-reduce across ranks (gloo on CPU tensors) when N > 1."""

    def __init__(self, world):
        self.world = world
        self.dist = None
        if world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, x):
        if not self.dist:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x):
        if not self.dist:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return float(t.item())


class ClockSampler:
    """nvidia-smi clock/throttle samples while the timed region runs."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = os.path.join("/tmp", f"phj_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        self.proc.wait()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def launch_overlaps(run, i, tol_ms=1e-3):
    """Whether launch i of one run's kernel times overlapped another launch
    (only launches on different streams can: one stream's run in order)."""
    a0 = run[i]["start_ms"]
    a1 = a0 + run[i]["ms"]
    for j, k in enumerate(run):
        if j != i and min(a1, k["start_ms"] + k["ms"]) - max(a0, k["start_ms"]) > tol_ms:
            return True
    return False


def measured_peak():
    try:
        d = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(d["hbm_gbs"]), "measured copy bandwidth (MEASURED_PEAKS.json, burst)"
    except Exception:
        return 6800.0, "fallback 6.8 TB/s (MEASURED_PEAKS.json absent)"


def profiled_traffic(kernel, workload, scale=1.0):
    """DRAM bytes per launch of `kernel` from the committed ncu summary: a
    full-size launch, scaled by the rows a `--scale`d run processes (the
    figures grow in proportion to the rows)."""
    try:
        d = json.load(open(os.path.join(ROOT, "profiles", "ncu_traffic.json")))
        e = d.get(workload, {}).get(kernel)
        return int(e["dram_bytes_per_launch"] * scale) if e else None
    except Exception:
        return None


def row_bytes(types):
    return 8 + sum(WIDTH[t] for t in types)


def make_tables(ctx, wl):
    _, _, bspec, pspec, _ = WORKLOADS[wl]
    b = ctx.generate(bspec["kind"], bspec["rows"], bspec["seed"], bspec["key_seed"], bspec["types"])
    pspec = dict(pspec)
    if pspec.get("domain") is None:
        pspec["domain"] = b.gen_distinct
    p = ctx.generate(pspec["kind"], pspec["rows"], pspec["seed"], pspec["key_seed"], pspec["types"], domain=pspec["domain"],
                     match_permille=pspec.get("match_permille", 1000), theta=pspec.get("theta", 1.0))
    return b, p


def scale_workload(name, f):
    desc, scheme, bspec, pspec, bits = WORKLOADS[name]
    bspec, pspec = dict(bspec), dict(pspec)
    bspec["rows"] = max(1, int(bspec["rows"] * f))
    pspec["rows"] = max(1, int(pspec["rows"] * f))
    if pspec.get("domain") and bspec["kind"] in (0, 1):
        pspec["domain"] = bspec["rows"]
    if name in BEP_BUDGET_PER_GROUP:
        BEP_BUDGET_PER_GROUP[name] = max(1, int(BEP_BUDGET_PER_GROUP[name] * f))
    WORKLOADS[name] = (f"{desc} [rows scaled by {f:g}]", scheme, bspec, pspec, bits)


def run_scheme(ctx, scheme, b, p, bits, budget_mib=0):
    if scheme == "chj":
        return ctx.run_chj(b, p)
    if scheme == "phj":
        return ctx.run_phj_bep(b, p, bits, budget_mib)
    return ctx.run_phj_pure(b, p, bits)


def cpu_budget_mib(workload, threads):
    """PHJ (BEP) budget of the CPU run: the per-worker budget times the
    worker threads (the GPU run gives each CTA group the same share)."""
    return BEP_BUDGET_PER_GROUP.get(workload, 32) * threads


def sample_text(build_rows, n_p, probe_rows, scheme, threads, runs, stat):
    """What the CPU runs covered, for the JSON line."""
    part = "the whole workload" if n_p == probe_rows else f"the full build side and the first {n_p} of {probe_rows} probe rows"
    import platform
    arch = platform.machine()
    simd = ("the scalar intHash64Batch, the reference's path on a host without AVX-512 (src/Hash.h:35-58)" if arch in ("aarch64", "arm64")
            else "a scalar intHash64Batch (the reference would take its AVX-512 path here, src/Hash.h:35-58)")
    return (f"{scheme} on {part} ({build_rows} + {n_p} rows); {stat} of {runs} runs on {threads} threads of this {arch} host; C++ port "
            f"of the reference's scheme (oracle/cpu_port.cpp; the reference's sources are not on this machine) with {simd}")


def cpu_baseline(bhost, phost, bits, frac, threads, scheme, reps=3, budget_mib=512):
    import oracle
    n_p = max(1, int(len(phost.keys) * frac))
    probe = phost if n_p == len(phost.keys) else type(phost)(phost.types, phost.keys[:n_p], [c[:n_p] for c in phost.payloads])
    times = []
    for _ in range(reps):
        _, ms = oracle.port_run(scheme, bhost, probe, bits, threads, budget_mib)
        times.append(ms["e2e"])
    t = statistics.median(times) / 1e3
    return {"value": (len(bhost.keys) + n_p) / t, "unit": "tuples/s", "cores": threads, "kind": "port",
            "sample": sample_text(len(bhost.keys), n_p, len(phost.keys), scheme, threads, reps, "median"),
            "ms_per_run": statistics.median(times)}


def host_tables(wl, probe_rows=None):
    """The workload's build and probe sides generated on the host (the same
    integers as the device generator, phj_table_generate), optionally only
    the first `probe_rows` probe rows."""
    import phj_datagen as G
    import phj_gpu as P
    _, _, bspec, pspec, _ = WORKLOADS[wl]
    if bspec["kind"] == 2:
        bk, used = G.gen_multi_match_keys(bspec["rows"], bspec["seed"], bspec["key_seed"])
    else:
        bk, used = G.parallel_keys(bspec["kind"], bspec["rows"], bspec["seed"], bspec["key_seed"]), bspec["rows"]
    b = P.BlockStream(bspec["types"], bk, G.parallel_payloads(bspec["seed"], bspec["types"], bspec["rows"]))
    n_p = pspec["rows"] if probe_rows is None else probe_rows
    dom = pspec.get("domain") or used
    pk = G.parallel_keys(pspec["kind"], n_p, pspec["seed"], pspec["key_seed"], domain=dom,
                         match_permille=pspec.get("match_permille", 1000), theta=pspec.get("theta", 1.0))
    return b, P.BlockStream(pspec["types"], pk, G.parallel_payloads(pspec["seed"], pspec["types"], n_p))


def golden_fingerprint(wl):
    """The oracle's fingerprint of a full-size workload's join, as
    tests/golden/gen_fullsize.py recorded it (None if absent)."""
    try:
        d = json.load(open(os.path.join(ROOT, "tests", "golden", "fullsize.json")))
        return tuple(int(v) for v in d[wl]["fingerprint"])
    except Exception:
        return None


def workload_config(desc, scheme, build_rows, probe_rows, output_rows, bits, probe_types, world, n_p=None):
    """The `config` object of both arms' JSON lines: the same workload gives
    the same object on the GPU and on the host cores."""
    cfg = {"workload": desc, "scheme": scheme, "build_rows": build_rows, "probe_rows": probe_rows if n_p is None else n_p,
           "output_rows": output_rows, "radix_pass_bits": list(bits),
           "l2": f"probe side {probe_rows * row_bytes(probe_types) / 1e9:.2f} GB; an L2 flush (a write larger than L2) between steps"}
    if n_p is not None and n_p != probe_rows:
        cfg["probe_sample_of"] = probe_rows
    if world > 1:
        cfg["parallelism"] = f"{world} replicas"
    return cfg


def host_streams_from_device(ctx, b, p):
    return b.download(), p.download()


def reference_arm(args, rank, world, dist):
    """The reference's CPU implementation (its C++ port) on the host cores."""
    if rank != 0:
        return
    import oracle
    import phj_gpu as P
    if args.scale != 1.0:
        scale_workload(args.workload, args.scale)
    desc, scheme, bspec, pspec, bits = WORKLOADS[args.workload]
    scheme = args.scheme or scheme
    threads = os.cpu_count() or 1
    frac = args.cpu_probe_frac
    if args.pass_bits:
        bits = [int(x) for x in args.pass_bits.split(",")]
    if bits is None:
        bits = P.autotune_radix(bspec["rows"])
    # the same seeded inputs as the GPU arm's device generator, made on the
    # host in parallel chunks (not timed)
    n_p = max(1, int(pspec["rows"] * frac))
    b, p = host_tables(args.workload, n_p)
    cs = scheme
    budget = cpu_budget_mib(args.workload, threads)
    # one untimed run checks the port's rows against the oracle's answer for
    # the full workload (tests/golden/fullsize.json)
    _, ms = oracle.port_run(cs, b, p, bits, threads, budget, fingerprint=True)
    checked = None
    golden = golden_fingerprint(args.workload)
    if golden is not None and n_p == pspec["rows"] and args.scale == 1.0:
        checked = tuple(ms["fingerprint"]) == golden
    for _ in range(max(0, args.warmup - 1)):
        oracle.port_run(cs, b, p, bits, threads, budget)
    times = []
    for _ in range(args.steps):
        out_rows, ms = oracle.port_run(cs, b, p, bits, threads, budget)
        times.append(ms["e2e"])
    t = statistics.mean(times)
    value = (len(b.keys) + n_p) / (t / 1e3)
    line = {
        "impl": "reference", "metric": "join tuples/s (build+probe)", "value": value, "unit": "tuples/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64", "data": "synthetic (seeded, same generator specification as the GPU arm)",
        "config": workload_config(desc, scheme, len(b.keys), pspec["rows"], int(out_rows), bits, pspec["types"], world, n_p),
        "cpu_baseline": {"value": value, "unit": "tuples/s", "cores": threads, "kind": "port",
                         "sample": sample_text(len(b.keys), n_p, pspec["rows"], cs, threads, args.steps, "mean")},
        "e2e": {"value": value, "unit": "tuples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "output_equals_oracle": checked,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c2", choices=sorted(WORKLOADS))
    ap.add_argument("--scheme", default=None, choices=["phj-pure", "chj", "phj"])
    ap.add_argument("--bep-budget-mib", type=int, default=0, help="PHJ (BEP) whole-run probe budget (default: per-group budget x SMs)")
    ap.add_argument("--pass-bits", default=None, help="radix bits per pass, e.g. 8,8 (overrides the workload's; no autotuning)")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-probe-frac", type=float, default=1.0, help="fraction of the probe side the CPU runs take (default: all of it)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-chj", action="store_true")
    ap.add_argument("--scale", type=float, default=1.0, help="multiply both sides' rows (profiling on a smaller case)")
    ap.add_argument("--set", action="append", default=[], metavar="NAME=VALUE", help="context option (phj_ctx_set_int)")
    ap.add_argument("--serve-requests", type=int, default=2048, help="requests of the batched/served stream (0: skip it)")
    ap.add_argument("--serve-only", action="store_true", help="run only the batched/served stream")
    ap.add_argument("--serve-batch-rows", type=int, default=1 << 18, help="served form: requests of at most this many build rows are batched")
    ap.add_argument("--serve-slots", type=int, default=4, help="served form: execution slots (contexts with their own streams)")
    ap.add_argument("--csv", default=None, help="append the timed runs to this CSV (the reference's columns + GPU columns)")
    args = ap.parse_args()
    rank, world, local = env_rank()
    dist = Dist(world)
    if args.impl == "reference":
        reference_arm(args, rank, world, dist)
        return
    if args.serve_only:
        print(json.dumps({"serving": serving_benchmark(args.serve_requests, args.serve_slots, args.serve_batch_rows)}), flush=True)
        return

    import phj_gpu as P
    desc, scheme, bspec, pspec, bits = WORKLOADS[args.workload]
    scheme = args.scheme or scheme
    if args.pass_bits:
        bits = [int(x) for x in args.pass_bits.split(",")]
    if args.scale != 1.0:
        scale_workload(args.workload, args.scale)
        desc, _, bspec, pspec, _ = WORKLOADS[args.workload]
    ctx = P.Context(local)
    for kv in args.set:
        k, v = kv.split("=")
        ctx.set_int(k, int(v))
    b, p = make_tables(ctx, args.workload)
    B, Pn = b.rows, p.rows
    tuples = B + Pn
    tuned = None
    if bits is None:
        import autotune
        tuned = autotune.tune(ctx, b, p, scheme=scheme, reps=2, cache_path=None)
        bits = tuned["pass_bits"]
    budget = args.bep_budget_mib or BEP_BUDGET_PER_GROUP.get(args.workload, 32) * ctx.get_int("num_sms")

    # -------- device-resident timing --------
    sampler = ClockSampler(local)
    for _ in range(args.warmup):
        out, _ = run_scheme(ctx, scheme, b, p, bits, budget)
        out.free()
    sampler.start()
    dist.barrier()
    launches0 = ctx.launch_count()
    step_ms, kernel_runs, out_rows, step_results = [], [], 0, []
    t_wall0 = time.perf_counter()
    for _ in range(args.steps):
        ctx.flush_l2()
        out, res = run_scheme(ctx, scheme, b, p, bits, budget)
        step_ms.append(res.e2e_wall_ms)
        step_results.append(res)
        kernel_runs.append(ctx.kernel_times())
        out_rows = out.rows
        if _ == args.steps - 1:
            launches = ctx.launch_count() - launches0  # joins only (the L2 flush is a memset)
            fp_main = out.fingerprint()
        out.free()
    wall = time.perf_counter() - t_wall0
    dist.barrier()
    clocks = sampler.stop()
    ms_per_step = dist.max(statistics.mean(step_ms))
    total_tuples = dist.sum(tuples)
    value = total_tuples / (ms_per_step / 1e3)

    # dominant kernel: the largest time per step in launches that ran alone
    # (a launch that overlapped one on another stream shares the GPU, so its
    # event span is not its own cost), then its per-launch average over them
    per_name, alone = {}, {}
    for run in kernel_runs:
        for i, k in enumerate(run):
            d = per_name.setdefault(k["name"], {"ms": 0.0, "launches": 0, "bytes": 0})
            d["ms"] += k["ms"]
            d["launches"] += 1
            d["bytes"] += k["bytes"]
            if not launch_overlaps(run, i):
                e = alone.setdefault(k["name"], {"ms": 0.0, "launches": 0, "bytes": 0})
                e["ms"] += k["ms"]
                e["launches"] += 1
                e["bytes"] += k["bytes"]
    pool = alone if alone else per_name
    dom_name = max(pool, key=lambda n: pool[n]["ms"])
    dom = pool[dom_name]
    peak, peak_src = measured_peak()
    avg_ms = dom["ms"] / dom["launches"]
    bytes_per_launch = dom["bytes"] / dom["launches"]
    achieved = bytes_per_launch / (avg_ms / 1e3) / 1e9
    bmin = B * row_bytes(bspec["types"]) + Pn * row_bytes(pspec["types"]) + out_rows * (
        8 + sum(WIDTH[t] for t in bspec["types"]) + sum(WIDTH[t] for t in pspec["types"]))
    join_gbs = bmin / (statistics.mean(step_ms) / 1e3) / 1e9
    kernel_share = {n: round(d["ms"] / sum(x["ms"] for x in per_name.values()), 4) for n, d in
                    sorted(per_name.items(), key=lambda kv: -kv[1]["ms"])}

    line = {
        "metric": "join tuples/s (build+probe)", "value": value, "unit": "tuples/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u64", "data": "synthetic (seeded device generator; keys, payloads and match rate as specified)",
        "config": workload_config(desc, scheme, B, Pn, out_rows, bits, pspec["types"], world),
        "tuning": {"options": args.set, "autotuned": tuned},
        "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": profiled_traffic(dom_name, args.workload, args.scale),
                     "bytes_per_launch": bytes_per_launch, "ms_per_launch": avg_ms, "launches_timed": dom["launches"],
                     "selection": "largest time in launches that overlapped no other launch", "peak_source": peak_src},
        "join_roofline": {"bytes_min": bmin, "achieved_gbs": join_gbs, "frac": join_gbs / peak,
                          "definition": "B*(8+sum w_b) + P*(8+sum w_p) + O*(8+sum w_b+sum w_p) over the join's device time"},
        "kernel_share": kernel_share,
        "gpu_launches": int(launches),
        "clocks": clocks,
        "wall_s_timed": wall,
        "fingerprint": [str(v) for v in fp_main],
    }

    if scheme == "phj":
        line["bep"] = {k: getattr(res, k) for k in ("bep_evictions", "bep_refinements", "bep_peak_bytes", "bep_build_skip_retries")}
        line["bep"]["budget_mib"] = budget
        line["bep"]["budget_mib_per_group"] = BEP_BUDGET_PER_GROUP.get(args.workload, 32)
        line["bep"]["phase_ms"] = {k: getattr(res, k).wall_ms for k in
                                   ("build_shuffle", "build", "probe_shuffle", "probe", "eviction_overhead")}
        line["bep"]["form"] = ("device budget engine (per-group unrefined chains, water marks, refinement, round-robin "
                               "eviction, lazy builds)" if ctx.get_int("bep_engine") == 0 else "budget-sized probe batches")
        # the other form on the same inputs: budget-sized probe batches
        if ctx.get_int("bep_engine") == 0:
            ctx.set_int("bep_engine", 1)
            try:
                out, _ = run_scheme(ctx, scheme, b, p, bits, budget)
                out.free()
                bms = []
                for _ in range(3):
                    ctx.flush_l2()
                    out, bres = run_scheme(ctx, scheme, b, p, bits, budget)
                    bms.append(bres.e2e_wall_ms)
                    fp_b = out.fingerprint()
                    out.free()
            finally:
                ctx.set_int("bep_engine", 0)
            line["bep_batches"] = {"value": tuples / (statistics.mean(bms) / 1e3), "ms_per_step": statistics.mean(bms),
                                   "fingerprint_equals_engine": fp_b == fp_main,
                                   "bep_evictions": bres.bep_evictions, "bep_peak_bytes": bres.bep_peak_bytes}

    # -------- CHJ on the same inputs (extra line item) --------
    if not args.no_chj and scheme != "chj":
        for _ in range(2):
            out, _ = ctx.run_chj(b, p)
            out.free()
        cms, chj_results = [], []
        for _ in range(max(3, args.steps // 2)):
            ctx.flush_l2()
            out, cres = ctx.run_chj(b, p)
            cms.append(cres.e2e_wall_ms)
            chj_results.append(cres)
            fp_chj = out.fingerprint()
            out.free()
        line["chj"] = {"value": tuples / (statistics.mean(cms) / 1e3), "ms_per_step": statistics.mean(cms),
                       "fingerprint_equals_phj_pure": fp_chj == fp_main}
        # the unpartitioned probe in sweeps over groups of sub-tables small
        # enough for L2 (cells ~48 B a build row at the reference's load)
        l2 = ctx.get_int("l2_bytes")
        windows = 2
        while windows < 256 and B * 48 // windows > l2 // 2:
            windows *= 2
        ctx.set_int("chj_windows", windows)
        try:
            out, _ = ctx.run_chj(b, p)
            out.free()
            wms = []
            for _ in range(3):
                ctx.flush_l2()
                out, cres = ctx.run_chj(b, p)
                wms.append(cres.e2e_wall_ms)
                fp_w = out.fingerprint()
                out.free()
        finally:
            ctx.set_int("chj_windows", 0)
        line["chj_windowed"] = {"windows": windows, "value": tuples / (statistics.mean(wms) / 1e3), "ms_per_step": statistics.mean(wms),
                                "fingerprint_equals_phj_pure": fp_w == fp_main}

    hb = hp = None
    if not (args.no_e2e and (args.no_cpu or rank != 0 or world != 1)):
        hb, hp = host_streams_from_device(ctx, b, p)
    # -------- end to end through the C ABI with host buffers --------
    if not args.no_e2e:
        pin = []
        for s in (hb, hp):
            keys = ctx.pinned((len(s.keys),), np.uint64)
            keys[:] = s.keys
            cols = []
            for c in s.payloads:
                a = ctx.pinned(c.shape, c.dtype)
                a[...] = c
                cols.append(a)
            pin.append(P.BlockStream(s.types, keys, cols, block_rows=s.block_rows))
        cap = out_rows
        okeys = ctx.pinned((cap,), np.uint64)
        oleft = [ctx.pinned((cap, 2), np.uint64) if t == 4 else ctx.pinned((cap,), P.TYPE_DTYPE[t]) for t in bspec["types"]]
        oright = [ctx.pinned((cap, 2), np.uint64) if t == 4 else ctx.pinned((cap,), P.TYPE_DTYPE[t]) for t in pspec["types"]]
        h2d = sum(s.keys.nbytes + sum(c.nbytes for c in s.payloads) for s in pin)
        d2h = out_rows * (8 + sum(WIDTH[t] for t in bspec["types"]) + sum(WIDTH[t] for t in pspec["types"]))
        e2e_t, e2e_warm = [], []
        n_warm = max(1, args.warmup)  # as the device-resident steps: the first calls warm the host paths
        for i in range(args.e2e_steps + n_warm):
            dist.barrier()
            t0 = time.perf_counter()
            if scheme == "phj-pure":
                # runPHJ with host buffers: chunked probe upload, join and
                # output download overlapped inside the call
                rows_e2e, _ = ctx.run_phj_pure_host(pin[0], pin[1], bits, okeys, oleft, oright)
                t1 = time.perf_counter()
                assert rows_e2e == out_rows
            elif scheme == "phj":
                # runPhjBep with host buffers: batch uploads, joins and
                # downloads overlapped inside the call
                rows_e2e, _ = ctx.run_phj_bep_host(pin[0], pin[1], bits, budget, okeys, oleft, oright)
                t1 = time.perf_counter()
                assert rows_e2e == out_rows
            else:
                tb, tp = ctx.upload(pin[0]), ctx.upload(pin[1])
                out, _ = run_scheme(ctx, scheme, tb, tp, bits, budget)
                out.download((okeys, oleft, oright))
                t1 = time.perf_counter()
                out.free(), tb.free(), tp.free()
            (e2e_t if i >= n_warm else e2e_warm).append(t1 - t0)
        e2e_s = dist.max(statistics.mean(e2e_t))
        line["e2e"] = {"value": total_tuples / e2e_s, "unit": "tuples/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                       "ms_per_step": e2e_s * 1e3, "runs_ms": [round(t * 1e3, 2) for t in e2e_t],
                       "warmup_runs_ms": [round(t * 1e3, 2) for t in e2e_warm],
                       "path": {"phj-pure": "phj_run_phj_pure_host (pinned host inputs and output columns)",
                                "phj": "phj_run_phj_bep_host (pinned host inputs and output columns)"}.get(
                                    scheme, "phj_table_upload + scheme + phj_output_download")}
        del pin

    # -------- CPU baseline (rank 0, N = 1 only) --------
    if rank == 0 and world == 1 and not args.no_cpu:
        try:
            ncpu = os.cpu_count() or 1
            line["cpu_baseline"] = cpu_baseline(hb, hp, bits, args.cpu_probe_frac, ncpu, scheme,
                                                budget_mib=cpu_budget_mib(args.workload, ncpu))
        except Exception as e:  # the baseline is reported, never the target
            line["cpu_baseline"] = {"value": None, "error": str(e)}
    if args.csv and rank == 0:
        import report
        common = dict(threads=1, build_rows=B, probe_rows=Pn, build_types=bspec["types"], probe_types=pspec["types"],
                      partitions=1 << sum(bits), distribution="synthetic", match_rate=pspec.get("match_permille", 1000) / 1000,
                      gpu_device="GB300")
        rows = [report.result_row(scheme, i, r, tuples_per_s=tuples / (r.e2e_wall_ms / 1e3), dominant_kernel=dom_name,
                                  roofline_frac=achieved / peak, dram_gbps=bmin / (r.e2e_wall_ms / 1e3) / 1e9, **common)
                for i, r in enumerate(step_results)]
        if "chj" in line:
            rows += [report.result_row("chj", i, r, tuples_per_s=tuples / (r.e2e_wall_ms / 1e3), **common)
                     for i, r in enumerate(chj_results)]
        report.write_csv(args.csv, rows)
    b.free(), p.free()
    ctx.close()
    # -------- batched / served request stream versus the plain form --------
    if rank == 0 and args.serve_requests > 0:
        line["batched_serving"] = serving_benchmark(args.serve_requests, args.serve_slots, args.serve_batch_rows)
    if rank == 0:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
