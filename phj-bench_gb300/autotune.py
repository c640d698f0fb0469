"""Measuring autotuner for the device join.

For a (build, probe) pair resident on the device it times candidate
configurations of one scheme and keeps the fastest: radix bits and pass
count, leaf-table load factor (table_cap_pct), the first radix pass's tile
rows and bulk-copy ring depth, whether the probe side's pass is written
out, and its width (probe_pass_bits).  The search is coordinate descent from the heuristic start
(phj_autotune_radix): each knob in turn is swept with the others held, and
the best value is kept.  Results are cached per (scheme, log2 build rows,
log2 probe rows, build/probe row widths) in a JSON file, so a later join of
the same shape reuses them without measuring.

Every candidate runs through the same C ABI as a normal join; the outputs
of all candidates are the same multiset of rows (the configuration changes
the speed only), which `tune` checks through the device fingerprint.
"""
from __future__ import annotations

import json
import math
import os
import statistics
from typing import Dict, List, Optional, Sequence

import phj_gpu as P

KNOBS = ("pass_bits", "table_cap_pct", "p1_tile_rows", "p1_stages", "probe_materialize", "probe_pass_bits")
DEFAULT_CACHE = os.path.join(os.path.expanduser("~"), ".cache", "phj_gb300_tune.json")


def shape_key(scheme: str, build_rows: int, probe_rows: int, build_types: Sequence[int], probe_types: Sequence[int]) -> str:
    wb = 8 + sum(P.TYPE_WIDTH[t] for t in build_types)
    wp = 8 + sum(P.TYPE_WIDTH[t] for t in probe_types)
    lb = int(math.log2(max(build_rows, 1)))
    lp = int(math.log2(max(probe_rows, 1)))
    return f"{scheme}:b{lb}:p{lp}:w{wb}x{wp}"


def split_bits(total: int, passes: int) -> List[int]:
    """The CLI's split (src/CLI.cpp:330-348): extra bits to the earlier passes."""
    return [total // passes + (1 if i < total % passes else 0) for i in range(passes)]


def radix_candidates(build_rows: int) -> List[List[int]]:
    """Total bits around the heuristic (leaves of ~256 rows) and 1-3 passes."""
    start = sum(P.autotune_radix(build_rows))
    out = []
    for total in range(max(1, start - 2), min(24, start + 2) + 1):
        for passes in (1, 2, 3):
            if passes > total:
                continue
            bits = split_bits(total, passes)
            if max(bits) <= 16 and bits not in out:
                out.append(bits)
    return out


def knob_values(build_rows: int) -> Dict[str, list]:
    return {
        "pass_bits": radix_candidates(build_rows),
        "table_cap_pct": [200, 300, 150],
        "p1_tile_rows": [0, 4096, 2048, 1024],
        "p1_stages": [0, 2, 3, 4],
        "probe_materialize": [-1, 1, 0],
        "probe_pass_bits": [0, 5, 6, 7, 8],
    }


def apply(ctx: "P.Context", cfg: dict) -> None:
    for k in ("table_cap_pct", "p1_tile_rows", "p1_stages", "probe_materialize", "probe_pass_bits"):
        if k in cfg:
            ctx.set_int(k, int(cfg[k]))


def reset(ctx: "P.Context") -> None:
    apply(ctx, {"table_cap_pct": 200, "p1_tile_rows": 0, "p1_stages": 0, "probe_materialize": -1, "probe_pass_bits": 0})


def _time(ctx, scheme, b, p, cfg, reps, budget_mib):
    apply(ctx, cfg)
    times, fp = [], None
    for i in range(reps + 1):
        ctx.flush_l2()
        if scheme == "phj":
            out, res = ctx.run_phj_bep(b, p, cfg["pass_bits"], budget_mib)
        else:
            out, res = ctx.run_phj_pure(b, p, cfg["pass_bits"])
        if i == 0:
            fp = out.fingerprint()
        else:
            times.append(res.e2e_wall_ms)
        out.free()
    return statistics.median(times), fp


def tune(ctx: "P.Context", build: "P.Table", probe: "P.Table", scheme: str = "phj-pure", reps: int = 3, budget_mib: int = 512,
         cache_path: Optional[str] = DEFAULT_CACHE, use_cache: bool = True, log=None) -> dict:
    """Returns the fastest configuration found (and applies its context
    options to `ctx`): {"pass_bits", "table_cap_pct", "p1_tile_rows",
    "p1_stages", "probe_materialize", "probe_pass_bits", "ms", "trials"}."""
    key = shape_key(scheme, build.rows, probe.rows, build.types, probe.types)
    cache = {}
    if cache_path and use_cache and os.path.exists(cache_path):
        try:
            cache = json.load(open(cache_path))
        except (OSError, ValueError):
            cache = {}
        if key in cache:
            apply(ctx, cache[key])
            return dict(cache[key], cached=True)
    values = knob_values(build.rows)
    best = {"pass_bits": P.autotune_radix(build.rows), "table_cap_pct": 200, "p1_tile_rows": 0, "p1_stages": 0,
            "probe_materialize": -1, "probe_pass_bits": 0}
    best_ms, ref_fp = _time(ctx, scheme, build, probe, best, reps, budget_mib)
    trials = 1
    for knob in KNOBS:
        for v in values[knob]:
            if v == best[knob]:
                continue
            cand = dict(best, **{knob: v})
            try:
                ms, fp = _time(ctx, scheme, build, probe, cand, reps, budget_mib)
            except P.PhjError:
                continue  # a candidate the device rejects (e.g. a tile that does not fit)
            trials += 1
            if fp != ref_fp:
                raise RuntimeError(f"autotune: candidate {cand} changed the join's output")
            if log:
                log(f"{knob}={v}: {ms:.3f} ms (best {best_ms:.3f})")
            if ms < best_ms:
                best, best_ms = cand, ms
    reset(ctx)
    apply(ctx, best)
    result = dict(best, ms=best_ms, trials=trials)
    if cache_path:
        cache[key] = result
        os.makedirs(os.path.dirname(cache_path), exist_ok=True)
        with open(cache_path, "w") as f:
            json.dump(cache, f, indent=1)
    return result
