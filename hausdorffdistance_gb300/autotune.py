"""Autotuner for the AUTO selector (project-written; replaces the reference's
-vary_params sweep, src/autotune_hausdorff_distance.cu:208-299, and the
XGBoost trees trained from it, src/models/tree_*.h).

    python -m hausdorffdistance_gb300.autotune [--quick] [--write]

For a sweep of synthetic workloads (uniform 2-D, Gaussian clusters 3-D,
LiDAR-like planes 3-D, coherent polylines 2-D; several sizes; both
directions) it times every index-free and index-based variant on the GPU
(device-resident inputs, CUDA-event time reported by the library) and records
the statistics the selector sees: the mean (and the 80th percentile, p80) of
sampled early-break iteration counts and ratio = |A| * mean / (|A| + |B|); the
fraction of
sampled queries outside the target's box (outside) and the target's cell
occupancy skew (skew).  It then fits the selector's table:

  eb_small_pairs
               size band (|A| * |B|) below which EB is chosen without
               sampling (index_min_pairs, above which the LBVH is chosen
               without sampling, and eb_sample_max_pairs, the largest problem
               the EB sample runs on, are fixed by design);
  eb_ratio     the threshold on ratio below which EB is chosen;
  grid_max_outside, grid_max_skew
               the grid is chosen when both statistics are at or below them;
  (each minimising the total time of the sweep's choices).

The batch sweep (skipped with --no-batch) times the batched solver on the
lognormal polyline batch for each schedule (one-warp threshold
batch_small_rows x items per warp step batch_chunk x bound-window half-width
batch_window) and keeps the fastest.  The budget sweep (--no-budget) times
undirected LBVH solves on clustered, planar and uniform sets for each
per-packet traversal budget (lbvh_budget) and keeps the smallest total.

--write regenerates hausdorffdistance_gb300/csrc/hd_tuning_table.h and
records the sweep in hausdorffdistance_gb300/tuning_sweep.json (or both in
--out DIR).
"""
from __future__ import annotations

import argparse
import itertools
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import hausdorffdistance_gb300 as hd  # noqa: E402
from hausdorffdistance_gb300 import synth  # noqa: E402

TABLE_NAME = "hd_tuning_table.h"
SWEEP_NAME = "tuning_sweep.json"


def workloads(quick: bool):
    sizes2 = [1_000, 3_000, 20_000, 200_000] if quick else [1_000, 3_000, 20_000, 200_000,
                                                            2_000_000]
    sizes3 = [2_000, 10_000, 100_000, 1_000_000] if quick else [2_000, 10_000, 100_000,
                                                               1_000_000, 10_000_000]
    for n in sizes2:
        a, b = synth.uniform2d(n, seed=101)
        yield f"uniform2d_{n}", a, b
    for n in sizes3:
        a, b = synth.clusters3d(n, seed=102)
        yield f"clusters3d_{n}", a, b
    for n in ([1_000_000] if quick else [1_000_000, 10_000_000]):
        a, b = synth.planes3d(n, seed=103, n_planes=max(10, n // 100_000))
        yield f"planes3d_{n}", a, b
    a, b, _ = synth.polylines(sizes=[50_000], seed=104)
    yield "polyline_50000", a, b
    for n in ([100_000] if quick else [100_000, 1_000_000]):
        a, b = duplicated3d(n, seed=105)
        yield f"duplicated3d_{n}", a, b


def duplicated3d(n, seed=105, sites=16):
    """Heavily duplicated 3-D data: every point is one of `sites` locations
    (both sets), the case where the early break stops after a few pairs."""
    rng = np.random.default_rng(seed)
    c = rng.random((sites, 3)).astype(np.float32)
    return (np.ascontiguousarray(c[rng.integers(0, sites, n)]),
            np.ascontiguousarray(c[rng.integers(0, sites, n)]))


def time_variant(eng, ta, tb, variant, reps=3):
    best = float("inf")
    for _ in range(reps):
        r = eng.solve(ta, tb, variant=variant, timing=True)
        best = min(best, r.ms)
    return best, r


def sweep(quick: bool):
    import torch
    rows = []
    with hd.Engine(always_sample=True) as eng:
        for name, a, b in workloads(quick):
            for direction, (x, y) in enumerate([(a, b), (b, a)]):
                tx = torch.from_numpy(np.ascontiguousarray(x)).cuda()
                ty = torch.from_numpy(np.ascontiguousarray(y)).cuda()
                rec = {"case": name, "direction": direction, "n_a": len(x), "n_b": len(y)}
                r = eng.solve(tx, ty, variant="auto")
                rec["p80"] = r.sample_p80[0]
                rec["mean"] = r.sample_mean[0]
                rec["ratio"] = len(x) * r.sample_mean[0] / (len(x) + len(y))
                rec["outside"] = r.grid_outside[0]
                rec["skew"] = r.grid_skew[0]
                for v in ("eb", "lbvh", "grid"):
                    ms, rv = time_variant(eng, tx, ty, v)
                    rec[v] = ms
                    assert rv.hd_f32 == r.hd_f32
                rows.append(rec)
                print(json.dumps(rec), flush=True)
    return rows


INDEX_MIN_PAIRS = 1e13
EB_SAMPLE_MAX_PAIRS = 1e10


def choose(r, small, eb_ratio, max_outside, max_skew):
    """The selector's choice for a sweep row under a table."""
    if r["pairs"] <= small:
        return "eb"
    if r["pairs"] >= INDEX_MIN_PAIRS:
        return "lbvh"
    if r["pairs"] <= EB_SAMPLE_MAX_PAIRS and r["ratio"] < eb_ratio:
        return "eb"
    if r.get("outside", 1.0) <= max_outside and r.get("skew", 1e30) <= max_skew:
        return "grid"
    return "lbvh"


def fit(rows):
    """Fits the selector table: each parameter is chosen from the sweep's own
    values to minimise the sweep's total time (coordinate search, three
    rounds)."""
    for r in rows:
        r.setdefault("pairs", float(r.get("n_a", 1)) * float(r.get("n_b", 1)))

    def cost(*p):
        return sum(r[choose(r, *p)] for r in rows)

    pair_c = sorted({0.0} | {r["pairs"] for r in rows})
    ratio_c = sorted({0.0} | {r["ratio"] * 1.0001 for r in rows})
    out_c = sorted({0.0} | {r.get("outside", 0.0) * 1.0001 for r in rows})
    skew_c = sorted({0.0} | {r.get("skew", 0.0) * 1.0001 for r in rows})
    p = [0.0, 0.0, 0.0, 0.0]
    for _ in range(3):
        for i, cands in enumerate((pair_c, ratio_c, out_c, skew_c)):
            p[i] = min(cands, key=lambda x: (cost(*(p[:i] + [x] + p[i + 1:])), x))
    return {"eb_small_pairs": p[0], "index_min_pairs": INDEX_MIN_PAIRS, "eb_ratio": p[1],
            "eb_sample_max_pairs": EB_SAMPLE_MAX_PAIRS, "grid_max_outside": p[2],
            "grid_max_skew": p[3], "total_ms_chosen": cost(*p),
            "total_ms_oracle_choice": sum(min(r["eb"], r["lbvh"], r["grid"]) for r in rows)}


BATCH_SMALL_ROWS = (512, 1024, 2048, 4096, 8192)
BATCH_CHUNKS = (8,)
BATCH_WINDOWS = (1, 2, 4)
BATCH_DEFAULT = {"batch_small_rows": 8192, "batch_chunk": 8, "batch_window": 4}
LBVH_BUDGET_DEFAULT = 256
EB_CAP_DEFAULT = {"eb_cap_div": 512, "eb_cap_min": 4096, "eb_cap_max": 65536}
LBVH_BUDGETS = (128, 256, 512, 1024, 4096)


def batch_sweep(quick: bool, reps: int = 9):
    """Times every batch schedule on the polyline batch (device-resident
    inputs, wall time around the synchronous call); all schedules must give
    identical results."""
    import time
    import torch
    n = 20_000 if quick else 100_000
    a, b, off = synth.polylines(n_problems=n, seed=104)
    ta, tb = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    rows, ref = [], None
    for small, chunk, window in itertools.product(BATCH_SMALL_ROWS, BATCH_CHUNKS, BATCH_WINDOWS):
        with hd.Engine(batch_small_rows=small, batch_chunk=chunk, batch_window=window) as eng:
            out = eng.solve_batch(ta, tb, off, off, undirected=True)
            if ref is None:
                ref = out["hd_f32"].copy()
            assert np.array_equal(out["hd_f32"], ref), (small, chunk, window)
            best = float("inf")
            for _ in range(reps):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                eng.solve_batch(ta, tb, off, off, undirected=True)
                best = min(best, (time.perf_counter() - t0) * 1e3)
        rec = {"batch_small_rows": small, "batch_chunk": chunk, "batch_window": window,
               "ms": best, "problems": n}
        rows.append(rec)
        print(json.dumps(rec), flush=True)
    return rows


def budget_sweep(quick: bool, reps: int = 7):
    """Times undirected LBVH solves for each per-packet traversal budget on
    the clustered, planar and uniform workloads (CUDA-event time reported by
    the library); every budget must give the same distance."""
    import torch
    cases = [("clusters3d", synth.clusters3d(1_000_000 if quick else 10_000_000, seed=102)),
             ("planes3d", synth.planes3d(1_000_000 if quick else 10_000_000, seed=103,
                                         n_planes=100)),
             ("uniform2d", synth.uniform2d(200_000, seed=101))]
    rows = []
    for name, (a, b) in cases:
        ta, tb = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
        ref = None
        for budget in LBVH_BUDGETS:
            with hd.Engine(lbvh_budget=budget) as eng:
                eng.solve(ta, tb, undirected=True, variant="lbvh")
                best = float("inf")
                for _ in range(reps):
                    r = eng.solve(ta, tb, undirected=True, variant="lbvh", timing=True)
                    best = min(best, r.ms)
            if ref is None:
                ref = r.hd_f32
            assert r.hd_f32 == ref, (name, budget)
            rec = {"case": name, "lbvh_budget": budget, "ms": best, "deferred": int(r.rechecked)}
            rows.append(rec)
            print(json.dumps(rec), flush=True)
    return rows


def fit_budget(rows):
    """The budget with the smallest total time over the sweep's cases."""
    totals = {}
    for r in rows:
        totals[r["lbvh_budget"]] = totals.get(r["lbvh_budget"], 0.0) + r["ms"]
    best = min(totals, key=lambda k: (totals[k], k))
    return {"lbvh_budget": best, "lbvh_budget_total_ms": totals[best]}


def fit_batch(rows):
    best = min(rows, key=lambda r: r["ms"])
    return {"batch_small_rows": best["batch_small_rows"], "batch_chunk": best["batch_chunk"],
            "batch_window": best.get("batch_window", BATCH_DEFAULT["batch_window"]),
            "batch_ms": best["ms"]}


def read_table(path):
    """The parameters of an existing table (sweeps that are skipped keep them)."""
    import re
    vals = dict(re.findall(r"#define HD_TUNED_(\w+) (\S+)", open(path).read()))
    out = {"eb_small_pairs": float(vals["EB_SMALL_PAIRS"]),
           "index_min_pairs": float(vals["INDEX_MIN_PAIRS"]),
           "eb_ratio": float(vals["EB_RATIO"]),
           "eb_sample_max_pairs": float(vals["EB_SAMPLE_MAX_PAIRS"]),
           "grid_max_outside": float(vals["GRID_MAX_OUTSIDE"]),
           "grid_max_skew": float(vals["GRID_MAX_SKEW"])}
    for key, name in (("batch_small_rows", "BATCH_SMALL_ROWS"), ("batch_chunk", "BATCH_CHUNK"),
                      ("batch_window", "BATCH_WINDOW"), ("lbvh_budget", "LBVH_BUDGET"),
                      ("eb_cap_div", "EB_CAP_DIV"), ("eb_cap_min", "EB_CAP_MIN"),
                      ("eb_cap_max", "EB_CAP_MAX")):
        if name in vals:
            out[key] = int(vals[name])
    return out


def write_table(params, path):
    with open(path, "w") as f:
        f.write("// Generated by hausdorffdistance_gb300/autotune.py — do not edit by hand.\n")
        f.write("#pragma once\n")
        f.write(f"#define HD_TUNED_EB_SMALL_PAIRS {params['eb_small_pairs']:.6g}\n")
        f.write(f"#define HD_TUNED_INDEX_MIN_PAIRS {params['index_min_pairs']:.6g}\n")
        f.write(f"#define HD_TUNED_EB_RATIO {params['eb_ratio']:.6g}\n")
        f.write("#define HD_TUNED_BF16_MIN_PAIRS 67108864.0\n")
        f.write(f"#define HD_TUNED_EB_SAMPLE_MAX_PAIRS {params['eb_sample_max_pairs']:.6g}\n")
        f.write(f"#define HD_TUNED_GRID_MAX_OUTSIDE {params['grid_max_outside']:.6g}\n")
        f.write(f"#define HD_TUNED_GRID_MAX_SKEW {params['grid_max_skew']:.6g}\n")
        f.write("#define HD_TUNED_LEAF_SIZE 16\n")
        f.write(f"#define HD_TUNED_BATCH_SMALL_ROWS "
                f"{params.get('batch_small_rows', BATCH_DEFAULT['batch_small_rows'])}\n")
        f.write(f"#define HD_TUNED_BATCH_CHUNK "
                f"{params.get('batch_chunk', BATCH_DEFAULT['batch_chunk'])}\n")
        f.write(f"#define HD_TUNED_BATCH_WINDOW "
                f"{params.get('batch_window', BATCH_DEFAULT['batch_window'])}\n")
        f.write(f"#define HD_TUNED_LBVH_BUDGET {params.get('lbvh_budget', LBVH_BUDGET_DEFAULT)}\n")
        for key, name in (("eb_cap_div", "EB_CAP_DIV"), ("eb_cap_min", "EB_CAP_MIN"),
                          ("eb_cap_max", "EB_CAP_MAX")):
            f.write(f"#define HD_TUNED_{name} {params.get(key, EB_CAP_DEFAULT[key])}\n")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--quick", action="store_true")
    ap.add_argument("--write", action="store_true")
    ap.add_argument("--out", default=None,
                    help="directory for the table and the sweep record (default: in place)")
    ap.add_argument("--no-batch", action="store_true", help="skip the batch schedule sweep")
    ap.add_argument("--no-budget", action="store_true", help="skip the LBVH budget sweep")
    ap.add_argument("--batch-only", action="store_true",
                    help="only the schedule sweeps (batch, LBVH budget); the selector keeps "
                         "the current table")
    args = ap.parse_args()
    if args.batch_only:
        # The selector keeps the committed table and sweep record.
        params = read_table(os.path.join(HERE, "csrc", TABLE_NAME))
        with open(os.path.join(HERE, SWEEP_NAME)) as f:
            rows = json.load(f)["rows"]
    else:
        rows = sweep(args.quick)
        params = fit(rows)
        # Schedule values whose sweeps are skipped keep what the table holds.
        kept = read_table(os.path.join(HERE, "csrc", TABLE_NAME))
        for key in ("batch_small_rows", "batch_chunk", "batch_window", "lbvh_budget",
                    "eb_cap_div", "eb_cap_min", "eb_cap_max"):
            if key in kept:
                params.setdefault(key, kept[key])
    batch_rows, budget_rows = [], []
    if not args.no_batch:
        batch_rows = batch_sweep(args.quick)
        params.update(fit_batch(batch_rows))
    if not args.no_budget:
        budget_rows = budget_sweep(args.quick)
        params.update(fit_budget(budget_rows))
    print(json.dumps(params))
    if args.write:
        table_dir = args.out or os.path.join(HERE, "csrc")
        sweep_dir = args.out or HERE
        os.makedirs(table_dir, exist_ok=True)
        write_table(params, os.path.join(table_dir, TABLE_NAME))
        with open(os.path.join(sweep_dir, SWEEP_NAME), "w") as f:
            json.dump({"rows": rows, "batch_rows": batch_rows, "budget_rows": budget_rows,
                       "fit": params}, f, indent=1)


if __name__ == "__main__":
    main()
