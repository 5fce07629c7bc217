"""Autotuner for the AUTO selector (project-written; replaces the reference's
-vary_params sweep, src/autotune_hausdorff_distance.cu:208-299, and the
XGBoost trees trained from it, src/models/tree_*.h).

    python -m hausdorffdistance_gb300.autotune [--quick] [--write]

For a sweep of synthetic workloads (uniform 2-D, Gaussian clusters 3-D,
LiDAR-like planes 3-D, coherent polylines 2-D; several sizes; both
directions) it times every index-free and index-based variant on the GPU
(device-resident inputs, CUDA-event time reported by the library) and records
the sampler statistic the selector sees: the 80th percentile of sampled
early-break iteration counts, p80, and ratio = |A| * p80 / (|A| + |B|).
It then fits the selector's table:

  eb_ratio     the threshold on ratio below which EB is chosen: the value
               minimising the total time of the sweep's choices;
  prefer_grid  whether the grid beats the LBVH in total over the sweep.

--write regenerates hausdorffdistance_gb300/csrc/hd_tuning_table.h and
records the sweep in hausdorffdistance_gb300/tuning_sweep.json (or both in
--out DIR).
"""
from __future__ import annotations

import argparse
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
    sizes2 = [20_000, 200_000] if quick else [20_000, 200_000, 2_000_000]
    sizes3 = [100_000, 1_000_000] if quick else [100_000, 1_000_000, 10_000_000]
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


def time_variant(eng, ta, tb, variant, reps=3):
    best = float("inf")
    for _ in range(reps):
        r = eng.solve(ta, tb, variant=variant, timing=True)
        best = min(best, r.ms)
    return best, r


def sweep(quick: bool):
    import torch
    rows = []
    with hd.Engine() as eng:
        for name, a, b in workloads(quick):
            for direction, (x, y) in enumerate([(a, b), (b, a)]):
                tx = torch.from_numpy(np.ascontiguousarray(x)).cuda()
                ty = torch.from_numpy(np.ascontiguousarray(y)).cuda()
                rec = {"case": name, "direction": direction, "n_a": len(x), "n_b": len(y)}
                r = eng.solve(tx, ty, variant="auto")
                rec["p80"] = r.sample_p80[0]
                rec["ratio"] = len(x) * r.sample_p80[0] / (len(x) + len(y))
                for v in ("eb", "lbvh", "grid"):
                    ms, rv = time_variant(eng, tx, ty, v)
                    rec[v] = ms
                    assert rv.hd_f32 == r.hd_f32
                rows.append(rec)
                print(json.dumps(rec), flush=True)
    return rows


def fit(rows):
    index_best = {}
    grid_total = sum(r["grid"] for r in rows)
    lbvh_total = sum(r["lbvh"] for r in rows)
    prefer_grid = grid_total < lbvh_total
    idx = "grid" if prefer_grid else "lbvh"
    cands = sorted({0.0} | {r["ratio"] * 1.0001 for r in rows} | {1e30})
    best_t, best_cost = None, float("inf")
    for t in cands:
        cost = sum(r["eb"] if r["ratio"] < t else r[idx] for r in rows)
        if cost < best_cost:
            best_t, best_cost = t, cost
    index_best["total_ms_chosen"] = best_cost
    index_best["total_ms_oracle_choice"] = sum(min(r["eb"], r["lbvh"], r["grid"]) for r in rows)
    return {"eb_ratio": best_t, "prefer_grid": prefer_grid, **index_best}


def write_table(params, path):
    with open(path, "w") as f:
        f.write("// Generated by hausdorffdistance_gb300/autotune.py — do not edit by hand.\n")
        f.write("#pragma once\n")
        f.write("#define HD_TUNED_EB_SMALL_PAIRS 4194304.0\n")
        f.write(f"#define HD_TUNED_EB_RATIO {params['eb_ratio']:.6g}\n")
        f.write("#define HD_TUNED_BF16_MIN_PAIRS 67108864.0\n")
        f.write(f"#define HD_TUNED_PREFER_GRID {1 if params['prefer_grid'] else 0}\n")
        f.write("#define HD_TUNED_LEAF_SIZE 16\n")
        f.write("#define HD_TUNED_BATCH_SMALL 512\n")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--quick", action="store_true")
    ap.add_argument("--write", action="store_true")
    ap.add_argument("--out", default=None,
                    help="directory for the table and the sweep record (default: in place)")
    args = ap.parse_args()
    rows = sweep(args.quick)
    params = fit(rows)
    print(json.dumps(params))
    if args.write:
        table_dir = args.out or os.path.join(HERE, "csrc")
        sweep_dir = args.out or HERE
        os.makedirs(table_dir, exist_ok=True)
        write_table(params, os.path.join(table_dir, TABLE_NAME))
        with open(os.path.join(sweep_dir, SWEEP_NAME), "w") as f:
            json.dump({"rows": rows, "fit": params}, f, indent=1)


if __name__ == "__main__":
    main()
