"""Benchmark: Hausdorff solves/s (and Gpairs/s) on one GB300 per rank.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload clusters3d|uniform2d|planes3d] [--n POINTS]
                    [--variant auto|eb|lbvh|grid] [--directed]

A step is one undirected Hausdorff solve H(A,B) = max(h(A,B), h(B,A)) of the
workload through libhdgpu.so's C ABI.  The default workload is the 3-D
Gaussian mixture: |A| = |B| = 10,000,000 points, 64 clusters, sigma 0.01, B
shifted by (0.05, 0, 0) (seeded synthetic data standing in for the
reference's real datasets).  Inputs are larger than L2 (2 x 120 MB), so no
flush is needed between steps.

value   solves/s with A and B already resident in HBM (device pointers),
        CUDA events on the library's stream, max over ranks, x N ranks.
e2e     the same solve through the C ABI from pinned host buffers: the H2D
        copies of A and B and the D2H read of the result are inside the
        timed region.
Multi-GPU: each rank solves its own replica (the solve does not shard); the
whole-job value is the number of solves all ranks completed / max time.

--impl reference times the reference's CPU early-break (the oracle's
restatement of src/hd_impl/hausdorff_distance_early_break.h:44-115) on the
host cores, on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PEAKS_PATH = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0
METRIC = "Hausdorff solves/s & Gpairs/s at rel err<=1e-6, chosen vs plain FP32, 1 GB300"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="clusters3d",
                   choices=["clusters3d", "uniform2d", "planes3d", "unit64", "polylines"])
    p.add_argument("--n", type=int, default=0, help="points per set (default: workload size)")
    p.add_argument("--variant", default="auto")
    p.add_argument("--directed", action="store_true")
    p.add_argument("--no-compare", action="store_true", help="skip the plain-EB comparison")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    p.add_argument("--profile", action="store_true",
                   help="one solve and exit (the command profiled under ncu)")
    return p.parse_args()


WORKLOAD_SIZES = {"clusters3d": 10_000_000, "uniform2d": 200_000, "planes3d": 50_000_000,
                  "unit64": 1_000_000, "polylines": 100_000}


def make_data(name, n):
    from hausdorffdistance_gb300 import synth
    seed = {"clusters3d": 2, "uniform2d": 1, "planes3d": 5, "unit64": 3}[name]
    return getattr(synth, name)(n, seed=seed)


def workload_desc(name, n):
    return {
        "clusters3d": f"3-D Gaussian mixture, 64 clusters sigma 0.01, |A|=|B|={n}, B shifted (0.05,0,0)",
        "uniform2d": f"2-D uniform, |A|=|B|={n}, B = jittered permutation of A + 5% outliers",
        "planes3d": f"3-D LiDAR-like planes, |A|=|B|={n}, B = A rotated 1 deg + 0.1% outliers",
        "unit64": f"64-D unit rows, |A|=|B|={n}, B = A with 1% of rows replaced",
        "polylines": f"{n} 2-D polyline-pair problems, lognormal sizes (median 200, sigma 1.2)",
    }[name]


class ClockSampler:
    """nvidia-smi clock / throttle-reason sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def load_peaks():
    try:
        with open(PEAKS_PATH) as f:
            pk = json.load(f)
        return float(pk["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def traffic_from_profiles(kernel_tag, units):
    """Per-launch DRAM bytes of the dominant kernel from the committed ncu
    summary (profiles/<kernel>.txt, a line 'dram_bytes_per_unit: X'),
    scaled to this launch's units; None if no summary exists."""
    path = os.path.join(ROOT, "profiles", f"{kernel_tag}.txt")
    try:
        for ln in open(path):
            if ln.startswith("dram_bytes_per_unit:"):
                return float(ln.split(":", 1)[1]) * units
    except OSError:
        pass
    return None


def cpu_baseline(a, b, undirected, max_seconds=25.0):
    """The reference's CPU early-break (oracle restatement) on all host cores
    over bounded samples of A (first k points of the seeded shuffle), per
    direction, extrapolated to the full set from the marginal cost between two
    sample sizes.  Returns the baseline dict (solves/s)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import hd_oracle
    cores = os.cpu_count() or 1
    dirs = [(a, b), (b, a)] if undirected else [(a, b)]
    if a.shape[1] not in (2, 3):
        # The reference has no path for n_dims other than 2 and 3: time the
        # oracle's exact FP32 max-min (not reference code) on the first k rows
        # of A against all of B and extrapolate linearly (no early break).
        total_ms = 0.0
        detail = []
        for x, y in dirs:
            k = max(16, min(len(x), 64))
            t0 = time.perf_counter()
            hd_oracle.exact(x[:k], y, 32, n_threads=cores)
            ms = (time.perf_counter() - t0) * 1e3
            est = ms * len(x) / k
            total_ms += est
            detail.append({"sample_rows": k, "sample_ms": ms, "extrapolated_ms": est})
        return {"value": 1000.0 / total_ms, "unit": "solves/s", "cores": cores, "kind": "port",
                "sample": ("oracle exact FP32 max-min restatement (not reference code: the "
                           "reference supports n_dims 2 and 3 only), all host threads, first k "
                           "rows of A against all of B, extrapolated linearly: "
                           + json.dumps(detail))}
    total_ms = 0.0
    detail = []
    budget = max_seconds / len(dirs)
    for x, y in dirs:
        k1 = max(64, min(len(x), 2048))
        r1 = hd_oracle.eb(x, y, seed=0, n_threads=cores, limit_a=k1)
        # Grow the second sample while it stays well inside the budget.
        k2 = min(len(x), k1 * 4)
        if r1["compute_ms"] * 4 > budget * 1e3:
            k2 = k1
        r2 = hd_oracle.eb(x, y, seed=0, n_threads=cores, limit_a=k2) if k2 > k1 else r1
        if k2 >= len(x):
            est = r2["compute_ms"]
        else:
            marginal = max(0.0, (r2["compute_ms"] - r1["compute_ms"]) / max(1, k2 - k1))
            est = r2["compute_ms"] + marginal * (len(x) - k2)
        total_ms += est
        detail.append({"sample_points": [k1, k2], "sample_ms": [r1["compute_ms"], r2["compute_ms"]],
                       "extrapolated_ms": est})
    return {"value": 1000.0 / total_ms, "unit": "solves/s", "cores": cores, "kind": "port",
            "sample": ("reference CPU early-break restated (oracle/hd_oracle.cpp), all host "
                       "threads, per direction the first k of the seeded shuffle of A against all "
                       "of B for two k, extrapolated linearly from the marginal cost: "
                       + json.dumps(detail))}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    n = args.n or WORKLOAD_SIZES[args.workload]
    undirected = not args.directed
    if args.workload == "polylines":
        from hausdorffdistance_gb300 import synth
        a, b, off = synth.polylines(n_problems=n, seed=4)
        measure = lambda: cpu_baseline_batch(a, b, off, undirected, max_seconds=8.0)  # noqa: E731
    else:
        a, b = make_data(args.workload, n)
        measure = lambda: cpu_baseline(a, b, undirected, max_seconds=8.0)  # noqa: E731
    vals = []
    base = None
    for i in range(args.warmup + args.steps):
        base = measure()
        if i >= args.warmup:
            vals.append(base["value"])
    v = float(np.median(vals))
    base["value"] = v
    line = {"metric": METRIC, "value": v, "unit": "solves/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / v,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": workload_desc(args.workload, n),
                       "undirected": undirected, "l2": "inputs larger than L2"},
            "cpu_baseline": base,
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def cpu_baseline_batch(a, b, off, undirected, max_seconds=20.0):
    """Reference CPU early-break (oracle restatement), one thread per problem,
    problems spread over all host cores, on the first k problems of the
    (randomly ordered) batch; extrapolated to the whole batch by pair count."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import concurrent.futures as cf
    import hd_oracle
    cores = os.cpu_count() or 1
    sizes = np.diff(off)
    pairs = sizes.astype(np.float64) ** 2
    k = 0
    acc = 0.0
    budget_pairs = 4e9 * max_seconds / 20.0  # ~ what the cores finish in the budget
    while k < len(sizes) and acc < budget_pairs:
        acc += pairs[k]
        k += 1

    def one(p):
        x, y = a[off[p]:off[p + 1]], b[off[p]:off[p + 1]]
        hd_oracle.eb(x, y, n_threads=1)
        if undirected:
            hd_oracle.eb(y, x, n_threads=1)

    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=cores) as ex:
        list(ex.map(one, range(k)))
    t = time.perf_counter() - t0
    est = t * pairs.sum() / pairs[:k].sum()
    return {"value": len(sizes) / est, "unit": "solves/s", "cores": cores, "kind": "port",
            "sample": (f"reference CPU early-break restated (oracle/hd_oracle.cpp), n_threads=1 "
                       f"per problem, problems spread over {cores} host threads; first {k} of "
                       f"{len(sizes)} problems ({t:.2f} s), extrapolated by pair count")}


def main_batch(args):
    import torch

    import hausdorffdistance_gb300 as hd
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    n = args.n or WORKLOAD_SIZES["polylines"]
    from hausdorffdistance_gb300 import synth
    a, b, off = synth.polylines(n_problems=n, seed=4)
    undirected = not args.directed
    stream = torch.cuda.current_stream()
    eng = hd.Engine(device=local)
    eng.set_stream(stream.cuda_stream)
    ta = torch.from_numpy(a).cuda()
    tb = torch.from_numpy(b).cuda()
    if args.profile:
        eng.solve_batch(ta, tb, off, off, undirected=undirected)
        torch.cuda.synchronize()
        print(json.dumps({"profile_solve": True}), flush=True)
        return
    for _ in range(args.warmup):
        ref = eng.solve_batch(ta, tb, off, off, undirected=undirected)
    clocks = ClockSampler(local)
    clocks.start()
    l0 = eng.kernel_launches
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        res = eng.solve_batch(ta, tb, off, off, undirected=undirected)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    clk = clocks.stop()
    launches = eng.kernel_launches - l0
    assert np.array_equal(res["hd_f32"], ref["hd_f32"])
    value = world * n / (ms / 1e3)
    pa = torch.from_numpy(a).pin_memory().numpy()
    pb = torch.from_numpy(b).pin_memory().numpy()
    eng.solve_batch(pa, pb, off, off, undirected=undirected)
    t0 = time.perf_counter()
    ke = max(3, args.steps // 2)
    for _ in range(ke):
        eng.solve_batch(pa, pb, off, off, undirected=undirected)
    t_e2e = (time.perf_counter() - t0) / ke
    plain = None
    if not args.no_compare:
        t0 = time.perf_counter()
        rp = eng.solve_batch(ta, tb, off, off, undirected=undirected, plain=True)
        torch.cuda.synchronize()
        tp = time.perf_counter() - t0
        assert np.array_equal(rp["hd_f32"], res["hd_f32"]), "plain and batched disagree"
        plain = {"variant": "per-problem plain EB launches", "ms_per_step": tp * 1e3,
                 "solves_per_s": n / tp, "speedup_batched_vs_plain": tp * 1e3 / ms}
    peak, peak_kind = load_peaks()
    sizes = np.diff(off)
    alg = float((2 if undirected else 1) * (2 * sizes).sum() * 8)  # both sets, both directions
    achieved = alg / (ms / 1e3) / 1e9
    roof = {"bound": "hbm", "kernel": "batch_graph", "achieved": achieved, "peak": peak,
            "unit": "GB/s", "frac": achieved / peak, "traffic": traffic_from_profiles("batch", float(sizes.sum())),
            "algorithmic_bytes": alg, "kernel_ms": ms, "peak_source": peak_kind + " hbm_gbs"}
    base = None if (args.no_cpu or world > 1) else cpu_baseline_batch(a, b, off, undirected)
    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded numpy PCG64)",
            "config": {"workload": (f"{n} 2-D polyline-pair problems, sizes round(LogNormal(ln 200,"
                                    f" 1.2)) clipped to [8, 50000], {int(sizes.sum())} points "
                                    "per side"), "undirected": undirected,
                       "l2": "inputs larger than L2 (no flush)", "parallelism": f"replicas x{world}"},
            "gpairs_per_s_effective": float((sizes.astype(np.float64) ** 2).sum()
                                            * (2 if undirected else 1) / (ms / 1e3) / 1e9),
            "plain_per_problem": plain,
            "e2e": {"value": world * n / t_e2e, "unit": "solves/s",
                    "h2d_bytes_per_step": int(a.nbytes + b.nbytes + n * 32),
                    "d2h_bytes_per_step": int(n * 16)},
            "gpu_launches": int(launches), "roofline": roof, "cpu_baseline": base, "clocks": clk,
        }), flush=True)
    eng.close()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload == "polylines":
        main_batch(args)
        return
    import torch
    import torch.distributed as dist

    import hausdorffdistance_gb300 as hd

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if world > 1:
            dist.barrier()

    n = args.n or WORKLOAD_SIZES[args.workload]
    a, b = make_data(args.workload, n)
    undirected = not args.directed
    dims = a.shape[1]
    stream = torch.cuda.current_stream()
    eng = hd.Engine(device=local, variant=args.variant)
    eng.set_stream(stream.cuda_stream)
    ta = torch.from_numpy(a).cuda()
    tb = torch.from_numpy(b).cuda()
    if args.profile:
        r = eng.solve(ta, tb, undirected=undirected)
        torch.cuda.synchronize()
        print(json.dumps({"profile_solve": True, "hd_f32": float(r.hd_f32),
                          "variant_used": int(r.variant_used)}), flush=True)
        eng.close()
        return

    # Instrumented run (outside the timed region): visited pairs / nodes for
    # the algorithmic byte counts of the roofline.
    rc = eng.solve(ta, tb, undirected=undirected, count_pairs=True, timing=True)
    for _ in range(args.warmup):
        eng.solve(ta, tb, undirected=undirected)
    torch.cuda.synchronize()

    clocks = ClockSampler(local)
    clocks.start()
    launches0 = eng.kernel_launches
    phase = np.zeros(8)
    barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    res = None
    for _ in range(args.steps):
        res = eng.solve(ta, tb, undirected=undirected, timing=True)
        phase += np.array(res.phase_ms[:8])
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    elapsed_ms = ev0.elapsed_time(ev1)
    launches = eng.kernel_launches - launches0
    clk = clocks.stop()
    if world > 1:
        t = torch.tensor([elapsed_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed_ms = float(t.item())
    ms_step = elapsed_ms / args.steps
    value = world * args.steps / (elapsed_ms / 1e3)
    pairs_eff = (2 if undirected else 1) * float(n) * float(n)

    # End to end through the C ABI from pinned host buffers.
    pa = torch.from_numpy(a).pin_memory()
    pb = torch.from_numpy(b).pin_memory()
    na, nb = pa.numpy(), pb.numpy()
    for _ in range(2):
        eng.solve(na, nb, undirected=undirected)
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_steps = max(3, args.steps // 2)
    for _ in range(e2e_steps):
        re2e = eng.solve(na, nb, undirected=undirected)
    t_e2e = time.perf_counter() - t0
    if world > 1:
        t = torch.tensor([t_e2e], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_e2e = float(t.item())
    assert re2e.hd_f32 == res.hd_f32

    # Plain FP32 early-break on the same inputs ("chosen vs plain FP32").
    plain = None
    if not args.no_compare and args.variant != "eb":
        eng.solve(ta, tb, undirected=undirected, variant="eb")
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        ksteps = 2
        e0.record(stream)
        for _ in range(ksteps):
            rp = eng.solve(ta, tb, undirected=undirected, variant="eb")
        e1.record(stream)
        torch.cuda.synchronize()
        pms = e0.elapsed_time(e1) / ksteps
        assert rp.hd_f32 == res.hd_f32, "plain EB and chosen variant disagree"
        plain = {"variant": "eb", "ms_per_step": pms, "solves_per_s": 1e3 / pms,
                 "speedup_chosen_vs_plain": pms / ms_step}

    # Roofline of the dominant kernel of the chosen variant.
    peak, peak_kind = load_peaks()
    phase_avg = phase / args.steps
    names = ["prep", "build", "sample", "main_pass", "tail", "certify"]
    roof = None
    if res.variant_used in (hd._lib.VARIANT_LBVH, hd._lib.VARIANT_GRID):
        # Query pass (phase 3): algorithmic bytes = query points (16 B each)
        # + internal nodes visited (64 B) + leaf points scanned (16 B each).
        leaf = 16 if res.variant_used == hd._lib.VARIANT_LBVH else 0
        lf = rc.visited_leaves
        alg = (2 if undirected else 1) * n * 16 + rc.visited_nodes * 64 + lf * 16 * 16
        t_ms = phase_avg[3]
        tag = "lbvh_query" if res.variant_used == hd._lib.VARIANT_LBVH else "grid_query"
        achieved = alg / (t_ms / 1e3) / 1e9
        # An undirected LBVH solve answers both directions' queries in one
        # launch (the fused pass); otherwise one launch per direction.
        fused = (undirected and res.variant_used == hd._lib.VARIANT_LBVH
                 and res.variant_used_ba == hd._lib.VARIANT_LBVH)
        nl = 1 if (fused or not undirected) else 2
        tr = traffic_from_profiles(tag, float(n) * (2 if fused else 1))
        roof = {"bound": "hbm", "kernel": tag, "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "traffic": tr,
                "algorithmic_bytes_per_launch": alg / nl, "kernel_ms_per_launch": t_ms / nl,
                "launches": nl, "peak_source": peak_kind + " hbm_gbs"}
    elif res.variant_used == hd._lib.VARIANT_EB:
        # The EB scan is FP32-issue bound; its HBM view counts the B tiles each
        # CTA streams (16 B per point, one 256-point tile per 256 x 4 x 256
        # slot-pairs), reported with the pair rate beside it.
        t_ms = phase_avg[3]
        alg = rc.visited_pairs * 16.0 / (256 * 4)
        achieved = alg / (t_ms / 1e3) / 1e9
        roof = {"bound": "hbm", "kernel": "eb_main", "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "traffic": None,
                "kernel_ms": t_ms, "peak_source": peak_kind + " hbm_gbs",
                "pairs_per_s": rc.visited_pairs / (t_ms / 1e3)}

    if res.variant_used == hd._lib.VARIANT_BF16:
        # Split-BF16 contraction: 3 products x 2 K FLOP per (a, b) pair per
        # direction, against the sustained dense BF16 rate (a long kernel).
        K = ((dims + 15) // 16) * 16
        flops = (2 if undirected else 1) * 3.0 * 2.0 * K * float(n) * float(n)
        t_ms = phase_avg[3]
        try:
            with open(PEAKS_PATH) as f:
                pk = json.load(f)
            tpeak, tkind = float(pk["bf16_tflops_sustained"]), "measured bf16_tflops_sustained"
        except Exception:
            tpeak, tkind = 1700.0, "fallback sustained bf16"
        achieved = flops / (t_ms / 1e3) / 1e12
        roof = {"bound": "tensor", "kernel": "bf16_rowmin", "achieved": achieved, "peak": tpeak,
                "unit": "TFLOP/s", "frac": achieved / tpeak,
                "traffic": traffic_from_profiles("bf16_rowmin", float(n) * float(n)),
                "algorithmic_flops_per_launch": flops / (2 if undirected else 1),
                "kernel_ms_per_launch": t_ms / (2 if undirected else 1), "peak_source": tkind,
                "rechecked_rows": int(res.rechecked), "err_bound": res.err_bound}
    base = None
    if rank == 0 and world == 1 and not args.no_cpu:
        base = cpu_baseline(a, b, undirected)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded numpy PCG64)",
            "config": {"workload": workload_desc(args.workload, n), "n_a": n, "n_b": n,
                       "n_dims": dims, "undirected": undirected, "variant": args.variant,
                       "variant_used": [hd._lib.VARIANT_NAMES.get(res.variant_used),
                                        hd._lib.VARIANT_NAMES.get(res.variant_used_ba)],
                       "l2": "inputs larger than L2 (no flush)",
                       "parallelism": f"replicas x{world}"},
            "gpairs_per_s_effective": value * pairs_eff / 1e9,
            "gpairs_per_s_visited": (rc.visited_pairs * value / 1e9) if rc.visited_pairs else None,
            "hd_f32": float(res.hd_f32), "hd64_certified": res.hd,
            "certifying_pair": [int(res.ia), int(res.ib), int(res.direction)],
            "phase_ms": {nm: float(phase_avg[i]) for i, nm in enumerate(names)},
            "plain_fp32_eb": plain,
            "e2e": {"value": world * e2e_steps / t_e2e, "unit": "solves/s",
                    "h2d_bytes_per_step": int(a.nbytes + b.nbytes),
                    "d2h_bytes_per_step": 2 * 160},
            "gpu_launches": int(launches),
            "roofline": roof,
            "cpu_baseline": base,
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    eng.close()
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
