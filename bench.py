"""Benchmark: Hausdorff solves/s (and Gpairs/s) on one GB300 per rank.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload all|clusters3d|uniform2d|planes3d|unit64|polylines|
                                clusters3d_f64]
                    [--n POINTS] [--variant auto|eb|lbvh|grid|bf16] [--directed]

A step is one undirected Hausdorff solve H(A,B) = max(h(A,B), h(B,A)) of a
workload through libhdgpu.so's C ABI (for the polyline workload: one batched
solve of all its problems).  Workloads (seeded synthetic data with the shapes,
sizes and distributions of the benchmark configurations; the reference's real
datasets are not available):

  clusters3d  3-D Gaussian mixture, |A| = |B| = 10,000,000, 64 clusters,
              sigma 0.01, B shifted (0.05, 0, 0)          (the headline)
  uniform2d   2-D, |A| = |B| = 200,000, B a jittered permutation of A plus
              5% outliers
  unit64      64-D unit rows, |A| = |B| = 1,000,000, 1% of B replaced
  polylines   100,000 2-D polyline-pair problems, lognormal sizes
  planes3d    3-D LiDAR-like planes, |A| = |B| = 50,000,000, B rotated
              1 degree plus 0.1% outliers
  clusters3d_f64  the clusters3d sets in float64 with N(0, 1e-7) jitter (true
              double coordinates), solved exactly in FP64 (hd_solve_f64)

The default (--workload all) measures the headline at the top level of the
JSON line and the other five under "workloads", each with the same keys.
Inputs are larger than L2 (or the step's working set is), so no flush runs
between steps; "config.l2" says so per workload.

value     solves/s with A and B resident in HBM (device pointers), CUDA
          events on the library's stream around K steps, the same call a user
          makes (no timing instrumentation), max over ranks, x N ranks.
e2e       the same solve through the C ABI from pinned host buffers: the H2D
          copies of A and B and the D2H read of the result are inside the
          timed region.
phase_ms  per-phase device times from a separate instrumented run (HD_TIMING).
rel_err_vs_oracle  |hd - H64| / H64 where H64 is the oracle's independent FP64
          max-min (k-d tree, computed outside the timed region).
Multi-GPU: each rank solves its own replica (the solve does not shard); the
whole-job value is the number of solves all ranks completed / max time.

--impl reference runs the reference's CPU early-break (the oracle's
restatement of src/hd_impl/hausdorff_distance_early_break.h:44-115) on all host
cores: each step is one whole undirected solve of the headline workload when
it fits the step budget, else a bounded estimate (see cpu_eb_baseline).
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
FALLBACK = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}
METRIC = "Hausdorff solves/s & Gpairs/s at rel err<=1e-6, chosen vs plain FP32, 1 GB300"
ALL = ["clusters3d", "uniform2d", "unit64", "polylines", "planes3d", "clusters3d_f64"]
WORKLOAD_SIZES = {"clusters3d": 10_000_000, "uniform2d": 200_000, "planes3d": 50_000_000,
                  "unit64": 1_000_000, "polylines": 100_000, "clusters3d_f64": 10_000_000}
SEEDS = {"clusters3d": 2, "uniform2d": 1, "planes3d": 5, "unit64": 3, "polylines": 4,
         "clusters3d_f64": 2}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="all", choices=["all"] + ALL)
    p.add_argument("--n", type=int, default=0, help="points per set (default: workload size)")
    p.add_argument("--variant", default="auto")
    p.add_argument("--directed", action="store_true")
    p.add_argument("--no-compare", action="store_true", help="skip the plain-EB comparison")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    p.add_argument("--no-oracle", action="store_true", help="skip the FP64 oracle check")
    p.add_argument("--profile", action="store_true",
                   help="one solve of one workload and exit (the command profiled under ncu)")
    return p.parse_args()


def make_data(name, n):
    from hausdorffdistance_gb300 import synth
    if name == "polylines":
        return synth.polylines(n_problems=n, seed=SEEDS[name])
    if name == "clusters3d_f64":
        # The mixture in double precision: jitter below float resolution
        # makes every coordinate a true double.
        a, b = synth.clusters3d(n, seed=SEEDS[name])
        rng = np.random.default_rng(SEEDS[name] + 100)
        return (a.astype(np.float64) + rng.normal(0.0, 1e-7, a.shape),
                b.astype(np.float64) + rng.normal(0.0, 1e-7, b.shape))
    return getattr(synth, name)(n, seed=SEEDS[name])


def workload_desc(name, n):
    return {
        "clusters3d": f"3-D Gaussian mixture, 64 clusters sigma 0.01, |A|=|B|={n}, B shifted (0.05,0,0)",
        "uniform2d": f"2-D uniform, |A|=|B|={n}, B = jittered permutation of A + 5% outliers",
        "planes3d": f"3-D LiDAR-like planes, |A|=|B|={n}, B = A rotated 1 deg + 0.1% outliers",
        "unit64": f"64-D unit rows, |A|=|B|={n}, B = A with 1% of rows replaced",
        "polylines": (f"{n} 2-D polyline-pair problems, sizes round(LogNormal(ln 200, 1.2)) "
                      "clipped to [8, 50000]"),
        "clusters3d_f64": (f"clusters3d in float64 (+N(0, 1e-7) jitter), |A|=|B|={n}, exact "
                           "FP64 distance (hd_solve_f64)"),
    }[name]


class ClockSampler:
    """nvidia-smi clock / throttle-reason sampling during the timed region
    (a read-only query)."""
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
        return self

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
        return {k: float(pk[k]) for k in FALLBACK}, "measured"
    except Exception:
        return dict(FALLBACK), "fallback"


def profile_figures(tag):
    """'key: value' lines of the committed ncu summary profiles/<tag>.txt
    (dram_bytes_per_unit, issue_active, ...)."""
    out = {}
    try:
        for ln in open(os.path.join(ROOT, "profiles", f"{tag}.txt")):
            if ":" in ln and not ln.startswith((" ", "\t")):
                k, v = ln.split(":", 1)
                try:
                    out[k.strip()] = float(v.split()[0])
                except (ValueError, IndexError):
                    pass
    except OSError:
        pass
    return out


def traffic_from_profiles(tag, units):
    """Per-launch DRAM bytes of a kernel from its committed ncu summary
    (dram_bytes_per_unit) scaled to this launch's units; None without one."""
    v = profile_figures(tag).get("dram_bytes_per_unit")
    return None if v is None else v * units


def host_cpu():
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name:"):
                model = ln.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    return int(cores or 1), model


# ---------------------------------------------------------------------------
# Oracle and CPU baseline (test infrastructure; never part of a timed GPU step)

def _oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import hd_oracle
    return hd_oracle


def oracle_hd64(a, b, undirected):
    """The oracle's independent FP64 max-min (k-d tree with early break, all
    host threads): (H64, seconds)."""
    o = _oracle()
    t0 = time.perf_counter()
    h2 = o.exact(a, b, 64)[0]
    if undirected:
        h2 = max(h2, o.exact(b, a, 64)[0])
    return float(np.sqrt(h2)), time.perf_counter() - t0


def oracle_batch_hd64(a, b, off, undirected):
    o = _oracle()
    t0 = time.perf_counter()
    h2 = o.exact_batch(a, b, off, off, 64, undirected=undirected)[0]
    return np.sqrt(h2), time.perf_counter() - t0


def _eb_direction(o, x, y, d2_final, cores, budget_s):
    """One direction of the reference CPU early-break (oracle restatement) on
    all host cores.  The whole scan runs when a probe says it fits budget_s;
    otherwise its time is estimated as (measured time of the first k points
    of the seeded shuffle) + (n - k) x (mean per-point time of a window of
    later points scanned from the final running maximum).  A point's scan can
    only get shorter as the running maximum rises, so the window's per-point
    time is at most the same points' time in the whole run: the estimate is
    biased low (the CPU figure is, if anything, too fast)."""
    n = len(x)
    k = min(n, 4096)
    r1 = o.eb_window(x, y, 0, k, 0.0, n_threads=cores)
    if k >= n:
        return {"ms": r1["compute_ms"], "shuffle_ms": r1["shuffle_ms"], "full": True,
                "pairs": r1["compared_pairs"]}
    c2 = np.float32(d2_final) * np.float32(1.0 + 1e-6)
    m = min(n - k, 16384)
    while True:
        r2 = o.eb_window(x, y, k, k + m, c2, n_threads=cores)
        if r2["compute_ms"] > 300.0 or k + m >= n or m >= 4_000_000:
            break
        m = min(n - k, m * 4)
    per_point = r2["compute_ms"] / m
    est = r1["compute_ms"] + per_point * (n - k)
    if est <= budget_s * 1e3:
        r = o.eb(x, y, seed=0, n_threads=cores)
        return {"ms": r["compute_ms"], "shuffle_ms": r["shuffle_ms"], "full": True,
                "pairs": r["compared_pairs"]}
    return {"ms": est, "shuffle_ms": r1["shuffle_ms"], "full": False,
            "first_k": k, "first_k_ms": r1["compute_ms"], "window": m,
            "window_ms": r2["compute_ms"]}


def cpu_eb_baseline(a, b, undirected, d2_final, budget_s=20.0):
    """The reference's CPU early-break (restated in oracle/hd_oracle.cpp; for
    n_dims other than 2 and 3, which the reference does not support, the same
    algorithm applied to rows, not reference code) on all host cores, per
    direction, whole runs where they fit budget_s, else the bounded estimate
    of _eb_direction.  d2_final: the final squared maxima per direction
    (from the GPU result).  Times are compute times, the reference's own
    ReportedTime (early_break.h:106); the shuffle is listed beside them."""
    o = _oracle()
    cores, model = host_cpu()
    dirs = [(a, b, d2_final[0]), (b, a, d2_final[1])] if undirected else [(a, b, d2_final[0])]
    parts = [_eb_direction(o, x, y, d2, cores, budget_s) for x, y, d2 in dirs]
    total = sum(p["ms"] for p in parts)
    full = all(p["full"] for p in parts)
    ref = "reference CPU early-break restated (oracle/hd_oracle.cpp)"
    if a.shape[1] not in (2, 3):
        ref = ("the reference's early-break algorithm applied to 64-D rows (oracle/hd_oracle.cpp; "
               "not reference code: the reference supports n_dims 2 and 3 only)")
    how = ("whole solve measured" if full else
           "estimated per direction: measured first k points of the seeded shuffle + remaining "
           "points at the per-point time of a window scanned from the final running maximum "
           "(a lower bound on the reference's time)")
    return {"value": 1000.0 / total, "unit": "solves/s", "cores": cores, "cpu_model": model,
            "kind": "port", "ms_per_solve": total, "measured_whole_solve": full,
            "sample": f"{ref}, {cores} host threads, {how}: " + json.dumps(parts)}


def cpu_batch_baseline(a, b, off, undirected, budget_s=20.0):
    """Reference CPU early-break (oracle restatement), n_threads = 1 per
    problem, problems spread over all host cores: the whole batch when the
    first problems' rate says it fits budget_s, else those first problems
    extrapolated by pair count."""
    import concurrent.futures as cf
    o = _oracle()
    cores, model = host_cpu()
    sizes = np.diff(off)
    pairs = sizes.astype(np.float64) ** 2

    def one(p):
        x, y = a[off[p]:off[p + 1]], b[off[p]:off[p + 1]]
        o.eb(x, y, n_threads=1)
        if undirected:
            o.eb(y, x, n_threads=1)

    def run(k):
        t0 = time.perf_counter()
        with cf.ThreadPoolExecutor(max_workers=cores) as ex:
            list(ex.map(one, range(k)))
        return time.perf_counter() - t0

    k = min(len(sizes), 4000)
    t = run(k)
    est = t * pairs.sum() / pairs[:k].sum()
    full = False
    if est <= budget_s:
        t, k, full = run(len(sizes)), len(sizes), True
        est = t
    return {"value": len(sizes) / est, "unit": "solves/s", "cores": cores, "cpu_model": model,
            "kind": "port", "ms_per_step": est * 1e3, "measured_whole_batch": full,
            "sample": (f"reference CPU early-break restated (oracle/hd_oracle.cpp), n_threads=1 "
                       f"per problem, problems spread over {cores} host threads; "
                       + ("the whole batch measured" if full else
                          f"first {k} of {len(sizes)} problems ({t:.2f} s), extrapolated by "
                          "pair count"))}


# ---------------------------------------------------------------------------
# GPU workloads

def _events_ms(stream, fn, steps):
    """Average device time per call of fn() over `steps` calls: CUDA events on
    the library's stream, synchronised on both sides."""
    import torch
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    r = None
    for _ in range(steps):
        r = fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps, r


def _fp32_issue_peak(local, sm_mhz):
    """Non-fused FP32 operations per second: SMs x 128 FP32 lanes x SM clock
    (the sampled clock; nominal maximum 2070 MHz when unsampled)."""
    import torch
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    return sms * 128 * (sm_mhz or 2070.0) * 1e6


def _lbvh_phases(n_a, n_b, dims, undirected, rc, phase):
    """Roofline entries of the LBVH path's three phases, algorithmic bytes as
    the measurement plan defines them: sort (per set: read the points twice,
    two 8-byte key/index passes read and written, write the sorted points),
    tree build ((2 n/16) nodes x 32 B per set), query (queries x n_dims x 4 +
    visited nodes x 32 + visited leaf points x n_dims x 4)."""
    sets = [n_a, n_b]
    sort_b = sum(n * (dims * 4 * 2 + 2 * 16 + dims * 4) for n in sets)
    build_b = sum((2 * ((n + 15) // 16)) * 32 for n in sets)
    queries = (n_a + n_b) if undirected else n_a
    query_b = queries * dims * 4 + rc.visited_nodes * 32 + rc.visited_leaves * 16 * dims * 4
    return [("morton_sort", sort_b, phase[0]), ("lbvh_build", build_b, phase[1]),
            ("lbvh_query", query_b, phase[3])]


def bench_single(eng, name, n, steps, warmup, args, ctx):
    import torch
    import hausdorffdistance_gb300 as hd
    stream, local, world, barrier = ctx["stream"], ctx["local"], ctx["world"], ctx["barrier"]
    t_gen = time.perf_counter()
    a, b = make_data(name, n)
    t_gen = time.perf_counter() - t_gen
    undirected = not args.directed
    dims = a.shape[1]
    ta = torch.from_numpy(a).cuda()
    tb = torch.from_numpy(b).cuda()
    variant = args.variant

    def solve():
        return eng.solve(ta, tb, undirected=undirected, variant=variant)

    # Instrumented runs (outside the timed region): visited pairs / nodes for
    # the algorithmic byte counts, per-phase event times.
    rc = eng.solve(ta, tb, undirected=undirected, variant=variant, count_pairs=True)
    phase = np.zeros(8)
    n_inst = 3
    for _ in range(n_inst):
        ri = eng.solve(ta, tb, undirected=undirected, variant=variant, timing=True)
        phase += np.array(ri.phase_ms[:8])
    phase /= n_inst
    for _ in range(warmup):
        solve()
    clocks = ClockSampler(local).start()
    launches0 = eng.kernel_launches
    barrier()
    ms, res = _events_ms(stream, solve, steps)
    barrier()
    launches = eng.kernel_launches - launches0
    clk = clocks.stop()
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = world * 1e3 / ms

    # End to end from pinned host buffers (copies and result read inside).
    pa = torch.from_numpy(a).pin_memory()
    pb = torch.from_numpy(b).pin_memory()
    na, nb = pa.numpy(), pb.numpy()
    for _ in range(2):
        eng.solve(na, nb, undirected=undirected, variant=variant)
    e2e_steps = max(3, steps // 2)
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        re2e = eng.solve(na, nb, undirected=undirected, variant=variant)
    t_e2e = (time.perf_counter() - t0) / e2e_steps
    assert re2e.hd_f32 == res.hd_f32

    # Plain FP32 early-break on the same inputs ("chosen vs plain FP32").
    plain = None
    if not args.no_compare and res.variant_used != hd._lib.VARIANT_EB:
        eng.solve(ta, tb, undirected=undirected, variant="eb")
        ksteps = 2 if dims <= 3 else 1
        pms, rp = _events_ms(stream, lambda: eng.solve(ta, tb, undirected=undirected,
                                                       variant="eb"), ksteps)
        assert rp.hd_f32 == res.hd_f32, "plain EB and chosen variant disagree"
        plain = {"variant": "eb", "ms_per_step": pms, "solves_per_s": 1e3 / pms,
                 "speedup_chosen_vs_plain": pms / ms}

    peaks, pkind = load_peaks()
    used = (hd._lib.VARIANT_NAMES.get(res.variant_used),
            hd._lib.VARIANT_NAMES.get(res.variant_used_ba) if undirected else None)
    roof, phases = None, []
    if res.variant_used == hd._lib.VARIANT_LBVH:
        for tag, alg, t_ms in _lbvh_phases(n, n, dims, undirected, rc, phase):
            if t_ms <= 0:
                continue
            ach = alg / (t_ms / 1e3) / 1e9
            fig = profile_figures(tag)
            units = 2.0 * n if undirected else float(n)
            phases.append({"bound": "hbm", "kernel": tag, "achieved": ach,
                           "peak": peaks["hbm_gbs"], "unit": "GB/s",
                           "frac": ach / peaks["hbm_gbs"],
                           "traffic": (fig["dram_bytes_per_unit"] * units
                                       if "dram_bytes_per_unit" in fig else None),
                           "algorithmic_bytes": alg, "ms": t_ms,
                           "issue_active_ncu": fig.get("issue_active"),
                           "peak_source": pkind + " hbm_gbs"})
        if phases:
            roof = max(phases, key=lambda p: p["ms"])
    elif res.variant_used in (hd._lib.VARIANT_EB, hd._lib.VARIANT_GRID):
        # FP32-issue bound: 3 n_dims - 1 non-fused FLOP per visited pair.
        t_ms = phase[3] + phase[4]
        flops = rc.visited_pairs * (3 * dims - 1)
        pk = _fp32_issue_peak(local, clk.get("sm_mhz"))
        ach = flops / (t_ms / 1e3) / 1e12
        roof = {"bound": "fp32_issue", "kernel": "eb_main+eb_heavy", "achieved": ach,
                "peak": pk / 1e12, "unit": "TFLOP/s", "frac": ach / (pk / 1e12),
                "traffic": None, "ms": t_ms, "visited_pairs": int(rc.visited_pairs),
                "issue_active_ncu": profile_figures("eb_main").get("issue_active"),
                "peak_source": "SMs x 128 FP32 lanes x sampled SM clock (non-fused ops)"}
    elif res.variant_used == hd._lib.VARIANT_BF16:
        # Split-BF16 contraction: 3 products x 2 K FLOP per pair and direction.
        K = ((dims + 15) // 16) * 16
        dirs = 2 if undirected else 1
        flops = dirs * 3.0 * 2.0 * K * float(n) * float(n)
        t_ms = phase[3]
        ach = flops / (t_ms / 1e3) / 1e12
        fig = profile_figures("bf16_rowmin")
        roof = {"bound": "tensor", "kernel": "bf16_rowmin", "achieved": ach,
                "peak": peaks["bf16_tflops"], "unit": "TFLOP/s",
                "frac": ach / peaks["bf16_tflops"],
                "frac_of_sustained": ach / peaks["bf16_tflops_sustained"],
                "traffic": traffic_from_profiles("bf16_rowmin", float(n) * float(n)),
                "algorithmic_flops_per_launch": flops / dirs, "ms": t_ms,
                "tensor_pipe_active_ncu": fig.get("tensor_pipe_active"),
                "peak_source": pkind + " bf16_tflops (burst); frac_of_sustained against "
                               "bf16_tflops_sustained",
                "rechecked_rows": int(res.rechecked), "err_bound": res.err_bound}

    # Relative error against the oracle's independent FP64 max-min.
    oracle = None
    if not args.no_oracle and ctx["rank"] == 0:
        h64, t_or = oracle_hd64(a, b, undirected)
        oracle = {"hd64": h64, "rel_err_vs_oracle": abs(res.hd - h64) / h64,
                  "hd_f32_rel_err_vs_oracle": abs(float(res.hd_f32) - h64) / h64,
                  "oracle_s": t_or}

    base = None
    if ctx["rank"] == 0 and world == 1 and not args.no_cpu:
        d2f = [np.float32(res.hd_ab) ** 2, np.float32(max(res.hd_ba, 0.0)) ** 2]
        base = cpu_eb_baseline(a, b, undirected, d2f)

    pairs_eff = (2 if undirected else 1) * float(n) * float(n)
    return {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": steps, "warmup": warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded numpy PCG64)",
        "config": {"workload": workload_desc(name, n), "n_a": n, "n_b": n, "n_dims": dims,
                   "undirected": undirected, "l2": l2_note(a.nbytes + b.nbytes),
                   "parallelism": f"replicas x{world}"},
        "variant": variant, "variant_used": list(used),
        "gpairs_per_s_effective": value * pairs_eff / 1e9,
        "gpairs_per_s_visited": (rc.visited_pairs * value / 1e9) if rc.visited_pairs else None,
        "hd_f32": float(res.hd_f32), "hd64_certified": res.hd,
        "certifying_pair": [int(res.ia), int(res.ib), int(res.direction)],
        "rel_err_vs_oracle": None if not oracle or "hd64" not in oracle
        else oracle["rel_err_vs_oracle"],
        "oracle": oracle,
        "phase_ms": {nm: float(phase[i]) for i, nm in
                     enumerate(["prep", "build", "sample", "main_pass", "tail", "certify"])},
        "instrumented_ms": float(ri.ms),
        "plain_fp32_eb": plain,
        "e2e": {"value": world / t_e2e, "unit": "solves/s",
                # D2H: the two per-direction result records.
                "h2d_bytes_per_step": int(a.nbytes + b.nbytes), "d2h_bytes_per_step": 2 * 152},
        "gpu_launches": int(launches),
        "roofline": roof, "phases_roofline": phases or None,
        "cpu_baseline": base, "clocks": clk, "data_gen_s": t_gen,
    }


def bench_batch(eng, n, steps, warmup, args, ctx):
    import torch
    stream, local, world, barrier = ctx["stream"], ctx["local"], ctx["world"], ctx["barrier"]
    t_gen = time.perf_counter()
    a, b, off = make_data("polylines", n)
    t_gen = time.perf_counter() - t_gen
    undirected = not args.directed
    ta = torch.from_numpy(a).cuda()
    tb = torch.from_numpy(b).cuda()

    def solve():
        return eng.solve_batch(ta, tb, off, off, undirected=undirected)

    for _ in range(warmup):
        ref = solve()
    clocks = ClockSampler(local).start()
    l0 = eng.kernel_launches
    barrier()
    ms, res = _events_ms(stream, solve, steps)
    barrier()
    clk = clocks.stop()
    launches = eng.kernel_launches - l0
    assert np.array_equal(res["hd_f32"], ref["hd_f32"])
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = world * n / (ms / 1e3)
    pa = torch.from_numpy(a).pin_memory().numpy()
    pb = torch.from_numpy(b).pin_memory().numpy()
    eng.solve_batch(pa, pb, off, off, undirected=undirected)
    ke = max(3, steps // 2)
    t0 = time.perf_counter()
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
    peaks, pkind = load_peaks()
    sizes = np.diff(off)
    alg = float((2 if undirected else 1) * (2 * sizes).sum() * 8)  # both sets, both directions
    achieved = alg / (ms / 1e3) / 1e9
    fig = profile_figures("batch")
    roof = {"bound": "hbm", "kernel": "batch_graph", "achieved": achieved,
            "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"],
            "traffic": traffic_from_profiles("batch", float(sizes.sum())),
            "algorithmic_bytes": alg, "ms": ms, "issue_active_ncu": fig.get("issue_active"),
            "peak_source": pkind + " hbm_gbs"}
    oracle = None
    if not args.no_oracle and ctx["rank"] == 0:
        h64, t_or = oracle_batch_hd64(a, b, off, undirected)
        rel = np.abs(res["hd_f32"].astype(np.float64) - h64) / np.maximum(h64, 1e-30)
        oracle = {"max_rel_err_vs_oracle": float(rel.max()), "oracle_s": t_or,
                  "what": "per problem |hd_f32 - H64| / H64, maximum over the batch"}
    base = None
    if ctx["rank"] == 0 and world == 1 and not args.no_cpu:
        base = cpu_batch_baseline(a, b, off, undirected)
    return {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": steps, "warmup": warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded numpy PCG64)",
        "config": {"workload": workload_desc("polylines", n) + f", {int(sizes.sum())} points per side",
                   "undirected": undirected, "l2": "inputs larger than L2 (no flush)",
                   "parallelism": f"replicas x{world}"},
        "variant_used": ["batch", "batch"],
        "gpairs_per_s_effective": float((sizes.astype(np.float64) ** 2).sum()
                                        * (2 if undirected else 1) / (ms / 1e3) / 1e9),
        "rel_err_vs_oracle": oracle["max_rel_err_vs_oracle"] if oracle else None,
        "oracle": oracle,
        "plain_per_problem": plain,
        "e2e": {"value": world * n / t_e2e, "unit": "solves/s",
                "h2d_bytes_per_step": int(a.nbytes + b.nbytes + n * 32),
                "d2h_bytes_per_step": int(n * 16)},
        "gpu_launches": int(launches), "roofline": roof, "cpu_baseline": base, "clocks": clk,
        "data_gen_s": t_gen,
    }


def bench_f64(eng, name, n, steps, warmup, args, ctx):
    """FP64 input path (hd_solve_f64) on double-precision sets: device-resident
    solves/s, end to end from pinned float64 host buffers, the oracle's exact
    FP64 value (must match bit for bit), and the FP32 solve of the same sets
    rounded to float for comparison."""
    import torch
    stream, local, world, barrier = ctx["stream"], ctx["local"], ctx["world"], ctx["barrier"]
    a, b = make_data(name, n)
    undirected = not args.directed
    ta = torch.from_numpy(a).cuda()
    tb = torch.from_numpy(b).cuda()

    def solve():
        return eng.solve_f64(ta, tb, undirected=undirected)

    ri = eng.solve_f64(ta, tb, undirected=undirected, timing=True)
    for _ in range(warmup):
        solve()
    clocks = ClockSampler(local).start()
    launches0 = eng.kernel_launches
    barrier()
    ms, res = _events_ms(stream, solve, steps)
    barrier()
    launches = eng.kernel_launches - launches0
    clk = clocks.stop()
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = world * 1e3 / ms
    pa = torch.from_numpy(a).pin_memory()
    pb = torch.from_numpy(b).pin_memory()
    na, nb = pa.numpy(), pb.numpy()
    eng.solve_f64(na, nb, undirected=undirected)
    e2e_steps = max(3, steps // 2)
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        re2e = eng.solve_f64(na, nb, undirected=undirected)
    t_e2e = (time.perf_counter() - t0) / e2e_steps
    assert re2e.hd == res.hd
    # The FP32 solve of the same sets rounded to float.
    fa, fb = ta.float(), tb.float()
    eng.solve(fa, fb, undirected=undirected)
    ms32, _ = _events_ms(stream, lambda: eng.solve(fa, fb, undirected=undirected), 3)
    oracle = None
    if not args.no_oracle and ctx["rank"] == 0:
        o = _oracle()
        t_or = time.perf_counter()
        h2 = o.exact_f64(a, b)[0]
        if undirected:
            h2 = max(h2, o.exact_f64(b, a)[0])
        h64 = float(np.sqrt(h2))
        oracle = {"hd64": h64, "rel_err_vs_oracle": abs(res.hd - h64) / h64,
                  "bit_identical": res.hd == h64, "oracle_s": time.perf_counter() - t_or}
    return {
        "metric": "exact FP64 Hausdorff solves/s, 1 GB300", "value": value, "unit": "solves/s",
        "n_gpus": world, "steps": steps, "warmup": warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded numpy PCG64)",
        "config": {"workload": workload_desc(name, n), "n_a": n, "n_b": n, "n_dims": 3,
                   "undirected": undirected, "l2": l2_note(a.nbytes + b.nbytes),
                   "parallelism": f"replicas x{world}"},
        "variant_used": int(res.variant_used),
        "hd64": res.hd, "certifying_pair": [int(res.ia), int(res.ib), int(res.direction)],
        "rows_walked_in_fp64": int(res.rechecked),
        "rel_err_vs_oracle": None if not oracle else oracle["rel_err_vs_oracle"],
        "oracle": oracle,
        "fp32_solve_of_rounded_sets_ms": ms32,
        "fp64_over_fp32_time": ms / ms32,
        "instrumented_ms": float(ri.ms),
        "e2e": {"value": 1.0 / t_e2e, "unit": "solves/s",
                "h2d_bytes_per_step": int(a.nbytes + b.nbytes),
                # three read-backs of the FP64 scalars (152 B) and one of the
                # FP32 stage's two DevScalars (152 B each)
                "d2h_bytes_per_step": 3 * 152 + 2 * 152, "ms_per_step": t_e2e * 1e3},
        "cpu_baseline": None,
        "cpu_baseline_note": "not measured: the reference has no double build of its CPU "
                             "path (its -is_double dispatch is disabled)",
        "clocks": clk, "gpu_launches": launches,
    }


def l2_note(nbytes):
    if nbytes > 130e6:
        return "inputs larger than L2 (no flush)"
    return ("inputs smaller than L2, no flush: every step re-sorts or re-packs both sets, so "
            "the solve rebuilds its own working set each step")


def sub_steps(name, steps, warmup):
    """Steps for a workload measured beside the headline: K and W as given,
    except that the long 64-D solves (~0.4 s each) keep their timed region to
    a few seconds."""
    if name == "unit64":
        return max(3, min(steps, 8)), max(3, min(warmup, 3))
    return steps, warmup


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
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

    stream = torch.cuda.current_stream()
    eng = hd.Engine(device=local, variant=args.variant)
    eng.set_stream(stream.cuda_stream)
    ctx = {"stream": stream, "local": local, "world": world, "rank": rank, "barrier": barrier}
    names = ALL if args.workload == "all" else [args.workload]

    if args.profile:
        name = names[0]
        n = args.n or WORKLOAD_SIZES[name]
        if name == "polylines":
            a, b, off = make_data(name, n)
            eng.solve_batch(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda(), off, off,
                            undirected=not args.directed)
            out = {"profile_solve": True, "workload": name}
        elif name == "clusters3d_f64":
            a, b = make_data(name, n)
            r = eng.solve_f64(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda(),
                              undirected=not args.directed)
            out = {"profile_solve": True, "workload": name, "hd64": r.hd,
                   "rows_walked_in_fp64": int(r.rechecked)}
        else:
            a, b = make_data(name, n)
            r = eng.solve(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda(),
                          undirected=not args.directed)
            out = {"profile_solve": True, "workload": name, "hd_f32": float(r.hd_f32),
                   "variant_used": int(r.variant_used)}
        torch.cuda.synchronize()
        print(json.dumps(out), flush=True)
        eng.close()
        return

    records = {}
    for i, name in enumerate(names):
        n = args.n or WORKLOAD_SIZES[name]
        steps, warmup = (args.steps, args.warmup) if i == 0 else sub_steps(name, args.steps,
                                                                           args.warmup)
        if name == "polylines":
            records[name] = bench_batch(eng, n, steps, warmup, args, ctx)
        elif name == "clusters3d_f64":
            records[name] = bench_f64(eng, name, n, steps, warmup, args, ctx)
        else:
            records[name] = bench_single(eng, name, n, steps, warmup, args, ctx)
        torch.cuda.empty_cache()
    if rank == 0:
        line = dict(records[names[0]])
        if len(names) > 1:
            line["workloads"] = {nm: records[nm] for nm in names[1:]}
        print(json.dumps(line), flush=True)
    eng.close()
    if world > 1:
        dist.destroy_process_group()


def run_reference(args):
    """The reference arm: the reference's CPU early-break on all host cores
    (oracle restatement; the reference's own x86 build cannot run on an Arm
    host), for the headline workload, one undirected solve per step."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    name = ALL[0] if args.workload == "all" else args.workload
    n = args.n or WORKLOAD_SIZES[name]
    undirected = not args.directed
    o = _oracle()
    if name == "polylines":
        a, b, off = make_data(name, n)

        def measure():
            return cpu_batch_baseline(a, b, off, undirected)
    else:
        a, b = make_data(name, n)
        # Final squared maxima per direction (only used when a whole solve does
        # not fit the step budget and the bounded estimate runs instead).
        d2f = [np.float32(o.exact(a, b, 32)[0])]
        if undirected:
            d2f.append(np.float32(o.exact(b, a, 32)[0]))

        def measure():
            return cpu_eb_baseline(a, b, undirected, d2f, budget_s=8.0)
    vals, base = [], None
    for i in range(args.warmup + args.steps):
        base = measure()
        if i >= args.warmup:
            vals.append(base["value"])
    v = float(np.median(vals))
    base["value"] = v
    line = {"metric": METRIC, "value": v, "unit": "solves/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / v,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded numpy PCG64)", "impl": "reference",
            "config": {"workload": workload_desc(name, n), "n_a": n, "n_b": n,
                       "n_dims": int(a.shape[1]), "undirected": undirected,
                       "l2": l2_note(a.nbytes + b.nbytes), "parallelism": "replicas x1"},
            "variant": "reference CPU early-break (host cores)",
            "cpu_baseline": base,
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
