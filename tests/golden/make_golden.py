"""Generates the golden vectors in tests/golden/ from the reference's own CPU
early-break implementation (src/hd_impl/hausdorff_distance_early_break.h:44-115),
compiled from the reference sources by oracle/build_ref.sh into
oracle/_ref/ref_eb.

For every case it writes the two inputs in the reference's point-cache layout
(inputs/<name>_{a,b}.bin) and records, in golden.json, what the reference
returned: the float distance (and its bit pattern) and the compared-pair
count for n_threads=1 (deterministic: it depends only on the seeded shuffle),
and the distance for n_threads=4; likewise, for double inputs, the
reference's double instantiation (oracle/_ref/ref_eb64).  It also runs some of
those float inputs through
the reference's -normalize / -translate preprocessing (oracle/_ref/ref_prep)
and records a SHA-256 of each result's float32 points, and records the
reference's statistics-grid shape of every input (oracle/_ref/ref_stats).

Run from the repository root, in a container that has the reference sources:
    oracle/build_ref.sh <reference src directory> && python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from hausdorffdistance_gb300 import synth  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref", "ref_eb")
REF64 = os.path.join(ROOT, "oracle", "_ref", "ref_eb64")
REF_PREP = os.path.join(ROOT, "oracle", "_ref", "ref_prep")
REF_STATS = os.path.join(ROOT, "oracle", "_ref", "ref_stats")

# -normalize / -translate settings run through the reference's own
# NormalizePoints / TranslatePoints (src/loaders/translate_points.h:42-79).
PREP_CASES = ["uniform2d_3k_ab", "clusters3d_4k_ab", "offset_large_3d", "negative_2d",
              "coplanar_3d", "all_equal_2d", "collinear_2d", "planes3d_3k_ab"]
PREP_SETTINGS = [(1, 0.0), (0, 0.37), (1, 0.1234567), (0, -2.5)]


def cases():
    rng = np.random.Generator(np.random.PCG64(20240601))
    out = []

    def add(name, a, b, dims, seed=0):
        out.append((name, np.ascontiguousarray(a, np.float32),
                    np.ascontiguousarray(b, np.float32), dims, seed))

    a, b = synth.uniform2d(3000, seed=11)
    add("uniform2d_3k_ab", a, b, 2, 0)
    add("uniform2d_3k_ba", b, a, 2, 7)
    a, b = synth.clusters3d(4000, seed=12)
    add("clusters3d_4k_ab", a, b, 3, 0)
    add("clusters3d_4k_ba", b, a, 3, 3)
    add("uniform3d_2000x1500", rng.random((2000, 3)), rng.random((1500, 3)), 3, 5)
    add("uniform2d_1000x1000", rng.random((1000, 2)), rng.random((1000, 2)), 2, 1)
    a, b = synth.planes3d(3000, seed=13, n_planes=20)
    add("planes3d_3k_ab", a, b, 3, 0)
    add("planes3d_3k_ba", b, a, 3, 0)
    a, b, off = synth.polylines(sizes=[300, 8], seed=14)
    add("polyline_300", a[:300], b[:300], 2, 0)
    add("polyline_8", a[300:], b[300:], 2, 0)
    # Edge cases: single points, one side single, exact duplicates.
    add("single_single_2d", [[0.25, 0.5]], [[0.75, -0.5]], 2, 0)
    add("single_vs_many_3d", [[0.5, 0.5, 0.5]], rng.random((100, 3)), 3, 0)
    add("many_vs_single_3d", rng.random((100, 3)), [[0.5, 0.5, 0.5]], 3, 0)
    d = rng.random((500, 2))
    add("identical_2d", d, d[rng.permutation(500)], 2, 0)
    # Ties: integer lattice against a shifted lattice, all distances equal.
    g = np.stack(np.meshgrid(np.arange(12), np.arange(12)), -1).reshape(-1, 2)
    add("lattice_ties_2d", g, g + 0.5, 2, 0)
    g3 = np.stack(np.meshgrid(np.arange(6), np.arange(6), np.arange(6)), -1).reshape(-1, 3)
    add("lattice_ties_3d", g3, g3[::2] + 0.5, 3, 0)
    # Degenerate extents: all-equal points, collinear sets, coplanar 3-D.
    add("all_equal_2d", np.full((50, 2), 3.0), np.full((40, 2), 3.0), 2, 0)
    t = rng.random(400)
    add("collinear_2d", np.stack([t, 2 * t], 1), np.stack([t[::-1] * 0.9, 1.8 * t[::-1]], 1), 2, 0)
    add("coplanar_3d", np.c_[rng.random((300, 2)), np.zeros(300)],
        np.c_[rng.random((200, 2)), np.full(200, 0.1)], 3, 0)
    # Large offsets and negative coordinates.
    add("offset_large_3d", rng.random((800, 3)) * 10 + 1.0e4,
        rng.random((700, 3)) * 10 + 1.0e4 - 3.0, 3, 0)
    add("negative_2d", -rng.random((600, 2)) * 5, -rng.random((900, 2)) * 5 + 0.25, 2, 0)
    # The Spider distributions of the reference's synthetic experiments
    # (expr/for_the_paper/data_gen.sh), seed 1 against seed 2.
    for dist, n in (("uniform", 4000), ("gaussian", 4000), ("bit", 5000), ("diagonal", 4000),
                    ("sierpinski", 5000)):
        dims = 2 if dist == "sierpinski" else 3
        add(f"spider_{dist}_{dims}d", synth.spider(dist, n, dims, seed=1),
            synth.spider(dist, n, dims, seed=2), dims, 0)
    return out


def cases_f64():
    """Double inputs for the reference's double instantiation (ref_eb64):
    values that need double precision, points distinct only below float
    precision, exact ties, large offsets, a single point."""
    rng = np.random.Generator(np.random.PCG64(20261204))
    out = []

    def add(name, a, b, dims, seed=0):
        out.append((name, np.ascontiguousarray(a, np.float64),
                    np.ascontiguousarray(b, np.float64), dims, seed))

    a, b = synth.clusters3d(3000, seed=21)
    a = a.astype(np.float64) + rng.normal(0.0, 1e-9, a.shape)
    b = b.astype(np.float64) + rng.normal(0.0, 1e-9, b.shape)
    add("f64_clusters3d_3k_ab", a, b, 3, 0)
    add("f64_clusters3d_3k_ba", b, a, 3, 3)
    add("f64_uniform2d_2500x2000", rng.random((2500, 2)), rng.random((2000, 2)) * 1.05, 2, 1)
    base = rng.random((1500, 3))
    add("f64_subfloat_3d", base, base + rng.normal(0.0, 3e-9, base.shape), 3, 0)
    g = np.stack(np.meshgrid(np.arange(10), np.arange(10)), -1).reshape(-1, 2).astype(np.float64)
    add("f64_lattice_ties_2d", g, g + 0.5, 2, 0)
    add("f64_offset_3d", rng.random((1200, 3)) * 10 + 1.0e6, rng.random((1000, 3)) * 10 + 1.0e6 - 2.0,
        3, 5)
    add("f64_single_vs_many_3d", [[0.1, 0.2, 0.3]], rng.random((300, 3)), 3, 0)
    return out


def write_bin64(path, pts):
    with open(path, "wb") as f:
        f.write(np.uint64(len(pts)).tobytes())
        f.write(np.ascontiguousarray(pts, np.float64).tobytes())


def run_ref(a_path, b_path, dims, seed, threads, exe=REF):
    r = subprocess.run([exe, a_path, b_path, str(dims), str(seed), str(threads)],
                       check=True, capture_output=True, text=True)
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1]
    return json.loads(line)["runs"][0]


def run_prep(records, inp):
    """The reference's preprocessing of each input file of PREP_CASES under
    PREP_SETTINGS, recorded as a SHA-256 of the resulting float32 points."""
    import hashlib
    import tempfile
    out = []
    by_name = {r["name"]: r for r in records}
    with tempfile.TemporaryDirectory() as tmp:
        for name in PREP_CASES:
            rec = by_name[name]
            for side in ("a", "b"):
                src = os.path.join(HERE, rec[side])
                for normalize, translate in PREP_SETTINGS:
                    dst = os.path.join(tmp, "out.bin")
                    subprocess.run([REF_PREP, src, dst, str(rec["dims"]), str(normalize),
                                    repr(translate)], check=True)
                    pts = synth.read_bin(dst, rec["dims"])
                    out.append({"input": rec[side], "dims": rec["dims"], "normalize": normalize,
                                "translate": translate, "n": int(pts.shape[0]),
                                "sha256": hashlib.sha256(pts.tobytes()).hexdigest()})
    return out


def run_stats(records):
    """The reference's statistics-grid shape (non-empty box, resolution,
    density) of every input file, for n_points_cell 10 (hd_exec's default)
    and, on the first cases, 8."""
    out = []
    for i, rec in enumerate(records):
        for side in ("a", "b"):
            for npc in ((10, 8) if i < 6 else (10,)):
                r = subprocess.run([REF_STATS, os.path.join(HERE, rec[side]), str(rec["dims"]),
                                    str(npc)], check=True, capture_output=True, text=True)
                v = r.stdout.split()
                d = rec["dims"]
                out.append({"input": rec[side], "dims": d, "n_points_cell": npc,
                            "lower": [float(x) for x in v[:d]],
                            "upper": [float(x) for x in v[d:2 * d]],
                            "size": [int(x) for x in v[2 * d:3 * d]],
                            "density": float(v[3 * d])})
    return out


def main():
    if not os.path.exists(REF):
        sys.exit("oracle/_ref/ref_eb is missing: run oracle/build_ref.sh <reference src directory> first")
    inp = os.path.join(HERE, "inputs")
    os.makedirs(inp, exist_ok=True)
    records = []
    for name, a, b, dims, seed in cases():
        pa = os.path.join(inp, f"{name}_a.bin")
        pb = os.path.join(inp, f"{name}_b.bin")
        synth.write_bin(pa, a)
        synth.write_bin(pb, b)
        r1 = run_ref(pa, pb, dims, seed, 1)
        r4 = run_ref(pa, pb, dims, seed, 4)
        records.append({
            "name": name, "dims": dims, "seed": seed,
            "n_a": int(a.shape[0]), "n_b": int(b.shape[0]),
            "a": f"inputs/{name}_a.bin", "b": f"inputs/{name}_b.bin",
            "hd": r1["hd"], "hd_bits": r1["hd_bits"],
            "compared_pairs_t1": r1["compared_pairs"],
            "hd_bits_t4": r4["hd_bits"],
        })
        print(name, r1["hd"], r1["compared_pairs"])
    records64 = []
    if os.path.exists(REF64):
        for name, a, b, dims, seed in cases_f64():
            pa = os.path.join(inp, f"{name}_a.bin")
            pb = os.path.join(inp, f"{name}_b.bin")
            write_bin64(pa, a)
            write_bin64(pb, b)
            r1 = run_ref(pa, pb, dims, seed, 1, REF64)
            r4 = run_ref(pa, pb, dims, seed, 4, REF64)
            records64.append({
                "name": name, "dims": dims, "seed": seed,
                "n_a": int(a.shape[0]), "n_b": int(b.shape[0]),
                "a": f"inputs/{name}_a.bin", "b": f"inputs/{name}_b.bin",
                "hd": r1["hd"], "hd_bits": r1["hd_bits"],
                "compared_pairs_t1": r1["compared_pairs"],
                "hd_bits_t4": r4["hd_bits"],
            })
            print(name, r1["hd"], r1["compared_pairs"])
    prep = run_prep(records, inp) if os.path.exists(REF_PREP) else []
    stats = run_stats(records) if os.path.exists(REF_STATS) else []
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py",
                   "reference": "src/hd_impl/hausdorff_distance_early_break.h:44-115 "
                                "built by oracle/build_ref.sh",
                   "cases": records,
                   "reference_f64": "the same early-break in the reference's double "
                                    "instantiation (ref_eb64); inputs hold doubles",
                   "cases_f64": records64,
                   "preprocessing_reference": "src/loaders/translate_points.h:42-79 "
                                              "(ref_prep, built by oracle/build_ref.sh)",
                   "preprocessing": prep,
                   "stats_grid_reference": "src/geoms/mbr.h:288-296, "
                                           "src/index/uniform_grid.h:222-244 "
                                           "(ref_stats, built by oracle/build_ref.sh)",
                   "stats_grid": stats}, f, indent=1)


if __name__ == "__main__":
    main()
