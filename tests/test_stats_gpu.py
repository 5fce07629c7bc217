"""hd_compute_stats: the reference's per-file statistics (bounding box,
density, statistics-grid occupancy, Gini index, median, percentile table;
src/run_hausdorff_distance.cu:150-185, src/index/uniform_grid.h:222-244,
343-484, 673-693, src/running_stats.h:33-62) computed on the GPU, checked
against the same quantities computed here with numpy."""
import json
import os
import subprocess

import numpy as np
import pytest

from hausdorffdistance_gb300 import synth

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def expected(P, npc):
    """The reference's statistics in its arithmetic (float box and extents, a
    flat axis widened by 1e-5 in float, cell side sqrt/cbrt in double, float
    density and cell diagonal; a point's cell (p - lower) / extent * size in
    float, clamped and truncated)."""
    n, d = P.shape
    lo = P.min(0)
    hi = P.max(0)
    hi = np.where(hi - lo == 0, (lo.astype(np.float64) + 1e-5).astype(np.float32), hi)
    hi = np.where(hi - lo == 0, np.nextafter(lo, np.float32(np.inf)), hi)
    ext = hi - lo
    vol, vol32 = 1.0, np.float32(1)
    for e in ext:
        vol *= float(e)
        vol32 = np.float32(vol32 * e)
    q = vol * npc / n
    side = np.sqrt(q) if d == 2 else np.cbrt(q)
    size = np.array([max(1, int(np.ceil(float(e) / side))) for e in ext], np.int64)
    cells = np.zeros(n, np.int64)
    for k in reversed(range(d)):
        c = ((P[:, k] - lo[k]) / ext[k]) * np.float32(size[k])
        c = np.minimum(np.maximum(c, np.float32(0)), np.float32(size[k]) - np.float32(1))
        cells = cells * size[k] + c.astype(np.int64)
    counts = np.bincount(cells, minlength=int(np.prod(size)))
    ne = np.sort(counts[counts > 0]).astype(np.float64)
    m = len(ne)
    gini = float(((2 * np.arange(m) - m + 1) * ne).sum() / (m * ne.sum()))
    sum2 = np.float32(0)
    for e, z in zip(ext, size):
        u = np.float32(e / np.float32(z))
        sum2 = np.float32(sum2 + np.float32(u * u))
    # HdrHistogram (hdr_init(1, non-empty cells, 3)) records only values below
    # the smallest power-of-two multiple of 2048 beyond the non-empty count.
    untrackable = 2048
    while untrackable <= max(m, 2):
        untrackable <<= 1
    rec = ne[ne < untrackable].astype(np.int64)
    return {"lower": lo.astype(np.float64), "upper": hi.astype(np.float64),
            "hdr_first": hdr_highest_equivalent(int(rec[0])),
            "hdr_last": hdr_highest_equivalent(int(rec[-1])), "hdr_total": len(rec),
            "density": float(np.float32(np.float32(n) / vol32)), "size": size,
            "total": int(np.prod(size)), "nonempty": m, "max": int(ne[-1]),
            "median": int(ne[m // 2]), "gini": gini, "diag": float(np.sqrt(sum2))}


def hdr_highest_equivalent(v):
    """HdrHistogram with 3 significant figures: values from 2048 on share
    buckets of 2^b values and are reported as the bucket's highest."""
    if v < 2048:
        return v
    b = v.bit_length() - 11
    return ((v >> b) << b) + (1 << b) - 1


@pytest.mark.parametrize("name", ["uniform2d", "clusters3d", "planes3d"])
def test_point_stats_match_numpy(engine, name):
    if name == "uniform2d":
        P = synth.uniform2d(100_000, seed=11)[1]
    elif name == "clusters3d":
        P = synth.clusters3d(200_000, seed=12)[0]
    else:
        P = synth.planes3d(150_000, seed=13, n_planes=20)[1]
    st = engine.point_stats(P, 10)
    want = expected(P, 10)
    d = P.shape[1]
    assert np.array_equal(np.array(st.lower[:d]), want["lower"])
    assert np.array_equal(np.array(st.upper[:d]), want["upper"])
    assert st.density == want["density"]
    assert list(st.grid_size[:d]) == list(want["size"])
    assert st.total_cells == want["total"]
    assert st.nonempty_cells == want["nonempty"]
    assert st.max_points == want["max"] and st.median_points == want["median"]
    assert st.gini_index == pytest.approx(want["gini"], rel=1e-9, abs=1e-12)
    assert st.cell_diagonal == want["diag"]
    # Percentile table (HdrHistogram's iteration; its exact rows are pinned to
    # the reference's logs in test_stats_host.py): values ascending, possibly
    # repeated, at strictly rising targets from 0, ending at the largest
    # recorded count (in its HdrHistogram bucket) with every recorded cell
    # counted.
    k = st.n_hist
    vals = np.array(st.hist_value[:k])
    pct = np.array(st.hist_percentile[:k])
    assert k >= 2 and np.all(np.diff(vals) >= 0) and np.all(np.diff(pct) > 0)
    assert pct[0] == 0.0 and vals[0] == want["hdr_first"]
    assert vals[-1] == want["hdr_last"] and st.hist_count[k - 1] == want["hdr_total"]
    assert pct[-1] == 1.0


def test_hd_exec_writes_reference_statistics(tmp_path):
    from hausdorffdistance_gb300 import build
    build.build_lib()
    exe = build.build_exec()
    a, b = synth.clusters3d(20_000, seed=14)
    pa, pb = tmp_path / "a.bin", tmp_path / "b.bin"
    synth.write_bin(str(pa), a)
    synth.write_bin(str(pb), b)
    out = tmp_path / "run.json"
    r = subprocess.run([exe, "-input1", str(pa), "-input2", str(pb), "-input_type", "bin",
                        "-n_dims", "3", "-variant", "hybrid", "-repeat", "2", "-check",
                        "-json", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "HausdorffDistance is checked" in r.stdout
    st = json.load(open(out))
    assert st["Check"]["Pass"] is True
    for j in st["Input"]["Files"] + [st["Input"]]:
        assert {"Grid", "MBR", "Density", "StatsGridNumPointsPerCell"} <= set(j)
        assert {"TotalCells", "NonEmptyCells", "MaxPoints", "GiniIndex", "GridSize",
                "CellDiagonalLength", "MedianPointsPerCell", "Histogram"} <= set(j["Grid"])
        assert len(j["MBR"]) == 3 and j["Density"] > 0
    want = expected(np.concatenate([a, b]), 10)
    assert st["Input"]["Grid"]["MaxPoints"] == want["max"]
