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
    n, d = P.shape
    lo = P.min(0).astype(np.float64)
    hi = P.max(0).astype(np.float64)
    ext = np.where(hi > lo, hi - lo, 1e-5)
    vol = float(np.prod(ext))
    side = (vol * npc / n) ** (1.0 / d)
    size = np.maximum(1, np.ceil(ext / side)).astype(np.int64)
    scale = (size / ext).astype(np.float32)
    lo32 = lo.astype(np.float32)
    cells = np.zeros(n, np.int64)
    for k in reversed(range(d)):
        c = np.floor((P[:, k] - lo32[k]) * scale[k])
        c = np.clip(c, 0, size[k] - 1).astype(np.int64)
        cells = cells * size[k] + c
    counts = np.bincount(cells, minlength=int(np.prod(size)))
    ne = np.sort(counts[counts > 0]).astype(np.float64)
    m = len(ne)
    gini = float(((2 * np.arange(m) - m + 1) * ne).sum() / (m * ne.sum()))
    return {"lower": lo, "upper": lo + ext, "density": n / vol, "size": size,
            "total": int(np.prod(size)), "nonempty": m, "max": int(ne[-1]),
            "median": int(ne[m // 2]), "gini": gini,
            "diag": float(np.sqrt(((ext / size) ** 2).sum()))}


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
    assert np.allclose(np.array(st.upper[:d]), want["upper"], rtol=0, atol=1e-12)
    assert st.density == pytest.approx(want["density"], rel=1e-12)
    assert list(st.grid_size[:d]) == list(want["size"])
    assert st.total_cells == want["total"]
    assert st.nonempty_cells == want["nonempty"]
    assert st.max_points == want["max"] and st.median_points == want["median"]
    assert st.gini_index == pytest.approx(want["gini"], rel=1e-9, abs=1e-12)
    assert st.cell_diagonal == pytest.approx(want["diag"], rel=1e-12)
    # Percentile table: ascending values and percentiles, ending at the
    # largest count with every non-empty cell counted.
    k = st.n_hist
    vals = np.array(st.hist_value[:k])
    pct = np.array(st.hist_percentile[:k])
    assert k >= 2 and np.all(np.diff(vals) >= 0) and np.all(np.diff(pct) > 0)
    assert vals[-1] == want["max"] and st.hist_count[k - 1] == want["nonempty"]
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
