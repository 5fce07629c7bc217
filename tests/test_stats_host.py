"""Host-side statistics of hd_compute_stats (csrc/hd_stats_host.h), on the CPU.

The percentile table is pinned to the reference's own output: the fixture
tests/golden/hdr_percentiles.json holds 150 of the ~1,900 distinct tables that
its experiment logs record (expr/for_the_paper/logs/**.json, Grid.Histogram,
printed there by HdrHistogram_c).  A table fixes the cumulative count at every
value it reports; a histogram with its cells only at those values yields the
same rows under the same iteration, so each logged table is replayed from its
own rows and must come back digit for digit."""
import json
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "hausdorffdistance_gb300", "csrc")
TABLES = json.load(open(os.path.join(ROOT, "tests", "golden", "hdr_percentiles.json")))["tables"]


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("hdr") / "hdr_probe")
    subprocess.run(["g++", "-std=c++17", "-O2", f"-I{CSRC}",
                    os.path.join(ROOT, "tests", "hdr_probe.cpp"), "-o", out], check=True)
    return out


def replay(probe, rows):
    cells, prev = {}, 0
    for v, _, c in rows:
        if c > prev:
            cells[int(v)] = cells.get(int(v), 0) + c - prev
            prev = c
    n = rows[-1][2]
    text = f"{n} {max(cells, default=0) + 1}\n" + "".join(f"{v} {c}\n" for v, c in cells.items())
    r = subprocess.run([probe, "rows"], input=text, capture_output=True, text=True, check=True)
    return [(float(a), float(b), int(c)) for a, b, c in (ln.split() for ln in r.stdout.split("\n")
                                                          if ln)]


def test_percentile_rows_match_the_reference_logs(probe):
    assert len(TABLES) == 150
    for t in TABLES:
        want = [(float(v), float(p), int(c)) for v, p, c in t["rows"]]
        assert replay(probe, t["rows"]) == want, t["log"]


def test_percentile_rows_shapes(probe):
    """Repeated values at successive targets, bucketed large values, and the
    final 100 % row."""
    big = [t for t in TABLES if max(r[0] for r in t["rows"]) >= 2048]
    assert len(big) >= 50
    # 123230 points in one cell is logged in its 64-wide bucket as 123263
    # (recorded because the histogram tracks up to the non-empty cell count).
    text = "3029223 123231\n1 1\n5 1\n123230 1\n"
    r = subprocess.run([probe, "rows"], input=text, capture_output=True, text=True, check=True)
    rows = [ln.split() for ln in r.stdout.split("\n") if ln]
    assert rows[-1] == ["123263.000", "1.000000", "3"]
    # One cell in three is at 1: it is reported at the 0 % and 16.7 % targets.
    assert rows[:2] == [["1.000", "0.000000", "1"], ["1.000", "0.166667", "1"]]
    assert "5.000" in [x[0] for x in rows]


def grid(probe, dims, n, npc, lo, hi):
    text = f"{dims} {n} {npc}\n" + " ".join(map(repr, lo)) + "\n" + " ".join(map(repr, hi)) + "\n"
    r = subprocess.run([probe, "grid"], input=text, capture_output=True, text=True, check=True)
    ln = r.stdout.split("\n")
    axes = [ln[k].split() for k in range(dims)]
    total, density, diag = ln[dims].split()
    return ([int(a[0]) for a in axes], [float(a[1]) for a in axes], int(total), float(density),
            float(diag))


def reference_grid(dims, n, npc, lo, hi):
    """src/index/uniform_grid.h:222-244,695-705 and mbr.h:288-296 in numpy."""
    lo = np.float32(lo)
    hi = np.array(hi, np.float32)
    hi = np.where(hi - lo == 0, (lo.astype(np.float64) + 1e-5).astype(np.float32), hi)
    # Where lower + 1e-5 rounds back to lower the reference stops on a zero
    # volume (CHECK_GT); the library then gives the axis one float step.
    hi = np.where(hi - lo == 0, np.nextafter(lo, np.float32(np.inf)), hi)
    ext = hi - lo
    vol = 1.0
    vol32 = np.float32(1)
    for e in ext:
        vol *= float(e)
        vol32 = np.float32(vol32 * e)
    q = vol * npc / n
    s = np.sqrt(q) if dims == 2 else np.cbrt(q)
    size = [max(1, int(np.ceil(float(e) / s))) for e in ext]
    unit = [np.float32(e / np.float32(z)) for e, z in zip(ext, size)]
    sum2 = np.float32(0)
    for u in unit:
        sum2 = np.float32(sum2 + np.float32(u * u))
    return (size, [float(h) for h in hi], int(np.prod(size)),
            float(np.float32(np.float32(n) / vol32)), float(np.sqrt(sum2)))


@pytest.mark.parametrize("dims,n,npc,lo,hi", [
    (3, 200000, 10, [0.013, -0.02, 0.1], [1.07, 0.98, 1.02]),
    (2, 100000, 10, [0.0, 0.0], [1.2, 1.19]),
    (3, 5000, 10, [3.0, 1.0, 2.0], [3.0, 4.5, 2.5]),    # a flat axis: + 1e-5
    (2, 7, 10, [1e4, -5.0], [1e4, -5.0]),                # a single point
    (3, 1, 10, [0.5, 0.5, 0.5], [0.5, 0.5, 0.5]),
    (2, 3, 10, [-2e4, 7.0], [-2e4, 9.0]),                # flat at a large negative x
    (3, 3029223, 10, [-124.7, 24.5, 0.0], [-66.9, 49.4, 0.0]),
])
def test_grid_shape_matches_the_reference_rule(probe, dims, n, npc, lo, hi):
    got = grid(probe, dims, n, npc, lo, hi)
    want = reference_grid(dims, n, npc, lo, hi)
    assert got[0] == want[0] and got[2] == want[2]
    assert np.array_equal(np.float32(got[1]), np.float32(want[1]))  # %.9g round-trips float
    assert got[3] == want[3] and got[4] == want[4]


GRID = json.load(open(os.path.join(ROOT, "tests", "golden", "golden.json"))).get("stats_grid", [])


@pytest.mark.parametrize("rec", GRID, ids=[f"{r['input'].split('/')[-1][:-4]}-k{r['n_points_cell']}"
                                          for r in GRID])
def test_grid_shape_matches_the_reference_build(probe, rec):
    """The statistics grid's non-empty box, resolution and density equal what
    the reference's own Mbr::ToNonemptyMBR / CalculateGridResolution /
    get_volume give on the golden inputs (built from its sources)."""
    from hausdorffdistance_gb300 import synth
    d = rec["dims"]
    P = synth.read_bin(os.path.join(ROOT, "tests", "golden", rec["input"]), d)
    size, upper, _, density, _ = grid(probe, d, len(P), rec["n_points_cell"],
                                      [float(x) for x in P.min(0)], [float(x) for x in P.max(0)])
    assert size == rec["size"]
    assert np.array_equal(np.float32(upper), np.float32(rec["upper"]))
    assert np.float32(density) == np.float32(rec["density"])


LOGGED = json.load(open(os.path.join(ROOT, "tests", "golden", "log_grid_stats.json")))["records"]


def test_grid_shape_matches_the_reference_logs(probe):
    """The statistics grid's cells per axis, cell diagonal and (per file)
    density equal what the reference logged in its real runs for the same
    box, point count and n_points_cell (tests/golden/log_grid_stats.json)."""
    assert len(LOGGED) >= 150
    for r in LOGGED:
        d = len(r["lower"])
        size, _, _, density, diag = grid(probe, d, r["n"], r["n_points_cell"],
                                         r["lower"], r["upper"])
        assert size == r["grid_size"], r["log"]
        assert np.float32(diag) == np.float32(r["cell_diagonal"]), r["log"]
        if "density" in r:
            assert np.float32(density) == np.float32(r["density"]), r["log"]
