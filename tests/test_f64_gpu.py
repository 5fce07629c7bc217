"""FP64 input path (hd_solve_f64) against the oracle's exact FP64 max-min of
double coordinates (hd_oracle_exact_f64: the reference's distance formula in
double, the instantiation its disabled -is_double switch would select,
src/run_hausdorff_distance.cu:56-62).

Bar: the FP64 distance is bit-identical to the oracle's (sqrt of the same
double), and the certifying pair is the oracle's (lowest row, then lowest
column among ties).  Cases cover sets whose rounding to float matters (points
distinct in double and equal in float), sets that are exactly float values,
a lattice and its translate (every row ties: the candidate list overflows and
every row is walked), the scan route (eb, brute, other n_dims, coordinates
beyond the LBVH route's range), device pointers, and the errors.
"""
import json
import math
import os

import numpy as np
import pytest

import hd_oracle
from hausdorffdistance_gb300 import synth

pytestmark = pytest.mark.gpu

CORES = os.cpu_count() or 1


def oracle(a, b, undirected):
    h0, i0, j0 = hd_oracle.exact_f64(a, b, n_threads=CORES)
    out = {"h2": h0, "ia": i0, "ib": j0, "direction": 0, "h_ab": math.sqrt(h0), "h_ba": -1.0}
    if undirected:
        h1, i1, j1 = hd_oracle.exact_f64(b, a, n_threads=CORES)
        out["h_ba"] = math.sqrt(h1)
        if h1 > h0:
            out.update(h2=h1, ia=i1, ib=j1, direction=1)
    return out


def check(r, want):
    assert r.hd == math.sqrt(want["h2"]), (r.hd, math.sqrt(want["h2"]))
    assert r.hd_ab == want["h_ab"]
    if want["h_ba"] >= 0:
        assert r.hd_ba == want["h_ba"]
    assert (r.direction, int(r.ia), int(r.ib)) == (want["direction"], want["ia"], want["ib"])


def clusters(n, d, seed, sigma=0.01, k=32):
    rng = np.random.default_rng(seed)
    centers = rng.random((k, d))
    lab = rng.integers(0, k, n)
    return centers[lab] + rng.normal(0.0, sigma, (n, d))


CASES = {
    # (n_a, n_b, n_dims): double-precision clusters, B shifted
    "small2d": (1000, 800, 2),
    "mid3d": (50_000, 40_000, 3),
    "big3d": (1_000_000, 900_000, 3),
    "big2d": (600_000, 700_000, 2),
}


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("undirected", [False, True])
def test_f64_clusters_match_oracle(engine, case, undirected):
    na, nb, d = CASES[case]
    a = clusters(na, d, seed=na)
    b = clusters(nb, d, seed=nb + 1) + 0.003
    r = engine.solve_f64(a, b, undirected=undirected)
    check(r, oracle(a, b, undirected))
    assert r.variant_used == 3  # LBVH route
    # The FP64 work is a handful of rows, not the sets.
    assert r.rechecked <= max(32, (na + nb) // 100)


def test_f64_float_valued_inputs(engine):
    # Coordinates that are exactly floats: rounding moves nothing.
    a32, b32 = synth.clusters3d(300_000, seed=7)
    a, b = a32.astype(np.float64), b32.astype(np.float64)
    r = engine.solve_f64(a, b, undirected=True)
    check(r, oracle(a, b, True))


def test_f64_distinct_only_in_double(engine):
    # B = A moved by ~1e-10: in float most pairs coincide, in double every
    # nearest distance is ~1e-10, far below the float rounding of the
    # coordinates (~6e-8).  Every row is listed and walked in FP64.
    rng = np.random.default_rng(11)
    a = 1.0 + rng.random((20_000, 3))
    b = a + rng.normal(0.0, 1e-10, a.shape)
    r = engine.solve_f64(a, b, undirected=True)
    check(r, oracle(a, b, True))
    assert r.hd < 1e-8


def test_f64_lattice_translate_all_rows_tie(engine):
    # A lattice and its translate: every row's nearest distance is the same,
    # the candidate list (2^20 rows) overflows and every row is walked.
    g = np.arange(1100, dtype=np.float64)
    xx, yy = np.meshgrid(g, g[:1000], indexing="ij")
    a = np.stack([xx.ravel(), yy.ravel()], 1) * 0.001
    b = a + np.array([0.0003, 0.0001])
    r = engine.solve_f64(a, b)
    want = oracle(a, b, False)
    check(r, want)
    assert r.rechecked >= a.shape[0]


@pytest.mark.parametrize("variant", ["eb", "brute"])
def test_f64_scan_variants(engine, variant):
    a = clusters(30_000, 3, seed=5)
    b = clusters(20_000, 3, seed=6) + 0.002
    r = engine.solve_f64(a, b, undirected=True, variant=variant)
    check(r, oracle(a, b, True))
    assert r.variant_used == (1 if variant == "eb" else 5)


@pytest.mark.parametrize("d", [1, 5, 17])
def test_f64_other_dims(engine, d):
    rng = np.random.default_rng(d)
    a = rng.random((4000, d))
    b = rng.random((3000, d)) * 1.05
    r = engine.solve_f64(a, b, undirected=True)
    check(r, oracle(a, b, True))


def test_f64_large_coordinates_take_the_scan(engine):
    rng = np.random.default_rng(3)
    a = rng.random((5000, 2)) * 1e20
    b = rng.random((4000, 2)) * 1e20
    r = engine.solve_f64(a, b, undirected=True)
    check(r, oracle(a, b, True))
    assert r.variant_used == 1  # EB scan


def test_f64_device_pointers(engine):
    import torch
    a = clusters(200_000, 3, seed=21)
    b = clusters(150_000, 3, seed=22) + 0.004
    r = engine.solve_f64(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda(), undirected=True)
    check(r, oracle(a, b, True))


def test_f64_errors(engine):
    import hausdorffdistance_gb300 as hd
    a = np.zeros((10, 3))
    b = np.ones((10, 3))
    bad = a.copy()
    bad[3, 1] = np.nan
    with pytest.raises(hd.HDError):
        engine.solve_f64(bad, b)
    bad[3, 1] = np.inf
    with pytest.raises(hd.HDError):
        engine.solve_f64(bad, b)
    for v in ("grid", "bf16"):
        with pytest.raises(hd.HDError):
            engine.solve_f64(a, b, variant=v)
    with pytest.raises(hd.HDError):
        engine.solve_f64(np.zeros((10, 4)), np.ones((10, 4)), variant="lbvh")
    # The context stays usable.
    r = engine.solve_f64(a, b)
    assert r.hd == math.sqrt(3.0)


def test_f64_reference_mirror_class(built_lib):
    # The COORD_T = double instantiation of the reference's seam class.
    import hausdorffdistance_gb300 as hd
    a = clusters(40_000, 2, seed=31)
    b = clusters(30_000, 2, seed=32) + 0.001
    h = hd.HausdorffDistanceHybrid(coord_type="float64")
    got = h.CalculateDistance(a, b)
    assert isinstance(got, np.float64)
    assert got == math.sqrt(hd_oracle.exact_f64(a, b, n_threads=CORES)[0])
    assert {"Algorithm", "Execution", "ReportedTime"} <= set(h.get_stats())


EDGE = {
    "single_points": lambda rng: (np.array([[0.25, -1.5, 3.0]]), np.array([[1.0, 2.0, -0.5]])),
    "one_vs_many": lambda rng: (np.array([[0.5, 0.5, 0.5]]), rng.random((5000, 3))),
    "many_vs_one": lambda rng: (rng.random((5000, 3)), np.array([[0.5, 0.5, 0.5]])),
    "all_identical": lambda rng: (np.full((3000, 3), 0.3), np.full((2000, 3), 0.3)),
    "duplicates_with_ties": lambda rng: (np.repeat(rng.random((50, 2)), 40, axis=0),
                                         np.repeat(rng.random((60, 2)), 30, axis=0)),
    # Float rounding (ulp 0.0625 at 1e6) swamps the distances: every row is
    # listed and settled in FP64.
    "large_offset": lambda rng: (1e6 + clusters(100_000, 3, seed=41, sigma=0.001),
                                 1e6 + clusters(80_000, 3, seed=42, sigma=0.001) + 0.0005),
    "negative_coords": lambda rng: (-5.0 + clusters(60_000, 2, seed=43),
                                    -5.0 + clusters(50_000, 2, seed=44) - 0.002),
    # A exactly float-valued, B genuinely double.
    "mixed_precision": lambda rng: (clusters(70_000, 3, seed=45).astype(np.float32).astype(np.float64),
                                    clusters(60_000, 3, seed=46) + 1e-9),
}


@pytest.mark.parametrize("case", sorted(EDGE))
def test_f64_edge_cases(engine, case):
    rng = np.random.default_rng(7)
    a, b = EDGE[case](rng)
    for undirected in (False, True):
        r = engine.solve_f64(a, b, undirected=undirected, count_pairs=True, timing=True)
        check(r, oracle(a, b, undirected))
        assert r.ms > 0


def test_f64_repeated_calls_and_sizes(engine):
    # Buffers grow and shrink across calls; results stay exact.
    for n, m, seed in [(200_000, 150_000, 51), (3_000, 9_000, 52), (400_000, 20, 53)]:
        a = clusters(n, 3, seed=seed)
        b = clusters(m, 3, seed=seed + 100) + 0.001
        r = engine.solve_f64(a, b, undirected=True)
        check(r, oracle(a, b, True))


GOLDEN64 = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                                       "golden.json"))).get("cases_f64", [])


@pytest.mark.parametrize("case", GOLDEN64, ids=[c["name"] for c in GOLDEN64])
def test_f64_matches_reference_double_golden(engine, case):
    """hd_solve_f64 returns, bit for bit, the distance of the reference's own
    double instantiation (golden vectors of oracle/_ref/ref_eb64)."""
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

    def rd(p):
        with open(os.path.join(here, p), "rb") as f:
            n = int(np.frombuffer(f.read(8), np.uint64)[0])
            return np.frombuffer(f.read(), np.float64)[: n * case["dims"]].reshape(n, case["dims"])
    a, b = rd(case["a"]).copy(), rd(case["b"]).copy()
    r = engine.solve_f64(a, b)
    assert int(np.float64(r.hd).view(np.uint64)) == case["hd_bits"]
