"""Seeded random sweep: many small-to-large shapes, distributions and variants
against the oracle in one run.  Each case draws its sizes (1 point to 2.1M
per set), n_dims (2 or 3), distribution (uniform, Gaussian clusters, points on
a line, heavy duplicates, a lattice with ties) and variant, and checks the
FP32 result bit for bit, the certifying pair and direction; the FP64 input
path is checked on a subset.  Sizes of 2M per set reach the two-queries-per-
lane LBVH launches and the per-set sorts; the small ones the fused sort."""
import math
import os

import numpy as np
import pytest

import hd_oracle

pytestmark = pytest.mark.gpu

CORES = os.cpu_count() or 1


def draw(rng, kind, n, d):
    if kind == "uniform":
        return rng.random((n, d))
    if kind == "clusters":
        c = rng.random((16, d))
        return c[rng.integers(0, 16, n)] + rng.normal(0.0, 0.01, (n, d))
    if kind == "line":
        t = rng.random((n, 1))
        return np.hstack([t, 0.5 * t] + ([0.25 * t] if d == 3 else [])) + rng.normal(0, 1e-4, (n, d))
    if kind == "duplicates":
        base = rng.random((max(1, n // 50), d))
        return base[rng.integers(0, len(base), n)]
    # lattice: many equal nearest distances
    k = int(math.ceil(n ** (1.0 / d))) + 1
    g = np.stack(np.meshgrid(*([np.arange(k)] * d), indexing="ij"), -1).reshape(-1, d)[:n]
    return g * 0.01 + (0.003 if rng.random() < 0.5 else 0.0)


def oracle32(a, b, undirected):
    h0, i0, j0 = hd_oracle.exact(a, b, 32, n_threads=CORES)
    want = {"d2": np.float32(h0), "direction": 0}
    if undirected:
        h1, _, _ = hd_oracle.exact(b, a, 32, n_threads=CORES)
        if np.float32(h1) > np.float32(h0):
            want = {"d2": np.float32(h1), "direction": 1}
    return want


def cases():
    rng = np.random.default_rng(2026)
    out = []
    sizes = [1, 2, 7, 31, 33, 64, 65, 500, 3000, 40_000, 250_000]
    for i in range(44):
        kind = ["uniform", "clusters", "line", "duplicates", "lattice"][i % 5]
        d = 2 + (i // 5) % 2
        na = int(rng.choice(sizes))
        nb = int(rng.choice(sizes))
        variant = ["auto", "lbvh", "grid", "eb"][i % 4]
        out.append((i, kind, d, na, nb, variant, bool(i % 3), 1000 + i))
    # Large: two-queries-per-lane launches and per-set sorts.
    out.append((100, "clusters", 3, 2_100_000, 2_000_000, "auto", True, 7))
    out.append((101, "uniform", 2, 2_000_000, 2_100_000, "lbvh", True, 8))
    return out


@pytest.mark.parametrize("case", cases(), ids=lambda c: f"{c[0]}-{c[1]}-{c[2]}d-{c[3]}x{c[4]}-{c[5]}")
def test_random_case_matches_oracle(engine, case):
    _, kind, d, na, nb, variant, undirected, seed = case
    rng = np.random.default_rng(seed)
    a = draw(rng, kind, na, d).astype(np.float32)
    b = (draw(rng, kind, nb, d) + rng.normal(0, 0.002, (nb, d))).astype(np.float32)
    r = engine.solve(a, b, undirected=undirected, variant=variant)
    want = oracle32(a, b, undirected)
    assert np.float32(r.hd_f32) == np.sqrt(want["d2"])
    assert r.direction == want["direction"]
    src, dst = (a, b) if r.direction == 0 else (b, a)
    assert hd_oracle.dist2_f32(src[int(r.ia)], dst[int(r.ib)]) == want["d2"]


@pytest.mark.parametrize("case", [c for c in cases() if c[0] % 4 == 1 or c[0] >= 100],
                         ids=lambda c: f"f64-{c[0]}-{c[1]}-{c[2]}d-{c[3]}x{c[4]}")
def test_random_case_f64_matches_oracle(engine, case):
    _, kind, d, na, nb, _, undirected, seed = case
    rng = np.random.default_rng(seed + 7)
    a = draw(rng, kind, na, d)
    b = draw(rng, kind, nb, d) + rng.normal(0, 0.002, (nb, d))
    r = engine.solve_f64(a, b, undirected=undirected)
    h0, i0, j0 = hd_oracle.exact_f64(a, b, n_threads=CORES)
    want = (h0, 0, i0, j0)
    if undirected:
        h1, i1, j1 = hd_oracle.exact_f64(b, a, n_threads=CORES)
        if h1 > h0:
            want = (h1, 1, i1, j1)
    assert r.hd == math.sqrt(want[0])
    assert (r.direction, int(r.ia), int(r.ib)) == want[1:]
