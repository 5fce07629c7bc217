"""The oracle (oracle/hd_oracle.cpp) against golden vectors produced by the
reference's own CPU early-break code (tests/golden/make_golden.py)."""
import json
import os

import numpy as np
import pytest

import hd_oracle
from hausdorffdistance_gb300 import synth

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = json.load(open(os.path.join(HERE, "golden", "golden.json")))
CASES = GOLDEN["cases"]


def load_case(c):
    a = synth.read_bin(os.path.join(HERE, "golden", c["a"]), c["dims"])
    b = synth.read_bin(os.path.join(HERE, "golden", c["b"]), c["dims"])
    return a, b


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_eb_port_matches_reference_bit_for_bit(case):
    a, b = load_case(case)
    r = hd_oracle.eb(a, b, seed=case["seed"], n_threads=1)
    assert int(np.float32(r["hd"]).view(np.uint32)) == case["hd_bits"]
    # The compared-pair count depends on the seeded shuffle of both inputs and
    # on the break rule, so equality pins the whole restatement.
    assert r["compared_pairs"] == case["compared_pairs_t1"]
    r4 = hd_oracle.eb(a, b, seed=case["seed"], n_threads=4)
    assert int(np.float32(r4["hd"]).view(np.uint32)) == case["hd_bits_t4"]


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_exact_oracle_matches_reference(case):
    a, b = load_case(case)
    h2, ia, ib = hd_oracle.exact(a, b, 32)
    assert int(np.sqrt(np.float32(h2)).view(np.uint32)) == case["hd_bits"]
    # Certifying pair: achieves the maximum and is A[ia]'s nearest neighbour.
    assert hd_oracle.dist2_f32(a[ia], b[ib]) == np.float32(h2)
    d = ((a[ia].astype(np.float64) - b.astype(np.float64)) ** 2).sum(1)
    assert d.min() == pytest.approx(float(h2), rel=1e-6, abs=1e-30)


def brute_f64(a, b):
    a = a.astype(np.float64)
    b = b.astype(np.float64)
    best = np.full(len(a), np.inf)
    for s in range(0, len(b), 4096):
        d = ((a[:, None, :] - b[None, s:s + 4096, :]) ** 2).sum(-1)
        best = np.minimum(best, d.min(1))
    return best.max(), int(best.argmax())


@pytest.mark.parametrize("dims,na,nb,seed", [(2, 700, 900, 1), (3, 800, 500, 2),
                                             (5, 300, 400, 3), (64, 200, 300, 4)])
def test_exact_fp64_against_numpy(dims, na, nb, seed):
    rng = np.random.default_rng(seed)
    a = rng.random((na, dims)).astype(np.float32)
    b = rng.random((nb, dims)).astype(np.float32)
    h2, ia, ib = hd_oracle.exact(a, b, 64)
    want, wia = brute_f64(a, b)
    assert h2 == pytest.approx(want, rel=1e-12)
    assert ia == wia


def brute_f64_rows(a, b):
    """Exact FP64 max-min of double rows by numpy (the same left-to-right
    formula: difference, square, sum over dims in order), with the lowest
    row among equal maxima and its lowest column."""
    best = np.full(len(a), np.inf)
    col = np.zeros(len(a), np.int64)
    for s in range(0, len(b), 2048):
        diff = a[:, None, :] - b[None, s:s + 2048, :]
        d = diff[..., 0] * diff[..., 0]
        for k in range(1, a.shape[1]):
            d = d + diff[..., k] * diff[..., k]
        m = d.min(1)
        better = m < best
        col[better] = s + d.argmin(1)[better]
        best = np.minimum(best, m)
    i = int(np.flatnonzero(best == best.max())[0])
    return best[i], i, int(col[i])


@pytest.mark.parametrize("dims,na,nb,seed", [(2, 900, 700, 5), (3, 600, 800, 6), (5, 300, 400, 7)])
def test_exact_f64_inputs_against_numpy(dims, na, nb, seed):
    """The FP64-input oracle (double coordinates) against numpy, including a
    set whose points differ only below float precision."""
    rng = np.random.default_rng(seed)
    a = rng.random((na, dims))
    b = rng.random((nb, dims)) * 1.1
    assert hd_oracle.exact_f64(a, b) == brute_f64_rows(a, b)
    b2 = a[: nb // 2] + rng.normal(0.0, 1e-12, (nb // 2, dims))
    assert hd_oracle.exact_f64(a[: nb // 2 + 7], b2) == brute_f64_rows(a[: nb // 2 + 7], b2)


def test_exact_clustered_kdtree_vs_brute():
    a, b = synth.clusters3d(20000, seed=9)
    h2, ia, ib = hd_oracle.exact(a, b, 32)
    a64 = a.astype(np.float64)
    # Check the certifying pair by brute force on A[ia] and a sample of rows.
    d = ((a64[ia] - b) ** 2).sum(1)
    assert d.argmin() == ib
    rows = np.random.default_rng(0).choice(len(a), 200, replace=False)
    for r in rows:
        assert ((a64[r] - b) ** 2).sum(1).min() <= h2 * (1 + 1e-6)


def test_bounded_sample_eb():
    a, b = synth.uniform2d(5000, seed=5)
    full = hd_oracle.eb(a, b, n_threads=2)
    part = hd_oracle.eb(a, b, n_threads=2, limit_a=500)
    assert part["compared_pairs"] < full["compared_pairs"]
    assert part["hd"] <= full["hd"]


CASES64 = GOLDEN.get("cases_f64", [])


def load_case64(c):
    def rd(p):
        with open(os.path.join(HERE, "golden", p), "rb") as f:
            n = int(np.frombuffer(f.read(8), np.uint64)[0])
            return np.frombuffer(f.read(), np.float64)[: n * c["dims"]].reshape(n, c["dims"])
    return rd(c["a"]), rd(c["b"])


@pytest.mark.parametrize("case", CASES64, ids=[c["name"] for c in CASES64])
def test_exact_f64_oracle_matches_reference_double_build(case):
    """The FP64 oracle's exact max-min equals, bit for bit, what the
    reference's own early-break returns in its double instantiation (built
    from its sources as oracle/_ref/ref_eb64), including points distinct only
    below float precision, exact ties and large offsets."""
    a, b = load_case64(case)
    h2, ia, ib = hd_oracle.exact_f64(a, b)
    assert int(np.float64(np.sqrt(h2)).view(np.uint64)) == case["hd_bits"]
    assert case["hd_bits_t4"] == case["hd_bits"]
