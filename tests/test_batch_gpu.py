"""Batched solves (one graph-captured persistent launch) against the oracle
per problem and against the per-problem plain solves."""
import numpy as np
import pytest

import hd_oracle
from hausdorffdistance_gb300 import synth

pytestmark = pytest.mark.gpu


def small_batch(n_problems=300, seed=44, cap=3000):
    sizes = np.minimum(synth.polyline_sizes(n_problems, seed=seed), cap)
    a, b, off = synth.polylines(sizes=sizes, seed=seed)
    return a, b, off


@pytest.mark.parametrize("undirected", [True, False])
def test_batch_matches_oracle(engine, undirected):
    a, b, off = small_batch()
    out = engine.solve_batch(a, b, off, off, undirected=undirected)
    for p in range(len(off) - 1):
        x, y = a[off[p]:off[p + 1]], b[off[p]:off[p + 1]]
        want = hd_oracle.hd_f32(x, y, undirected=undirected)
        assert out["hd_f32"][p] == want["hd_f32"], p
        src, dst = (x, y) if out["direction"][p] == 0 else (y, x)
        assert hd_oracle.dist2_f32(src[out["ia"][p]], dst[out["ib"][p]]) == want["d2"]


def test_batch_equals_plain_and_device_inputs(engine):
    torch = pytest.importorskip("torch")
    a, b, off = small_batch(120, seed=45)
    # Uneven sizes per side: B of problem p is a prefix of its walk.
    offb = off.copy()
    nb = np.maximum(np.diff(off) // 2, 1)
    bparts = [b[off[p]:off[p] + nb[p]] for p in range(len(nb))]
    bb = np.concatenate(bparts)
    offb = np.concatenate([[0], np.cumsum(nb)])
    batched = engine.solve_batch(a, bb, off, offb, undirected=True)
    plain = engine.solve_batch(a, bb, off, offb, undirected=True, plain=True)
    assert np.array_equal(batched["hd_f32"], plain["hd_f32"])
    dev = engine.solve_batch(torch.from_numpy(a).cuda(), torch.from_numpy(bb).cuda(), off, offb,
                             undirected=True)
    assert np.array_equal(dev["hd_f32"], batched["hd_f32"])


def test_batch_3d_and_single_points(engine):
    rng = np.random.default_rng(7)
    sizes = [1, 2, 31, 32, 33, 700, 1]
    a = rng.random((sum(sizes), 3)).astype(np.float32)
    b = rng.random((sum(sizes), 3)).astype(np.float32)
    off = np.concatenate([[0], np.cumsum(sizes)])
    out = engine.solve_batch(a, b, off, off, undirected=True)
    for p in range(len(sizes)):
        want = hd_oracle.hd_f32(a[off[p]:off[p + 1]], b[off[p]:off[p + 1]], undirected=True)
        assert out["hd_f32"][p] == want["hd_f32"]


def test_batch_rejects_empty_problem(engine):
    import hausdorffdistance_gb300 as hd
    a = np.ones((4, 2), np.float32)
    with pytest.raises(hd.HDError) as ei:
        engine.solve_batch(a, a, [0, 2, 2], [0, 2, 4])
    assert ei.value.status == 1
