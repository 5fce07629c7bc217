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


@pytest.mark.parametrize("dims", [2, 3])
@pytest.mark.parametrize("small_rows", [0, 1024])
def test_batch_incoherent_sets(dims, small_rows):
    """Random (not spatially ordered) sets: most rows do not settle in their
    short scan and go through the warp-wide scans."""
    import hausdorffdistance_gb300 as hd
    engine = hd.Engine(batch_small_rows=small_rows)  # 0: the tuned threshold
    rng = np.random.default_rng(9 + dims)
    # With a threshold of 1024, directions of <= 1024 query rows take the
    # one-warp path and larger ones the multi-pass pipeline; 1024/1025
    # straddle the boundary, 100 x 20000 sends open rows of a one-warp
    # direction through its warp-wide scan.
    na = [5000, 2000, 65, 64, 63, 1, 3000, 33, 1024, 1025, 100]
    nb = [4000, 2500, 64, 65, 1, 63, 3000, 97, 1025, 1024, 20000]
    a = rng.random((sum(na), dims)).astype(np.float32)
    b = rng.random((sum(nb), dims)).astype(np.float32)
    oa = np.concatenate([[0], np.cumsum(na)])
    ob = np.concatenate([[0], np.cumsum(nb)])
    for undirected in (False, True):
        out = engine.solve_batch(a, b, oa, ob, undirected=undirected)
        for p in range(len(na)):
            x, y = a[oa[p]:oa[p + 1]], b[ob[p]:ob[p + 1]]
            want = hd_oracle.hd_f32(x, y, undirected=undirected)
            assert out["hd_f32"][p] == want["hd_f32"], (p, undirected)


def test_batch_rejects_out_of_range_offsets(engine):
    import hausdorffdistance_gb300 as hd
    a = np.ones((4, 2), np.float32)
    # A huge offset whose sum with the count wraps around 2^64.
    with pytest.raises(hd.HDError):
        engine.solve_batch(a, a, np.array([2**63, 2**63 + 2], np.uint64).astype(np.int64),
                           [0, 2])
    with pytest.raises(ValueError):
        engine.solve_batch(a, a, [0, 2, 4], [0, 4])


def test_batch_reuses_graph_across_calls(engine):
    """Same launch shape, different problems: the cached graph re-plans from
    the problems on the device."""
    rng = np.random.default_rng(21)
    a = rng.random((3000, 2)).astype(np.float32)
    b = rng.random((3000, 2)).astype(np.float32)
    # Sizes (1000, 2000) then (2000, 1000): same item total and largest
    # problem, so the second and third calls run the first call's graph.
    for cut, shift in ((1000, 0.0), (2000, 0.0), (2000, 0.25)):
        off = np.array([0, cut, 3000])
        bb = b + np.float32(shift)
        out = engine.solve_batch(a, bb, off, off, undirected=True)
        for p in range(2):
            want = hd_oracle.hd_f32(a[off[p]:off[p + 1]], bb[off[p]:off[p + 1]], undirected=True)
            assert out["hd_f32"][p] == want["hd_f32"], (cut, shift, p)


def test_batch_schedules_agree():
    """Every schedule (one-warp threshold, items per warp step) gives the
    oracle's distances: all directions one-warp, none, and mixed."""
    import hausdorffdistance_gb300 as hd
    a, b, off = small_batch(150, seed=46)
    want = [hd_oracle.hd_f32(a[off[p]:off[p + 1]], b[off[p]:off[p + 1]], undirected=True)["hd_f32"]
            for p in range(len(off) - 1)]
    for small, chunk, window in ((1, 1, 1), (64, 8, 4), (8192, 3, 8), (65536, 64, 2)):
        with hd.Engine(batch_small_rows=small, batch_chunk=chunk, batch_window=window) as eng:
            out = eng.solve_batch(a, b, off, off, undirected=True)
        assert np.array_equal(out["hd_f32"], np.array(want, np.float32)), (small, chunk, window)


def test_batch_threshold_boundary_and_many_tiny_problems(engine):
    """Sizes straddling the tuned one-warp threshold (4096 rows) in the same
    batch as 200,000 problems of 1 to 3 points."""
    rng = np.random.default_rng(77)
    sizes = [4095, 4096, 4097, 8191] + list(rng.integers(1, 4, size=200_000))
    a, b, off = synth.polylines(sizes=sizes, seed=78)
    out = engine.solve_batch(a, b, off, off, undirected=True)
    check = list(range(4)) + list(rng.integers(4, len(sizes), size=300))
    for p in check:
        x, y = a[off[p]:off[p + 1]], b[off[p]:off[p + 1]]
        want = hd_oracle.hd_f32(x, y, undirected=True)
        assert out["hd_f32"][p] == want["hd_f32"], p


def test_batch_problem_array_abi_matches_offsets(engine):
    """hd_solve_batch (an hd_problem array) and hd_solve_batch_offsets (two
    offset arrays, what Engine.solve_batch calls) give the same results."""
    import ctypes
    from hausdorffdistance_gb300 import _lib
    a, b, off = small_batch(200, seed=47)
    offb = np.concatenate([[0], np.cumsum(np.maximum(np.diff(off) - 3, 1))])
    bb = np.concatenate([b[off[p]:off[p] + (offb[p + 1] - offb[p])] for p in range(len(off) - 1)])
    via_offsets = engine.solve_batch(a, bb, off, offb, undirected=True)
    n = len(off) - 1
    probs = (_lib.Problem * n)()
    for i in range(n):
        probs[i].offset_a, probs[i].n_a = int(off[i]), int(off[i + 1] - off[i])
        probs[i].offset_b, probs[i].n_b = int(offb[i]), int(offb[i + 1] - offb[i])
    out = np.empty(n, dtype=via_offsets.dtype)
    st = engine.lib.hd_solve_batch(engine._h, ctypes.c_void_p(a.ctypes.data), len(a),
                                   ctypes.c_void_p(bb.ctypes.data), len(bb), 2, probs, n,
                                   _lib.HD_UNDIRECTED,
                                   out.ctypes.data_as(ctypes.POINTER(_lib.BatchResult)))
    assert st == _lib.HD_OK
    assert np.array_equal(out["hd_f32"], via_offsets["hd_f32"])
    assert np.array_equal(out["direction"], via_offsets["direction"])


@pytest.mark.parametrize("undirected", [True, False])
def test_host_batch_runs_in_groups(engine, undirected):
    """Host points of at least 2 x 96 MB, given by offsets, run as groups of
    consecutive problems whose copies overlap the solves of earlier groups
    (here about 290 MB: three groups).  Every problem's result equals the
    device-input solve of the whole batch at once; a sample is checked
    against the oracle."""
    import torch
    rng = np.random.default_rng(91)
    n = 3000
    sizes = rng.integers(3000, 9000, n)
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    total = int(off[-1])
    a = rng.random((total, 2), dtype=np.float32)
    b = (a + rng.normal(0, 1e-3, a.shape)).astype(np.float32)
    far = rng.choice(total, 500, replace=False)
    b[far] = rng.random((500, 2), dtype=np.float32) * 1.5
    host = engine.solve_batch(a, b, off, off, undirected=undirected)
    dev = engine.solve_batch(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda(), off, off,
                             undirected=undirected)
    for f in ("hd_f32", "ia", "ib", "direction"):
        assert np.array_equal(host[f], dev[f]), f
    for i in (0, 1234, n - 1):
        sa, sb = a[off[i]:off[i + 1]], b[off[i]:off[i + 1]]
        want = hd_oracle.hd_f32(sa, sb, undirected=undirected)["hd_f32"]
        assert host["hd_f32"][i] == want, i
