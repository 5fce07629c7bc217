import numpy as np

from hausdorffdistance_gb300 import synth


def test_shapes_and_determinism(tmp_path):
    a, b = synth.uniform2d(1000, seed=1)
    a2, b2 = synth.uniform2d(1000, seed=1)
    assert a.shape == (1000, 2) and b.shape == (1000, 2)
    assert a.dtype == np.float32 and np.array_equal(a, a2) and np.array_equal(b, b2)
    # 5% outliers in [0, 1.2]^2 outside the unit square are possible.
    assert b.max() <= 1.2 + 1e-2
    a, b = synth.clusters3d(5000, seed=2)
    assert a.shape == (5000, 3)
    assert abs(float(b[:, 0].mean() - a[:, 0].mean()) - 0.05) < 0.03
    a, b = synth.unit64(2000, seed=3)
    assert np.allclose(np.linalg.norm(a, axis=1), 1.0, atol=1e-5)
    assert (np.abs(a - b).sum(1) > 0).sum() == 20
    a, b, off = synth.polylines(n_problems=50, seed=4)
    assert off[-1] == len(a) == len(b) and len(off) == 51
    assert np.diff(off).min() >= 8
    a, b = synth.planes3d(20000, seed=5, n_planes=10)
    assert a.shape == b.shape == (20000, 3)
    p = tmp_path / "x.bin"
    synth.write_bin(str(p), a)
    assert np.array_equal(synth.read_bin(str(p), 3), a)


def test_polyline_sizes_distribution():
    s = synth.polyline_sizes(100000, seed=4)
    assert s.min() >= 8 and s.max() <= 50000
    assert 150 <= np.median(s) <= 250


def test_spider_distributions():
    """The Spider point sets of the reference's synthetic experiments."""
    for dist in synth.SPIDER:
        a = synth.spider(dist, 20000, 3, seed=1)
        assert a.dtype == np.float32 and np.array_equal(a, synth.spider(dist, 20000, 3, seed=1))
        assert not np.array_equal(a, synth.spider(dist, 20000, 3, seed=2))
        assert a.min() >= 0.0 and a.max() <= 1.0
        assert a.shape == ((20000, 2) if dist == "sierpinski" else (20000, 3))
    g = synth.spider("gaussian", 50000, 3)
    assert abs(float(g.mean()) - 0.5) < 0.01 and abs(float(g.std()) - 0.1) < 0.01
    bit = synth.spider("bit", 50000, 3)
    # Multiples of 2^-10 with ~0.8^30 of the points at the origin; heavy duplicates.
    assert np.array_equal(bit * 1024, np.round(bit * 1024))
    assert len(np.unique(bit, axis=0)) < 0.95 * len(bit)
    assert abs(float((bit * 1024).astype(int).__and__(512).astype(bool).mean()) - 0.2) < 0.01
    diag = synth.spider("diagonal", 50000, 3)
    on = (diag[:, 0] == diag[:, 1]) & (diag[:, 1] == diag[:, 2])
    # 20% drawn on the diagonal, always kept; ~11% of the others rejected.
    assert 0.2 <= float(on.mean()) <= 0.25
    s = synth.spider("sierpinski", 50000)
    assert np.allclose(s[:3], [[0, 0], [1, 0], [0.5, np.sqrt(3) / 2]])
    # Every point lies in the triangle.
    assert (s[:, 1] <= np.sqrt(3) * np.minimum(s[:, 0], 1 - s[:, 0]) + 1e-6).all()
