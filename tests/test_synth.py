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
