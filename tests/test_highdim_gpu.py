"""High-dimensional inputs: the FP32 scans (EB, brute) for any n_dims up to
128 and the split-BF16 tcgen05 tiles, against the oracle.  The BF16 kernel's
raw approximate row minima are also checked against FP64 minima within the
error bound the certification relies on."""
import ctypes

import numpy as np
import pytest

import hd_oracle
from hausdorffdistance_gb300 import synth

pytestmark = pytest.mark.gpu
REL_TOL_F64 = 1e-6


def row_bound(a, b, K):
    """Python copy of the kernel's per-row bound (hd_bf16.cu, row_bound)."""
    c = 4.0 * 2.0 ** -18 + (3.0 * K + 16.0) * 2.0 ** -23
    s = (a + b) ** 2
    e = 2.0 * c * a * b + 2.0 ** -21 * s + (K + 2.0) * 2.0 ** -24 * s
    return 2.0 * e + 1e-30


def exact_rowmin(a, b):
    a64 = a.astype(np.float64)
    b64 = b.astype(np.float64)
    out = np.empty(len(a))
    for s in range(0, len(a), 256):
        d = ((a64[s:s + 256, None, :] - b64[None, :, :]) ** 2).sum(-1)
        out[s:s + 256] = d.min(1)
    return out


@pytest.mark.parametrize("dims", [16, 32, 48, 64])
def test_bf16_rowmin_within_certified_bound(engine, dims):
    from hausdorffdistance_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(dims)
    a = (rng.standard_normal((700, dims)) * rng.uniform(0.2, 3.0, (700, 1))).astype(np.float32)
    b = (rng.standard_normal((900, dims)) * rng.uniform(0.2, 3.0, (900, 1))).astype(np.float32)
    b[:50] = a[:50]  # exact duplicates: minima of 0
    rowmin = np.zeros(len(a), np.float32)
    st = lib.hd_debug_bf16_rowmin(engine._h, a.ctypes.data, len(a), b.ctypes.data, len(b), dims,
                                  rowmin.ctypes.data)
    assert st == 0, lib.hd_last_error(engine._h)
    want = exact_rowmin(a, b)
    bmax = np.linalg.norm(b.astype(np.float64), axis=1).max()
    an = np.linalg.norm(a.astype(np.float64), axis=1)
    err = np.abs(rowmin.astype(np.float64) - want)
    assert np.all(err <= row_bound(an, bmax, dims)), err.max()
    # The bound is loose; the split products are far more accurate than it.
    assert err.max() < 1e-3 * (an.max() * bmax)


@pytest.mark.parametrize("variant", ["bf16", "eb", "brute", "auto"])
@pytest.mark.parametrize("dims", [16, 64])
def test_highdim_matches_oracle(engine, variant, dims):
    a, b = synth.unit64(3000, seed=30 + dims, dims=dims, replace_frac=0.02)
    b = b[:2500]
    r = engine.solve(a, b, undirected=True, variant=variant)
    want = hd_oracle.hd_f32(a, b, undirected=True)
    assert np.float32(r.hd_f32) == want["hd_f32"]
    assert r.hd == pytest.approx(hd_oracle.hd_f64(a, b, True), rel=REL_TOL_F64)
    src, dst = (a, b) if r.direction == 0 else (b, a)
    assert hd_oracle.dist2_f32(src[r.ia], dst[r.ib]) == want["d2"]
    if variant == "bf16":
        assert r.rechecked >= 1 and r.err_bound > 0


@pytest.mark.parametrize("dims", [1, 4, 5, 7, 24, 100, 128])
@pytest.mark.parametrize("variant", ["eb", "brute"])
def test_fp32_scans_any_dims(engine, dims, variant):
    rng = np.random.default_rng(dims * 3)
    a = rng.random((1500, dims)).astype(np.float32)
    b = rng.random((1300, dims)).astype(np.float32) * 1.05
    r = engine.solve(a, b, undirected=True, variant=variant)
    want = hd_oracle.hd_f32(a, b, undirected=True)
    assert np.float32(r.hd_f32) == want["hd_f32"]


def test_bf16_rejects_unsupported_dims(engine):
    import hausdorffdistance_gb300 as hd
    a = np.ones((10, 20), np.float32)
    with pytest.raises(hd.HDError) as ei:
        engine.solve(a, a, variant="bf16")
    assert ei.value.status == 5
