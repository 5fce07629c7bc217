"""Seeded synthetic point sets for the five benchmark workloads.

The reference measures on real datasets (MRI volumes, CAD meshes, PLY scans,
WKT geometries) that are not available offline; these generators stand in for
them with the shapes, sizes and value distributions of the five workloads:

  uniform2d   2-D, A uniform in [0,1]^2; B = a permutation of A jittered by
              N(0, 1e-3) per coordinate, 5% of B replaced by U[0,1.2]^2.
  clusters3d  3-D Gaussian mixture of 64 isotropic clusters (centres uniform in
              the unit cube, sigma 0.01, equal weights); B an independent draw
              from the same mixture translated by (0.05, 0, 0).
  unit64      64-D rows ~ N(0, I) normalised to unit length; B = A with 1% of
              its rows replaced by fresh unit vectors.
  polylines   many 2-D problems: sizes round(LogNormal(ln 200, 1.2)) clipped
              to [8, 50000]; A a random walk from U[0,100]^2 with N(0, 0.01^2)
              steps; B the same vertices re-noised with N(0, 0.002^2).
  planes3d    LiDAR-like: 500 planes (centres U[0,100]^3, normals uniform on
              the sphere), points uniform on 10x10 in-plane patches plus
              N(0, 0.02) along the normal; B = A rotated 1 degree about z
              around the centroid, then 0.1% replaced by U[0,100]^3.

The reference's own synthetic experiments (expr/for_the_paper/data_gen.sh)
draw single point sets from the Spider generator of Katiyar et al.
(SpiderWeb, SIGSPATIAL 2020), one file per seed, and pair the seeds; ``spider``
restates its point distributions in the unit cube:

  uniform     every coordinate U[0,1).
  gaussian    every coordinate N(0.5, 0.1); points with a coordinate outside
              [0,1] are drawn again.
  bit         every coordinate sum_{i=1..digits} Bernoulli(prob) * 2^-i (the
              experiments use prob 0.2, digits 10): a skewed lattice with heavy
              exact duplicates.
  diagonal    with probability `prob` a point of the diagonal (c, c, ...),
              else c plus alternating +-N(0, buffer/5)/sqrt(2) per coordinate
              (buffer 0.5), points outside the cube drawn again.
  sierpinski  the chaos game on the triangle (0,0), (1,0), (1/2, sqrt(3)/2):
              the first three points are its corners, each next point the
              midpoint of the previous one and a corner chosen with
              probabilities 2/5, 2/5, 1/5.  Two-dimensional whatever the
              requested dimension, as in the generator.

Every generator draws from numpy's PCG64 with the given seed and returns
C-contiguous float32 arrays of shape (n, n_dims).  ``write_bin``/``read_bin``
use the reference's point-cache layout (src/loaders/loader.h:150-185): a
64-bit count followed by the packed float32 points.
"""
from __future__ import annotations

import numpy as np


def _rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def uniform2d(n: int = 200_000, seed: int = 1, outlier_frac: float = 0.05):
    rng = _rng(seed)
    a = rng.random((n, 2))
    b = a[rng.permutation(n)] + rng.normal(0.0, 1e-3, size=(n, 2))
    k = int(round(outlier_frac * n))
    if k:
        idx = rng.choice(n, size=k, replace=False)
        b[idx] = rng.random((k, 2)) * 1.2
    return np.ascontiguousarray(a, np.float32), np.ascontiguousarray(b, np.float32)


def clusters3d(n: int = 10_000_000, seed: int = 2, n_clusters: int = 64,
               sigma: float = 0.01, shift=(0.05, 0.0, 0.0)):
    rng = _rng(seed)
    centres = rng.random((n_clusters, 3))

    def draw():
        k = rng.integers(0, n_clusters, size=n)
        return centres[k] + rng.normal(0.0, sigma, size=(n, 3))

    a = draw()
    b = draw() + np.asarray(shift, np.float64)
    return np.ascontiguousarray(a, np.float32), np.ascontiguousarray(b, np.float32)


def unit64(n: int = 1_000_000, seed: int = 3, dims: int = 64,
           replace_frac: float = 0.01):
    rng = _rng(seed)
    a = rng.standard_normal((n, dims), dtype=np.float32)
    a /= np.linalg.norm(a, axis=1, keepdims=True)
    b = a.copy()
    k = int(round(replace_frac * n))
    if k:
        idx = rng.choice(n, size=k, replace=False)
        r = rng.standard_normal((k, dims), dtype=np.float32)
        r /= np.linalg.norm(r, axis=1, keepdims=True)
        b[idx] = r
    return np.ascontiguousarray(a, np.float32), np.ascontiguousarray(b, np.float32)


def polyline_sizes(n_problems: int = 100_000, seed: int = 4, median: float = 200.0,
                   sigma: float = 1.2, lo: int = 8, hi: int = 50_000):
    rng = _rng(seed)
    s = np.rint(rng.lognormal(np.log(median), sigma, size=n_problems))
    return np.clip(s, lo, hi).astype(np.int64)


def polylines(n_problems: int = 100_000, seed: int = 4, sizes=None):
    """Returns (A, B, offsets): problem p owns rows offsets[p]:offsets[p+1] of
    both A and B (B is A's walk re-noised, so both sets have the same size)."""
    if sizes is None:
        sizes = polyline_sizes(n_problems, seed)
    sizes = np.asarray(sizes, np.int64)
    rng = _rng(seed + 1_000_003)
    total = int(sizes.sum())
    offsets = np.zeros(len(sizes) + 1, np.int64)
    np.cumsum(sizes, out=offsets[1:])
    steps = rng.normal(0.0, 0.01, size=(total, 2))
    starts = rng.random((len(sizes), 2)) * 100.0
    # Each walk starts at its own origin: zero the first step of every problem
    # and add the start point, then cumulative-sum within problems.
    steps[offsets[:-1]] = 0.0
    walk = np.cumsum(steps, axis=0)
    base = walk[offsets[:-1]]
    owner = np.repeat(np.arange(len(sizes)), sizes)
    a = walk - base[owner] + starts[owner]
    b = a + rng.normal(0.0, 0.002, size=a.shape)
    return (np.ascontiguousarray(a, np.float32), np.ascontiguousarray(b, np.float32),
            offsets)


def planes3d(n: int = 50_000_000, seed: int = 5, n_planes: int = 500,
             patch: float = 10.0, noise: float = 0.02, angle_deg: float = 1.0,
             outlier_frac: float = 0.001, chunk: int = 5_000_000):
    rng = _rng(seed)
    centres = rng.random((n_planes, 3)) * 100.0
    normals = rng.standard_normal((n_planes, 3))
    normals /= np.linalg.norm(normals, axis=1, keepdims=True)
    # Orthonormal in-plane basis (u, v) per plane.
    helper = np.where(np.abs(normals[:, :1]) < 0.9, [[1.0, 0.0, 0.0]], [[0.0, 1.0, 0.0]])
    u = np.cross(normals, helper)
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    v = np.cross(normals, u)
    a = np.empty((n, 3), np.float32)
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        m = e - s
        k = rng.integers(0, n_planes, size=m)
        st = (rng.random((m, 2)) - 0.5) * patch
        h = rng.normal(0.0, noise, size=m)
        a[s:e] = (centres[k] + st[:, :1] * u[k] + st[:, 1:] * v[k]
                  + h[:, None] * normals[k]).astype(np.float32)
    centroid = a.mean(axis=0, dtype=np.float64)
    th = np.deg2rad(angle_deg)
    c, sn = np.cos(th), np.sin(th)
    b = np.empty_like(a)
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        x = a[s:e, 0].astype(np.float64) - centroid[0]
        y = a[s:e, 1].astype(np.float64) - centroid[1]
        b[s:e, 0] = (c * x - sn * y + centroid[0]).astype(np.float32)
        b[s:e, 1] = (sn * x + c * y + centroid[1]).astype(np.float32)
        b[s:e, 2] = a[s:e, 2]
    k = int(round(outlier_frac * n))
    if k:
        idx = rng.choice(n, size=k, replace=False)
        b[idx] = (rng.random((k, 3)) * 100.0).astype(np.float32)
    return a, b


WORKLOADS = {
    "uniform2d": uniform2d,
    "clusters3d": clusters3d,
    "unit64": unit64,
    "planes3d": planes3d,
}


SPIDER = ("uniform", "gaussian", "bit", "diagonal", "sierpinski")


def spider(dist: str, n: int, dims: int = 3, seed: int = 1, prob: float = 0.2,
           digits: int = 10, buffer: float = 0.5) -> np.ndarray:
    """One Spider point set (see the module docstring), float32 (n, dims);
    (n, 2) for sierpinski."""
    rng = _rng(seed)
    if dist == "uniform":
        out = rng.random((n, dims))
    elif dist in ("gaussian", "diagonal"):
        out = np.empty((0, dims))
        while len(out) < n:
            m = n - len(out) + 64
            if dist == "gaussian":
                p = rng.normal(0.5, 0.1, (m, dims))
            else:
                c = rng.random((m, 1))
                on = rng.random(m) < prob
                d = rng.normal(0.0, buffer / 5.0, (m, 1)) / np.sqrt(2.0)
                sign = 1.0 - 2.0 * (np.arange(dims) % 2)
                p = np.where(on[:, None], np.repeat(c, dims, 1), c + sign * d)
            p = p[np.all((p >= 0.0) & (p <= 1.0), axis=1)]
            out = np.concatenate([out, p])[:n]
    elif dist == "bit":
        weights = 0.5 ** np.arange(1, digits + 1)
        out = np.zeros((n, dims))
        for w in weights:
            out += (rng.random((n, dims)) < prob) * w
    elif dist == "sierpinski":
        corners = np.array([[0.0, 0.0], [1.0, 0.0], [0.5, np.sqrt(3.0) / 2.0]])
        pick = np.minimum(rng.integers(0, 5, n) // 2, 2)  # 2/5, 2/5, 1/5
        # Unrolled recurrence p_i = (p_{i-1} + v_i) / 2: p_i is the sum of
        # v_{i-k} / 2^(k+1); 60 terms exhaust double precision.
        v = corners[pick]
        out = np.zeros((n, 2))
        for k in range(60):
            out[k:] += v[: n - k] * 0.5 ** (k + 1)
        out[: min(n, 3)] = corners[: min(n, 3)]
    else:
        raise ValueError(f"unknown Spider distribution {dist!r}")
    return np.ascontiguousarray(out, np.float32)


def write_bin(path: str, pts: np.ndarray) -> None:
    pts = np.ascontiguousarray(pts, np.float32)
    with open(path, "wb") as f:
        f.write(np.uint64(pts.shape[0]).tobytes())
        f.write(pts.tobytes())


def read_bin(path: str, n_dims: int) -> np.ndarray:
    raw = np.fromfile(path, dtype=np.uint8)
    n = int(raw[:8].view(np.uint64)[0])
    return raw[8:8 + 4 * n * n_dims].view(np.float32).reshape(n, n_dims).copy()
