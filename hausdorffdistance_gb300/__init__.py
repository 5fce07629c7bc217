"""GB300-native Hausdorff distance (directed and undirected) behind the
reference's algorithm interface.

The reference's seam is the C++ class template
``hd::HausdorffDistance<COORD_T,N_DIMS>`` with ``CalculateDistance(points_a,
points_b)`` and ``get_stats()`` (src/hausdorff_distance.h:15-43), implemented
by one class per variant (src/hd_impl/*.h).  The classes below keep those
names, argument meanings and the required stats keys ("Algorithm",
"Execution", "ReportedTime"); all compute goes through libhdgpu.so's C ABI
(include/hd_gpu.h) on the GPU.  There is no CPU fallback.

Differences from the reference, all deliberate:
  * inputs are never permuted in place (the reference shuffles them,
    early_break.h:50-52 and :132-136);
  * ``CalculateDistance(..., undirected=True)`` computes max(h(A,B), h(B,A)),
    which the reference can only do with two calls;
  * errors raise ``HDError`` with the library's status instead of aborting.
"""
from __future__ import annotations

import ctypes
import time

import numpy as np

from . import _lib
from ._lib import (HD_COUNT_PAIRS, HD_DEVICE_PTRS, HD_TIMING, HD_UNDIRECTED, HDError,
                   VARIANT_NAMES, VARIANTS)

__all__ = ["Engine", "HDError", "HausdorffDistance", "HausdorffDistanceEarlyBreak",
           "HausdorffDistanceHybrid", "HausdorffDistanceRayTracing",
           "HausdorffDistanceGrid", "HausdorffDistanceLBVH", "HausdorffDistanceBF16",
           "HausdorffDistanceBrute", "solve"]


def _as_points(x, name, dtype="float32"):
    """Returns (pointer, n, dims, is_device, keepalive) for a numpy array or a
    CUDA torch tensor of shape (n, dims) (dtype float32, or float64)."""
    mod = type(x).__module__
    if mod.startswith("torch"):
        if str(x.dtype) != "torch." + dtype:
            raise TypeError(f"{name} must be {dtype}")
        if x.dim() != 2:
            raise ValueError(f"{name} must have shape (n, n_dims)")
        x = x.contiguous()
        return x.data_ptr(), x.shape[0], x.shape[1], x.is_cuda, x
    a = np.ascontiguousarray(x, dtype=np.float32 if dtype == "float32" else np.float64)
    if a.ndim != 2:
        raise ValueError(f"{name} must have shape (n, n_dims)")
    return a.ctypes.data, a.shape[0], a.shape[1], False, a


class Engine:
    """One libhdgpu context: a CUDA stream plus a cached device arena.
    Mirrors one reference variant instance (not thread-safe, one per thread)."""

    def __init__(self, device: int = 0, variant: str | int = "auto", seed: int = 0,
                 sample_rate: float = 0.01, n_points_cell: int = 8, leaf_size: int = 16,
                 eb_only_threshold: int = 0, always_sample: bool = False,
                 batch_small_rows: int = 0, batch_chunk: int = 0, batch_window: int = 0,
                 lbvh_budget: int = 0, eb_cap_pairs: int = 0):
        self.lib = _lib.load()
        opt = _lib.Options()
        self.lib.hd_default_options(ctypes.byref(opt))
        opt.device = device
        opt.variant = VARIANTS[variant] if isinstance(variant, str) else int(variant)
        opt.seed = seed
        opt.sample_rate = sample_rate
        opt.n_points_cell = n_points_cell
        opt.leaf_size = leaf_size
        opt.eb_only_threshold = eb_only_threshold
        opt.always_sample = 1 if always_sample else 0
        opt.batch_small_rows = batch_small_rows  # 0: tuned table value
        opt.batch_chunk = batch_chunk            # 0: tuned table value
        opt.batch_window = batch_window          # 0: tuned table value
        opt.lbvh_budget = lbvh_budget            # 0: tuned table value
        opt.eb_cap_pairs = eb_cap_pairs          # 0: tuned table value
        h = ctypes.c_void_p()
        st = self.lib.hd_create(ctypes.byref(h), ctypes.byref(opt))
        if st != _lib.HD_OK:
            raise HDError(st, "hd_create failed (no sm_103a device?)")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self.lib.hd_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_stream(self, stream_handle: int | None):
        self.lib.hd_set_stream(self._h, ctypes.c_void_p(stream_handle or 0))

    @property
    def kernel_launches(self) -> int:
        return int(self.lib.hd_kernel_launches(self._h))

    def _check(self, st):
        if st != _lib.HD_OK:
            raise HDError(st, self.lib.hd_last_error(self._h).decode())

    def solve(self, A, B, undirected: bool = False, variant: str | int | None = None,
              count_pairs: bool = False, timing: bool = False) -> _lib.Result:
        pa, na, da, deva, ka = _as_points(A, "A")
        pb, nb, db, devb, kb = _as_points(B, "B")
        if da != db:
            raise ValueError("A and B must have the same n_dims")
        if deva != devb:
            raise ValueError("A and B must both be host arrays or both device tensors")
        flags = (HD_UNDIRECTED if undirected else 0) | (HD_DEVICE_PTRS if deva else 0)
        flags |= (HD_COUNT_PAIRS if count_pairs else 0) | (HD_TIMING if timing else 0)
        v = -1 if variant is None else (VARIANTS[variant] if isinstance(variant, str)
                                        else int(variant))
        res = _lib.Result()
        st = self.lib.hd_solve(self._h, ctypes.c_void_p(pa), na, ctypes.c_void_p(pb), nb,
                               da, flags, v, ctypes.byref(res))
        del ka, kb
        self._check(st)
        return res

    def solve_f64(self, A, B, undirected: bool = False, variant: str | int | None = None,
                  count_pairs: bool = False, timing: bool = False) -> _lib.Result:
        """Exact FP64 Hausdorff distance of float64 point sets (hd_solve_f64:
        the reference's double instantiations behind its disabled -is_double
        switch).  variant: auto, lbvh, eb or brute."""
        pa, na, da, deva, ka = _as_points(A, "A", "float64")
        pb, nb, db, devb, kb = _as_points(B, "B", "float64")
        if da != db:
            raise ValueError("A and B must have the same n_dims")
        if deva != devb:
            raise ValueError("A and B must both be host arrays or both device tensors")
        flags = (HD_UNDIRECTED if undirected else 0) | (HD_DEVICE_PTRS if deva else 0)
        flags |= (HD_COUNT_PAIRS if count_pairs else 0) | (HD_TIMING if timing else 0)
        v = -1 if variant is None else (VARIANTS[variant] if isinstance(variant, str)
                                        else int(variant))
        res = _lib.Result()
        st = self.lib.hd_solve_f64(self._h, ctypes.c_void_p(pa), na, ctypes.c_void_p(pb), nb,
                                   da, flags, v, ctypes.byref(res))
        del ka, kb
        self._check(st)
        return res

    def point_stats(self, P, n_points_cell: int = 10) -> _lib.PointStats:
        """Bounding box, density and statistics-grid occupancy of one 2-D or
        3-D point set (hd_compute_stats; the reference's per-file "Grid",
        "MBR" and "Density" log entries)."""
        pp, n, d, dev, keep = _as_points(P, "P")
        out = _lib.PointStats()
        st = self.lib.hd_compute_stats(self._h, ctypes.c_void_p(pp), n, d, n_points_cell,
                                       HD_DEVICE_PTRS if dev else 0, ctypes.byref(out))
        del keep
        self._check(st)
        return out

    def solve_batch(self, A, B, offsets_a, offsets_b, undirected=False, plain=False):
        """Many independent problems: problem i owns rows offsets_a[i]:offsets_a[i+1]
        of A and offsets_b[i]:offsets_b[i+1] of B.  Returns a structured numpy
        array with fields hd_f32, ia, ib, direction."""
        pa, na, da, deva, ka = _as_points(A, "A")
        pb, nb, db, devb, kb = _as_points(B, "B")
        oa = np.ascontiguousarray(offsets_a, np.int64)
        ob = np.ascontiguousarray(offsets_b, np.int64)
        n = len(oa) - 1
        if len(ob) - 1 != n:
            raise ValueError("offsets_a and offsets_b must describe the same number of problems")
        out = np.empty(n, dtype=[("hd_f32", "<f4"), ("ia", "<u4"), ("ib", "<u4"),
                                 ("direction", "<i4")])
        flags = (HD_UNDIRECTED if undirected else 0) | (HD_DEVICE_PTRS if deva else 0)
        res = out.ctypes.data_as(ctypes.POINTER(_lib.BatchResult))
        if plain:
            # hd_problem rows: offset_a, n_a, offset_b, n_b (uint64; negative
            # counts wrap to huge values and are rejected by the library).
            probs = np.empty((n, 4), np.int64)
            probs[:, 0] = oa[:-1]
            np.subtract(oa[1:], oa[:-1], out=probs[:, 1])
            probs[:, 2] = ob[:-1]
            np.subtract(ob[1:], ob[:-1], out=probs[:, 3])
            st = self.lib.hd_solve_batch_plain(
                self._h, ctypes.c_void_p(pa), na, ctypes.c_void_p(pb), nb, da,
                probs.ctypes.data_as(ctypes.POINTER(_lib.Problem)), n, flags, res)
        else:
            # Offsets go to the library as they are (int64 viewed as uint64).
            st = self.lib.hd_solve_batch_offsets(
                self._h, ctypes.c_void_p(pa), na, ctypes.c_void_p(pb), nb, da,
                ctypes.c_void_p(oa.ctypes.data), ctypes.c_void_p(ob.ctypes.data), n, flags, res)
        del ka, kb
        self._check(st)
        return out


def solve(A, B, undirected=False, variant="auto", **kw) -> _lib.Result:
    with Engine(variant=variant, **kw) as e:
        return e.solve(A, B, undirected=undirected)


class HausdorffDistance:
    """Mirror of hd::HausdorffDistance<COORD_T,N_DIMS> (src/hausdorff_distance.h:15-43).

    ``CalculateDistance(points_a, points_b)`` returns the directed distance
    h(A,B) as float32 (bit-identical to the reference's -execution=cpu
    result); the inputs may be numpy arrays (host, copied to the device
    inside the call) or CUDA float32 torch tensors (the reference's
    device_vector overload).  ``coord_type="float64"`` is the COORD_T =
    double instantiation: float64 inputs, the exact FP64 distance as
    float64 (hd_solve_f64).  ``get_stats()`` returns the per-call stats with
    the keys the reference requires."""

    algorithm = "?"
    variant = "auto"

    def __init__(self, seed: int = 0, device: int = 0, coord_type: str = "float32", **kw):
        if coord_type not in ("float32", "float64"):
            raise ValueError("coord_type is float32 or float64")
        self.coord_type = coord_type
        self._engine = Engine(device=device, variant=self.variant, seed=seed, **kw)
        self.stats_: dict = {}
        self.last_result: _lib.Result | None = None

    def CalculateDistance(self, points_a, points_b, undirected: bool = False):
        t0 = time.perf_counter()
        solve = self._engine.solve_f64 if self.coord_type == "float64" else self._engine.solve
        res = solve(points_a, points_b, undirected=undirected, count_pairs=True, timing=True)
        wall_ms = (time.perf_counter() - t0) * 1e3
        self.last_result = res
        on_device = type(points_a).__module__.startswith("torch") and points_a.is_cuda
        self.stats_ = {
            "Algorithm": self.algorithm,
            "Execution": "GPU",
            "ReportedTime": res.ms if res.ms > 0 else wall_ms,
            "WallTime": wall_ms,
            "InputsOnDevice": bool(on_device),
            "ComparedPairs": int(res.visited_pairs),
            "VisitedNodes": int(res.visited_nodes),
            "VariantUsed": VARIANT_NAMES.get(res.variant_used, "?"),
            "HD64": res.hd,
            "CertifyingPair": [int(res.ia), int(res.ib)],
            "Direction": int(res.direction),
        }
        return np.float64(res.hd) if self.coord_type == "float64" else np.float32(res.hd_f32)

    def get_stats(self) -> dict:
        for k in ("Algorithm", "Execution", "ReportedTime"):
            if k not in self.stats_:
                raise RuntimeError(f"stats missing {k}: call CalculateDistance first")
        return self.stats_


class HausdorffDistanceEarlyBreak(HausdorffDistance):
    """src/hd_impl/hausdorff_distance_early_break.h — persistent EB scan."""
    algorithm = "Early Break"
    variant = "eb"


class HausdorffDistanceHybrid(HausdorffDistance):
    """src/hd_impl/hausdorff_distance_hybrid.h — sampler-driven selector."""
    algorithm = "Hybrid"
    variant = "auto"


class HausdorffDistanceLBVH(HausdorffDistance):
    """LBVH nearest-neighbour search with early break; stands in for the
    OptiX variant src/hd_impl/hausdorff_distance_ray_tracing.h."""
    algorithm = "LBVH"
    variant = "lbvh"


HausdorffDistanceRayTracing = HausdorffDistanceLBVH


class HausdorffDistanceGrid(HausdorffDistance):
    """Morton-sorted uniform grid (src/index/uniform_grid.h) with ring search."""
    algorithm = "Uniform Grid"
    variant = "grid"


class HausdorffDistanceBF16(HausdorffDistance):
    """Split-BF16 tcgen05 tiles with exact FP32 recheck (high n_dims)."""
    algorithm = "Split BF16"
    variant = "bf16"


class HausdorffDistanceBrute(HausdorffDistance):
    """Plain FP32 all-pairs max-min (no early break)."""
    algorithm = "Brute Force"
    variant = "brute"
