"""ctypes binding of libhdgpu.so's C ABI (include/hd_gpu.h).

The library is built in-tree by hausdorffdistance_gb300.build into
hausdorffdistance_gb300/_build/libhdgpu.so.  There is no CPU fallback: if the
library is missing, or no sm_103a device is present, calls fail loudly.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libhdgpu.so")

HD_OK = 0
STATUS_NAMES = {
    0: "HD_OK", 1: "HD_ERR_INVALID_ARG", 2: "HD_ERR_OOM", 3: "HD_ERR_DEVICE_TIMEOUT",
    4: "HD_ERR_CUDA", 5: "HD_ERR_UNSUPPORTED", 6: "HD_ERR_NO_DEVICE",
}

VARIANT_AUTO, VARIANT_EB, VARIANT_GRID, VARIANT_LBVH, VARIANT_BF16, VARIANT_BRUTE = range(6)
VARIANTS = {"auto": VARIANT_AUTO, "hybrid": VARIANT_AUTO, "eb": VARIANT_EB,
            "grid": VARIANT_GRID, "lbvh": VARIANT_LBVH, "rt": VARIANT_LBVH,
            "bf16": VARIANT_BF16, "brute": VARIANT_BRUTE}
VARIANT_NAMES = {VARIANT_AUTO: "auto", VARIANT_EB: "eb", VARIANT_GRID: "grid",
                 VARIANT_LBVH: "lbvh", VARIANT_BF16: "bf16", VARIANT_BRUTE: "brute"}

HD_DIRECTED = 0
HD_UNDIRECTED = 1
HD_DEVICE_PTRS = 2
HD_COUNT_PAIRS = 4
HD_TIMING = 8

# Every symbol include/hd_gpu.h declares.
EXPORTED = ["hd_default_options", "hd_create", "hd_destroy", "hd_set_stream",
            "hd_solve", "hd_solve_f64", "hd_solve_batch", "hd_solve_batch_offsets", "hd_solve_batch_plain",
            "hd_last_error",
            "hd_status_string", "hd_kernel_launches", "hd_version", "hd_solve_eb_noalloc",
            "hd_debug_bf16_rowmin", "hd_compute_stats"]

HD_STATS_HIST_ROWS = 96


class Options(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("variant", ctypes.c_int),
                ("seed", ctypes.c_uint64), ("sample_rate", ctypes.c_double),
                ("n_points_cell", ctypes.c_uint32), ("leaf_size", ctypes.c_uint32),
                ("eb_only_threshold", ctypes.c_uint32), ("always_sample", ctypes.c_uint32),
                ("batch_small_rows", ctypes.c_uint32), ("batch_chunk", ctypes.c_uint32),
                ("batch_window", ctypes.c_uint32), ("lbvh_budget", ctypes.c_uint32),
                ("eb_cap_pairs", ctypes.c_uint32), ("reserved", ctypes.c_uint32 * 2)]


class PointStats(ctypes.Structure):
    _fields_ = [("n_dims", ctypes.c_int32), ("n_points_cell", ctypes.c_uint32),
                ("n_points", ctypes.c_uint64), ("lower", ctypes.c_double * 3),
                ("upper", ctypes.c_double * 3), ("density", ctypes.c_double),
                ("grid_size", ctypes.c_uint32 * 3), ("max_points", ctypes.c_uint32),
                ("total_cells", ctypes.c_uint64), ("nonempty_cells", ctypes.c_uint64),
                ("median_points", ctypes.c_uint32), ("n_hist", ctypes.c_uint32),
                ("gini_index", ctypes.c_double), ("cell_diagonal", ctypes.c_double),
                ("build_ms", ctypes.c_double),
                ("hist_value", ctypes.c_double * HD_STATS_HIST_ROWS),
                ("hist_percentile", ctypes.c_double * HD_STATS_HIST_ROWS),
                ("hist_count", ctypes.c_uint64 * HD_STATS_HIST_ROWS)]


class Result(ctypes.Structure):
    _fields_ = [("hd", ctypes.c_double), ("hd_f32", ctypes.c_float),
                ("direction", ctypes.c_int32), ("ia", ctypes.c_uint64),
                ("ib", ctypes.c_uint64), ("hd_ab", ctypes.c_double),
                ("hd_ba", ctypes.c_double), ("visited_pairs", ctypes.c_uint64),
                ("visited_nodes", ctypes.c_uint64), ("ms", ctypes.c_double),
                ("phase_ms", ctypes.c_double * 8), ("variant_used", ctypes.c_int32),
                ("variant_used_ba", ctypes.c_int32), ("err_bound", ctypes.c_double),
                ("rechecked", ctypes.c_uint64), ("visited_leaves", ctypes.c_uint64),
                ("sample_p80", ctypes.c_double * 2), ("grid_outside", ctypes.c_double * 2),
                ("grid_skew", ctypes.c_double * 2), ("sample_mean", ctypes.c_double * 2)]


class Problem(ctypes.Structure):
    _fields_ = [("offset_a", ctypes.c_uint64), ("n_a", ctypes.c_uint64),
                ("offset_b", ctypes.c_uint64), ("n_b", ctypes.c_uint64)]


class BatchResult(ctypes.Structure):
    _fields_ = [("hd_f32", ctypes.c_float), ("ia", ctypes.c_uint32),
                ("ib", ctypes.c_uint32), ("direction", ctypes.c_int32)]


class HDError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


_lib = None


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Loads libhdgpu.so (once).  Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with "
                           "`python -m hausdorffdistance_gb300.build`")
    lib = ctypes.CDLL(path)
    P = ctypes.c_void_p
    lib.hd_default_options.argtypes = [ctypes.POINTER(Options)]
    lib.hd_default_options.restype = None
    lib.hd_create.argtypes = [ctypes.POINTER(P), ctypes.POINTER(Options)]
    lib.hd_create.restype = ctypes.c_int
    lib.hd_destroy.argtypes = [P]
    lib.hd_destroy.restype = ctypes.c_int
    lib.hd_set_stream.argtypes = [P, P]
    lib.hd_set_stream.restype = ctypes.c_int
    lib.hd_solve.argtypes = [P, P, ctypes.c_uint64, P, ctypes.c_uint64, ctypes.c_int,
                             ctypes.c_uint32, ctypes.c_int, ctypes.POINTER(Result)]
    lib.hd_solve.restype = ctypes.c_int
    lib.hd_solve_f64.argtypes = lib.hd_solve.argtypes
    lib.hd_solve_f64.restype = ctypes.c_int
    for name in ("hd_solve_batch", "hd_solve_batch_plain"):
        f = getattr(lib, name)
        f.argtypes = [P, P, ctypes.c_uint64, P, ctypes.c_uint64, ctypes.c_int,
                      ctypes.POINTER(Problem), ctypes.c_uint64, ctypes.c_uint32,
                      ctypes.POINTER(BatchResult)]
        f.restype = ctypes.c_int
    lib.hd_solve_batch_offsets.argtypes = [P, P, ctypes.c_uint64, P, ctypes.c_uint64,
                                           ctypes.c_int, P, P, ctypes.c_uint64, ctypes.c_uint32,
                                           ctypes.POINTER(BatchResult)]
    lib.hd_solve_batch_offsets.restype = ctypes.c_int
    lib.hd_last_error.argtypes = [P]
    lib.hd_last_error.restype = ctypes.c_char_p
    lib.hd_status_string.argtypes = [ctypes.c_int]
    lib.hd_status_string.restype = ctypes.c_char_p
    lib.hd_kernel_launches.argtypes = [P]
    lib.hd_kernel_launches.restype = ctypes.c_uint64
    lib.hd_solve_eb_noalloc.argtypes = [P, ctypes.c_uint64, P, ctypes.c_uint64, ctypes.c_int,
                                        ctypes.c_uint32, P, ctypes.POINTER(Result)]
    lib.hd_solve_eb_noalloc.restype = ctypes.c_int
    lib.hd_debug_bf16_rowmin.argtypes = [P, P, ctypes.c_uint64, P, ctypes.c_uint64, ctypes.c_int, P]
    lib.hd_debug_bf16_rowmin.restype = ctypes.c_int
    lib.hd_compute_stats.argtypes = [P, P, ctypes.c_uint64, ctypes.c_int, ctypes.c_uint32,
                                     ctypes.c_uint32, ctypes.POINTER(PointStats)]
    lib.hd_compute_stats.restype = ctypes.c_int
    lib.hd_version.argtypes = []
    lib.hd_version.restype = ctypes.c_char_p
    _lib = lib
    return lib
