"""ORACLE — test infrastructure, not product code.

ctypes wrapper of oracle/hd_oracle.cpp (the CPU restatement of the reference's
early-break path plus an exact max-min with the certifying pair).  Only
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it, and
only to check results or as the timed CPU baseline.  Parity is pinned against
the reference's own compiled CPU code through tests/golden/ (see
tests/test_oracle.py).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(_HERE, "_build", "liboracle.so")
REF_EB = os.path.join(_HERE, "_ref", "ref_eb")
_lib = None


def _load():
    global _lib
    if _lib is None:
        src = os.path.join(_HERE, "hd_oracle.cpp")
        if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
            os.makedirs(os.path.dirname(LIB), exist_ok=True)
            subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-pthread",
                            "-shared", "-fPIC", os.path.join(_HERE, "hd_oracle.cpp"),
                            "-o", LIB], check=True)
        lib = ctypes.CDLL(LIB)
        P = ctypes.c_void_p
        lib.hd_oracle_eb.argtypes = [P, ctypes.c_uint64, P, ctypes.c_uint64, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_int, ctypes.c_uint64, P, P, P, P]
        lib.hd_oracle_eb.restype = ctypes.c_int
        lib.hd_oracle_eb_window.argtypes = [P, ctypes.c_uint64, P, ctypes.c_uint64,
                                            ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_uint64, ctypes.c_uint64, ctypes.c_float,
                                            P, P, P, P]
        lib.hd_oracle_eb_window.restype = ctypes.c_int
        lib.hd_oracle_exact.argtypes = [P, ctypes.c_uint64, P, ctypes.c_uint64, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_int, P, P, P]
        lib.hd_oracle_exact.restype = ctypes.c_int
        lib.hd_oracle_exact_batch.argtypes = [P, P, P, P, ctypes.c_uint64, ctypes.c_int,
                                              ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P, P,
                                              P]
        lib.hd_oracle_exact_batch.restype = ctypes.c_int
        lib.hd_oracle_exact_f64.argtypes = [P, ctypes.c_uint64, P, ctypes.c_uint64, ctypes.c_int,
                                            ctypes.c_int, P, P, P]
        lib.hd_oracle_exact_f64.restype = ctypes.c_int
        lib.hd_oracle_dist2_f32.argtypes = [P, P, ctypes.c_int]
        lib.hd_oracle_dist2_f32.restype = ctypes.c_float
        _lib = lib
    return _lib


def _f32(x):
    return np.ascontiguousarray(x, dtype=np.float32)


def eb(A, B, seed=0, n_threads=1, limit_a=0):
    """Restatement of the reference CPU early-break (early_break.h:44-115).
    Returns dict(hd=float32, compared_pairs, compute_ms, shuffle_ms)."""
    lib = _load()
    A = _f32(A)
    B = _f32(B)
    hd = ctypes.c_float()
    pairs = ctypes.c_uint64()
    cm = ctypes.c_double()
    sm = ctypes.c_double()
    st = lib.hd_oracle_eb(A.ctypes.data, A.shape[0], B.ctypes.data, B.shape[0], A.shape[1],
                          seed, n_threads, limit_a, ctypes.byref(hd), ctypes.byref(pairs),
                          ctypes.byref(cm), ctypes.byref(sm))
    if st != 0:
        raise ValueError("oracle eb: unsupported input")
    return {"hd": np.float32(hd.value), "compared_pairs": int(pairs.value),
            "compute_ms": cm.value, "shuffle_ms": sm.value}


def eb_window(A, B, begin, end, cmax2_init, seed=0, n_threads=1):
    """The reference CPU early-break restated, over the window [begin, end)
    of the seeded shuffle of A, starting from the running maximum cmax2_init
    (a squared distance).  Returns the same dict as eb()."""
    lib = _load()
    A = _f32(A)
    B = _f32(B)
    hd = ctypes.c_float()
    pairs = ctypes.c_uint64()
    cm = ctypes.c_double()
    sm = ctypes.c_double()
    st = lib.hd_oracle_eb_window(A.ctypes.data, A.shape[0], B.ctypes.data, B.shape[0],
                                 A.shape[1], seed, n_threads, begin, end, float(cmax2_init),
                                 ctypes.byref(hd), ctypes.byref(pairs), ctypes.byref(cm),
                                 ctypes.byref(sm))
    if st != 0:
        raise ValueError("oracle eb_window: unsupported input")
    return {"hd": np.float32(hd.value), "compared_pairs": int(pairs.value),
            "compute_ms": cm.value, "shuffle_ms": sm.value}


def exact(A, B, precision=32, n_threads=None):
    """Exact directed max-min: returns (hd2, ia, ib) with hd2 the squared
    distance (FP32 formula for precision=32, FP64 for 64) and the certifying
    pair (lowest indices on ties)."""
    lib = _load()
    A = _f32(A)
    B = _f32(B)
    if n_threads is None:
        n_threads = os.cpu_count() or 1
    h2 = ctypes.c_double()
    ia = ctypes.c_uint64()
    ib = ctypes.c_uint64()
    st = lib.hd_oracle_exact(A.ctypes.data, A.shape[0], B.ctypes.data, B.shape[0],
                             A.shape[1], precision, n_threads, ctypes.byref(h2),
                             ctypes.byref(ia), ctypes.byref(ib))
    if st != 0:
        raise ValueError("oracle exact: unsupported input")
    return h2.value, int(ia.value), int(ib.value)


def exact_f64(A, B, n_threads=None):
    """Exact directed max-min of FP64 points with FP64 squared distances:
    returns (hd2, ia, ib), the certifying pair with the lowest indices on
    ties."""
    lib = _load()
    A = np.ascontiguousarray(A, dtype=np.float64)
    B = np.ascontiguousarray(B, dtype=np.float64)
    if n_threads is None:
        n_threads = os.cpu_count() or 1
    h2 = ctypes.c_double()
    ia = ctypes.c_uint64()
    ib = ctypes.c_uint64()
    st = lib.hd_oracle_exact_f64(A.ctypes.data, A.shape[0], B.ctypes.data, B.shape[0],
                                 A.shape[1], n_threads, ctypes.byref(h2), ctypes.byref(ia),
                                 ctypes.byref(ib))
    if st != 0:
        raise ValueError("oracle exact_f64: unsupported input")
    return h2.value, int(ia.value), int(ib.value)


def exact_batch(A, B, offsets_a, offsets_b, precision=32, undirected=True, n_threads=None):
    """Exact max-min of many independent problems (problem p owns rows
    offsets_a[p]..offsets_a[p+1]-1 of A and the same of B).  Returns arrays
    (hd2, ia, ib, direction); ia/ib are relative to the problem's start and
    index the direction's own source/target set."""
    lib = _load()
    A = _f32(A)
    B = _f32(B)
    oa = np.ascontiguousarray(offsets_a, dtype=np.uint64)
    ob = np.ascontiguousarray(offsets_b, dtype=np.uint64)
    n = len(oa) - 1
    if n_threads is None:
        n_threads = os.cpu_count() or 1
    h2 = np.zeros(n, np.float64)
    ia = np.zeros(n, np.uint64)
    ib = np.zeros(n, np.uint64)
    dr = np.zeros(n, np.int32)
    st = lib.hd_oracle_exact_batch(A.ctypes.data, B.ctypes.data, oa.ctypes.data, ob.ctypes.data,
                                   n, A.shape[1], precision, int(undirected), n_threads,
                                   h2.ctypes.data, ia.ctypes.data, ib.ctypes.data, dr.ctypes.data)
    if st != 0:
        raise ValueError("oracle exact_batch: unsupported input")
    return h2, ia, ib, dr


def dist2_f32(a, b):
    """FP32 squared distance of one pair, formed as the reference forms it."""
    lib = _load()
    a = _f32(a)
    b = _f32(b)
    return np.float32(lib.hd_oracle_dist2_f32(a.ctypes.data, b.ctypes.data, a.shape[0]))


def hd_f32(A, B, undirected=False):
    """Reference-exact float32 Hausdorff distance and its certifying data."""
    h2, ia, ib = exact(A, B, 32)
    out = {"hd_f32": np.sqrt(np.float32(h2)), "d2": np.float32(h2), "ia": ia, "ib": ib,
           "direction": 0}
    if undirected:
        h2b, ja, jb = exact(B, A, 32)
        if np.float32(h2b) > np.float32(h2):
            out = {"hd_f32": np.sqrt(np.float32(h2b)), "d2": np.float32(h2b), "ia": ja,
                   "ib": jb, "direction": 1}
    return out


def hd_f64(A, B, undirected=False):
    """FP64 Hausdorff distance (squared distances in FP64)."""
    h2, _, _ = exact(A, B, 64)
    if undirected:
        h2 = max(h2, exact(B, A, 64)[0])
    return float(np.sqrt(h2))
