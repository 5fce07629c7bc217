"""hd_solve_eb_noalloc — the early-break solve for callers that cannot
allocate device memory during the call (a process whose HBM is all handed to
its own pool at start-up, or host code that must not let a cudaMalloc/cudaFree
synchronise the device).  It keeps all scratch in one fixed array inside the
library, so these checks call it through the C ABI twice in a row (the second
call finds the first call's leftovers in that array) and compare each result
with the oracle and with hd_solve's early-break variant on the same inputs:
the FP32 distance must be bit-identical and the FP64 distance within the
suite's 1e-6 relative bound of the oracle's FP64 max-min.  The capacity itself
(2^20 points per set) is run in 2-D and 3-D, and the device's free memory is
sampled around the second call to show that the call allocates nothing.

This file is named to be collected last: if it fails, a run that stops at
the first failure has already run every other test.
"""
import ctypes
import os

import numpy as np
import pytest

import hd_oracle
from hausdorffdistance_gb300 import synth

pytestmark = pytest.mark.gpu

REL_TOL_F64 = 1e-6
MAX_POINTS = 1 << 20  # the documented capacity of the fixed scratch array
CORES = os.cpu_count() or 1


def _pair_d2(src, dst, ia, ib):
    return hd_oracle.dist2_f32(src[ia], dst[ib])


def _oracle(a, b, undirected):
    want = hd_oracle.hd_f32(a, b, undirected=undirected)
    want["hd64"] = hd_oracle.hd_f64(a, b, undirected=undirected)
    return want


def _call(lib, _lib, ta, na, tb, nb, dims, flags, stream):
    out = _lib.Result()
    st = lib.hd_solve_eb_noalloc(ctypes.c_void_p(ta.data_ptr()), na, ctypes.c_void_p(tb.data_ptr()),
                                 nb, dims, flags, ctypes.c_void_p(stream), ctypes.byref(out))
    return st, out


def _run_twice(a, b, undirected, want, ref=None):
    torch = pytest.importorskip("torch")
    from hausdorffdistance_gb300 import _lib
    lib = _lib.load()
    flags = _lib.HD_UNDIRECTED if undirected else 0
    ta = torch.from_numpy(a).cuda()
    tb = torch.from_numpy(b).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    torch.cuda.synchronize()
    free = []
    for _ in range(2):
        free.append(torch.cuda.mem_get_info()[0])
        st, out = _call(lib, _lib, ta, len(a), tb, len(b), a.shape[1], flags, stream)
        assert st == _lib.HD_OK
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
        assert np.float32(out.hd_f32) == want["hd_f32"]
        assert out.direction == want["direction"]
        assert abs(out.hd - want["hd64"]) <= REL_TOL_F64 * want["hd64"]
        src, dst = (a, b) if out.direction == 0 else (b, a)
        assert _pair_d2(src, dst, out.ia, out.ib) == want["d2"]
        if ref is not None:
            assert np.float32(out.hd_f32) == np.float32(ref.hd_f32)
            assert out.hd == pytest.approx(ref.hd, rel=REL_TOL_F64)
    # The first call may load the library's kernels (lazy module loading
    # takes device memory once); the second call must not change the
    # device's free memory at all.
    assert free[3] == free[2], f"free device memory changed by {free[2] - free[3]} bytes"
    # Inputs are left untouched.
    assert np.array_equal(ta.cpu().numpy(), a) and np.array_equal(tb.cpu().numpy(), b)


@pytest.mark.parametrize("undirected", [False, True])
def test_noalloc_matches_oracle_and_hd_solve_on_two_calls(undirected):
    import hausdorffdistance_gb300 as hd
    cases = [synth.uniform2d(60_000, seed=21), synth.clusters3d(50_000, seed=22),
             synth.planes3d(30_000, seed=23, n_planes=12)]
    with hd.Engine(device=0) as eng:
        for a, b in cases:
            ref = eng.solve(a, b, undirected=undirected, variant="eb")
            _run_twice(a, b, undirected, _oracle(a, b, undirected), ref)


@pytest.mark.parametrize("dims", [2, 3])
def test_noalloc_at_capacity(dims):
    if dims == 2:
        a, b = synth.uniform2d(MAX_POINTS, seed=24)
    else:
        a, b = synth.clusters3d(MAX_POINTS, seed=25)
    assert len(a) == len(b) == MAX_POINTS
    _run_twice(a, b, True, _oracle(a, b, True))


def test_noalloc_rejects_inputs_beyond_capacity():
    from hausdorffdistance_gb300 import _lib
    lib = _lib.load()
    out = _lib.Result()
    # The size check comes before any device work, so these pointers are
    # never dereferenced.
    fake = ctypes.c_void_p(16)
    assert lib.hd_solve_eb_noalloc(fake, MAX_POINTS + 1, fake, 10, 3, 0, None,
                                   ctypes.byref(out)) == 1  # HD_ERR_INVALID_ARG
    assert lib.hd_solve_eb_noalloc(fake, 10, fake, MAX_POINTS + 1, 2, 0, None,
                                   ctypes.byref(out)) == 1  # HD_ERR_INVALID_ARG
    assert lib.hd_solve_eb_noalloc(fake, 10, fake, 10, 5, 0, None,
                                   ctypes.byref(out)) == 1  # HD_ERR_INVALID_ARG
