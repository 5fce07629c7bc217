"""The C-ABI library builds, loads and exports every symbol include/hd_gpu.h
declares; host-side argument handling (no GPU needed)."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "hd_gpu.h")).read()
    return sorted(set(re.findall(r"HD_API\s+[\w\s\*]+?\b(hd_\w+)\s*\(", src)))


def test_header_and_binding_agree():
    from hausdorffdistance_gb300 import _lib
    assert declared_symbols() == sorted(_lib.EXPORTED)


def test_library_exports_every_declared_symbol(built_lib):
    lib = ctypes.CDLL(built_lib)
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_defaults_and_strings(built_lib):
    from hausdorffdistance_gb300 import _lib
    lib = _lib.load()
    opt = _lib.Options()
    lib.hd_default_options(ctypes.byref(opt))
    assert opt.leaf_size == 16 and opt.n_points_cell == 8 and abs(opt.sample_rate - 0.01) < 1e-12
    assert lib.hd_status_string(3) == b"HD_ERR_DEVICE_TIMEOUT"
    assert b"sm_103a" in lib.hd_version()
    assert lib.hd_last_error(None) == b"null context"
    res = _lib.Result()
    # A null context is rejected before any device work.
    assert lib.hd_solve(None, None, 0, None, 0, 2, 0, 0, ctypes.byref(res)) == 1


def test_struct_layouts_match_header():
    from hausdorffdistance_gb300 import _lib
    assert ctypes.sizeof(_lib.Problem) == 32
    assert ctypes.sizeof(_lib.BatchResult) == 16
    assert ctypes.sizeof(_lib.Options) == 4 + 4 + 8 + 8 + 4 * 3 + 4 * 8 + 4


def test_no_device_is_reported_loudly(built_lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import hausdorffdistance_gb300 as hd
    with pytest.raises(hd.HDError) as ei:
        hd.Engine()
    assert ei.value.status == 6


def test_struct_layouts_match_the_header(tmp_path):
    """The ctypes mirrors of hd_result, hd_options and hd_point_stats have the
    sizes and field offsets the C compiler gives the header's structs."""
    import shutil
    import subprocess
    from hausdorffdistance_gb300 import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    include = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    checks = [("hd_result", _lib.Result), ("hd_options", _lib.Options),
              ("hd_point_stats", _lib.PointStats)]
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "hd_gpu.h"', 'int main(void) {']
    for cname, ct in checks:
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in ct._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", include, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    got = {}
    for ln in out.splitlines():
        c, f, v = ln.split()
        got[(c, f)] = int(v)
    for cname, ct in checks:
        assert got[(cname, "size")] == ctypes.sizeof(ct), cname
        for fname, _ in ct._fields_:
            assert got[(cname, fname)] == getattr(ct, fname).offset, (cname, fname)
