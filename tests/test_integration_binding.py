"""The binding INTEGRATION.md documents (section 1: a HausdorffDistance
subclass over the C ABI) compiles against the reference's own seam header,
src/hausdorff_distance.h, with the project-written stand-ins for glog and
nlohmann::json the oracle's reference build uses (oracle/shim/).  Needs the
reference sources (present where the library is developed; the test is
skipped elsewhere) and nvcc; it compiles only, no GPU."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_SRC = os.environ.get("HD_REFERENCE_SRC", "/root/reference/src")


def test_documented_subclass_compiles_against_the_reference_seam(tmp_path):
    if not os.path.isfile(os.path.join(REF_SRC, "hausdorff_distance.h")):
        pytest.skip("reference sources not present")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not present")
    doc = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    section = doc.split("## 1.", 1)[1].split("## 2.", 1)[0]
    code = re.search(r"```cpp\n(.*?)```", section, re.S).group(1)
    hdr = tmp_path / "hausdorff_distance_gb300.h"
    hdr.write_text(code)
    unit = tmp_path / "binding.cu"
    unit.write_text('#include "hausdorff_distance_gb300.h"\n'
                    "template class hd::HausdorffDistanceGB300<float, 2>;\n"
                    "template class hd::HausdorffDistanceGB300<float, 3>;\n")
    shim = os.path.join(ROOT, "oracle", "shim")
    r = subprocess.run([nvcc, "-std=c++17", "--extended-lambda", "--expt-relaxed-constexpr",
                        "-I", str(tmp_path), "-I", shim, "-I", REF_SRC,
                        "-I", os.path.join(ROOT, "include"),
                        "-include", os.path.join(shim, "prelude.h"),
                        "-c", str(unit), "-o", str(tmp_path / "binding.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
