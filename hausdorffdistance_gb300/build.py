"""In-tree build of the native parts: libhdgpu.so (CUDA, sm_103a only), the
hd_exec driver (C++, links libhdgpu.so through its C ABI) and the oracle's
CPU library (test infrastructure, oracle/).

    python -m hausdorffdistance_gb300.build [--no-exec] [--no-oracle]

Translation units compile in parallel; outputs go to
hausdorffdistance_gb300/_build/ and oracle/_build/ (both git-ignored).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
OUT = os.path.join(PKG, "_build")
ORACLE = os.path.join(ROOT, "oracle")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-fvisibility=hidden", "--expt-relaxed-constexpr",
              f"-I{INCLUDE}", f"-I{CSRC}"] + ARCH

LIB = os.path.join(OUT, "libhdgpu.so")
EXE = os.path.join(OUT, "hd_exec")
ORACLE_LIB = os.path.join(ORACLE, "_build", "liboracle.so")


def _nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return p


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs + [os.path.join(INCLUDE, "hd_gpu.h")]


def build_lib(verbose=False) -> str:
    os.makedirs(os.path.join(OUT, "obj"), exist_ok=True)
    srcs = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))
    hdrs = _headers()
    objs = []
    jobs = []
    for s in srcs:
        o = os.path.join(OUT, "obj", os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if not _newer(o, [s] + hdrs):
            jobs.append([_nvcc()] + NVCC_FLAGS + ["-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for r in ex.map(_run, jobs):
                if verbose and r.stderr:
                    print(r.stderr)
    if jobs or not _newer(LIB, objs):
        _run([_nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcuda"])
    return LIB


def build_exec() -> str:
    srcs = [os.path.join(HOST, f) for f in sorted(os.listdir(HOST)) if f.endswith(".cpp")]
    hdrs = [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".h")]
    if _newer(EXE, srcs + hdrs + [LIB, os.path.join(INCLUDE, "hd_gpu.h")]):
        return EXE
    cuda = os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))
    libdir = next((d for d in (os.path.join(cuda, "lib64"), os.path.join(cuda, "lib"))
                   if os.path.isdir(d)), os.path.join(cuda, "lib64"))
    # -ffp-contract=off: the CPU early-break forms squared distances without
    # fused multiply-adds, as the reference does.
    _run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-pthread", f"-I{INCLUDE}", f"-I{HOST}",
          f"-I{os.path.join(cuda, 'include')}"] + srcs
         + ["-o", EXE, f"-L{OUT}", "-lhdgpu", f"-L{libdir}", "-lcudart",
            "-Wl,-rpath,$ORIGIN", f"-Wl,-rpath,{libdir}"])
    return EXE


def build_oracle() -> str:
    """The oracle's CPU library (test infrastructure only)."""
    os.makedirs(os.path.dirname(ORACLE_LIB), exist_ok=True)
    src = os.path.join(ORACLE, "hd_oracle.cpp")
    if not _newer(ORACLE_LIB, [src]):
        _run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-pthread", "-shared",
              "-fPIC", src, "-o", ORACLE_LIB])
    return ORACLE_LIB


# Where the reference checkout lies in the build container (read-only); a
# different location can be given with HD_REFERENCE_SRC.
REFERENCE_SRC = os.environ.get("HD_REFERENCE_SRC", "/root/reference/src")


def build_reference() -> None:
    """Builds the reference's own CPU early-break path (float and double), its
    -normalize/-translate preprocessing and its statistics-grid shape into
    oracle/_ref when the reference sources are present (test infrastructure
    only: they generate tests/golden/)."""
    script = os.path.join(ORACLE, "build_ref.sh")
    targets = [os.path.join(ORACLE, "_ref", t) for t in ("ref_eb", "ref_eb64", "ref_prep",
                                                          "ref_stats")]
    if all(os.path.exists(t) for t in targets) or not os.path.isdir(REFERENCE_SRC):
        return
    subprocess.run(["bash", script, REFERENCE_SRC], check=False, capture_output=True)


def build_all(exec_=True, oracle=True) -> None:
    build_lib()
    if exec_ and os.path.isdir(HOST):
        build_exec()
    if oracle:
        build_oracle()
        build_reference()


if __name__ == "__main__":
    build_all(exec_="--no-exec" not in sys.argv, oracle="--no-oracle" not in sys.argv)
    print("built", LIB)
