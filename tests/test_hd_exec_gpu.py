"""The hd_exec driver and the C++ seam mirror, end to end on the golden
inputs (GPU), plus argument handling that needs no GPU."""
import json
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HERE = os.path.join(ROOT, "tests")
BUILD = os.path.join(ROOT, "hausdorffdistance_gb300", "_build")
EXE = os.path.join(BUILD, "hd_exec")
GOLDEN = json.load(open(os.path.join(HERE, "golden", "golden.json")))["cases"]


@pytest.fixture(scope="module")
def exe():
    from hausdorffdistance_gb300 import build
    build.build_lib()
    build.build_exec()
    return EXE


def bits(x):
    return int(np.float32(x).view(np.uint32))


@pytest.mark.parametrize("case", GOLDEN, ids=[c["name"] for c in GOLDEN])
def test_cpu_execution_matches_reference_golden(exe, case, tmp_path):
    """-execution cpu (the driver's CPU early-break, product code written
    apart from the oracle) gives the reference's own CPU result bit for bit
    and, on one thread, its compared-pair count (which pins the seeded
    shuffle and the break rule).  Needs no GPU."""
    out = tmp_path / "run.json"
    r = subprocess.run([exe, "-input1", os.path.join(HERE, "golden", case["a"]), "-input2",
                        os.path.join(HERE, "golden", case["b"]), "-input_type", "bin",
                        "-n_dims", str(case["dims"]), "-execution", "cpu", "-repeat", "1",
                        "-parallelism", "1", "-seed", str(case["seed"]), "-json", str(out)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    st = json.load(open(out))
    assert bits(st["HDResult"]) == case["hd_bits"]
    rep = st["Running"]["Repeats"][0]
    assert rep["Execution"] == "CPU" and rep["Algorithm"] == "Early Break"
    assert rep["ComparedPairs"] == case["compared_pairs_t1"]
    assert {"Threads", "ShuffleTime", "ComputeTime", "ReportedTime"} <= set(rep)
    # The reference's "Running" configuration keys, whatever the execution.
    assert {"Seed", "FastBuildBVH", "RebuildBVH", "SampleRate", "NumPointsPerCell", "MaxHit",
            "EBOnlyThreshold", "AutoTune", "Repeats", "AvgTime"} <= set(st["Running"])
    assert {"DateTime", "Input", "Running", "HDResult"} <= set(st)
    assert {"Files", "Normalize", "Translate", "SerializationPrefix", "Limit", "NumDims",
            "Type"} <= set(st["Input"])


GOLDEN64 = json.load(open(os.path.join(HERE, "golden", "golden.json"))).get("cases_f64", [])


@pytest.mark.parametrize("case", GOLDEN64, ids=[c["name"] for c in GOLDEN64])
def test_cpu_execution_is_double_matches_reference_golden(exe, case, tmp_path):
    """-is_double -execution cpu gives the distance bits of the reference's own
    double instantiation and, on one thread, its compared-pair count.  Needs
    no GPU."""
    out = tmp_path / "run.json"
    r = subprocess.run([exe, "-input1", os.path.join(HERE, "golden", case["a"]), "-input2",
                        os.path.join(HERE, "golden", case["b"]), "-input_type", "bin",
                        "-n_dims", str(case["dims"]), "-execution", "cpu", "-is_double",
                        "-repeat", "1", "-parallelism", "1", "-seed", str(case["seed"]),
                        "-json", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    st = json.load(open(out))
    assert int(np.float64(st["HDResult"]).view(np.uint64)) == case["hd_bits"]
    assert st["Running"]["Repeats"][0]["ComparedPairs"] == case["compared_pairs_t1"]


def write_wkt(path, pts):
    with open(path, "w") as f:
        for p in pts:
            f.write("POINT (" + " ".join("%.17g" % v for v in p) + ")\n")


@pytest.fixture(scope="module")
def double_inputs(tmp_path_factory):
    """Two 3-D WKT files whose coordinates need double precision (17
    significant digits), and the oracle's exact FP64 directed/undirected
    distances of the parsed doubles."""
    import hd_oracle
    d = tmp_path_factory.mktemp("f64")
    rng = np.random.default_rng(4)
    a = rng.random((3000, 3))
    b = rng.random((2500, 3)) * 1.1
    pa, pb = str(d / "a.wkt"), str(d / "b.wkt")
    write_wkt(pa, a)
    write_wkt(pb, b)
    h_ab = np.sqrt(hd_oracle.exact_f64(a, b)[0])
    h_ba = np.sqrt(hd_oracle.exact_f64(b, a)[0])
    return pa, pb, float(h_ab), float(max(h_ab, h_ba))


@pytest.mark.parametrize("undirected", [False, True])
def test_cpu_execution_is_double(exe, double_inputs, undirected, tmp_path):
    """-is_double -execution cpu: the CPU early-break over the parsed doubles
    gives the oracle's exact FP64 distance (printed with 17 digits)."""
    pa, pb, h_ab, h_und = double_inputs
    out = tmp_path / "run.json"
    r = subprocess.run([exe, "-input1", pa, "-input2", pb, "-input_type", "wkt", "-n_dims", "3",
                        "-execution", "cpu", "-is_double", "-repeat", "1", "-json", str(out)]
                       + (["-undirected"] if undirected else []), capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    want = h_und if undirected else h_ab
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("HausdorffDistance")][0]
    assert float(line.split()[-1]) == want
    st = json.loads(out.read_text())
    assert st["HDResult"] == want
    assert st["Input"]["Type"] == "Double"


@pytest.mark.parametrize("fmt", ["off", "ply"])
def test_cpu_execution_is_double_off_ply(exe, fmt, tmp_path):
    """-is_double through the OFF loader (each number parsed once as float,
    once as double) and the ASCII PLY loader (doubles shifted so that every
    axis starts at 0, as the reference's PLY loader does): the CPU
    early-break gives the oracle's exact FP64 distance of the parsed doubles."""
    import hd_oracle
    rng = np.random.default_rng(12)
    a = 3.0 + rng.random((700, 3))
    b = 3.0 + rng.random((600, 3)) * 1.05
    paths = []
    for name, pts in (("a", a), ("b", b)):
        p = str(tmp_path / f"{name}.{fmt}")
        with open(p, "w") as f:
            if fmt == "off":
                f.write(f"OFF\n{len(pts)} 0 0\n")
            else:
                f.write(f"ply\nformat ascii 1.0\nelement vertex {len(pts)}\nproperty double x\n"
                        "property double y\nproperty double z\nend_header\n")
            for q in pts:
                f.write(" ".join("%.17g" % v for v in q) + "\n")
        paths.append(p)
    if fmt == "ply":
        # The PLY loader shifts each set to its own minimum per axis.
        a, b = a - a.min(0), b - b.min(0)
    want = float(np.sqrt(hd_oracle.exact_f64(a, b)[0]))
    r = subprocess.run([exe, "-input1", paths[0], "-input2", paths[1], "-input_type", fmt,
                        "-n_dims", "3", "-execution", "cpu", "-is_double", "-repeat", "1"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("HausdorffDistance")][0]
    assert float(line.split()[-1]) == want


@pytest.fixture(scope="module")
def image_inputs(tmp_path_factory):
    """Two 3-D int16 volumes shaped like the reference's medical-image inputs
    (NIfTI-1 files, a noisy ellipsoid of intensities in each, some of them
    multiples of 256 that the unsigned-char conversion drops), with the point
    sets the loader must take from them and the oracle's FP32 distances."""
    import hd_oracle
    from image_files import image_points, write_nifti
    d = tmp_path_factory.mktemp("img")
    rng = np.random.default_rng(21)
    z, y, x = np.meshgrid(np.arange(30), np.arange(34), np.arange(38), indexing="ij")
    vols = []
    for c, r in (((15, 17, 19), (11, 13, 15)), ((14, 18, 20), (12, 12, 16))):
        inside = ((z - c[0]) / r[0]) ** 2 + ((y - c[1]) / r[1]) ** 2 + ((x - c[2]) / r[2]) ** 2 < 1
        v = np.where(inside, rng.integers(1, 1200, inside.shape), 0)
        v[rng.random(inside.shape) < 0.002] = 700  # stray voxels outside the body
        v[inside & (rng.random(inside.shape) < 0.05)] = 512
        vols.append(v.astype(np.int16))
    paths = [str(d / "a.nii"), str(d / "b.nii")]
    for pth, v in zip(paths, vols):
        write_nifti(pth, v)
    a, b = (image_points(v, 3).astype(np.float32) for v in vols)
    h_ab = np.sqrt(np.float32(hd_oracle.exact(a, b, 32)[0]))
    h_ba = np.sqrt(np.float32(hd_oracle.exact(b, a, 32)[0]))
    return paths, len(a), len(b), h_ab, max(h_ab, h_ba)


@pytest.mark.parametrize("undirected", [False, True])
def test_cpu_execution_image(exe, image_inputs, undirected, tmp_path):
    """-input_type image -execution cpu on NIfTI volumes: the voxel points the
    reference's ITK loader takes, and the oracle's FP32 distance bit for bit."""
    paths, na, nb, h_ab, h_und = image_inputs
    out = tmp_path / "run.json"
    r = subprocess.run([exe, "-input1", paths[0], "-input2", paths[1], "-input_type", "image",
                        "-n_dims", "3", "-execution", "cpu", "-repeat", "1", "-json", str(out)]
                       + (["-undirected"] if undirected else []), capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    st = json.loads(out.read_text())
    assert [f["NumPoints"] for f in st["Input"]["Files"]] == [na, nb]
    assert bits(st["HDResult"]) == bits(h_und if undirected else h_ab)


@pytest.mark.gpu
@pytest.mark.parametrize("variant", ["hybrid", "eb"])
def test_hd_exec_image(exe, image_inputs, variant, tmp_path):
    """-input_type image on the GPU: the oracle's FP32 distance bit for bit."""
    paths, _, _, _, h_und = image_inputs
    out = tmp_path / "run.json"
    r = subprocess.run([exe, "-input1", paths[0], "-input2", paths[1], "-input_type", "image",
                        "-n_dims", "3", "-variant", variant, "-undirected", "-repeat", "2",
                        "-json", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert bits(json.loads(out.read_text())["HDResult"]) == bits(h_und)


@pytest.mark.gpu
@pytest.mark.parametrize("max_hit", [0, 1, 40])
def test_hd_exec_max_hit(exe, max_hit, tmp_path):
    """-max_hit caps an LBVH packet's visits before its open queries go to the
    deferred pass (0: no cap, as in the reference; 1: every packet deferred):
    the distance stays the oracle's, and the JSON logs the cap."""
    import hd_oracle
    rng = np.random.default_rng(31)
    c = rng.random((12, 3))
    a = (c[rng.integers(0, 12, 20000)] + rng.normal(0, 0.01, (20000, 3))).astype(np.float32)
    b = (c[rng.integers(0, 12, 18000)] + rng.normal(0, 0.01, (18000, 3)) + [0.02, 0, 0]).astype(np.float32)
    paths = []
    for name, pts in (("a", a), ("b", b)):
        p = str(tmp_path / f"{name}.bin")
        with open(p, "wb") as f:
            f.write(np.uint64(len(pts)).tobytes() + pts.tobytes())
        paths.append(p)
    h = max(np.sqrt(np.float32(hd_oracle.exact(a, b, 32)[0])),
            np.sqrt(np.float32(hd_oracle.exact(b, a, 32)[0])))
    out = tmp_path / "run.json"
    r = subprocess.run([exe, "-input1", paths[0], "-input2", paths[1], "-input_type", "bin",
                        "-n_dims", "3", "-variant", "rt", "-undirected", "-repeat", "2",
                        "-max_hit", str(max_hit), "-json", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    st = json.loads(out.read_text())
    assert bits(st["HDResult"]) == bits(h)
    assert st["Running"]["MaxHit"] == max_hit
    assert st["Running"]["LBVHBudget"] == (max_hit or 0xFFFFFFFF)
    # The sweep form: one JSON file per -max_hit_list entry.
    prefix = str(tmp_path / "sweep")
    r = subprocess.run([exe, "-input1", paths[0], "-input2", paths[1], "-input_type", "bin",
                        "-n_dims", "3", "-variant", "rt", "-undirected", "-repeat", "1",
                        "-vary_params", "-max_hit_list", f"{max_hit},7", "-json", prefix],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for mh in (max_hit, 7):
        sw = json.loads(open(f"{prefix}_sr0.01_th0_np8_mh{mh}.json").read())
        assert bits(sw["HDResult"]) == bits(h) and sw["Running"]["MaxHit"] == mh


@pytest.mark.gpu
@pytest.mark.parametrize("variant", ["hybrid", "rt", "eb"])
def test_hd_exec_is_double(exe, double_inputs, variant, tmp_path):
    """-is_double on the GPU (hd_solve_f64): the oracle's exact FP64 value, and
    the driver's own -check (the CPU early-break in double) agrees."""
    pa, pb, _, h_und = double_inputs
    out = tmp_path / "run.json"
    r = subprocess.run([exe, "-input1", pa, "-input2", pb, "-input_type", "wkt", "-n_dims", "3",
                        "-variant", variant, "-is_double", "-undirected", "-repeat", "2",
                        "-json", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("HausdorffDistance: distance")][0]
    assert float(line.split()[-1]) == h_und
    js = json.loads(out.read_text())
    assert js["HDResult"] == h_und and js["Check"]["Pass"] is True


def test_bad_flags_rejected(exe):
    c = GOLDEN[0]
    base = [exe, "-input1", os.path.join(HERE, "golden", c["a"]), "-input2",
            os.path.join(HERE, "golden", c["b"]), "-n_dims", str(c["dims"])]
    r = subprocess.run(base + ["-input_type", "bin", "-execution", "tpu"], capture_output=True,
                       text=True)
    assert r.returncode == 1 and "Unknown execution" in r.stderr
    r = subprocess.run(base + ["-input_type", "shp"], capture_output=True, text=True)
    assert r.returncode == 1 and "Unsupported input type" in r.stderr
    r = subprocess.run(base + ["-input_type", "bin", "-variant", "itk"], capture_output=True, text=True)
    assert r.returncode == 1 and "variant" in r.stderr


@pytest.mark.parametrize("style", [
    ["-input_type", "bin", "-seed", "{seed}", "-parallelism", "1", "-execution", "cpu"],
    ["--input_type=bin", "--seed={seed}", "-parallelism=1", "--execution", "cpu"],
    ["-input_type=BIN", "-seed", "{seed}", "--parallelism", "1", "-execution=CPU", "-nocheck"],
    ["-input_type", "bin", "-seed={seed}", "-parallelism", "1", "-execution", "cpu",
     "-check=F", "-normalize=False", "-v=1", "-rt_prune=false"],
])
def test_cpu_execution_gflags_syntax(exe, tmp_path, style):
    """The reference's flags are gflags: -name value, -name=value,
    --name=value and -noboolflag all parse, and give the same run."""
    c = GOLDEN[1]
    out = tmp_path / "run.json"
    args = [a.format(seed=c["seed"]) for a in style]
    r = subprocess.run([exe, "-input1", os.path.join(HERE, "golden", c["a"]), "-input2",
                        os.path.join(HERE, "golden", c["b"]), "-n_dims", str(c["dims"]),
                        "-repeat", "1", "-json", str(out)] + args, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    st = json.load(open(out))
    assert bits(st["HDResult"]) == c["hd_bits"]
    assert st["Running"]["Repeats"][0]["ComparedPairs"] == c["compared_pairs_t1"]
    assert st["Running"]["Seed"] == c["seed"]


@pytest.mark.gpu
@pytest.mark.parametrize("variant", ["eb", "hybrid", "rt", "grid"])
@pytest.mark.parametrize("case", GOLDEN[:8], ids=[c["name"] for c in GOLDEN[:8]])
def test_hd_exec_matches_reference_golden(exe, tmp_path, case, variant):
    out = tmp_path / "run.json"
    r = subprocess.run([exe, "-input1", os.path.join(HERE, "golden", case["a"]),
                        "-input2", os.path.join(HERE, "golden", case["b"]), "-input_type", "bin",
                        "-n_dims", str(case["dims"]), "-variant", variant, "-repeat", "2",
                        "-json", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("HausdorffDistance: distance is")][0]
    assert bits(float(line.split()[-1])) == case["hd_bits"]
    assert "Time:" in r.stdout and "HausdorffDistance is checked" in r.stdout
    js = json.loads(out.read_text())
    assert js["Check"]["Pass"] is True
    assert len(js["Running"]["Repeats"]) == 2
    for rep in js["Running"]["Repeats"]:
        assert {"Algorithm", "Execution", "ReportedTime"} <= set(rep)
    assert js["Input"]["Files"][0]["NumPoints"] == case["n_a"]


@pytest.mark.gpu
def test_hd_exec_undirected(exe):
    c = [g for g in GOLDEN if g["name"] == "uniform2d_3k_ab"][0]
    d = [g for g in GOLDEN if g["name"] == "uniform2d_3k_ba"][0]
    r = subprocess.run([exe, "-input1", os.path.join(HERE, "golden", c["a"]), "-input2",
                        os.path.join(HERE, "golden", c["b"]), "-input_type", "bin", "-n_dims", "2",
                        "-variant", "hybrid", "-undirected", "-repeat", "1"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("HausdorffDistance")][0]
    assert bits(float(line.split()[-1])) == max(c["hd_bits"], d["hd_bits"])


def build_seam_probe(tmp_path):
    from hausdorffdistance_gb300 import build
    build.build_lib()
    probe = str(tmp_path / "seam_probe")
    r = subprocess.run(["g++", "-std=c++17", "-O1", f"-I{os.path.join(ROOT, 'include')}",
                        f"-I{os.path.join(ROOT, 'hausdorffdistance_gb300', 'host')}",
                        os.path.join(HERE, "seam_probe.cpp"), "-o", probe, f"-L{BUILD}",
                        "-lhdgpu", f"-Wl,-rpath,{BUILD}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return probe


def test_cpp_seam_mirror_compiles(tmp_path):
    """The C++ seam mirror and the driver's loaders compile and link against
    libhdgpu.so (no GPU needed)."""
    assert os.path.exists(build_seam_probe(tmp_path))


@pytest.mark.gpu
def test_cpp_seam_mirror(tmp_path):
    probe = build_seam_probe(tmp_path)
    c = [g for g in GOLDEN if g["name"] == "clusters3d_4k_ab"][0]
    r = subprocess.run([probe, os.path.join(HERE, "golden", c["a"]),
                        os.path.join(HERE, "golden", c["b"])], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.splitlines()
    assert all(bits(float(x)) == c["hd_bits"] for x in lines[0].split())
    stats = json.loads(lines[1])
    assert stats["Execution"] == "GPU" and stats["Algorithm"] == "LBVH" and stats["ReportedTime"] > 0
    assert lines[2] == "error 1"
    # The double instantiation: the oracle's exact FP64 max-min.
    import hd_oracle
    a = np.fromfile(os.path.join(HERE, "golden", c["a"]), dtype=np.float32, offset=8).reshape(-1, 3)
    b = np.fromfile(os.path.join(HERE, "golden", c["b"]), dtype=np.float32, offset=8).reshape(-1, 3)
    assert float(lines[3]) == float(np.sqrt(hd_oracle.exact_f64(a.astype(np.float64),
                                                                b.astype(np.float64))[0]))
