"""hd_exec's loaders (hausdorffdistance_gb300/host/loaders.h) on small files of
every supported format, through a tiny C++ probe (no GPU needed)."""
import os
import struct
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HOST = os.path.join(ROOT, "hausdorffdistance_gb300", "host")


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("probe") / "loader_probe")
    subprocess.run(["g++", "-std=c++17", "-O1", f"-I{HOST}",
                    os.path.join(ROOT, "tests", "loader_probe.cpp"), "-o", out], check=True)
    return out


def run(probe, path, typ, dims, limit=1 << 30, normalize=0, translate=None):
    args = [probe, str(path), typ, str(dims), str(limit), str(normalize)]
    if translate is not None:
        args.append(str(translate))
    r = subprocess.run(args, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stderr)
    lines = r.stdout.split("\n")
    n = int(lines[0])
    return np.array([[float(x) for x in ln.split()] for ln in lines[1:1 + n]]).reshape(n, dims)


def test_wkt_geometries(probe, tmp_path):
    p = tmp_path / "g.wkt"
    p.write_text("POINT (1 2)\n"
                 "LINESTRING (0 0, 1 1, 2 0.5)\n"
                 "POLYGON ((0 0, 4 0, 4 4, 0 0), (1 1, 2 1, 1 2, 1 1))\n"
                 "MULTIPOLYGON (((10 10, 11 10, 10 11, 10 10)), ((20 20, 21 20, 20 21, 20 20), (5 5, 6 6, 5 6, 5 5)))\n"
                 "MULTILINESTRING ((7 7, 8 8), (9 9, -1e1 3.5))\n"
                 "GEOMETRYCOLLECTION (POINT (100 100))\n")
    got = run(probe, p, "wkt", 2)
    want = [[1, 2], [0, 0], [1, 1], [2, 0.5], [0, 0], [4, 0], [4, 4], [0, 0],
            [10, 10], [11, 10], [10, 11], [10, 10], [20, 20], [21, 20], [20, 21], [20, 20],
            [7, 7], [8, 8], [9, 9], [-10, 3.5]]
    assert np.array_equal(got, np.array(want, float))
    assert len(run(probe, p, "wkt", 2, limit=5)) == 5


def test_off(probe, tmp_path):
    p = tmp_path / "m.off"
    p.write_text("OFF\n4 1 0\n0 0 0\n1 0 0\n0 1 0.5\n0 0 1\n3 0 1 2\n")
    assert np.array_equal(run(probe, p, "off", 3), [[0, 0, 0], [1, 0, 0], [0, 1, 0.5], [0, 0, 1]])
    q = tmp_path / "n.off"
    q.write_text("OFF 2 0 0\n5 6 7\n8 9 10\n")
    assert np.array_equal(run(probe, q, "off", 3), [[5, 6, 7], [8, 9, 10]])


@pytest.mark.parametrize("fmt", ["ascii", "binary_little_endian", "binary_big_endian"])
def test_ply_shifted_to_min(probe, tmp_path, fmt):
    v = np.array([[1.5, 2.0, -3.0], [4.0, 2.5, -1.0], [2.0, 7.0, 0.0]])
    p = tmp_path / "v.ply"
    head = (f"ply\nformat {fmt} 1.0\nelement vertex 3\nproperty float x\nproperty float y\n"
            "property float z\nproperty uchar red\nelement face 1\n"
            "property list uchar int vertex_indices\nend_header\n")
    if fmt == "ascii":
        body = "".join(f"{a} {b} {c} 7\n" for a, b, c in v) + "3 0 1 2\n"
        p.write_bytes(head.encode() + body.encode())
    else:
        e = "<" if fmt == "binary_little_endian" else ">"
        body = b"".join(struct.pack(e + "fffB", *row, 7) for row in v)
        body += struct.pack(e + "Biii", 3, 0, 1, 2)
        p.write_bytes(head.encode() + body)
    got = run(probe, p, "ply", 3)
    assert np.allclose(got, v - v.min(0))


def test_bin_normalize_translate(probe, tmp_path):
    pts = np.array([[0, 0], [2, 1], [4, 3]], np.float32)
    p = tmp_path / "x.bin"
    with open(p, "wb") as f:
        f.write(np.uint64(3).tobytes())
        f.write(pts.tobytes())
    assert np.array_equal(run(probe, p, "bin", 2), pts)
    assert np.allclose(run(probe, p, "bin", 2, normalize=1), pts / 4.0)
    assert np.allclose(run(probe, p, "bin", 2, translate=0.5)[:, 0], pts[:, 0] + 2.0)


def test_bad_inputs(probe, tmp_path):
    p = tmp_path / "bad.wkt"
    p.write_text("CIRCLE (1 2 3)\n")
    with pytest.raises(RuntimeError):
        run(probe, p, "wkt", 2)
    with pytest.raises(RuntimeError):
        run(probe, tmp_path / "missing.off", "off", 3)
