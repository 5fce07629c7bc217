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
    # -limit as the reference applies it (src/loaders/loader.h:38-96): the
    # count is tested after each vertex and only the innermost loop is left,
    # so each later ring or linestring still adds its first vertex.
    lim5 = [[1, 2], [0, 0], [1, 1], [2, 0.5], [0, 0], [10, 10], [20, 20], [7, 7], [9, 9]]
    assert np.array_equal(run(probe, p, "wkt", 2, limit=5), np.array(lim5, float))


def test_wkt_limit_stops_at_a_point_line(probe, tmp_path):
    """A POINT line that reaches the limit ends the file; polygons before it
    go on adding one vertex per ring."""
    p = tmp_path / "l.wkt"
    p.write_text("POLYGON ((0 0, 1 0, 1 1, 0 0))\n"
                 "POLYGON ((5 5, 6 5, 6 6, 5 5))\n"
                 "POINT (9 9)\n"
                 "POINT (8 8)\n"
                 "LINESTRING (3 3, 4 4)\n")
    assert np.array_equal(run(probe, p, "wkt", 2, limit=2), [[0, 0], [1, 0], [5, 5], [9, 9]])
    assert np.array_equal(run(probe, p, "wkt", 2, limit=7),
                          [[0, 0], [1, 0], [1, 1], [0, 0], [5, 5], [6, 5], [6, 6]] + [[9, 9]])


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


# Image inputs (-input_type image): NIfTI-1 and MetaImage read without ITK.
from image_files import image_points, write_meta, write_nifti  # noqa: E402


def test_nifti_uint8_mask(probe, tmp_path):
    rng = np.random.default_rng(3)
    vol = ((rng.random((5, 6, 7)) < 0.3) * rng.integers(1, 256, (5, 6, 7))).astype(np.uint8)
    p = tmp_path / "m.nii"
    write_nifti(p, vol)
    got = run(probe, p, "image", 3)
    assert len(got) == np.count_nonzero(vol)
    assert np.array_equal(got, image_points(vol, 3))
    # -limit keeps the first points in index order (x fastest).
    assert np.array_equal(run(probe, p, "image", 3, limit=10), image_points(vol, 3, limit=10))


def test_nifti_int16_low_byte_big_endian(probe, tmp_path):
    """Values reach the unsigned-char image through a static_cast: 256, 512
    and -256 have a zero low byte and give no point; 300 and -1 do."""
    vol = np.array([[[0, 256, 300, -1], [512, -256, 1, 255]]], np.int16)
    p = tmp_path / "be.nii"
    write_nifti(p, vol, big_endian=True)
    got = run(probe, p, "image", 3)
    assert np.array_equal(got, [[2, 0, 0], [3, 0, 0], [2, 1, 0], [3, 1, 0]])
    assert np.array_equal(got, image_points(vol, 3))


@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int16, np.uint16, np.int32])
def test_nifti_rescaled(probe, tmp_path, dtype):
    """scl_slope / scl_inter applied before the conversion (in float for all
    but double data), reals truncated toward zero."""
    rng = np.random.default_rng(5)
    if np.dtype(dtype).kind == "f":
        vol = (rng.random((3, 4, 5)) * 300 - 20).astype(dtype)
        vol.reshape(-1)[:4] = [0.5, 0.4, 1.0, 128.5]
    else:
        vol = rng.integers(0, 400, (3, 4, 5)).astype(dtype)
    p = tmp_path / "s.nii"
    write_nifti(p, vol, slope=2.0, inter=-1.0)
    got = run(probe, p, "image", 3)
    assert np.array_equal(got, image_points(vol, 3, slope=2.0, inter=-1.0))
    # Slope 1 and intercept 0 is no rescale.
    write_nifti(p, vol, slope=1.0, inter=0.0)
    assert np.array_equal(run(probe, p, "image", 3), image_points(vol, 3))


def test_image_dimensions(probe, tmp_path):
    rng = np.random.default_rng(6)
    flat = (rng.random((6, 9)) < 0.5).astype(np.uint8)
    p = tmp_path / "flat.nii"
    write_nifti(p, flat)
    got = run(probe, p, "image", 3)  # a 2-D image read as 3-D: k = 0
    assert np.array_equal(got, image_points(flat, 3)) and not got[:, 2].any()
    assert np.array_equal(run(probe, p, "image", 2), image_points(flat, 2))
    one = flat[None]  # 3-D with a single slice reads as 2-D
    q = tmp_path / "one.nii"
    write_nifti(q, one)
    assert np.array_equal(run(probe, q, "image", 2), image_points(flat, 2))
    thick = np.stack([flat, flat])
    r = tmp_path / "thick.nii"
    write_nifti(r, thick)
    with pytest.raises(RuntimeError, match="more than 2 dimensions"):
        run(probe, r, "image", 2)


@pytest.mark.parametrize("big_endian", [False, True])
def test_metaimage(probe, tmp_path, big_endian):
    rng = np.random.default_rng(7)
    vol = (rng.integers(-3, 3, (4, 5, 6)) * 128).astype(np.int16)
    p = tmp_path / "v.mha"
    write_meta(p, vol, big_endian=big_endian)
    assert np.array_equal(run(probe, p, "image", 3), image_points(vol, 3))
    fl = (rng.random((4, 5, 6)) * 3).astype(np.float32)
    q = tmp_path / "v.mhd"
    write_meta(q, fl, big_endian=big_endian, local=False, header_size=16,
               extra="ElementSpacing = 1 1 1\n")
    assert np.array_equal(run(probe, q, "image", 3), image_points(fl, 3))


def test_image_errors(probe, tmp_path):
    vol = np.ones((2, 3, 4), np.uint8)
    gz = tmp_path / "c.nii"
    gz.write_bytes(b"\x1f\x8b" + b"\0" * 400)
    with pytest.raises(RuntimeError, match="compressed"):
        run(probe, gz, "image", 3)
    cx = tmp_path / "cx.nii"
    write_nifti(cx, vol, datatype=32)  # complex64
    with pytest.raises(RuntimeError, match="datatype"):
        run(probe, cx, "image", 3)
    cm = tmp_path / "cm.mha"
    write_meta(cm, vol, extra="CompressedData = True\n")
    with pytest.raises(RuntimeError, match="compressed"):
        run(probe, cm, "image", 3)
    ch = tmp_path / "ch.mha"
    write_meta(ch, vol, extra="ElementNumberOfChannels = 3\n")
    with pytest.raises(RuntimeError, match="multi-channel"):
        run(probe, ch, "image", 3)
    png = tmp_path / "x.png"
    png.write_bytes(b"\x89PNG")
    with pytest.raises(RuntimeError, match="unsupported image format"):
        run(probe, png, "image", 2)
    short = tmp_path / "short.nii"
    write_nifti(short, vol)
    short.write_bytes(short.read_bytes()[:-5])
    with pytest.raises(RuntimeError, match="truncated"):
        run(probe, short, "image", 3)


def test_metaimage_oversized_header(probe, tmp_path):
    p = tmp_path / "huge.mha"
    p.write_bytes(b"NDims = 3\nDimSize = 100000 100000 100000\nElementType = MET_UCHAR\n"
                  b"ElementDataFile = LOCAL\n")
    with pytest.raises(RuntimeError, match="too large"):
        run(probe, p, "image", 3)


def test_translate_rounds_once_like_the_reference(probe, tmp_path):
    """-translate adds extent * ratio (a double) to each float coordinate and
    rounds the sum once, as the reference's `p += extent * ratio` does.  With
    extent 1 and ratio 2^-24 + 2^-49, x = 1 lands just above the halfway point
    to the next float: rounding the shift to float first would give 1.0."""
    pts = np.array([[0, 0], [1, 0]], np.float32)
    p = tmp_path / "t.bin"
    with open(p, "wb") as f:
        f.write(np.uint64(2).tobytes() + pts.tobytes())
    ratio = 2.0 ** -24 + 2.0 ** -49
    got = run(probe, p, "bin", 2, translate=repr(ratio))
    assert np.float32(got[1, 0]) == np.float32(1.0 + 2.0 ** -23)
    assert np.float32(got[0, 0]) == np.float32(ratio)


def test_wkt_parses_floats_directly(probe, tmp_path):
    """A coordinate just above the midpoint of two floats whose nearest double
    is the midpoint itself: parsed straight to float (as boost.geometry's
    reader does for float points) it rounds up; via double it would tie down."""
    p = tmp_path / "mid.wkt"
    p.write_text("POINT (1.00000005960464477539062500000000001 2)\n")
    assert float("1.00000005960464477539062500000000001") == 1.0 + 2.0 ** -24
    got = run(probe, p, "wkt", 2)
    assert np.float32(got[0, 0]) == np.float32(1.0 + 2.0 ** -23)


GOLDEN_JSON = os.path.join(ROOT, "tests", "golden", "golden.json")
PREP = __import__("json").load(open(GOLDEN_JSON)).get("preprocessing", [])


@pytest.mark.parametrize("rec", PREP, ids=[f"{r['input'].split('/')[-1][:-4]}-n{r['normalize']}-t{r['translate']}"
                                          for r in PREP])
def test_normalize_translate_match_the_reference(probe, rec):
    """-normalize and -translate give the float32 points the reference's own
    NormalizePoints / TranslatePoints give (golden hashes made by running
    them, built from the reference sources)."""
    import hashlib
    path = os.path.join(ROOT, "tests", "golden", rec["input"])
    got = run(probe, path, "bin", rec["dims"], normalize=rec["normalize"],
              translate=rec["translate"] if rec["translate"] != 0 else None)
    pts = np.ascontiguousarray(got, np.float32)
    assert len(pts) == rec["n"]
    assert hashlib.sha256(pts.tobytes()).hexdigest() == rec["sha256"]
