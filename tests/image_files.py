"""Small NIfTI-1 and MetaImage writers for the image-loader tests, and the
point set an image gives under the reference's image loader
(src/loaders/img_loader.h:13-63): every voxel whose value, converted to
unsigned char as ITK's reader converts pixel buffers (a static_cast), is
non-zero becomes the point of its index, index 0 fastest."""
import os
import struct

import numpy as np

NIFTI_CODES = {np.uint8: 2, np.int16: 4, np.int32: 8, np.float32: 16, np.float64: 64,
               np.int8: 256, np.uint16: 512, np.uint32: 768, np.int64: 1024, np.uint64: 1280}
MET_TYPES = {np.uint8: "MET_UCHAR", np.int8: "MET_CHAR", np.uint16: "MET_USHORT",
             np.int16: "MET_SHORT", np.uint32: "MET_UINT", np.int32: "MET_INT",
             np.uint64: "MET_ULONG_LONG", np.int64: "MET_LONG_LONG", np.float32: "MET_FLOAT",
             np.float64: "MET_DOUBLE"}


def _data(vol, big_endian):
    e = ">" if big_endian else "<"
    return np.ascontiguousarray(vol).astype(vol.dtype.newbyteorder(e)).tobytes()


def write_nifti(path, vol, big_endian=False, slope=0.0, inter=0.0, datatype=None):
    """A single-file NIfTI-1 image of `vol`, indexed [k, j, i] (or [j, i]):
    the last numpy axis is the file's fastest one (dim[1])."""
    e = ">" if big_endian else "<"
    dims = vol.shape[::-1]
    h = bytearray(348)
    struct.pack_into(e + "i", h, 0, 348)
    struct.pack_into(e + "8h", h, 40, len(dims), *dims, *([1] * (7 - len(dims))))
    code = datatype if datatype is not None else NIFTI_CODES[vol.dtype.type]
    struct.pack_into(e + "hh", h, 70, code, vol.dtype.itemsize * 8)
    struct.pack_into(e + "8f", h, 76, *([1.0] * 8))
    struct.pack_into(e + "fff", h, 108, 352.0, slope, inter)
    h[344:348] = b"n+1\0"
    with open(path, "wb") as f:
        f.write(bytes(h) + b"\0" * 4 + _data(vol, big_endian))


def write_meta(path, vol, big_endian=False, local=True, header_size=0, extra=""):
    """A MetaImage header at `path`; the voxels follow it (LOCAL, .mha) or sit
    in <path>.raw beside it, after `header_size` filler bytes."""
    dims = vol.shape[::-1]
    raw_name = os.path.basename(path) + ".raw"
    hdr = (f"ObjectType = Image\nNDims = {len(dims)}\nBinaryData = True\n"
           f"BinaryDataByteOrderMSB = {'True' if big_endian else 'False'}\n{extra}"
           f"DimSize = {' '.join(map(str, dims))}\n"
           f"ElementType = {MET_TYPES[vol.dtype.type]}\n"
           + (f"HeaderSize = {header_size}\n" if header_size else "")
           + f"ElementDataFile = {'LOCAL' if local else raw_name}\n").encode()
    body = b"\x07" * header_size + _data(vol, big_endian)
    if local:
        with open(path, "wb") as f:
            f.write(hdr + body)
    else:
        with open(path, "wb") as f:
            f.write(hdr)
        with open(os.path.join(os.path.dirname(path), raw_name), "wb") as f:
            f.write(body)


def _real_to_byte(r):
    ok = (r > -2147483649.0) & (r < 2147483648.0)
    return np.where(ok, np.trunc(np.where(ok, r, 0.0)), 0.0).astype(np.int64) & 0xFF


def voxel_bytes(vol, slope=0.0, inter=0.0):
    """Every voxel (index 0 fastest) as the unsigned char the loader sees."""
    v = np.ascontiguousarray(vol).reshape(-1)
    s, t = np.float32(slope), np.float32(inter)
    if s != 0 and (s != 1 or t != 0):
        if v.dtype == np.float64:
            return _real_to_byte(v * np.float64(s) + np.float64(t))
        r = v.astype(np.float32).astype(np.float64) * np.float64(s) + np.float64(t)
        return _real_to_byte(r.astype(np.float32).astype(np.float64))
    if v.dtype.kind == "f":
        return _real_to_byte(v.astype(np.float64))
    return v.astype(np.int64) & 0xFF


def image_points(vol, dims, limit=None, slope=0.0, inter=0.0):
    """The loader's points of `vol` as float64 rows (index 0 fastest)."""
    f = np.nonzero(voxel_bytes(vol, slope, inter))[0]
    if limit is not None:
        f = f[:limit]
    shape = vol.shape[::-1] + (1,) * (3 - vol.ndim)
    nx, ny = shape[0], shape[1]
    cols = [f % nx, (f // nx) % ny, f // (nx * ny)]
    return np.stack([c.astype(np.float64) for c in cols[:dims]]
                    + [np.zeros(len(f))] * max(0, dims - 3), 1)
