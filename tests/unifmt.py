"""A small independent writer/reader of the reference's .uni grid files
(source/fileio.cpp:38-44, 612-651, 834-880): a gzip stream with a 4-byte tag
(MNT2 3D, M4T2 4D), the 288-byte UniHeader {int dimX, dimY, dimZ, gridType,
elementType, bytesPerElement; char info[256]; uint64 timestamp}, for 4D an
int32 t extent, then float32 cells x fastest, one t slice after the other.
Used to check the library's C++ reader and writer against the layout."""
import gzip
import struct

import numpy as np

HEADER = struct.Struct("<6i256sQ")
assert HEADER.size == 288


def write(path, a, is4d, grid_type=None, info=b"unifmt test writer"):
    a = np.ascontiguousarray(a, dtype=np.float32)
    vec = a.ndim == (5 if is4d else 4)
    if is4d:
        t, z, y, x = a.shape[:4]
    else:
        z, y, x = a.shape[:3]
    nc = 4 if vec else 1
    gt = grid_type if grid_type is not None else (8 if vec else 1)
    with gzip.open(path, "wb", compresslevel=1) as f:
        f.write(b"M4T2" if is4d else b"MNT2")
        f.write(HEADER.pack(x, y, z, gt, 2 if vec else 1, 4 * nc, info, 1234567))
        if is4d:
            f.write(struct.pack("<i", t))
        f.write(a.tobytes())


def read(path):
    with gzip.open(path, "rb") as f:
        tag = f.read(4)
        x, y, z, gt, et, bpe, info, ts = HEADER.unpack(f.read(288))
        t = struct.unpack("<i", f.read(4))[0] if tag == b"M4T2" else None
        data = np.frombuffer(f.read(), dtype=np.float32)
    nc = bpe // 4
    shape = ((t,) if t is not None else ()) + (z, y, x) + ((nc,) if nc > 1 else ())
    return {"tag": tag, "dims": (x, y, z, t if t is not None else 1), "gridType": gt,
            "elementType": et, "bytesPerElement": bpe, "info": info.rstrip(b"\0"),
            "data": data.reshape(shape)}
