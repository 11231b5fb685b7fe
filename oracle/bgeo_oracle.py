"""Oracle of libmat's Houdini file writer (test infrastructure only).

Restates IO::GeometryWriter::OutputGeometry (src/IO/IO_CUDA/io_utils.cpp:106-231)
for the geometry save_convex_cells_houdini builds
(src/IO/IO_CUDA/io_cuda.cxx:156-187): the point attribute "P" alone and one
int primitive attribute "PrimAttr" (the polygon's site).  Everything is
big-endian:

  header   int 'Bgeo', char 'V', int 5, int points, int polygons, int 0
           (point groups), int 0 (primitive groups), int 0 (point
           attributes besides P), int 0 (vertex attributes), int 1
           (primitive attributes), int 0 (detail attributes)
  points   x, y, z, 1.0 as floats
  PrimAttr short 8, the name, unsigned short 1, int 1 (integer), int 0
           (default)
  polygons int 1, int vertex count, char '<', the point ids as 16-bit
           unsigned ints when there are at most 65536 points, else 32-bit,
           then the site as int
  footer   bytes 0x00, 0xff
"""
import numpy as np


def bgeo_bytes(points, poly_offsets, indices, poly_site):
    """The file image for a polygon soup: points (n, 3) float32,
    poly_offsets (m + 1) into indices, poly_site (m,)."""
    pts = np.asarray(points, np.float32).reshape(-1, 3)
    off = np.asarray(poly_offsets, np.int64)
    idx = np.asarray(indices, np.uint32)
    site = np.asarray(poly_site, np.int32)
    n_pts, n_polys = pts.shape[0], off.shape[0] - 1
    if n_pts == 0:
        raise ValueError("no points")  # the reference writer throws
    out = bytearray(b"Bgeo")
    out += b"V"
    out += np.array([5, n_pts, n_polys, 0, 0, 0, 0, 1, 0], ">i4").tobytes()
    out += np.concatenate([pts, np.ones((n_pts, 1), np.float32)], axis=1).astype(">f4").tobytes()
    out += np.array([8], ">i2").tobytes() + b"PrimAttr"
    out += np.array([1], ">u2").tobytes() + np.array([1, 0], ">i4").tobytes()
    it = ">u4" if n_pts > (1 << 16) else ">u2"
    for i in range(n_polys):
        a, b = int(off[i]), int(off[i + 1])
        out += np.array([1, b - a], ">i4").tobytes() + b"<"
        out += idx[a:b].astype(it).tobytes()
        out += np.array([site[i]], ">i4").tobytes()
    out += b"\x00\xff"
    return bytes(out)


def ref_bgeo_bytes(points, poly_offsets, indices, poly_site, folder):
    """The same file written by libmat's own GeometryWriter
    (oracle/_ref/librefbgeo.so, built from the reference's sources when they
    are present), or None without them.  folder: a scratch directory."""
    import ctypes
    import os
    from . import build
    path = build.build_ref_bgeo()
    if path is None:
        return None
    lib = ctypes.CDLL(path)
    lib.ref_write_bgeo.restype = ctypes.c_int
    vp = ctypes.c_void_p
    lib.ref_write_bgeo.argtypes = [ctypes.c_char_p, ctypes.c_char_p, vp, ctypes.c_longlong, vp, vp,
                                   ctypes.c_longlong, vp]
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
    off = np.ascontiguousarray(poly_offsets, np.int64)
    idx = np.ascontiguousarray(np.asarray(indices, np.uint32).reshape(-1) if len(indices) else
                               np.zeros(1, np.uint32))
    site = np.ascontiguousarray(poly_site, np.int32) if len(poly_site) else np.zeros(1, np.int32)
    p = lambda a: a.ctypes.data_as(vp)  # noqa: E731
    if lib.ref_write_bgeo(str(folder).encode(), b"ref", p(pts), pts.shape[0], p(off), p(idx),
                          off.shape[0] - 1, p(site)) != 0:
        raise RuntimeError("the reference writer failed")
    with open(os.path.join(str(folder), "ref.bgeo"), "rb") as f:
        return f.read()
