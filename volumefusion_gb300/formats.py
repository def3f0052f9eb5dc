"""The reference's on-disk formats from host arrays (afx_save_ply, afx_tsdf_save / afx_tsdf_load)."""
import ctypes as C

import numpy as np

from ._lib import check, lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def save_ply(path, vertices, faces, colors=None):
    """Mesh::savePly: vertices (N, 3) float32, faces (F, 3) int32, colors (N, 3) uint8 or None."""
    v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
    f = np.ascontiguousarray(faces, np.int32).reshape(-1, 3)
    c = None if colors is None else np.ascontiguousarray(colors, np.uint8).reshape(-1, 3)
    check(lib().afx_save_ply(str(path).encode(), _ptr(v), len(v), None if c is None else _ptr(c), _ptr(f), len(f)),
          "afx_save_ply")


def save_tsdf(path, tsdf, weights, volume_size, voxel_size, delta):
    """TSDFVolume::save of a volume; tsdf/weights shaped (Z, Y, X) or flat with dims given by shape."""
    t = np.ascontiguousarray(tsdf, np.float32)
    w = np.ascontiguousarray(weights, np.float32)
    dims = np.array(t.shape[::-1] if t.ndim == 3 else (t.size, 1, 1), np.int32)
    size = np.ascontiguousarray(volume_size, np.float32)
    vs = np.ascontiguousarray(voxel_size, np.float32)
    check(lib().afx_tsdf_save(str(path).encode(), _ptr(dims), _ptr(size), _ptr(vs), C.c_float(delta), _ptr(t), _ptr(w)),
          "afx_tsdf_save")


def load_tsdf(path):
    """(tsdf, weights, dims, volume_size, voxel_size, delta) of a TSDFVolume file; arrays (Z, Y, X)."""
    dims = np.zeros(3, np.int32)
    size, vs = np.zeros(3, np.float32), np.zeros(3, np.float32)
    delta = C.c_float(0)
    p = str(path).encode()
    check(lib().afx_tsdf_load_header(p, _ptr(dims), _ptr(size), _ptr(vs), C.byref(delta)), "afx_tsdf_load_header")
    n = int(np.prod(dims))
    t, w = np.empty(n, np.float32), np.empty(n, np.float32)
    check(lib().afx_tsdf_load(p, _ptr(t), _ptr(w), n), "afx_tsdf_load")
    shape = tuple(int(x) for x in dims[::-1])
    return t.reshape(shape), w.reshape(shape), dims, size, vs, float(delta.value)


__all__ = ["save_ply", "save_tsdf", "load_tsdf"]
