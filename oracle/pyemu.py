"""ctypes bindings to oracle/_ref/libvfemu.so: the reference's own CUDA kernels (src/*.cu)
executed on the host by the emulation runtime in oracle/ref_emu.  Test infrastructure only: it
pins the CPU oracle for the stages the reference has only as GPU code.  The library exists only
where the reference source tree is present (``python oracle/ref_emu/build_emu.py``); tests skip
without it and fall back to the committed fixtures.

Array conventions follow oracle/pyoracle.py: float32 row-major arrays, 3x3 matrices passed
column-major (Eigen layout), 4x4 transforms as column-major float[16] rows.
"""
import ctypes as C
import os

import numpy as np

from . import pyoracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_ref", "libvfemu.so")
_lib = None


def available():
    return os.path.exists(LIB)


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(LIB)
        for name in ("emu_correspondences",):
            getattr(L, name).restype = C.c_long
        for name in ("emu_mc_points", "emu_mc_full"):
            getattr(L, name).restype = C.c_uint
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


def knn_k():
    return lib().emu_knn_k()


def kreg():
    return lib().emu_kreg()


def filter_depth(depth, thr):
    d = _f32(depth).copy()
    lib().emu_filter_depth(_p(d), C.c_uint(d.size), C.c_float(thr))
    return d


def bilateral(depth, r, sigma_i, sigma_s, thr):
    d = _f32(depth)
    h, w = d.shape
    out = np.zeros_like(d)
    lib().emu_bilateral(_p(out), _p(d), h, w, r, C.c_double(sigma_i), C.c_double(sigma_s), C.c_float(thr))
    return out


def depth_to_mesh(depth, K):
    d = _f32(depth)
    h, w = d.shape
    out = np.zeros((h, w, 3), np.float32)
    lib().emu_depth_to_mesh(_p(out), _p(d), w, h, _p(O.kcol(K)))
    return out


def normals(verts, depth, lo, hi):
    """Returns (normals, vertices-after): the reference kernel also writes the vertex image."""
    v = _f32(verts).copy()
    d = _f32(depth)
    h, w = d.shape
    n = np.zeros_like(v)
    lib().emu_normals(_p(n), _p(v), _p(d), h, w, C.c_float(lo), C.c_float(hi))
    return n, v


def remove_without_normals(normals_, verts, depth):
    n = _f32(normals_).copy()
    v = _f32(verts).copy()
    d = _f32(depth).copy()
    h, w = d.shape
    lib().emu_remove(_p(n), _p(v), _p(d), h, w)
    return n, v, d


def integrate_rigid(tsdf, weights, depth, delta, dims, voxel_size, volume_size, R, t, K):
    h, w = depth.shape
    lib().emu_integrate_rigid(_p(tsdf), _p(weights), _p(_f32(depth)), w, h, C.c_float(delta), _p(_i32(dims)),
                              _p(_f32(voxel_size)), _p(_f32(volume_size)), _p(O.kcol(R)), _p(_f32(t)), _p(O.kcol(K)))


def warp_weights(radii, idx, dist):
    idx = _u32(idx)
    w = np.zeros(idx.shape, np.float32)
    lib().emu_warp_weights(_p(w), _p(_f32(radii)), _p(idx), _p(_f32(dist)), C.c_long(idx.shape[0]))
    return w


def warp(pts, transforms, idx, w):
    out = np.zeros((len(pts), 3), np.float32)
    lib().emu_warp(_p(out), _p(_f32(pts)), _p(_f32(transforms)), _p(_u32(idx)), _p(_f32(w)), C.c_long(len(pts)))
    return out


def correspondences(warped, K, depth, frame_mesh, thr):
    h, w = depth.shape
    m = len(warped)
    corr = np.zeros((max(m, 1), 2), np.int32)
    n = lib().emu_correspondences(_p(corr), _p(_f32(warped)), C.c_long(m), _p(O.kcol(K)), _p(_f32(depth)), h, w,
                                  _p(_f32(frame_mesh)), C.c_float(thr))
    return corr[:n].copy()


def gn_assemble(corr, canon, midx, mw, normals_, frame, warped, nodes, transforms, gidx, lam_d, lam_r):
    """Dense J^T J (6n x 6n), J^T r and the residual vector as the reference's
    MotionOptimization kernels build them (src/VolumeFusion.cu:454-646)."""
    n = len(nodes)
    C_ = len(corr)
    W = 6 * n
    jtj = np.zeros((W, W), np.float32)
    jtr = np.zeros(W, np.float32)
    r = np.zeros(C_ + 3 * kreg() * n, np.float32)
    lib().emu_gn_assemble(_p(jtj), _p(jtr), _p(r), _p(_i32(corr)), C.c_uint(C_), _p(_f32(canon)), _p(_u32(midx)),
                          _p(_f32(mw)), _p(_f32(normals_)), _p(_f32(frame)), _p(_f32(warped)), _p(_f32(nodes)),
                          _p(_f32(transforms)), C.c_uint(n), _p(_u32(gidx)), C.c_float(lam_d), C.c_float(lam_r))
    return jtj, jtr, r


def update_transforms(transforms, x):
    T = _f32(transforms).copy()
    lib().emu_update_transforms(_p(T), _p(_f32(x)), C.c_uint(len(T)))
    return T


def tsdf_knn(nodes, radii, voxel_size, volume_size, dims, per_node):
    S = int(np.prod(dims))
    k = knn_k()
    kidx = np.zeros((S, k), np.uint32)
    kdist = np.zeros((S, k), np.float32)
    kcount = np.zeros(S, np.int32)
    lib().emu_tsdf_knn(_p(kidx), _p(kdist), _p(kcount), _p(_f32(nodes)), _p(_f32(radii)), C.c_uint(len(nodes)),
                       _p(_f32(voxel_size)), _p(_f32(volume_size)), _p(_i32(dims)), _p(_i32(per_node)))
    return kidx, kdist, kcount


def tsdf_weights(radii, kidx, kdist, kcount):
    kw = np.zeros(kidx.shape, np.float32)
    lib().emu_tsdf_weights(_p(kw), _p(_f32(radii)), _p(_u32(kidx)), _p(_f32(kdist)), _p(_i32(kcount)),
                           C.c_long(kidx.shape[0]))
    return kw


def tsdf_vertices(voxel_size, volume_size, dims):
    S = int(np.prod(dims))
    v = np.zeros((S, 3), np.float32)
    lib().emu_tsdf_vertices(_p(v), _p(_f32(voxel_size)), _p(_f32(volume_size)), _p(_i32(dims)))
    return v


def translate(pts, t):
    p = _f32(pts).copy()
    lib().emu_translate(_p(p), C.c_uint(len(p)), _p(_f32(t)))
    return p


def warp_tsdf(verts, transforms, kidx, kw, kcount, voxel_size, volume_size, dims):
    v = _f32(verts).copy()
    lib().emu_warp_tsdf(_p(v), _p(_f32(transforms)), _p(_u32(kidx)), _p(_f32(kw)), _p(_i32(kcount)),
                        _p(_f32(voxel_size)), _p(_f32(volume_size)), _p(_i32(dims)))
    return v


def count_collisions(verts, kcount, voxel_size, volume_size, dims, Rinv, t):
    S = int(np.prod(dims))
    c = np.zeros(S, np.int32)
    lib().emu_count_collisions(_p(c), _p(_f32(verts)), _p(_i32(kcount)), _p(_f32(voxel_size)),
                               _p(_f32(volume_size)), _p(_i32(dims)), _p(O.kcol(Rinv)), _p(_f32(t)))
    return c


def integrate_warped(tsdf, weights, verts, collisions, kcount, depth, delta, voxel_size, volume_size, dims, Rinv, t,
                     K):
    h, w = depth.shape
    lib().emu_integrate_warped(_p(tsdf), _p(weights), _p(_f32(verts)), _p(_i32(collisions)), _p(_i32(kcount)),
                               _p(_f32(depth)), w, h, C.c_float(delta), _p(_f32(voxel_size)), _p(_f32(volume_size)),
                               _p(_i32(dims)), _p(O.kcol(Rinv)), _p(_f32(t)), _p(O.kcol(K)))


def mc_points(tsdf, weights, dims, voxel_size, volume_size, cap=None):
    cap = cap or max(1, int(np.prod(dims)) * 3)
    out = np.zeros((cap, 3), np.float32)
    n = lib().emu_mc_points(_p(out), _p(_f32(tsdf)), _p(_f32(weights)), _p(_i32(dims)), _p(_f32(voxel_size)),
                            _p(_f32(volume_size)))
    return out[:n].copy()


def mc_full(tsdf, weights, dims, voxel_size, volume_size, cap=None):
    cap = cap or max(3, int(np.prod(dims)) * 3)
    verts = np.zeros((cap, 3), np.float32)
    faces = np.zeros((cap, 3), np.int32)
    nf = C.c_uint(0)
    nv = lib().emu_mc_full(_p(verts), _p(faces), C.byref(nf), _p(_f32(tsdf)), _p(_f32(weights)), _p(_i32(dims)),
                           _p(_f32(voxel_size)), _p(_f32(volume_size)))
    return verts[:nv].copy(), faces[:nf.value].copy()
