"""ctypes bindings for the CPU oracle (oracle/liboracle.so).

Test infrastructure only: imported by tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg, never by the volumefusion_gb300 package.  Functions take and return
numpy arrays in the reference's layouts (see vf_oracle.h).
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
LIB64_PATH = os.path.join(HERE, "liboracle64.so")

f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
u16p = np.ctypeslib.ndpointer(np.uint16, flags="C_CONTIGUOUS")
INVALID = 0xFFFFFFFF


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        sig = {
            "vfo_expf": (C.c_float, [C.c_float]),
            "vfo_set_threads": (None, [C.c_int]),
            "vfo_threads": (C.c_int, []),
            "vfo_f2i_rz": (C.c_int, [C.c_float]),
            "vfo_depth_from_mm": (None, [u16p, C.c_long, f32p]),
            "vfo_filter_depth": (None, [f32p, C.c_long, C.c_float]),
            "vfo_bilateral": (None, [f32p, f32p, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_float]),
            "vfo_depth_to_mesh": (None, [f32p, f32p, C.c_int, C.c_int, f32p]),
            "vfo_normals": (None, [f32p, f32p, C.c_int, C.c_int, C.c_float, C.c_float]),
            "vfo_remove_without_normals": (None, [f32p, f32p, f32p, C.c_int, C.c_int]),
            "vfo_centroid": (None, [f32p, C.c_long, f32p]),
            "vfo_frame_prep": (None, [u16p, C.c_int, C.c_int, f32p, C.c_float, C.c_int, C.c_int, C.c_double,
                                      C.c_double, C.c_float, C.c_float, C.c_float, f32p, f32p, f32p, f32p]),
            "vfo_integrate_rigid": (None, [f32p, f32p, f32p, C.c_int, C.c_int, C.c_float, i32p, f32p, f32p, f32p,
                                           f32p, f32p, C.c_int]),
            "vfo_round_half": (C.c_float, [C.c_float]),
            "vfo_mc_pointcloud": (C.c_long, [f32p, f32p, i32p, f32p, f32p, C.c_float, f32p, C.c_long]),
            "vfo_sort_unique_vec3": (C.c_long, [f32p, C.c_long]),
            "vfo_transform_points": (None, [f32p, C.c_long, f32p]),
            "vfo_mc_full": (C.c_long, [f32p, f32p, i32p, f32p, f32p, C.c_float, f32p, C.c_long, i32p, C.c_long,
                                       C.POINTER(C.c_long)]),
            "vfo_translate": (None, [f32p, C.c_long, f32p]),
            "vfo_build_graph": (C.c_int, [f32p, f32p, f32p, C.c_int, C.c_int, f32p, C.c_long, C.c_int, C.c_float]),
            "vfo_knn": (None, [f32p, C.c_int, f32p, C.c_long, C.c_int, C.c_int, u32p, f32p]),
            "vfo_filter_disconnected": (None, [u32p, f32p, C.c_int, C.c_int, f32p]),
            "vfo_warp_weights": (None, [f32p, f32p, u32p, f32p, C.c_long, C.c_int, C.c_int]),
            "vfo_warp": (None, [f32p, f32p, C.c_long, f32p, u32p, f32p, C.c_int]),
            "vfo_warp_dqb": (None, [f32p, f32p, C.c_long, f32p, u32p, f32p, C.c_int]),
            "vfo_correspondences": (C.c_long, [i32p, C.c_long, f32p, C.c_long, f32p, f32p, C.c_int, C.c_int, f32p,
                                               C.c_float]),
            "vfo_residual_depth": (None, [f32p, i32p, C.c_long, f32p, f32p, f32p, C.c_float]),
            "vfo_residual_reg": (None, [f32p, f32p, f32p, C.c_int, u32p, C.c_int, C.c_float]),
            "vfo_energy": (C.c_double, [f32p, C.c_long]),
            "vfo_assemble": (C.c_int, [C.c_void_p, C.c_void_p, f32p, i32p, C.c_long, f32p, u32p, f32p, C.c_int, f32p,
                                       C.c_float, f32p, C.c_int, u32p, C.c_int, C.c_float, f32p, f32p]),
            "vfo_solve_dense": (C.c_int, [f64p, f32p, C.c_int, f64p]),
            "vfo_pcg": (C.c_int, [f64p, f32p, C.c_int, C.c_int, C.c_double, f64p, C.POINTER(C.c_int)]),
            "vfo_update_transforms": (None, [f32p, f32p, C.c_int]),
            "vfo_tsdf_knn": (None, [u32p, f32p, i32p, f32p, f32p, C.c_int, f32p, f32p, i32p, i32p, C.c_int]),
            "vfo_tsdf_weights": (None, [f32p, f32p, u32p, f32p, i32p, C.c_long, C.c_int]),
            "vfo_tsdf_vertices": (None, [f32p, f32p, f32p, i32p]),
            "vfo_warp_tsdf": (None, [f32p, f32p, u32p, f32p, i32p, C.c_long, C.c_int]),
            "vfo_count_collisions": (None, [i32p, f32p, i32p, f32p, f32p, i32p, f32p, f32p]),
            "vfo_integrate_warped": (None, [f32p, f32p, f32p, i32p, i32p, f32p, C.c_int, C.c_int, C.c_float, f32p,
                                            f32p, i32p, f32p, f32p, f32p, C.c_int]),
            "vfo_undistort_map": (None, [u32p, C.c_int, C.c_int, f32p, f32p, C.c_int]),
            "vfo_undistort_depth": (None, [f32p, f32p, C.c_int, C.c_int, u32p, C.c_int]),
            "vfo_xy_lookup_table": (None, [f32p, C.c_int, C.c_int, f32p, f32p]),
            "vfo_bc_unproject": (None, [f32p, i32p, f32p, f32p, C.c_long, f32p, f32p]),
            "vfo_bc_project": (None, [f32p, i32p, f32p, C.c_long, f32p, f32p]),
            "vfo_frame_prep_undistorted": (None, [u16p, C.c_int, C.c_int, f32p, C.c_float, C.c_int, C.c_int,
                                                  C.c_double, C.c_double, C.c_float, C.c_float, C.c_float, u32p,
                                                  f32p, f32p, f32p, f32p]),
            "vfo_fusion_create": (C.c_void_p, [C.c_void_p]),
            "vfo_fusion_destroy": (None, [C.c_void_p]),
            "vfo_fusion_process": (C.c_int, [C.c_void_p, u16p]),
            "vfo_fusion_num_nodes": (C.c_int, [C.c_void_p]),
            "vfo_fusion_mesh_size": (C.c_long, [C.c_void_p]),
            "vfo_fusion_num_corr": (C.c_long, [C.c_void_p]),
            "vfo_fusion_gn_done": (C.c_int, [C.c_void_p]),
            "vfo_fusion_energy": (C.c_double, [C.c_void_p]),
            "vfo_fusion_tsdf": (C.c_void_p, [C.c_void_p]),
            "vfo_fusion_weights": (C.c_void_p, [C.c_void_p]),
            "vfo_fusion_nodes": (C.c_void_p, [C.c_void_p]),
            "vfo_fusion_transforms": (C.c_void_p, [C.c_void_p]),
            "vfo_fusion_centroid": (C.c_void_p, [C.c_void_p]),
            "vfo_fusion_mesh": (C.c_void_p, [C.c_void_p]),
            "vfo_fusion_set_transforms": (None, [C.c_void_p, f32p, C.c_int]),
            "vfo_fusion_set_tsdf": (None, [C.c_void_p, f32p, f32p]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


_lib64 = None


def lib64():
    """The FP64 oracle: the same restatement evaluated in binary64 (whole-frame driver only)."""
    global _lib64
    if _lib64 is None:
        if not os.path.exists(LIB64_PATH):
            build()
        L = C.CDLL(LIB64_PATH)
        vp = C.c_void_p
        sig = {
            "vfo_fusion_create": (vp, [vp]),
            "vfo_fusion_destroy": (None, [vp]),
            "vfo_fusion_process": (C.c_int, [vp, u16p]),
            "vfo_fusion_num_nodes": (C.c_int, [vp]),
            "vfo_fusion_mesh_size": (C.c_long, [vp]),
            "vfo_fusion_num_corr": (C.c_long, [vp]),
            "vfo_fusion_gn_done": (C.c_int, [vp]),
            "vfo_fusion_energy": (C.c_double, [vp]),
            "vfo_fusion_tsdf": (vp, [vp]),
            "vfo_fusion_weights": (vp, [vp]),
            "vfo_fusion_nodes": (vp, [vp]),
            "vfo_fusion_transforms": (vp, [vp]),
            "vfo_fusion_centroid": (vp, [vp]),
            "vfo_fusion_mesh": (vp, [vp]),
            "vfo_fusion_set_transforms": (None, [vp, f64p, C.c_int]),
            "vfo_fusion_set_tsdf": (None, [vp, f64p, f64p]),
            "vfo_mc_pointcloud": (C.c_long, [f64p, f64p, i32p, f64p, f64p, C.c_double, f64p, C.c_long]),
            "vfo_sort_unique_vec3": (C.c_long, [f64p, C.c_long]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib64 = L
    return _lib64


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def kcol(K):
    """3x3 numpy matrix -> column-major float32[9] (Eigen layout)."""
    return _f32(np.asarray(K, dtype=np.float64).T.ravel())


I3 = kcol(np.eye(3))


def set_threads(n):
    """OpenMP threads of the oracle's parallel loops for later calls from this thread (a launcher
    such as torchrun may have set OMP_NUM_THREADS=1 for its processes)."""
    lib().vfo_set_threads(int(n))


def threads():
    """OpenMP threads the oracle's parallel loops use now."""
    return int(lib().vfo_threads())


def expf(x):
    return lib().vfo_expf(float(x))


def depth_from_mm(mm):
    mm = np.ascontiguousarray(mm, dtype=np.uint16)
    out = np.empty(mm.shape, np.float32)
    lib().vfo_depth_from_mm(mm.ravel(), mm.size, out.ravel())
    return out


def filter_depth(depth, threshold):
    d = _f32(depth).copy()
    lib().vfo_filter_depth(d.ravel(), d.size, threshold)
    return d


def bilateral(depth, r, sigma_i, sigma_s, thr):
    d = _f32(depth)
    h, w = d.shape
    out = np.empty_like(d)
    lib().vfo_bilateral(out, d, h, w, r, sigma_i, sigma_s, thr)
    return out


def depth_to_mesh(depth, K):
    d = _f32(depth)
    h, w = d.shape
    out = np.empty((h, w, 3), np.float32)
    lib().vfo_depth_to_mesh(out, d, w, h, kcol(K))
    return out


def normals(vertices, angle_lo, angle_hi):
    v = _f32(vertices)
    h, w, _ = v.shape
    out = np.empty_like(v)
    lib().vfo_normals(out, v, h, w, angle_lo, angle_hi)
    return out


def frame_prep(mm, K, depth_threshold=1.2, bilateral=1, r=2, sigma_i=0.03, sigma_s=2.0, thr=0.09,
               angle_lo=1.3, angle_hi=2.1):
    mm = np.ascontiguousarray(mm, dtype=np.uint16)
    h, w = mm.shape
    depth = np.empty((h, w), np.float32)
    verts = np.empty((h, w, 3), np.float32)
    nrm = np.empty((h, w, 3), np.float32)
    cen = np.empty(3, np.float32)
    lib().vfo_frame_prep(mm, w, h, kcol(K), depth_threshold, int(bilateral), r, float(np.float32(sigma_i)),
                         float(np.float32(sigma_s)), thr, angle_lo, angle_hi, depth, verts, nrm, cen)
    return depth, verts, nrm, cen


def integrate_rigid(tsdf, weights, depth, delta, dims, voxel_size, volume_size, R, t, K, half=False):
    h, w = depth.shape
    lib().vfo_integrate_rigid(tsdf, weights, _f32(depth), w, h, delta, _i32(dims), _f32(voxel_size),
                              _f32(volume_size), kcol(R), _f32(t), kcol(K), int(half))


def mc_pointcloud(tsdf, weights, dims, voxel_size, volume_size, iso=0.0, cap=None):
    cap = cap or max(1, int(np.prod(dims)) * 3)
    out = np.empty((cap, 3), np.float32)
    n = lib().vfo_mc_pointcloud(_f32(tsdf), _f32(weights), _i32(dims), _f32(voxel_size), _f32(volume_size), iso,
                                out, cap)
    assert n <= cap
    return out[:n].copy()


def sort_unique(pts):
    p = _f32(pts).copy()
    n = lib().vfo_sort_unique_vec3(p, len(p))
    return p[:n].copy()


def mc_full(tsdf, weights, dims, voxel_size, volume_size, iso=0.0, cap=None):
    cap = cap or max(3, int(np.prod(dims)) * 3)
    verts = np.empty((cap, 3), np.float32)
    faces = np.empty((cap, 3), np.int32)
    nf = C.c_long(0)
    nv = lib().vfo_mc_full(_f32(tsdf), _f32(weights), _i32(dims), _f32(voxel_size), _f32(volume_size), iso, verts,
                           cap, faces, cap, C.byref(nf))
    assert nv <= cap
    return verts[:nv].copy(), faces[:nf.value].copy()


def transform_points(pts, T):
    """(T * [p; 1]).head(3) for every point; T (4, 4) column-major flattened or a (4, 4) matrix."""
    p = _f32(pts).reshape(-1, 3).copy()
    lib().vfo_transform_points(p, len(p), kcol(T) if np.shape(T) == (4, 4) else _f32(T))
    return p


def translate(pts, t):
    p = _f32(pts).copy()
    lib().vfo_translate(p, len(p), _f32(t))
    return p


def build_graph(mesh, knn, radius, nodes=None, radii=None, transforms=None, cap=20000):
    nn = np.zeros((cap, 3), np.float32)
    rr = np.zeros(cap, np.float32)
    TT = np.zeros((cap, 16), np.float32)
    n0 = 0
    if nodes is not None and len(nodes):
        n0 = len(nodes)
        nn[:n0] = nodes
        rr[:n0] = radii
        TT[:n0] = np.asarray(transforms, np.float32).reshape(n0, 16)
    n = lib().vfo_build_graph(nn, rr, TT, n0, cap, _f32(mesh), len(mesh), knn, radius)
    if n < 0:
        raise RuntimeError("graph capacity exceeded")
    return nn[:n].copy(), rr[:n].copy(), TT[:n].copy()


def knn(nodes, pts, k, exclude_closest=False):
    m = len(pts)
    idx = np.empty((m, k), np.uint32)
    dist = np.empty((m, k), np.float32)
    lib().vfo_knn(_f32(nodes), len(nodes), _f32(pts), m, k, int(exclude_closest), idx, dist)
    return idx, dist


def filter_disconnected(idx, dist, radii):
    idx = np.ascontiguousarray(idx, np.uint32).copy()
    dist = _f32(dist).copy()
    lib().vfo_filter_disconnected(idx, dist, idx.shape[0], idx.shape[1], _f32(radii))
    return idx, dist


def warp_weights(radii, idx, dist):
    idx = np.ascontiguousarray(idx, np.uint32)
    w = np.empty(idx.shape, np.float32)
    lib().vfo_warp_weights(w, _f32(radii), idx, _f32(dist), idx.shape[0], idx.shape[1], len(radii))
    return w


def warp(pts, transforms, idx, w):
    idx = np.ascontiguousarray(idx, np.uint32)
    out = np.empty((len(pts), 3), np.float32)
    lib().vfo_warp(out, _f32(pts), len(pts), _f32(transforms), idx, _f32(w), idx.shape[1])
    return out


def warp_dqb(pts, transforms, idx, w):
    """Dual-quaternion blend of the node transforms (Kavan et al. 2007; no counterpart in the reference)."""
    idx = np.ascontiguousarray(idx, np.uint32)
    out = np.empty((len(pts), 3), np.float32)
    lib().vfo_warp_dqb(out, _f32(pts), len(pts), _f32(transforms), idx, _f32(w), idx.shape[1])
    return out


def correspondences(warped, K, depth, frame_mesh, thr):
    h, w = depth.shape
    m = len(warped)
    corr = np.empty((max(m, 1), 2), np.int32)
    n = lib().vfo_correspondences(corr, m, _f32(warped), m, kcol(K), _f32(depth), h, w, _f32(frame_mesh), thr)
    return corr[:n].copy()


def residual_depth(corr, warped, frame_mesh, normals_, lam):
    r = np.zeros(len(corr), np.float32)
    lib().vfo_residual_depth(r, _i32(corr), len(corr), _f32(warped), _f32(frame_mesh), _f32(normals_), lam)
    return r


def residual_reg(nodes, transforms, gidx, lam):
    n, kreg = gidx.shape
    r = np.zeros(n * kreg * 3, np.float32)
    lib().vfo_residual_reg(r, _f32(nodes), _f32(transforms), n, np.ascontiguousarray(gidx, np.uint32), kreg, lam)
    return r


def energy(r):
    return lib().vfo_energy(_f32(r), len(r))


def assemble(corr, canon, midx, mw, normals_, lam_d, nodes, gidx, lam_r, r_depth, r_reg):
    n, kreg = gidx.shape
    dim = 6 * n
    A = np.zeros((dim, dim), np.float32)
    b = np.zeros(dim, np.float32)
    empty = lib().vfo_assemble(None, A.ctypes.data, b, _i32(corr), len(corr), _f32(canon),
                               np.ascontiguousarray(midx, np.uint32), _f32(mw), midx.shape[1], _f32(normals_), lam_d,
                               _f32(nodes), n, np.ascontiguousarray(gidx, np.uint32), kreg, lam_r, _f32(r_depth),
                               _f32(r_reg))
    return A, b, empty


def solve_dense(A, b):
    A = np.ascontiguousarray(A, np.float64)
    x = np.zeros(len(b), np.float64)
    st = lib().vfo_solve_dense(A, _f32(b), len(b), x)
    if st:
        raise np.linalg.LinAlgError("not positive definite")
    return x


def pcg(A, b, iters, tol=0.0):
    A = np.ascontiguousarray(A, np.float64)
    x = np.zeros(len(b), np.float64)
    done = C.c_int(0)
    st = lib().vfo_pcg(A, _f32(b), len(b) // 6, iters, tol, x, C.byref(done))
    if st:
        raise np.linalg.LinAlgError("singular diagonal block")
    return x, done.value


def update_transforms(transforms, x):
    T = _f32(transforms).copy()
    lib().vfo_update_transforms(T, _f32(x), len(T))
    return T


def tsdf_knn(nodes, radii, voxel_size, volume_size, dims, per_node, k):
    S = int(np.prod(dims))
    kidx = np.empty((S, k), np.uint32)
    kdist = np.empty((S, k), np.float32)
    kcount = np.empty(S, np.int32)
    lib().vfo_tsdf_knn(kidx, kdist, kcount, _f32(nodes), _f32(radii), len(nodes), _f32(voxel_size),
                       _f32(volume_size), _i32(dims), _i32(per_node), k)
    return kidx, kdist, kcount


def tsdf_weights(radii, kidx, kdist, kcount):
    kw = np.empty(kidx.shape, np.float32)
    lib().vfo_tsdf_weights(kw, _f32(radii), kidx, _f32(kdist), _i32(kcount), kidx.shape[0], kidx.shape[1])
    return kw


def tsdf_vertices(voxel_size, volume_size, dims):
    S = int(np.prod(dims))
    v = np.empty((S, 3), np.float32)
    lib().vfo_tsdf_vertices(v, _f32(voxel_size), _f32(volume_size), _i32(dims))
    return v


def warp_tsdf(verts, transforms, kidx, kw, kcount):
    v = _f32(verts).copy()
    lib().vfo_warp_tsdf(v, _f32(transforms), kidx, _f32(kw), _i32(kcount), kidx.shape[0], kidx.shape[1])
    return v


def count_collisions(verts, kcount, voxel_size, volume_size, dims, Rinv, t):
    S = int(np.prod(dims))
    c = np.zeros(S, np.int32)
    lib().vfo_count_collisions(c, _f32(verts), _i32(kcount), _f32(voxel_size), _f32(volume_size), _i32(dims),
                               kcol(Rinv), _f32(t))
    return c


def integrate_warped(tsdf, weights, verts, collisions, kcount, depth, delta, voxel_size, volume_size, dims, Rinv, t,
                     K, half=False):
    h, w = depth.shape
    lib().vfo_integrate_warped(tsdf, weights, _f32(verts), _i32(collisions), _i32(kcount), _f32(depth), w, h, delta,
                               _f32(voxel_size), _f32(volume_size), _i32(dims), kcol(Rinv), _f32(t), kcol(K), int(half))


def round_half(x):
    """Nearest binary16 values of a float32 array (ties to even), as float32."""
    x = np.asarray(x, dtype=np.float32)
    return np.array([lib().vfo_round_half(float(v)) for v in x.ravel()], dtype=np.float32).reshape(x.shape)


def mc_pointcloud64(tsdf, weights, dims, voxel_size, volume_size, iso=0.0):
    """Sorted unique marching-cubes point cloud of a volume, evaluated in binary64 (FP64 oracle)."""
    L = lib64()
    cap = max(1, int(np.prod(dims)) * 3)
    out = np.zeros(3 * cap, np.float64)
    n = L.vfo_mc_pointcloud(np.ascontiguousarray(tsdf, np.float64).ravel(),
                            np.ascontiguousarray(weights, np.float64).ravel(), _i32(dims),
                            np.ascontiguousarray(voxel_size, np.float64), np.ascontiguousarray(volume_size, np.float64),
                            float(iso), out, cap)
    n = L.vfo_sort_unique_vec3(out, min(n, cap))
    return out[:3 * n].reshape(-1, 3)


# ---- depth ingest (OpenCV's undistortions and src/CameraCalibration.cpp, restated) ----

def dist_cv(d):
    """k1 k2 p1 p2 k3 k4 k5 k6 (OpenCV order) from a dict of coefficients."""
    return [float(d.get(k, 0.0)) for k in ("k1", "k2", "p1", "p2", "k3", "k4", "k5", "k6")]


def dist_bc(d):
    """k1..k6, codx, cody, p1, p2 (af::CameraDistortion order)."""
    return np.asarray([float(d.get(k, 0.0)) for k in ("k1", "k2", "k3", "k4", "k5", "k6", "codx", "cody", "p1",
                                                       "p2")], np.float32)


def undistort_map(K, d, width, height, mode):
    """Per-pixel source map (2 uint32 per pixel) of cv::undistort (mode 0) or of
    initUndistortRectifyMap(CV_32FC1) + remap(INTER_NEAREST) (mode 1)."""
    out = np.empty(2 * width * height, np.uint32)
    lib().vfo_undistort_map(out, width, height, kcol(K), np.asarray(dist_cv(d), np.float32), int(mode))
    return out


def undistort_depth(src, umap, mode):
    src = np.ascontiguousarray(src, np.float32)
    h, w = src.shape
    out = np.empty_like(src)
    lib().vfo_undistort_depth(out.ravel(), src.ravel(), w, h, np.ascontiguousarray(umap, np.uint32), int(mode))
    return out


def xy_lookup_table(intr, d, width, height):
    out = np.empty((height, width, 2), np.float32)
    lib().vfo_xy_lookup_table(out.ravel(), width, height, np.asarray(intr, np.float32), dist_bc(d))
    return out


def bc_unproject(pixels, depths, intr, d):
    pixels = np.ascontiguousarray(pixels, np.float32)
    depths = np.ascontiguousarray(depths, np.float32)
    n = depths.size
    pts = np.empty((n, 3), np.float32)
    valid = np.empty(n, np.int32)
    lib().vfo_bc_unproject(pts.ravel(), valid, pixels.ravel(), depths, n, np.asarray(intr, np.float32), dist_bc(d))
    return pts, valid


def bc_project(points, intr, d, out=None):
    points = np.ascontiguousarray(points, np.float32)
    n = points.shape[0]
    px = np.zeros((n, 2), np.float32) if out is None else np.ascontiguousarray(out, np.float32).copy()
    valid = np.empty(n, np.int32)
    lib().vfo_bc_project(px.ravel(), valid, points.ravel(), n, np.asarray(intr, np.float32), dist_bc(d))
    return px, valid


class VfoParams(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("K", C.c_float * 9), ("dims", C.c_int * 3),
                ("volume_size", C.c_float * 3), ("delta", C.c_float), ("depth_threshold", C.c_float),
                ("bilateral", C.c_int), ("bilateral_r", C.c_int), ("sigma_i", C.c_float), ("sigma_s", C.c_float),
                ("bilateral_thr", C.c_float), ("angle_lo", C.c_float), ("angle_hi", C.c_float),
                ("graph_radius", C.c_float), ("knn", C.c_int), ("kreg", C.c_int), ("update_graph", C.c_int),
                ("icp_iterations", C.c_int), ("gn_iterations", C.c_int), ("lambda_depth", C.c_float),
                ("lambda_reg", C.c_float), ("energy_min_step", C.c_float), ("corr_thresh", C.c_float),
                ("solver", C.c_int), ("pcg_iterations", C.c_int), ("pcg_tol", C.c_double), ("integrate", C.c_int),
                ("node_cap", C.c_int), ("mesh_cap", C.c_long), ("precision", C.c_int), ("blend", C.c_int),
                ("distorted", C.c_int), ("dist_cv", C.c_float * 8)]


class Fusion:
    """Whole-sequence oracle driver (af::runVolumeFusion's per-frame loop) over in-memory frames.
    fp64=True runs the binary64 build (liboracle64.so); arrays then come back as float64."""

    def __init__(self, cfg, fp64=False):
        self._L = lib64() if fp64 else lib()
        self._ct, self._dt = (C.c_double, np.float64) if fp64 else (C.c_float, np.float32)
        p = VfoParams()
        p.width, p.height = cfg["width"], cfg["height"]
        p.K[:] = list(kcol(cfg["K"]))
        p.dims[:] = list(cfg["dims"])
        p.volume_size[:] = list(cfg["volume_size"])
        for key in ("delta", "depth_threshold", "sigma_i", "sigma_s", "bilateral_thr", "angle_lo", "angle_hi",
                    "graph_radius", "lambda_depth", "lambda_reg", "energy_min_step", "corr_thresh"):
            setattr(p, key, float(cfg[key]))
        for key in ("bilateral", "bilateral_r", "knn", "kreg", "update_graph", "icp_iterations", "gn_iterations",
                    "solver", "pcg_iterations", "integrate", "node_cap", "mesh_cap"):
            setattr(p, key, int(cfg[key]))
        p.pcg_tol = float(cfg.get("pcg_tol", 0.0))
        p.precision = {"fp32": 0, "fp16": 1}[cfg.get("precision", "fp32")]
        p.blend = {"lbs": 0, "dqb": 1}[cfg.get("blend", "lbs")]
        if cfg.get("distortion"):
            p.distorted = 1
            p.dist_cv[:] = dist_cv(cfg["distortion"])
        self.cfg = cfg
        self._p = p
        self.h = self._L.vfo_fusion_create(C.byref(p))
        self.S = int(np.prod(cfg["dims"]))

    def close(self):
        if self.h:
            self._L.vfo_fusion_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def process(self, mm):
        st = self._L.vfo_fusion_process(self.h, np.ascontiguousarray(mm, np.uint16))
        if st:
            raise RuntimeError("oracle frame failed with status %d" % st)

    def _arr(self, ptr, n):
        if n == 0:
            return np.zeros(0, self._dt)
        return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(self._ct)), shape=(n,)).copy()

    @property
    def num_nodes(self):
        return self._L.vfo_fusion_num_nodes(self.h)

    @property
    def mesh_size(self):
        return self._L.vfo_fusion_mesh_size(self.h)

    @property
    def num_corr(self):
        return self._L.vfo_fusion_num_corr(self.h)

    @property
    def gn_done(self):
        return self._L.vfo_fusion_gn_done(self.h)

    @property
    def energy(self):
        return self._L.vfo_fusion_energy(self.h)

    def tsdf(self):
        return self._arr(self._L.vfo_fusion_tsdf(self.h), self.S)

    def weights(self):
        return self._arr(self._L.vfo_fusion_weights(self.h), self.S)

    def nodes(self):
        return self._arr(self._L.vfo_fusion_nodes(self.h), 3 * self.num_nodes).reshape(-1, 3)

    def transforms(self):
        return self._arr(self._L.vfo_fusion_transforms(self.h), 16 * self.num_nodes).reshape(-1, 16)

    def centroid(self):
        return self._arr(self._L.vfo_fusion_centroid(self.h), 3)

    def mesh(self):
        return self._arr(self._L.vfo_fusion_mesh(self.h), 3 * self.mesh_size).reshape(-1, 3)

    def set_transforms(self, T):
        T = np.ascontiguousarray(T, dtype=self._dt).reshape(-1, 16)
        self._L.vfo_fusion_set_transforms(self.h, T, len(T))

    def set_tsdf(self, tsdf, weights):
        self._L.vfo_fusion_set_tsdf(self.h, np.ascontiguousarray(tsdf, dtype=self._dt).ravel(),
                                  np.ascontiguousarray(weights, dtype=self._dt).ravel())
