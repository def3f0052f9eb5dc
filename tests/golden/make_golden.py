"""Generate the golden fixtures in tests/golden/ by running the reference's own CPU code.

Runs oracle/_ref/libvfref.so (built by ``make -C oracle -f Makefile.ref`` from the
reference source tree: TSDFVolume::integrate, MarchingCubes::computeIsoSurface /
computePointCloud, af::buildGraph, af::getKnnData, af::filterDisconnected,
MotionGraph::warp) on seeded synthetic inputs and stores inputs and outputs as
compressed .npz files.  The fixtures travel with the repository; the reference tree
does not, so tests read only the .npz files.

    python tests/golden/make_golden.py
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pyoracle as O  # noqa: E402
from volumefusion_gb300 import synth  # noqa: E402

REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libvfref.so")


def ref_lib():
    if not os.path.exists(REF_LIB):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "-f", "Makefile.ref"], check=True)
    return C.CDLL(REF_LIB)


def ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def ref_integrate(R, depth, K, dims, size, delta, pose):
    S = int(np.prod(dims))
    t = np.empty(S, np.float32)
    w = np.empty(S, np.float32)
    h, wd = depth.shape
    R.ref_integrate(ptr(t), ptr(w), ptr(np.ascontiguousarray(depth, np.float32)), wd, h, ptr(O.kcol(K)),
                    ptr(np.asarray(dims, np.int32)), ptr(np.asarray(size, np.float32)), C.c_float(delta),
                    ptr(np.ascontiguousarray(np.asarray(pose, np.float32).T).ravel()))
    return t, w


def ref_mc(R, tsdf, weights, dims, size, point_cloud):
    cap = 3_000_000
    v = np.empty((cap, 3), np.float32)
    f = np.empty((cap, 3), np.int32)
    nf = C.c_long(0)
    R.ref_marching_cubes.restype = C.c_long
    nv = R.ref_marching_cubes(ptr(tsdf), ptr(weights), ptr(np.asarray(dims, np.int32)),
                              ptr(np.asarray(size, np.float32)), C.c_float(0.0), int(point_cloud), ptr(v),
                              C.c_long(cap), ptr(f), C.c_long(cap), C.byref(nf))
    return v[:nv].copy(), f[:nf.value].copy()


def ref_build_graph(R, mesh, knn, radius, nodes=None, radii=None, T=None, cap=20000):
    nn = np.zeros((cap, 3), np.float32)
    rr = np.zeros(cap, np.float32)
    TT = np.zeros((cap, 16), np.float32)
    n0 = 0 if nodes is None else len(nodes)
    if n0:
        nn[:n0], rr[:n0], TT[:n0] = nodes, radii, T
    n = R.ref_build_graph(ptr(nn), ptr(rr), ptr(TT), n0, cap, ptr(np.ascontiguousarray(mesh, np.float32)),
                          C.c_long(len(mesh)), knn, C.c_float(radius))
    assert n > 0
    return nn[:n].copy(), rr[:n].copy(), TT[:n].copy()


def ref_knn(R, nodes, radii, pts, k, exclude):
    idx = np.empty((len(pts), k), np.uint32)
    dist = np.empty((len(pts), k), np.float32)
    st = R.ref_knn(ptr(np.ascontiguousarray(nodes, np.float32)), ptr(np.ascontiguousarray(radii, np.float32)),
                   len(nodes), ptr(np.ascontiguousarray(pts, np.float32)), C.c_long(len(pts)), k, int(exclude),
                   ptr(idx), ptr(dist))
    assert st == 0
    return idx, dist


def ref_filter(R, nodes, radii, idx, dist):
    idx = idx.copy()
    dist = dist.copy()
    st = R.ref_filter_disconnected(ptr(np.ascontiguousarray(nodes, np.float32)), ptr(radii), len(nodes), idx.shape[1],
                                   ptr(idx), ptr(dist))
    assert st == 0
    return idx, dist


def ref_warp(R, nodes, radii, T, pts, k):
    out = np.empty((len(pts), 3), np.float32)
    R.ref_warp(ptr(np.ascontiguousarray(nodes, np.float32)), ptr(np.ascontiguousarray(radii, np.float32)),
               ptr(np.ascontiguousarray(T, np.float32)), len(nodes), ptr(np.ascontiguousarray(pts, np.float32)),
               C.c_long(len(pts)), k, ptr(out))
    return out


def main():
    R = ref_lib()
    # 1. rigid integration of the 320x288 sphere frame (TSDFIntegrationTest.cu:12-59 on synthetic data)
    mm, K = synth.sphere_frame()
    depth = O.depth_from_mm(mm)  # the CPU reference treats 0 as "no depth"
    dims = np.array([64, 64, 64], np.int32)
    size = np.array([0.512, 0.512, 0.512], np.float32)
    delta = np.float32(0.016)
    _, verts, _, cen = O.frame_prep(mm, K, depth_threshold=1.2, bilateral=0)
    pose = np.eye(4, dtype=np.float32)
    pose[:3, 3] = cen
    t1, w1 = ref_integrate(R, depth, K, dims, size, delta, pose)
    np.savez_compressed(os.path.join(HERE, "integrate_sphere.npz"), mm=mm, K=K, dims=dims, size=size,
                        delta=np.float32(delta), centroid=cen, tsdf=t1, weights=w1)

    # 2. marching cubes on the reference's integrated volume (MarchingCubesTest.cu:27-115)
    pc, _ = ref_mc(R, t1, w1, dims, size, point_cloud=True)
    iv, fi = ref_mc(R, t1, w1, dims, size, point_cloud=False)
    np.savez_compressed(os.path.join(HERE, "marching_cubes.npz"), dims=dims, size=size, tsdf=t1, weights=w1,
                        pointcloud=pc, iso_verts=iv, iso_faces=fi)

    # 3. graph build + KNN on the canonical point cloud (src/VolumeFusion.cu:382-419)
    mesh = O.sort_unique(pc)
    mesh = O.translate(mesh, cen)
    radius = np.float32(0.025)
    nodes, radii, T = ref_build_graph(R, mesh, 4, radius)
    k4 = ref_knn(R, nodes, radii, mesh, 4, False)
    k6 = ref_knn(R, nodes, radii, mesh, 6, False)
    g8 = ref_knn(R, nodes, radii, nodes, 8, True)
    g8f = ref_filter(R, nodes, radii, *g8)
    # incremental build: transformed existing nodes, shifted point cloud (new nodes copy the
    # nearest node's transform, src/GraphBuilder.cpp:38-48)
    rng = np.random.default_rng(7)
    T_rand = np.tile(np.eye(4, dtype=np.float32).T.ravel(), (len(nodes), 1))
    T_rand[:, 12:15] = rng.normal(0, 0.01, (len(nodes), 3)).astype(np.float32)
    T_rand[:, 0] += rng.normal(0, 0.01, len(nodes)).astype(np.float32)
    mesh2 = mesh + np.array([0.03, 0.0, -0.01], np.float32)
    nodes2, radii2, T2 = ref_build_graph(R, mesh2, 4, radius, nodes, radii, T_rand)
    np.savez_compressed(os.path.join(HERE, "graph_knn.npz"), mesh=mesh, radius=radius, nodes=nodes, radii=radii,
                        transforms=T, k4_idx=k4[0], k4_dist=k4[1], k6_idx=k6[0], k6_dist=k6[1], g8_idx=g8[0],
                        g8_dist=g8[1], g8f_idx=g8f[0], g8f_dist=g8f[1], T_rand=T_rand, mesh2=mesh2, nodes2=nodes2,
                        radii2=radii2, transforms2=T2)

    # 4. CPU warp with non-trivial transforms (MotionGraph::warp, K=4) and the 4-node case of
    #    MotionGraphTest.cpp:98-133 (its hard-coded expectations are stale; the compiled code is the pin)
    W = ref_warp(R, nodes, radii, T_rand, mesh, 4)
    t1m = np.eye(4, dtype=np.float32); t1m[:3, 3] = 1.0
    t2m = np.eye(4, dtype=np.float32); t2m[:3, 3] = -1.0
    t3m = np.array([[2.0, 1.5, 1.5, 1.0], [1.0, 1.5, 2.5, 1.0], [2.0, 2.5, 4.0, 1.0], [0, 0, 0, 1]], np.float32)
    kn = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [0, 0, 2]], np.float32)
    kr = np.array([0.9, 0.9, 0.9, 1.1], np.float32)
    kT = np.stack([np.eye(4, dtype=np.float32).T.ravel(), t1m.T.ravel(), t2m.T.ravel(), t3m.T.ravel()])
    kp = np.array([[0, 0, 0], [0, 0.5, 0.5], [0, 0, 1.5], [0, 0, 1.2], [0, 0.5, 1.5]], np.float32)
    kw = ref_warp(R, kn, kr, kT, kp, 3)
    np.savez_compressed(os.path.join(HERE, "warp.npz"), nodes=nodes, radii=radii, transforms=T_rand, points=mesh,
                        warped=W, kat_nodes=kn, kat_radii=kr, kat_transforms=kT, kat_points=kp, kat_warped=kw)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
