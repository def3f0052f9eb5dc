"""Generate tests/golden/ref_kernels.npz: the reference's own CUDA kernels (src/*.cu), executed
on the host by oracle/_ref/libvfemu.so (``python oracle/ref_emu/build_emu.py``), on seeded
synthetic inputs.  These are the stages the reference has only as GPU code: depth filter,
bilateral filter, depth-to-vertices, normals, correspondences, the Gauss-Newton residuals /
J^T J / J^T r (with the thrust sort + reduce_by_key steps restated as stable sorts and
sequential sums), the transform update, per-voxel node support, TSDF warp weights, TSDF
vertices and warp, collision counts, warped integration and the GPU marching cubes.

The emulation runs the kernels' own source with host libm, so transcendental functions
(expf) round as glibc does, not as CUDA's device library does; outputs that go through expf
are compared within a few ulp, everything else bit-exactly.  The reference's compile-time
constants apply: K = 6 skinning neighbours, K_reg = 4 regularisation neighbours.

    python tests/golden/make_golden_kernels.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pyemu as E  # noqa: E402
from oracle import pyoracle as O  # noqa: E402
from volumefusion_gb300 import synth  # noqa: E402

OUT = os.path.join(HERE, "ref_kernels.npz")

# small capsule-pair view (quarter-resolution camera of the 640x576 workload)
W, H = 160, 144
KMAT = synth.intrinsics(126.0, 126.0, 80.0, 72.0)
DIMS = np.array([48, 40, 32], np.int32)
SIZE = np.array([0.576, 0.480, 0.384], np.float32)
RADIUS = 0.05


def inputs(frame=12):
    mm, K = synth.capsule_pair_frame(frame, width=W, height=H, fx=126.0, fy=126.0, cx=80.0, cy=72.0)
    return mm, K


def generate():
    if not E.available():
        raise SystemExit("oracle/_ref/libvfemu.so missing: python oracle/ref_emu/build_emu.py")
    k, kr = E.knn_k(), E.kreg()
    mm, K = inputs()
    out = {"mm": mm, "K": np.asarray(K, np.float64), "dims": DIMS, "size": SIZE, "radius": np.float32(RADIUS),
           "knn": np.int32(k), "kreg": np.int32(kr)}
    depth = O.depth_from_mm(mm)
    d0 = E.filter_depth(depth, 1.2)
    out["filtered"] = d0
    bil = E.bilateral(d0, 2, 0.03, 2.0, 0.09)
    out["bilateral"] = bil
    verts = E.depth_to_mesh(bil, K)
    out["vertices"] = verts
    nrm, verts2 = E.normals(verts, bil, 1.3, 2.1)
    nrm, verts3, depth3 = E.remove_without_normals(nrm, verts2, bil)
    out["normals"], out["vertices_kept"], out["depth_kept"] = nrm, verts3, depth3
    # volume around the frame centroid, rigid first frame
    _, _, _, c = O.frame_prep(mm, K)
    out["centroid"] = c
    vs = SIZE / DIMS.astype(np.float32)
    S = int(np.prod(DIMS))
    t0 = np.full(S, -1, np.float32)
    w0 = np.zeros(S, np.float32)
    E.integrate_rigid(t0, w0, depth3, 0.016, DIMS, vs, SIZE, np.eye(3), c, K)
    out["tsdf0"], out["weights0"] = t0, w0
    mv, mf = E.mc_full(t0, w0, DIMS, vs, SIZE)
    out["mc_vertices"], out["mc_faces"] = mv, mf
    pc = O.sort_unique(E.mc_points(t0, w0, DIMS, vs, SIZE))
    out["mc_points_sorted"] = pc
    mesh = E.translate(pc, c)
    nodes, radii, T = O.build_graph(mesh, 4, RADIUS)
    rng = np.random.default_rng(7)
    T = T.copy()
    T[:, 12:15] += rng.normal(0, 0.003, (len(T), 3)).astype(np.float32)
    out["mesh"], out["nodes"], out["radii"], out["T"] = mesh, nodes, radii, T
    midx, mdist = O.knn(nodes, mesh, k)
    out["midx"], out["mdist"] = midx, mdist
    mw = E.warp_weights(radii, midx, mdist)
    out["mw"] = mw
    warped = E.warp(mesh, T, midx, mw)
    out["warped"] = warped
    # second frame: correspondences and one Gauss-Newton system
    mm1, _ = inputs(14)
    d1, v1, n1, _ = O.frame_prep(mm1, K)
    out["mm1"] = mm1
    corr = E.correspondences(warped, K, d1, v1, 0.02)
    out["corr"] = corr
    gidx, gdist = O.knn(nodes, nodes, kr, exclude_closest=True)
    gidx, gdist = O.filter_disconnected(gidx, gdist, radii)
    out["gidx"] = gidx
    lam_d, lam_r = np.float32(1.0), np.float32(np.sqrt(200.0))
    jtj, jtr, r = E.gn_assemble(corr, mesh, midx, mw, n1, v1, warped, nodes, T, gidx, lam_d, lam_r)
    out["jtj"], out["jtr"], out["residuals"] = jtj, jtr, r
    x = rng.normal(0, 1e-3, 6 * len(nodes)).astype(np.float32)
    out["x"] = x
    out["T_updated"] = E.update_transforms(T, x)
    # voxel support, weights, warp, collisions, warped integration
    per = np.array([2 * (int(np.float32(RADIUS) / vs[i]) + 1) + 1 for i in range(3)], np.int32)
    nt = O.translate(nodes, -c)
    kidx, kdist, kcount = E.tsdf_knn(nt, radii, vs, SIZE, DIMS, per)
    out["per"], out["kidx"], out["kdist"], out["kcount"] = per, kidx, kdist, kcount
    kw = E.tsdf_weights(radii, kidx, kdist, kcount)
    out["kw"] = kw
    tv = E.tsdf_vertices(vs, SIZE, DIMS)
    out["tsdf_vertices"] = tv
    tvc = O.translate(tv, c)
    wv = E.warp_tsdf(tvc, T, kidx, kw, kcount, vs, SIZE, DIMS)
    out["warped_vertices"] = wv
    coll = E.count_collisions(wv, kcount, vs, SIZE, DIMS, np.eye(3), c)
    out["collisions"] = coll
    t1, w1 = t0.copy(), w0.copy()
    E.integrate_warped(t1, w1, wv, coll, kcount, d1, 0.016, vs, SIZE, DIMS, np.eye(3), c, K)
    out["tsdf1"], out["weights1"] = t1, w1
    np.savez_compressed(OUT, **out)
    print(OUT, os.path.getsize(OUT), "bytes;", len(corr), "correspondences,", len(nodes), "nodes,",
          int((kcount > 0).sum()), "supported voxels,", int((w1 != w0).sum()), "voxels updated")


if __name__ == "__main__":
    generate()
