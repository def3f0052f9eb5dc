"""Pins of the CPU oracle against the reference's own CUDA kernels (src/*.cu) executed on the
host (tests/golden/ref_kernels.npz, made by tests/golden/make_golden_kernels.py from
oracle/_ref/libvfemu.so).  Bit-exact except where the value goes through expf: the
emulation rounds expf as the host libm does and the oracle as the library's own exp, so
those outputs agree within 8 ulp.  The reference's constants apply: K = 6, K_reg = 4.

When the emulation library is present (only where the reference tree is), the same checks
also run live on a second frame."""
import os

import numpy as np
import pytest

from oracle import pyoracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
with np.load(os.path.join(HERE, "golden", "ref_kernels.npz")) as _z:
    G = {k: _z[k] for k in _z.files}


def ulp(a, b):
    a = np.ascontiguousarray(a, np.float32).view(np.int32).astype(np.int64)
    b = np.ascontiguousarray(b, np.float32).view(np.int32).astype(np.int64)
    return int(np.max(np.abs(a - b))) if a.size else 0


def vol():
    dims, size = G["dims"], G["size"]
    return dims, size, size / dims.astype(np.float32)


def test_depth_stages_match_reference_kernels():
    """filterDepthKernel, the shared-memory bilateral filter, depthToMeshKernel,
    depthVerticesNormalsKernel and removeDepthWithoutNormalsKernel (src/BilateralFilter.cu,
    src/VertexManipulation.cu)."""
    K = G["K"]
    depth = O.depth_from_mm(G["mm"])
    d0 = O.filter_depth(depth, 1.2)
    assert np.array_equal(d0, G["filtered"])
    bil = O.bilateral(d0, 2, 0.03, 2.0, 0.09)
    assert np.array_equal(bil, G["bilateral"])
    verts = O.depth_to_mesh(bil, K)
    assert np.array_equal(verts, G["vertices"])
    d, v, n, c = O.frame_prep(G["mm"], K)
    assert np.array_equal(n, G["normals"])
    assert np.array_equal(v, G["vertices_kept"])
    assert np.array_equal(d, G["depth_kept"])
    assert np.array_equal(c, G["centroid"])


def test_rigid_integration_and_gpu_marching_cubes_match_reference_kernels():
    """integrateTSDFFromFrameKernel and marchingCubesFullKernel / marchingCubesMeshKernel
    (src/TSDFIntegration.cu, src/MarchingCubes.cu); the GPU kernel appends in thread order, so
    faces are compared as sets of vertex triples."""
    dims, size, vs = vol()
    S = int(np.prod(dims))
    t, w = np.full(S, -1, np.float32), np.zeros(S, np.float32)
    O.integrate_rigid(t, w, G["depth_kept"], 0.016, dims, vs, size, np.eye(3), G["centroid"], G["K"])
    assert np.array_equal(t, G["tsdf0"]) and np.array_equal(w, G["weights0"])
    pc = O.sort_unique(O.mc_pointcloud(t, w, dims, vs, size))
    assert np.array_equal(pc, G["mc_points_sorted"])
    mv, mf = O.mc_full(t, w, dims, vs, size)
    rv, rf = G["mc_vertices"], G["mc_faces"]
    assert len(mf) == len(rf) and len(mv) == len(rv)
    tri = lambda V, F: sorted(map(tuple, np.sort(V[F].reshape(len(F), 9).view(np.int32), axis=1)))  # noqa: E731
    assert tri(mv, mf) == tri(rv, rf)


def test_skinning_warp_and_correspondences_match_reference_kernels():
    """computeWarpWeightsKernel, warpKernel, correspondencePairsKernel
    (src/VertexManipulation.cu, src/ComputeCorrespondence.cu)."""
    K = G["K"]
    mw = O.warp_weights(G["radii"], G["midx"], G["mdist"])
    assert ulp(mw, G["mw"]) <= 8
    warped = O.warp(G["mesh"], G["T"], G["midx"], G["mw"])
    assert np.array_equal(warped, G["warped"])
    d1, v1, _, _ = O.frame_prep(G["mm1"], K)
    corr = O.correspondences(G["warped"], K, d1, v1, 0.02)
    assert np.array_equal(corr, G["corr"])


def test_gauss_newton_system_matches_reference_kernels():
    """fill_r_*/fill_J_* kernels, computeJTJAndJTrContrib*, the sort / reduce_by_key steps,
    multiplyJTJContribPairsKernel / multiplyJTrContribElemsKernel, fillJTJKernel over the
    identity, fillJTrKernel (src/MotionOptimization.cu, src/VolumeFusion.cu:454-646) and
    updateTransformsKernel."""
    K = G["K"]
    d1, v1, n1, _ = O.frame_prep(G["mm1"], K)
    lam_d, lam_r = np.float32(1.0), np.float32(np.sqrt(200.0))
    corr, nodes, T, gidx = G["corr"], G["nodes"], G["T"], G["gidx"]
    rd = O.residual_depth(corr, G["warped"], v1, n1, lam_d)
    rr = O.residual_reg(nodes, T, gidx, lam_r)
    assert np.array_equal(np.concatenate([rd, rr]), G["residuals"])
    A, b, _ = O.assemble(corr, G["mesh"], G["midx"], G["mw"], n1, lam_d, nodes, gidx, lam_r, rd, rr)
    assert np.array_equal(A, G["jtj"])
    assert np.array_equal(b, G["jtr"])
    assert np.array_equal(O.update_transforms(T, G["x"]), G["T_updated"])


def test_voxel_stages_match_reference_kernels():
    """tsdfKNNGraph scatter (support counts; the node sets agree where a voxel has at most K
    supporting nodes, the reference keeps the first K in scatter order, the oracle the K
    nearest), computeTsdfWarpWeightsKernel, generateTsdfVerticesKernel, warpTsdfKernel,
    countCollisionsPerVoxelKernel, integrateWarpedTSDFFromFrameKernel
    (src/TSDFWarp.cu, src/TSDFIntegration.cu)."""
    K = G["K"]
    dims, size, vs = vol()
    c = G["centroid"]
    k = int(G["knn"])
    nt = O.translate(G["nodes"], -c)
    kidx, kdist, kcount = O.tsdf_knn(nt, G["radii"], vs, size, dims, G["per"], k)
    assert np.array_equal(kcount, G["kcount"])
    act = kcount > 0
    assert act.sum() > 1000
    # voxels whose support set is complete in both (fewer than K supporting nodes)
    few = np.where((kcount > 0) & (kcount < k))[0]
    assert len(few) > 100
    for i in few:
        c_ = kcount[i]
        assert sorted(zip(kidx[i, :c_], kdist[i, :c_])) == sorted(zip(G["kidx"][i, :c_], G["kdist"][i, :c_]))
    kw = O.tsdf_weights(G["radii"], G["kidx"], G["kdist"], G["kcount"])
    assert ulp(kw[act], G["kw"][act]) <= 8
    tv = O.tsdf_vertices(vs, size, dims)
    assert np.array_equal(tv, G["tsdf_vertices"])
    wv = O.warp_tsdf(O.translate(tv, c), G["T"], G["kidx"], G["kw"], G["kcount"])
    assert np.array_equal(wv, G["warped_vertices"])
    coll = O.count_collisions(G["warped_vertices"], G["kcount"], vs, size, dims, np.eye(3), c)
    assert np.array_equal(coll, G["collisions"])
    d1, _, _, _ = O.frame_prep(G["mm1"], K)
    t1, w1 = G["tsdf0"].copy(), G["weights0"].copy()
    O.integrate_warped(t1, w1, G["warped_vertices"], G["collisions"], G["kcount"], d1, 0.016, vs, size, dims,
                       np.eye(3), c, K)
    assert np.array_equal(t1, G["tsdf1"]) and np.array_equal(w1, G["weights1"])
    assert (w1 != G["weights0"]).sum() > 1000


def test_live_against_emulated_reference_when_present():
    from oracle import pyemu as E
    if not E.available():
        pytest.skip("reference emulation library not built (needs the reference source tree)")
    from volumefusion_gb300 import synth
    mm, K = synth.capsule_pair_frame(20, width=160, height=144, fx=126.0, fy=126.0, cx=80.0, cy=72.0)
    depth = O.filter_depth(O.depth_from_mm(mm), 1.2)
    assert np.array_equal(O.bilateral(depth, 2, 0.03, 2.0, 0.09), E.bilateral(depth, 2, 0.03, 2.0, 0.09))
    d, v, n, c = O.frame_prep(mm, K)
    pts = v.reshape(-1, 3)
    pts = pts[pts[:, 2] > 0][::3] + np.array([0.003, -0.002, 0.001], np.float32)
    assert np.array_equal(O.correspondences(pts, K, d, v, 0.01), E.correspondences(pts, K, d, v, 0.01))
