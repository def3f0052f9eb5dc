"""The af:: C++ surface run from a compiled C++ caller (tests/cpp/af_surface_check.cpp) on one
frame pair of the small non-rigid case, every intermediate compared with the CPU oracle:
DeviceTsdf::integrate / extractPointCloud, runTranslateKernel, buildGraph, getKnnData (both
layouts), filterDisconnected, MotionGraph::knnSearch / warp, WarpField (spreadMotionGraph,
weighted KNN, graph KNN, warp), runComputeWarpWeightsKernel, runCorrespondencePairsKernel,
GaussNewtonSystem (residuals and J^T J bit-exact, J^T r to rounding, 10 PCG iterations against the
oracle's FP64 PCG), runUpdateTransformsKernel, TSDFVolume integrate / save / load and
runFilterDepthKernel with a fill value."""
import json
import os
import subprocess

import numpy as np
import pytest

from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


# depthDistortion.txt order: k1 k2 p1 p2 k3 k4 k5 k6
INGEST_DIST = (-0.08, 0.02, 4e-4, -3e-4, 0.001, 0.0, 0.0, 0.0)


@pytest.fixture(scope="module")
def run(tmp_path_factory):
    pytest.importorskip("torch")
    import _cppcaller
    from volumefusion_gb300 import build, configs, synth
    build.build()
    work = tmp_path_factory.mktemp("cpp_surface")
    exe = str(work / "af_check")
    r = _cppcaller.compile_caller(exe)
    if r is None:
        pytest.skip("no g++ or CUDA runtime")
    assert r.returncode == 0, r.stderr
    cfg = configs.small_nonrigid(n_frames=30)
    K = cfg["K"]
    cam = dict(width=cfg["width"], height=cfg["height"], fx=float(K[0, 0]), fy=float(K[1, 1]), cx=float(K[0, 2]),
               cy=float(K[1, 2]))
    mm0, _ = synth.capsule_pair_frame(12, **cam)
    mm1, _ = synth.capsule_pair_frame(14, **cam)
    d0, _, _, c = O.frame_prep(mm0, K)
    d1, v1, n1, _ = O.frame_prep(mm1, K)
    dims = np.asarray(cfg["dims"], np.int32)
    size = np.asarray(cfg["volume_size"], np.float32)
    meta = np.array([cfg["width"], cfg["height"], K[0, 0], K[1, 1], K[0, 2], K[1, 2], *dims, *size, cfg["delta"],
                     cfg["graph_radius"], cfg["corr_thresh"], cfg["lambda_depth"], cfg["lambda_reg"], *c], np.float32)
    inp, out = work / "in", work / "out"
    inp.mkdir()
    out.mkdir()
    meta.tofile(inp / "meta.bin")
    for name, a in (("depth0", d0), ("depth1", d1), ("verts1", v1), ("normals1", n1)):
        np.ascontiguousarray(a, np.float32).tofile(inp / (name + ".bin"))
    # depth ingest inputs: frame 3 as a 16-bit PNG and the two calibration files
    import _depth_codecs
    mm3, _ = synth.capsule_pair_frame(16, **cam)
    (inp / "frame-000003.depth.png").write_bytes(_depth_codecs.png(mm3, 16, -1))
    (inp / "depthIntrinsics.txt").write_text("%r 0 %r\n0 %r %r\n0 0 1\n" % (float(K[0, 0]), float(K[0, 2]),
                                                                           float(K[1, 1]), float(K[1, 2])))
    (inp / "depthDistortion.txt").write_text(" ".join(repr(v) for v in INGEST_DIST))
    p = subprocess.run([exe, str(inp), str(out)], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stdout + p.stderr
    stats = json.loads(p.stdout.strip().splitlines()[-1])

    def load(name, dtype=np.float32, cols=None):
        a = np.fromfile(out / (name + ".bin"), dtype)
        return a.reshape(-1, cols) if cols else a

    return dict(cfg=cfg, K=K, d0=d0, d1=d1, v1=v1, n1=n1, c=c, dims=dims, size=size, vs=size / dims.astype(np.float32),
                stats=stats, load=load, out=out, mm3=mm3)


def test_volume_and_point_cloud(run):
    cfg, L = run["cfg"], run["load"]
    S = int(np.prod(run["dims"]))
    t, w = np.full(S, -1, np.float32), np.zeros(S, np.float32)
    O.integrate_rigid(t, w, run["d0"], cfg["delta"], run["dims"], run["vs"], run["size"], np.eye(3), run["c"],
                      run["K"])
    assert np.array_equal(L("tsdf"), t) and np.array_equal(L("weights"), w)
    cloud = O.sort_unique(O.mc_pointcloud(t, w, run["dims"], run["vs"], run["size"]))
    assert len(cloud) > 1000
    assert np.array_equal(L("cloud", cols=3), cloud)
    assert np.array_equal(L("mesh", cols=3), O.translate(cloud, run["c"]))
    # TSDFVolume through pose [I | c] is the same integration; its file round-trips
    assert np.array_equal(L("volume_tsdf"), t)
    assert run["stats"]["volume_roundtrip"] is True
    d = run["d0"].ravel()
    want = np.where((d > 0.9) | (d < 1e-4) | np.isnan(d), np.float32(0), d)
    assert np.array_equal(L("filtered"), want)


def test_graph_knn_and_warp(run):
    cfg, L = run["cfg"], run["load"]
    mesh = L("mesh", cols=3)
    nodes, radii, T = O.build_graph(mesh, 6, cfg["graph_radius"])
    assert len(nodes) > 10 and run["stats"]["nodes"] == len(nodes)
    assert np.array_equal(L("nodes", cols=3), nodes)
    assert np.array_equal(L("radii"), radii)
    assert np.array_equal(L("transforms", cols=16), T)
    midx, mdist = O.knn(nodes, mesh, 6)
    assert np.array_equal(L("midx", np.uint32, 6), midx)
    assert np.array_equal(L("mdist", cols=6), mdist)
    m = len(mesh)
    assert np.array_equal(L("one_idx", np.uint32), midx[m // 2])
    assert np.array_equal(L("one_dist"), mdist[m // 2])
    fidx, fdist = O.knn(nodes, nodes, 4, exclude_closest=True)
    assert np.array_equal(L("flat_idx", np.uint32), fidx.T.ravel())  # slot-major layout
    assert np.array_equal(L("flat_dist"), fdist.T.ravel())
    gidx, gdist = O.filter_disconnected(fidx, fdist, radii)
    assert np.array_equal(L("gidx", np.uint32, 4), gidx)
    assert np.array_equal(L("gdist", cols=4), gdist)
    Tm = L("transforms_moved", cols=16)
    assert np.abs(Tm - T).max() > 1e-3
    mw = O.warp_weights(radii, midx, mdist)
    warped = O.warp(mesh, Tm, midx, mw)
    assert np.array_equal(L("warped_motion_graph", cols=3), warped)
    # WarpField: the same graph, skinning and warp on the device
    assert np.array_equal(L("field_nodes", cols=3), nodes)
    assert np.array_equal(L("field_midx", np.uint32, 6), midx)
    assert np.array_equal(L("field_mw", cols=6), mw)
    assert np.array_equal(L("weights_op", cols=6), mw)
    assert np.array_equal(L("field_gidx", np.uint32, 4), fidx)
    assert np.array_equal(L("warped_field", cols=3), warped)


def test_correspondences_and_gauss_newton(run):
    cfg, L = run["cfg"], run["load"]
    mesh, nodes, radii = L("mesh", cols=3), L("nodes", cols=3), L("radii")
    Tm = L("transforms_moved", cols=16)
    midx = L("midx", np.uint32, 6)
    mw = L("field_mw", cols=6)
    warped = L("warped_field", cols=3)
    corr = O.correspondences(warped, run["K"], run["d1"], run["v1"], cfg["corr_thresh"])
    assert len(corr) > 100 and run["stats"]["correspondences"] == len(corr)
    assert np.array_equal(L("corr", np.int32, 2), corr)
    gidx = L("gidx", np.uint32, 4)
    lam_d, lam_r = np.float32(cfg["lambda_depth"]), np.float32(cfg["lambda_reg"])
    rd = O.residual_depth(corr, warped, run["v1"], run["n1"], lam_d)
    rr = O.residual_reg(nodes, Tm, gidx, lam_r)
    A, b, _ = O.assemble(corr, mesh, midx, mw, run["n1"], lam_d, nodes, gidx, lam_r, rd, rr)
    n = len(nodes)
    assert np.array_equal(L("r_depth"), rd)
    assert np.array_equal(L("r_reg"), rr)
    assert np.array_equal(L("jtj").reshape(6 * n, 6 * n), A)
    jb = L("jtr")
    assert np.abs(jb - b).max() <= 1e-5 * max(1.0, np.abs(b).max())
    x = L("x")
    x_o, _ = O.pcg(A, b, 10)
    assert np.linalg.norm(x - x_o) <= 3e-2 * np.linalg.norm(x_o)
    assert np.array_equal(L("transforms_updated", cols=16), O.update_transforms(Tm, x))


def test_depth_ingest(run):
    """loadDepthFrame (PNG by pattern -> metres), the calibration files, cv::undistort on the device
    and create_xy_lookup_table, from the C++ caller, against the oracle."""
    w, h, has_dist, table_ok, name = run["stats"]["ingest"]
    assert (w, h) == (run["cfg"]["width"], run["cfg"]["height"]) and has_dist and table_ok
    assert name == "frame-000042.depth.png"
    K = np.asarray(run["K"], np.float32)
    metres = O.depth_from_mm(run["mm3"])
    assert np.array_equal(run["load"]("ingest_depth"), metres.ravel())
    d = dict(zip(("k1", "k2", "p1", "p2", "k3", "k4", "k5", "k6"), INGEST_DIST))
    d = {k: float(np.float32(v)) for k, v in d.items()}
    umap = O.undistort_map(K, d, w, h, 0)
    assert np.array_equal(run["load"]("ingest_undistorted"), O.undistort_depth(metres, umap, 0).ravel())
    intr = np.array([K[0, 2], K[1, 2], K[0, 0], K[1, 1]], np.float32)
    assert np.array_equal(run["load"]("ingest_xy").reshape(h, w, 2), O.xy_lookup_table(intr, d, w, h))


def test_dense_operator_sequence(run):
    """The reference's dense Gauss-Newton sequence from the C++ caller (runFill_J_* / runFill_r_*,
    runComputeJTJAndJTrContrib*, runMultiply*, runFillJTJKernel / runFillJTrKernel with a host-side
    stable sort and sequential sums, then linearSolverLUStable): residuals, J^T J and J^T r equal the
    oracle's restatement of that sequence bit for bit (which the reference's own kernels pin), and
    the LU solution solves the system."""
    cfg, L = run["cfg"], run["load"]
    mesh, nodes = L("mesh", cols=3), L("nodes", cols=3)
    Tm = L("transforms_moved", cols=16)
    midx, mw = L("midx", np.uint32, 6), L("field_mw", cols=6)
    corr = L("corr", np.int32, 2)
    gidx = L("gidx", np.uint32, 4)
    lam_d, lam_r = np.float32(cfg["lambda_depth"]), np.float32(cfg["lambda_reg"])
    rd = O.residual_depth(corr, L("warped_field", cols=3), run["v1"], run["n1"], lam_d)
    rr = O.residual_reg(nodes, Tm, gidx, lam_r)
    A, b, _ = O.assemble(corr, mesh, midx, mw, run["n1"], lam_d, nodes, gidx, lam_r, rd, rr)
    n = len(nodes)
    assert np.array_equal(L("r_dense_ops"), np.concatenate([rd, rr]))
    assert np.array_equal(L("jtj_dense_ops").reshape(6 * n, 6 * n), A)
    assert np.array_equal(L("jtr_dense_ops"), b)
    x = L("x_lu").astype(np.float64)
    A64, b64 = A.astype(np.float64), b.astype(np.float64)
    assert np.linalg.norm(A64 @ x - b64) <= 1e-4 * np.linalg.norm(b64)
