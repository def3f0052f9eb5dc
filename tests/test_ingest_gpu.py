"""Depth undistortion on the GPU against the oracle, and the Brown-Conrady ray table against the
reference's own src/CameraCalibration.cpp (golden fixture):

  - the per-pixel maps of cv::undistort (fixed point, stripes) and of initUndistortRectifyMap(CV_32FC1)
    + INTER_NEAREST, word for word;
  - their application to a depth image, bit for bit;
  - a session with a distorted camera (af::loadProcessFrame undistorts before the filter) frame by
    frame against the oracle's driver, and the rigid stream with a distorted camera (the unfiltered
    metres remapped replace the filtered frame, src/MeshRecontructionStream.cu:91-101)."""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import pyoracle as O  # noqa: E402

pytestmark = pytest.mark.gpu

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

DISTORTIONS = [
    dict(k1=-0.05, k2=0.01, p1=5e-4, p2=-3e-4),
    dict(k1=0.6, k2=-0.2, k3=0.05, k4=0.7, k5=-0.1, k6=0.03, p1=2e-3, p2=1e-3),  # rational model
    dict(k1=-0.4, k2=0.2, p1=-4e-3, p2=3e-3),  # strong barrel: many pixels map outside the image
]


def _K(w, h):
    return np.array([[0.8 * w, 0, w / 2 - 0.5], [0, 0.8 * w + 1.5, h / 2 + 0.25], [0, 0, 1]], np.float32)


@pytest.mark.parametrize("mode", [0, 1])
def test_undistort_maps_and_remap_match_oracle(mode):
    from volumefusion_gb300 import ingest
    rng = np.random.default_rng(mode)
    for (w, h) in ((97, 61), (640, 576)):
        K = _K(w, h)
        src = (rng.random((h, w)) * 3).astype(np.float32)
        src[rng.random((h, w)) < 0.1] = 0
        for d in DISTORTIONS:
            u = ingest.Undistorter(K, d, w, h, mode=mode)
            torch.cuda.synchronize()
            expect = O.undistort_map(K, d, w, h, mode)
            got = u.map.cpu().numpy().view(np.uint32)
            assert np.array_equal(got, expect), (w, h, d)
            out = u(torch.from_numpy(src).cuda()).cpu().numpy()
            ref = O.undistort_depth(src, expect, mode)
            assert np.array_equal(out.view(np.uint32), ref.view(np.uint32)), (w, h, d)
            assert (out == 0).mean() < 0.6


def test_xy_table_and_projection_match_reference_fixture():
    from volumefusion_gb300 import ingest
    g = np.load(os.path.join(G, "camera_calibration.npz"))
    names = ("k1", "k2", "k3", "k4", "k5", "k6", "codx", "cody", "p1", "p2")
    for i in range(int(g["n"])):
        intr, dist = g["intr%d" % i], dict(zip(names, g["dist%d" % i].tolist()))
        W, H = (int(v) for v in g["size%d" % i])
        table = ingest.xy_lookup_table(intr, dist, W, H).cpu().numpy()
        assert np.array_equal(table.view(np.uint32), g["table%d" % i].view(np.uint32)), i
        pts, valid = ingest.unproject_points(torch.from_numpy(g["px%d" % i]).cuda(),
                                             torch.from_numpy(g["depth%d" % i]).cuda(), intr, dist)
        assert np.array_equal(pts.cpu().numpy().view(np.uint32), g["unproj%d" % i].view(np.uint32)), i
        assert np.array_equal(valid.cpu().numpy(), g["unproj_valid%d" % i]), i
        init = torch.full((len(valid), 2), -7.0, device="cuda")
        px, valid = ingest.project_points(torch.from_numpy(g["pts%d" % i]).cuda(), intr, dist, out=init)
        assert np.array_equal(px.cpu().numpy().view(np.uint32), g["proj%d" % i].view(np.uint32)), i
        assert np.array_equal(valid.cpu().numpy(), g["proj_valid%d" % i]), i


def test_session_with_distorted_camera_tracks_oracle():
    """af::loadProcessFrame with depthDistortion.txt present: each frame's metres go through
    cv::undistort before the filter.  Frame 0 is bit-exact; later frames are compared from a common
    state as in the undistorted session test."""
    from volumefusion_gb300 import configs
    from volumefusion_gb300.fusion import FusionSession
    cfg = dict(configs.small_nonrigid(n_frames=4))
    cfg["distortion"] = DISTORTIONS[0]
    frames = configs.small_frames(cfg)
    s = FusionSession(cfg, extract_mesh=True)
    o = O.Fusion(cfg)
    plain = O.Fusion(dict(cfg, distortion=None))
    for i, mm in enumerate(frames):
        s.process(mm)
        o.process(mm)
        st = s.stats()
        assert st["error"] == 0, st
        t, w = s.tsdf()
        t, w = t.cpu().numpy(), w.cpu().numpy()
        if i == 0:
            plain.process(mm)
            assert np.array_equal(s.centroid().cpu().numpy(), o.centroid())
            assert not np.array_equal(o.centroid(), plain.centroid())  # the undistortion took effect
            assert np.array_equal(t, o.tsdf()) and np.array_equal(w, o.weights())
        else:
            assert st["n_nodes"] == o.num_nodes and st["mesh_points"] == o.mesh_size, (i, st)
            assert np.array_equal(s.point_cloud().cpu().numpy(), o.mesh())
            assert st["correspondences"] == o.num_corr, (i, st, o.num_corr)
            nodes, radii, T = s.graph()
            dT = np.abs(T.cpu().numpy() - o.transforms()).max()
            assert dT < 1e-4, (i, dT)
            o.set_transforms(T.cpu().numpy())
        o.set_tsdf(t, w)
    s.close()


def test_rigid_stream_with_distorted_camera_matches_oracle():
    from volumefusion_gb300 import configs
    from volumefusion_gb300.rigid_stream import RigidStream
    cfg = configs.small_nonrigid(n_frames=4)
    frames = configs.small_frames(cfg)
    K = np.asarray(cfg["K"], np.float32)
    H, W = cfg["height"], cfg["width"]
    c2w = [np.eye(4, dtype=np.float32), np.eye(4, dtype=np.float32)]
    c2w[1][:3, 3] = [0.1, 0.0, 0.02]
    _, _, _, cen = O.frame_prep(frames[0], K)
    dims, size, delta = (64, 64, 64), (0.512, 0.512, 0.512), 0.032
    vs = np.float32(0.512) / np.float32(64)
    R = np.eye(3, dtype=np.float32)
    dist = [None, DISTORTIONS[0]]
    st = RigidStream([K, K], c2w, W, H, dims, size, delta, np.asarray(cen, np.float32), R, distortions=dist)
    umap = O.undistort_map(K, DISTORTIONS[0], W, H, 1)
    mms = [frames[0], frames[2]]
    st.process([torch.from_numpy(m.astype(np.int16)).cuda() for m in mms])
    cloud, verts, faces, tsdf, weights = (x.cpu().numpy() for x in st.outputs())
    clouds = []
    for c, mm in enumerate(mms):
        metres = O.depth_from_mm(mm).reshape(H, W)
        d = O.undistort_depth(metres, umap, 1) if dist[c] else O.filter_depth(metres, 1.2)
        d = O.bilateral(d, 2, 0.03, 2.0, 0.09)
        clouds.append(O.transform_points(O.depth_to_mesh(d, K).reshape(-1, 3), c2w[c]))
    expect = np.concatenate(clouds)
    assert np.array_equal(cloud, expect, equal_nan=True)
    t0 = np.full(int(np.prod(dims)), -1.0, np.float32)
    w0 = np.zeros_like(t0)
    d0 = O.bilateral(O.filter_depth(O.depth_from_mm(mms[0]).reshape(H, W), 1.2), 2, 0.03, 2.0, 0.09)
    O.integrate_rigid(t0, w0, d0, delta, dims, np.full(3, vs), size, R, np.asarray(cen, np.float32), K)
    assert np.array_equal(tsdf, t0) and np.array_equal(weights, w0)
    st.close()
