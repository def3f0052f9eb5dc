"""Rigid multi-camera reconstruction stream (af::startMeshReconstructionStream,
src/MeshRecontructionStream.cu:115-206): world point cloud of all cameras, camera 0 integrated into a
fresh volume at the volume pose, full mesh -- bit-identical to the oracle's restatement of the same
steps (triangles as a multiset), over two frames (the volume is re-initialised every frame)."""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import pyoracle as O  # noqa: E402

pytestmark = pytest.mark.gpu


def _rot(axis, deg):
    a = math.radians(deg)
    c, s = math.cos(a), math.sin(a)
    if axis == "x":
        return np.array([[1, 0, 0], [0, c, -s], [0, s, c]])
    if axis == "y":
        return np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])
    return np.array([[c, -s, 0], [s, c, 0], [0, 0, 1]])


def _pose(R, t):
    T = np.eye(4)
    T[:3, :3] = R
    T[:3, 3] = t
    return T.astype(np.float32)


def _tri_rows(v):
    t = np.ascontiguousarray(v, np.float32).reshape(-1, 9)
    return t[np.lexsort(t.T[::-1])]


def test_rigid_stream_matches_oracle():
    from volumefusion_gb300 import configs
    from volumefusion_gb300.rigid_stream import RigidStream
    cfg = configs.small_nonrigid(n_frames=6)
    frames = configs.small_frames(cfg)
    K = np.asarray(cfg["K"], np.float32)
    H, W = cfg["height"], cfg["width"]
    c2w = [np.eye(4, dtype=np.float32), _pose(_rot("y", 20), [0.15, 0.0, 0.05]),
           _pose(_rot("x", -15), [0.0, -0.1, 0.02])]
    Ks = [K, K * np.float32(1.0), K]
    _, _, _, cen = O.frame_prep(frames[0], K)
    center = np.asarray(cen, np.float32)
    R = _rot("z", 10).astype(np.float32)
    dims, size, delta = (64, 64, 64), (0.512, 0.512, 0.512), 0.032
    vs = np.float32(0.512) / np.float32(64)
    st = RigidStream(Ks, c2w, W, H, dims, size, delta, center, R)
    for step in range(2):
        mms = [frames[(2 * c + step) % len(frames)] for c in range(3)]
        st.process([torch.from_numpy(m.astype(np.int16)).cuda() for m in mms])
        cloud, verts, faces, tsdf, weights = (x.cpu().numpy() for x in st.outputs())
        # oracle: per camera depth, filter, bilateral, back-projection, camera-to-world
        clouds, depth0 = [], None
        for c, mm in enumerate(mms):
            d = O.filter_depth(O.depth_from_mm(mm), 1.2)
            d = O.bilateral(d, 2, 0.03, 2.0, 0.09)
            if c == 0:
                depth0 = d
            clouds.append(O.transform_points(O.depth_to_mesh(d, Ks[c]).reshape(-1, 3), c2w[c]))
        expect_cloud = np.concatenate(clouds)
        assert cloud.shape == expect_cloud.shape
        assert np.array_equal(cloud, expect_cloud, equal_nan=True)
        t0 = np.full(int(np.prod(dims)), -1.0, np.float32)
        w0 = np.zeros_like(t0)
        O.integrate_rigid(t0, w0, depth0, delta, dims, np.full(3, vs), size, R, center, K)
        assert np.array_equal(tsdf, t0) and np.array_equal(weights, w0)
        ev, ef = O.mc_full(t0, w0, dims, np.full(3, vs), size)
        assert len(verts) == len(ev) > 0
        assert np.array_equal(_tri_rows(verts), _tri_rows(ev))
        assert np.array_equal(faces.ravel(), np.arange(len(verts), dtype=np.int32))
    st.close()


def test_fresh_integration_equals_initialise_then_integrate():
    """afx_integrate_tsdf_fresh (one write-only pass) gives the values and weights of
    DeviceTsdf::initDefault followed by runIntegrateTSDFFromFrameKernel, at a rotated pose."""
    import ctypes as C

    from volumefusion_gb300 import af, configs
    from volumefusion_gb300._lib import check, lib
    cfg, [mm] = configs.rigid_sphere_128()
    depth, _, _, cen = O.frame_prep(mm, cfg["K"])
    d = torch.from_numpy(depth).cuda()
    dims, size = cfg["dims"], cfg["volume_size"]
    vs = configs.voxel_size(cfg)
    R = _rot("y", 12).astype(np.float32)
    S = int(np.prod(dims))
    t1 = torch.full((S,), -1.0, device="cuda")
    w1 = torch.zeros(S, device="cuda")
    af.runIntegrateTSDFFromFrameKernel(t1, w1, d, (cfg["width"], cfg["height"]), cfg["delta"], dims, vs, size, R, cen,
                                       cfg["K"])
    t2 = torch.full((S,), 7.0, device="cuda")  # garbage: every voxel must be written
    w2 = torch.full((S,), 7.0, device="cuda")
    f = lambda a: (C.c_float * len(a))(*[float(x) for x in a])  # noqa: E731
    col = lambda m: f(np.asarray(m, np.float64).T.ravel())  # noqa: E731
    check(lib().afx_integrate_tsdf_fresh(C.c_void_p(t2.data_ptr()), C.c_void_p(w2.data_ptr()), C.c_void_p(d.data_ptr()),
                                         cfg["width"], cfg["height"], C.c_float(cfg["delta"]),
                                         (C.c_int * 3)(*dims), f(vs), f(size), col(R), f(cen), col(cfg["K"]),
                                         C.c_void_p(torch.cuda.current_stream().cuda_stream)), "fresh")
    torch.cuda.synchronize()
    assert int((w1 > 0).sum()) > 1000
    assert torch.equal(t1.view(torch.int32), t2.view(torch.int32))  # bit for bit, signed zeros included
    assert torch.equal(w1.view(torch.int32), w2.view(torch.int32))
