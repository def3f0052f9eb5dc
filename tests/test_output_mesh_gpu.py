"""The session's output mesh as af::runVolumeFusion leaves it (src/VolumeFusion.cu:744-762): the
full marching-cubes mesh of the frame's volume, translated by the frame-0 centroid, and with
warp_mesh (settings.isMeshWarped) warped into the live frame by details::warpMeshGPU (:75-110).
Checked against the oracle on the GPU's own volume and graph; triangles are compared as a multiset
(their order comes from atomics in the reference too)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import pyoracle as O  # noqa: E402

pytestmark = pytest.mark.gpu


def _tri_rows(v):
    t = np.ascontiguousarray(v, np.float32).reshape(-1, 9)
    return t[np.lexsort(t.T[::-1])]


def test_output_mesh_translated_and_warped():
    from volumefusion_gb300 import configs
    from volumefusion_gb300.fusion import FusionSession
    cfg = configs.small_nonrigid(n_frames=5)
    frames = configs.small_frames(cfg)
    plain = FusionSession(cfg)
    warped = FusionSession(dict(cfg, warp_mesh=True))
    for mm in frames:
        plain.process(mm)
        warped.process(mm)
        assert plain.stats()["error"] == 0 and warped.stats()["error"] == 0
    t, w = (x.cpu().numpy() for x in plain.tsdf())
    c = plain.centroid().cpu().numpy()
    verts, faces = O.mc_full(t, w, cfg["dims"], configs.voxel_size(cfg), cfg["volume_size"])
    expect = O.translate(verts, c)
    v0, f0 = plain.mesh()
    v0 = v0.cpu().numpy()
    assert len(v0) == len(expect) and len(v0) > 0
    assert np.array_equal(_tri_rows(v0), _tri_rows(expect))
    # warp: K nearest graph nodes of each output vertex, skinning weights, committed transforms
    nodes, radii, T = (x.cpu().numpy() for x in plain.graph())
    idx, dist = O.knn(nodes, v0, cfg["knn"])
    ww = O.warp_weights(radii, idx, dist)
    expect_w = O.warp(v0, T, idx, ww)
    v1, _ = warped.mesh()
    v1 = v1.cpu().numpy()
    assert len(v1) == len(v0)
    assert np.array_equal(_tri_rows(v1), _tri_rows(expect_w))
    assert not np.array_equal(_tri_rows(v1), _tri_rows(v0))  # the graph has moved
    plain.close()
    warped.close()


@pytest.mark.parametrize("precision", ["fp32", "fp16"])
def test_session_volume_and_mesh_files(tmp_path, precision):
    """afx_fusion_save_volume writes the session's volume in TSDFVolume::save's format;
    afx_fusion_load_volume brings it back into a fresh session unchanged (FP16 values round-trip
    exactly through the widened file); afx_fusion_save_mesh_ply writes the frame's output mesh."""
    from volumefusion_gb300 import configs, formats
    from volumefusion_gb300.fusion import FusionSession
    cfg = dict(configs.small_nonrigid(n_frames=3), precision=precision)
    frames = configs.small_frames(cfg)
    s = FusionSession(cfg)
    for mm in frames:
        s.process(mm)
    t, w = (x.cpu().numpy() for x in s.tsdf())
    path = tmp_path / "vol.tsdf"
    s.save_volume(path)
    t2, w2, dims, size, vs, delta = formats.load_tsdf(path)
    assert np.array_equal(t2.ravel(), t) and np.array_equal(w2.ravel(), w)
    assert list(dims) == list(cfg["dims"]) and np.array_equal(vs, configs.voxel_size(cfg))
    assert delta == np.float32(cfg["delta"])
    s2 = FusionSession(cfg)
    s2.load_volume(path)
    t3, w3 = (x.cpu().numpy() for x in s2.tsdf())
    assert np.array_equal(t3, t) and np.array_equal(w3, w)
    ply = tmp_path / "mesh.ply"
    s.save_mesh_ply(ply)
    v, f = s.mesh()
    head = ply.read_text().split("end_header\n")[0]
    assert "element vertex %d\n" % len(v) in head and "element face %d\n" % len(f) in head
    s.close()
    s2.close()
