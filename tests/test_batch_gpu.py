"""Batched form (afx_batch_*): sessions of uneven size advanced one frame each per graph launch give
the same volumes, graphs and statistics as the same sessions processed one by one; the
marching-cubes tiles the autotuner chooses between give the same point clouds and triangle sets."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def _mix():
    from volumefusion_gb300 import configs
    a = configs.small_nonrigid(n_frames=8)
    b = configs.small_nonrigid(n_frames=8, dims=(48, 48, 48), voxel=0.011)
    c = configs.small_nonrigid(n_frames=8, dims=(80, 80, 80), voxel=0.0064)
    c["graph_radius"] = 0.04
    fa, fb, fc = configs.small_frames(a), configs.small_frames(b)[::-1], configs.small_frames(c)
    return [(a, fa), (b, fb), (c, fc)]


def _state(s):
    torch.cuda.synchronize()
    t, w = s.tsdf()
    nodes, _, T = s.graph()
    return [x.cpu().numpy() for x in (t, w, nodes, T, s.point_cloud())]


def test_batch_equals_sessions_alone():
    from volumefusion_gb300.batch import Batch
    from volumefusion_gb300.fusion import FusionSession
    mix = _mix()
    alone, alone_stats = [], []
    for cfg, frames in mix:
        s = FusionSession(cfg)
        for mm in frames:
            s.process(mm)
        alone_stats.append(s.stats())
        alone.append(_state(s))
        s.close()
    sessions = [FusionSession(cfg) for cfg, _ in mix]
    batch = Batch(sessions)
    dev = [[torch.from_numpy(mm.astype(np.int16)).cuda() for mm in frames] for _, frames in mix]
    n = len(mix[0][1])
    for i in range(n):
        batch.process([dev[k][i] for k in range(len(mix))])
    st = batch.stats()
    assert batch.graph_launches() == n - 3  # frames 3.. of every session in one launch each
    for k, s in enumerate(sessions):
        assert st[k]["error"] == 0 and st[k]["frame"] == alone_stats[k]["frame"], (st[k], alone_stats[k])
        for key in ("n_nodes", "mesh_points", "correspondences", "mesh_faces"):
            assert st[k][key] == alone_stats[k][key], (k, key, st[k], alone_stats[k])
        for x, y in zip(_state(s), alone[k]):
            assert np.array_equal(x, y), k
    batch.close()
    for s in sessions:
        s.close()


def test_every_mc_tile_gives_the_same_surface_and_autotune_picks_one():
    from volumefusion_gb300 import configs
    from volumefusion_gb300.fusion import FusionSession
    cfg = configs.small_nonrigid(n_frames=5)
    frames = configs.small_frames(cfg)
    ref = None
    for tile in range(7):
        s = FusionSession(cfg)
        s.set_tile(tile)
        for mm in frames:
            s.process(mm)
        assert s.stats()["error"] == 0
        v, f = s.mesh()
        tris = v.cpu().numpy().reshape(-1, 9)
        tris = tris[np.lexsort(tris.T[::-1])]  # the triangle multiset, rows in a fixed order
        out = _state(s) + [tris]
        if ref is None:
            ref = out
        else:
            for x, y in zip(out, ref):
                assert np.array_equal(x, y), tile
        if tile == 5:
            chosen, ms = s.autotune()
            print("\nMC_TILE_MS", chosen, [round(m, 4) for m in ms])
            assert 0 <= chosen < 6 and s.tile() == chosen and all(m > 0 for m in ms), (chosen, ms)
            s.process(frames[-1])  # graphs are captured again with the chosen tile
            assert s.stats()["error"] == 0
        s.close()
