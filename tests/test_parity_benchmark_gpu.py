"""Parity at the benchmarked configurations, against the CPU oracle, frame by frame from a common
state (after each frame the oracle continues from the GPU's volume and warp field):

* the headline workload (640x576 capsule pair, 256^3 at 4 mm, 25 mm graph), frames 0-3: node set,
  point cloud and correspondence count bit-exact; KNN of the point cloud bit-exact (up to exact
  distance ties); transforms within 1e-4; TSDF values and weights within 1e-5 relative except
  where a moved projection changes a voxel's update; marching cubes of the volume identical to the
  oracle's (triangle count and triangle multiset);
* the dense-graph variant (7 mm graph, more than 1024 nodes): everything up to the solve (node
  set, point cloud, correspondences, KNN) bit-exact.  Its normal equations are nearly singular
  (6x6 diagonal blocks with condition numbers up to 3e9: nodes whose only terms are regularisation
  edges), and ten block-Jacobi PCG iterations do not converge on them in binary64 either, so the
  solves of two arithmetics part there; the difference is reported, not bounded.  The PCG path used
  above 1024 nodes is pinned on a well-posed system of that size in test_gauss_newton_gpu.py."""
import json

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import pyoracle as O  # noqa: E402

pytestmark = pytest.mark.gpu


def _session(cfg):
    from volumefusion_gb300.fusion import FusionSession
    return FusionSession(cfg, extract_mesh=True)


def _tri_set(verts):
    """Triangles as a sorted array of rows (9 floats each, as bit patterns)."""
    v = np.ascontiguousarray(np.asarray(verts, np.float32).reshape(-1, 9)).view(np.uint32)
    return v[np.lexsort(v.T[::-1])]


def _knn_matches(nodes, points, k):
    """GPU getKnnData against the oracle: identical except where two nodes are at bit-identical
    distances from a point (equal distances are ordered by node index here, by the k-d tree in the
    reference).  Returns the number of rows that differ."""
    from volumefusion_gb300 import af
    idx_o, dist_o = O.knn(nodes, points, k)
    n = torch.tensor([len(nodes)], dtype=torch.int32, device="cuda")
    idx = torch.empty((len(points), k), dtype=torch.int32, device="cuda")
    dist = torch.empty((len(points), k), dtype=torch.float32, device="cuda")
    af.getKnnData(idx, dist, torch.from_numpy(nodes).cuda(), n, torch.from_numpy(points).cuda())
    idx = idx.cpu().numpy().view(np.uint32)
    dist = dist.cpu().numpy()
    assert np.array_equal(dist, dist_o)
    differ = np.any(idx != idx_o, axis=1)
    for r in np.nonzero(differ)[0]:  # every differing row is a tie
        assert sorted(idx[r]) == sorted(idx_o[r]) or len(set(dist[r])) < k, r
    return int(differ.sum())


def _track(cfg, frames, check_mesh=False, min_nodes=0, solve_bound=1e-4):
    s = _session(cfg)
    o = O.Fusion(cfg)
    report = []
    ident = np.eye(4, dtype=np.float32).T.ravel()
    for i, mm in enumerate(frames):
        s.process(mm)
        o.process(mm)
        st = s.stats()
        assert st["error"] == 0, st
        t, w = (x.cpu().numpy() for x in s.tsdf())
        row = {"frame": i}
        if i == 0:
            assert np.array_equal(t, o.tsdf()) and np.array_equal(w, o.weights())
        else:
            assert st["n_nodes"] == o.num_nodes, (i, st, o.num_nodes)
            assert st["n_nodes"] >= min_nodes, (i, st["n_nodes"])
            assert st["mesh_points"] == o.mesh_size, (i, st, o.mesh_size)
            pc = s.point_cloud().cpu().numpy()
            assert np.array_equal(pc, o.mesh())
            nodes, _, T = s.graph()
            nodes = nodes.cpu().numpy()
            assert np.array_equal(nodes, o.nodes())
            assert st["correspondences"] == o.num_corr, (i, st, o.num_corr)
            row["knn_ties"] = _knn_matches(nodes, pc, int(cfg["knn"]))
            T = T.cpu().numpy()
            row["nodes"] = int(st["n_nodes"])
            row["gn_iterations"] = int(st["gn_iterations_done"])
            row["motion"] = float(np.abs(T - ident).max())
            dT = float(np.abs(T - o.transforms()).max())
            row["warp_max"] = dT
            ot, ow = o.tsdf(), o.weights()
            bad = (np.abs(t - ot) > 1e-5 * np.maximum(1.0, np.abs(ot))) | (w != ow)
            row["tsdf_voxels_outside_1e-5"] = int(bad.sum())
            row["tsdf_updated"] = int((w > 0).sum())
            if solve_bound is not None:
                assert dT < solve_bound, (i, dT)
                assert bad.mean() < 1e-3, (i, int(bad.sum()))
            o.set_transforms(T)
        if check_mesh:
            v, _ = s.mesh()
            c = s.centroid().cpu().numpy()
            size = np.asarray(cfg["volume_size"], np.float32)
            vs = size / np.asarray(cfg["dims"], np.float32)
            mv, _ = O.mc_full(t, w, cfg["dims"], vs, size)
            mv = O.translate(mv, c)  # the output mesh is translated by the frame-0 centroid
            assert len(v) == len(mv), (i, len(v), len(mv))
            assert np.array_equal(_tri_set(v.cpu().numpy()), _tri_set(mv))
            row["triangles"] = len(v) // 3
        o.set_tsdf(t, w)
        report.append(row)
    s.close()
    o.close()
    return report


def test_headline_capsules_256_tracks_oracle():
    from volumefusion_gb300 import configs
    cfg = configs.nonrigid_capsules_256(n_frames=30)
    rows = _track(cfg, configs.capsule_frames(cfg, range(4)), check_mesh=True)
    print("\nPARITY_HEADLINE " + json.dumps(rows))


def test_dense_graph_tracks_oracle_up_to_the_solve():
    """More than 1024 nodes (the Gauss-Newton loop's global-memory path), every third frame of the
    sequence: graph, point cloud, correspondences and KNN bit-exact at each frame."""
    from volumefusion_gb300 import configs
    cfg = configs.nonrigid_capsules_256(n_frames=30)
    cfg["graph_radius"] = 0.007
    rows = _track(cfg, configs.capsule_frames(cfg, range(0, 24, 3)), min_nodes=1025, solve_bound=None)
    print("\nPARITY_DENSE_GRAPH " + json.dumps(rows))
