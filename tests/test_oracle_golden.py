"""The CPU oracle against golden vectors produced by the reference's own CPU code.

Fixtures come from tests/golden/make_golden.py (TSDFVolume::integrate, MarchingCubes,
af::buildGraph, af::getKnnData, af::filterDisconnected, MotionGraph::warp compiled from
the reference sources).  Rules follow the reference's tests: TSDF within 4 ULP
(TSDFIntegrationTest.cu:56-59), marching-cubes vertex sets exact
(MarchingCubesTest.cu:104-114), graph nodes and KNN indices exact.
"""
import os

import numpy as np
import pytest

from oracle import pyoracle as O

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(G, name))


def ulp_diff(a, b):
    a = np.ascontiguousarray(a, np.float32).view(np.int32).astype(np.int64)
    b = np.ascontiguousarray(b, np.float32).view(np.int32).astype(np.int64)
    a = np.where(a < 0, np.int64(-2**31) - a, a)
    b = np.where(b < 0, np.int64(-2**31) - b, b)
    return np.abs(a - b)


def test_rigid_integration_matches_reference_cpu():
    g = load("integrate_sphere.npz")
    depth = O.depth_from_mm(g["mm"])
    depth[depth == 0] = np.inf  # the GPU path marks missing depth with +inf, the CPU class with 0
    S = int(np.prod(g["dims"]))
    t = np.full(S, -1, np.float32)
    w = np.zeros(S, np.float32)
    vs = g["size"] / g["dims"].astype(np.float32)
    O.integrate_rigid(t, w, depth, float(g["delta"]), g["dims"], vs, g["size"], np.eye(3), g["centroid"], g["K"])
    assert np.array_equal(w, g["weights"])
    assert (w > 0).sum() > 10000
    assert ulp_diff(t, g["tsdf"]).max() <= 4


def test_marching_cubes_matches_reference_cpu():
    g = load("marching_cubes.npz")
    vs = g["size"] / g["dims"].astype(np.float32)
    pc = O.mc_pointcloud(g["tsdf"], g["weights"], g["dims"], vs, g["size"])
    # same cube order and edge order as computePointCloud: identical arrays
    assert np.array_equal(pc, g["pointcloud"])
    v, f = O.mc_full(g["tsdf"], g["weights"], g["dims"], vs, g["size"])
    assert np.array_equal(v, g["iso_verts"])
    assert np.array_equal(f, g["iso_faces"])
    # MarchingCubesTest: deduplicated iso-surface vertices == deduplicated point cloud
    assert np.array_equal(O.sort_unique(v), O.sort_unique(pc))


def test_graph_build_matches_reference_cpu():
    g = load("graph_knn.npz")
    nodes, radii, T = O.build_graph(g["mesh"], 4, float(g["radius"]))
    assert np.array_equal(nodes, g["nodes"])
    assert np.array_equal(radii, g["radii"])
    assert np.array_equal(T, g["transforms"])
    n2, r2, T2 = O.build_graph(g["mesh2"], 4, float(g["radius"]), g["nodes"], g["radii"], g["T_rand"])
    assert len(n2) > len(g["nodes"])
    assert np.array_equal(n2, g["nodes2"])
    assert np.array_equal(T2, g["transforms2"])


def assert_knn_equal_up_to_ties(idx, dist, ref_idx, ref_dist, max_tied_rows):
    """Distances bit-identical slot by slot; indices identical except among nodes at
    bit-identical distance, which we order by node index and the reference by its k-d tree
    traversal order (nanoflann KNNResultSet::addPoint keeps the first-found of equals)."""
    assert np.array_equal(dist, ref_dist)
    bad = np.where((idx != ref_idx).any(axis=1))[0]
    assert len(bad) <= max_tied_rows
    for i in bad:
        for s in np.where(idx[i] != ref_idx[i])[0]:
            d = dist[i, s]
            ties = (dist[i] == d).sum()
            # the differing slot must hold a distance shared with another slot or sitting at the
            # K-th boundary (where the reference dropped an equally distant node)
            assert ties > 1 or s == idx.shape[1] - 1, (i, idx[i], ref_idx[i], dist[i])


@pytest.mark.parametrize("k", [4, 6])
def test_mesh_knn_matches_reference_cpu(k):
    g = load("graph_knn.npz")
    idx, dist = O.knn(g["nodes"], g["mesh"], k)
    assert_knn_equal_up_to_ties(idx, dist, g["k%d_idx" % k], g["k%d_dist" % k], max_tied_rows=len(idx) // 100)


def test_graph_knn_and_filter_match_reference_cpu():
    g = load("graph_knn.npz")
    idx, dist = O.knn(g["nodes"], g["nodes"], 8, exclude_closest=True)
    assert_knn_equal_up_to_ties(idx, dist, g["g8_idx"], g["g8_dist"], max_tied_rows=len(idx) // 10)
    fi, fd = O.filter_disconnected(idx, dist, g["radii"])
    assert np.array_equal(fi, g["g8f_idx"])
    assert np.array_equal(fd, g["g8f_dist"])


def test_warp_matches_reference_cpu():
    # MotionGraph::warp evaluates the skinning weight in double precision; the GPU path (and
    # the oracle) evaluate it in binary32, so positions agree to a few ULP, not bit for bit.
    g = load("warp.npz")
    idx, dist = O.knn(g["nodes"], g["points"], 4)
    w = O.warp_weights(g["radii"], idx, dist)
    out = O.warp(g["points"], g["transforms"], idx, w)
    np.testing.assert_allclose(out, g["warped"], rtol=0, atol=2e-6)
    idx, dist = O.knn(g["kat_nodes"], g["kat_points"], 3)
    w = O.warp_weights(g["kat_radii"], idx, dist)
    out = O.warp(g["kat_points"], g["kat_transforms"], idx, w)
    np.testing.assert_allclose(out, g["kat_warped"], rtol=1e-6, atol=1e-6)
