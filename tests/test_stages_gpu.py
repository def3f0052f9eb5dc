"""Per-stage parity of the sm_103a kernels against the CPU oracle (bit-exact where the
stage is integer/index work or a fixed sequence of IEEE binary32 operations).

All calls go through the C ABI (libafx.so) via volumefusion_gb300.af."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import pyoracle as O  # noqa: E402

pytestmark = pytest.mark.gpu


def cu(a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a))
    if dtype is not None:
        t = t.to(dtype)
    return t.cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


@pytest.fixture(scope="module")
def af():
    from volumefusion_gb300 import af as _af
    return _af


@pytest.fixture(scope="module")
def frames():
    from volumefusion_gb300 import synth
    sphere, Ks = synth.sphere_frame()
    cap, Kc = synth.capsule_pair_frame(20, width=640, height=576, fx=504.0, fy=504.0, cx=320.0, cy=288.0)
    return [(sphere, Ks), (cap, Kc)]


def test_frame_prep_bit_exact(af, frames):
    for mm, K in frames:
        d_o, v_o, n_o, c_o = O.frame_prep(mm, K)
        d, v, n, c = af.loadProcessFrame(cu(mm.astype(np.int16)), K)
        assert np.array_equal(host(d), d_o)
        assert np.array_equal(host(v), v_o)
        assert np.array_equal(host(n), n_o)
        assert np.array_equal(host(c), c_o)
        assert (d_o < np.inf).sum() > 1000


def test_stage_kernels_bit_exact(af, frames):
    mm, K = frames[1]
    h, w = mm.shape
    d0 = O.filter_depth(O.depth_from_mm(mm), 1.2)
    dg = cu(O.depth_from_mm(mm))
    af.runFilterDepthKernel(dg, 1.2)
    assert np.array_equal(host(dg), d0)
    b0 = O.bilateral(d0, 2, float(np.float32(0.03)), 2.0, 0.09)
    bg = torch.empty_like(dg)
    af.bilateralFilterTextureOpmShared(bg, dg, h, w, 2, float(np.float32(0.03)), 2.0, 0.09)
    assert np.array_equal(host(bg), b0)
    v0 = O.depth_to_mesh(b0, K)
    vg = torch.empty((h, w, 3), dtype=torch.float32, device="cuda")
    af.runDepthToMeshKernel(vg, bg, w, h, K)
    assert np.array_equal(host(vg), v0)
    n0 = O.normals(v0, 1.3, 2.1)
    ng = torch.empty_like(vg)
    af.runDepthVerticesNormalsKernel(ng, vg, bg, h, w, (1.3, 2.1))
    assert np.array_equal(host(ng), n0)


def test_rigid_integration_bit_exact(af, frames):
    for (mm, K), dims, size, delta in ((frames[0], (128, 128, 128), 0.512, 0.016),
                                       (frames[1], (96, 80, 64), 0.6, 0.02)):
        d, _, _, c = O.frame_prep(mm, K)
        dims = np.array(dims, np.int32)
        vol = np.array([size] * 3, np.float32)
        vs = vol / dims.astype(np.float32)
        S = int(np.prod(dims))
        t0 = np.full(S, -1, np.float32)
        w0 = np.zeros(S, np.float32)
        for rep in range(2):  # second pass exercises the running average
            O.integrate_rigid(t0, w0, d, delta, dims, vs, vol, np.eye(3), c, K)
        tg = cu(np.full(S, -1, np.float32))
        wg = cu(np.zeros(S, np.float32))
        for rep in range(2):
            af.runIntegrateTSDFFromFrameKernel(tg, wg, cu(d), (mm.shape[1], mm.shape[0]), delta, dims, vs, vol,
                                               np.eye(3), c, K)
        assert np.array_equal(host(wg), w0)
        assert np.array_equal(host(tg), t0)
        assert (w0 > 0).sum() > 1000


def _sorted_rows(a):
    a = np.ascontiguousarray(a)
    return a[np.lexsort(a.T[::-1])]


def test_marching_cubes_and_sort_unique(af):
    g = np.load(__import__("os").path.join(__import__("os").path.dirname(__file__), "golden", "marching_cubes.npz"))
    dims, size = g["dims"], g["size"]
    vs = size / dims.astype(np.float32)
    pc_o = O.mc_pointcloud(g["tsdf"], g["weights"], dims, vs, size)
    cap = len(pc_o) + 1000
    pts = torch.zeros((cap, 3), dtype=torch.float32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    af.runMarchingCubesMeshKernel(pts, cnt, cu(g["tsdf"]), cu(g["weights"]), dims, vs, size)
    n = int(cnt.item())
    assert n == len(pc_o)
    assert np.array_equal(_sorted_rows(host(pts)[:n]), _sorted_rows(pc_o))
    # sort + unique equals the reference's thrust::sort/unique (and the golden computePointCloud)
    af.sortUnique(pts, cnt)
    u = host(pts)[:int(cnt.item())]
    assert np.array_equal(u, O.sort_unique(pc_o))
    assert np.array_equal(u, O.sort_unique(g["pointcloud"]))
    # full mesh: same multiset of triangles as the reference's computeIsoSurface
    v_o, f_o = O.mc_full(g["tsdf"], g["weights"], dims, vs, size)
    mv = torch.zeros((len(v_o) + 300, 3), dtype=torch.float32, device="cuda")
    mf = torch.zeros((len(f_o) + 100, 3), dtype=torch.int32, device="cuda")
    nv = torch.zeros(1, dtype=torch.int32, device="cuda")
    nf = torch.zeros(1, dtype=torch.int32, device="cuda")
    af.runMarchingCubesFullKernel(mv, nv, mf, nf, cu(g["tsdf"]), cu(g["weights"]), dims, vs, size)
    assert int(nf.item()) == len(f_o) and int(nv.item()) == len(v_o)
    tri_g = host(mv)[:len(v_o)].reshape(-1, 9)
    tri_o = v_o.reshape(-1, 9)
    assert np.array_equal(_sorted_rows(tri_g), _sorted_rows(tri_o))
    assert np.array_equal(_sorted_rows(tri_g), _sorted_rows(g["iso_verts"].reshape(-1, 9)))
    fg = host(mf)[:len(f_o)]
    assert np.array_equal(fg, np.arange(3 * len(f_o), dtype=np.int32).reshape(-1, 3))


def test_graph_knn_warp_bit_exact(af):
    g = np.load(__import__("os").path.join(__import__("os").path.dirname(__file__), "golden", "graph_knn.npz"))
    mesh = g["mesh"]
    radius = float(g["radius"])
    cap = 4096
    nodes = torch.zeros((cap, 3), dtype=torch.float32, device="cuda")
    radii = torch.zeros(cap, dtype=torch.float32, device="cuda")
    T = torch.zeros((cap, 16), dtype=torch.float32, device="cuda")
    nn = torch.zeros(1, dtype=torch.int32, device="cuda")
    mcount = cu(np.array([len(mesh)], np.int32))
    af.buildGraph(nodes, radii, T, nn, cu(mesh), mcount, 4, radius)
    n = int(nn.item())
    no, ro, To = O.build_graph(mesh, 4, radius)
    assert n == len(no)
    assert np.array_equal(host(nodes)[:n], no)
    assert np.array_equal(host(T)[:n], To)
    assert np.array_equal(host(nodes)[:n], g["nodes"])  # the reference's af::buildGraph
    # incremental build with transformed nodes (transform copy of the nearest node)
    T.zero_()
    T[:n] = cu(g["T_rand"])
    af.buildGraph(nodes, radii, T, nn, cu(g["mesh2"]), cu(np.array([len(g["mesh2"])], np.int32)), 4, radius)
    n2 = int(nn.item())
    assert n2 == len(g["nodes2"])
    assert np.array_equal(host(nodes)[:n2], g["nodes2"])
    assert np.array_equal(host(T)[:n2], g["transforms2"])
    # KNN: mesh -> 4 and 6 nodes, node -> 8 nodes excluding itself (ties ordered by index, as the oracle)
    nodes_g = cu(no)
    n_g = cu(np.array([len(no)], np.int32))
    for k in (4, 6):
        idx = torch.empty((len(mesh), k), dtype=torch.int32, device="cuda")
        dist = torch.empty((len(mesh), k), dtype=torch.float32, device="cuda")
        af.getKnnData(idx, dist, nodes_g, n_g, cu(mesh))
        io, do = O.knn(no, mesh, k)
        assert np.array_equal(host(idx).view(np.uint32), io)
        assert np.array_equal(host(dist), do)
    gi = torch.empty((len(no), 8), dtype=torch.int32, device="cuda")
    gd = torch.empty((len(no), 8), dtype=torch.float32, device="cuda")
    af.getKnnData(gi, gd, nodes_g, n_g, nodes_g, excludeClosest=True)
    gio, gdo = O.knn(no, no, 8, exclude_closest=True)
    assert np.array_equal(host(gi).view(np.uint32), gio)
    af.filterDisconnected(gi, gd, n_g, cu(ro))
    fio, fdo = O.filter_disconnected(gio, gdo, ro)
    assert np.array_equal(host(gi).view(np.uint32), fio)
    assert np.array_equal(host(gd), fdo)
    # weights and warp with non-trivial transforms
    idx = torch.empty((len(mesh), 4), dtype=torch.int32, device="cuda")
    dist = torch.empty((len(mesh), 4), dtype=torch.float32, device="cuda")
    af.getKnnData(idx, dist, nodes_g, n_g, cu(mesh))
    w = torch.empty_like(dist)
    af.runComputeWarpWeightsKernel(w, cu(ro), idx, dist, len(mesh), n_g)
    io, do = O.knn(no, mesh, 4)
    wo = O.warp_weights(ro, io, do)
    assert np.array_equal(host(w), wo)
    out = torch.empty((len(mesh), 3), dtype=torch.float32, device="cuda")
    af.runWarpKernel(out, cu(mesh), cu(g["T_rand"]), idx, w, len(mesh))
    assert np.array_equal(host(out), O.warp(mesh, g["T_rand"], io, wo))


def test_correspondences_bit_exact(af, frames):
    mm, K = frames[1]
    d, v, n, c = O.frame_prep(mm, K)
    pts = v.reshape(-1, 3)
    pts = pts[pts[:, 2] > 0][::7] + np.array([0.002, -0.001, 0.003], np.float32)
    corr_o = O.correspondences(pts, K, d, v, 0.01)
    corr = torch.empty((len(pts), 2), dtype=torch.int32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    af.runCorrespondencePairsKernel(corr, cnt, cu(pts), len(pts), K, cu(d), (mm.shape[0], mm.shape[1]), cu(v), 0.01)
    m = int(cnt.item())
    assert m == len(corr_o) and m > 100
    assert np.array_equal(host(corr)[:m], corr_o)


def test_voxel_warp_and_warped_integration_bit_exact(af, frames):
    from volumefusion_gb300 import configs
    mm, K = frames[1]
    d, v, n, c = O.frame_prep(mm, K)
    dims = np.array([64, 64, 48], np.int32)
    size = np.array([0.512, 0.512, 0.384], np.float32)
    vs = size / dims.astype(np.float32)
    S = int(np.prod(dims))
    t0 = np.full(S, -1, np.float32)
    w0 = np.zeros(S, np.float32)
    O.integrate_rigid(t0, w0, d, 0.016, dims, vs, size, np.eye(3), c, K)
    pc = O.sort_unique(O.mc_pointcloud(t0, w0, dims, vs, size))
    mesh = O.translate(pc, c)
    nodes, radii, T = O.build_graph(mesh, 4, 0.025)
    rng = np.random.default_rng(3)
    T = T.copy()
    T[:, 12:15] += rng.normal(0, 0.004, (len(T), 3)).astype(np.float32)
    per = np.array([2 * (int(np.float32(0.025) / vs[i]) + 1) + 1 for i in range(3)], np.int32)
    nt = O.translate(nodes, -c)
    for k in (4, 6):
        kidx, kdist, kcnt = O.tsdf_knn(nt, radii, vs, size, dims, per, k)
        gi = torch.empty((S, k), dtype=torch.int32, device="cuda")
        gd = torch.empty((S, k), dtype=torch.float32, device="cuda")
        gc = torch.empty(S, dtype=torch.int32, device="cuda")
        af.runTsdfKNNGraph(gi, gd, gc, cu(nt), cu(radii), len(nt), vs, size, dims, per)
        assert np.array_equal(host(gc), kcnt)
        act = kcnt > 0
        assert act.sum() > 1000
        assert np.array_equal(host(gi).view(np.uint32)[act], kidx[act])
        assert np.array_equal(host(gd)[act], kdist[act])
        kw = O.tsdf_weights(radii, kidx, kdist, kcnt)
        gw = torch.zeros((S, k), dtype=torch.float32, device="cuda")
        af.runComputeTsdfWarpWeightsKernel(gw, cu(radii), gi, gd, gc, S)
        assert np.array_equal(host(gw)[act], kw[act])
        verts = O.translate(O.tsdf_vertices(vs, size, dims), c)
        gv = torch.empty((S, 3), dtype=torch.float32, device="cuda")
        af.runGenerateTsdfVerticesKernel(gv, vs, size, dims)
        assert np.array_equal(host(gv), O.tsdf_vertices(vs, size, dims))
        gv = cu(verts)
        wv = O.warp_tsdf(verts, T, kidx, kw, kcnt)
        af.runWarpTsdfKernel(gv, cu(T), gi, gw, gc, vs, size, dims)
        assert np.array_equal(host(gv), wv)
        coll = O.count_collisions(wv, kcnt, vs, size, dims, np.eye(3), c)
        gcoll = torch.zeros(S, dtype=torch.int32, device="cuda")
        af.runCountCollisionsPerVoxelKernel(gcoll, gv, gc, vs, size, dims, np.eye(3), c)
        assert np.array_equal(host(gcoll), coll)
        t1, w1 = t0.copy(), w0.copy()
        O.integrate_warped(t1, w1, wv, coll, kcnt, d, 0.016, vs, size, dims, np.eye(3), c, K)
        tg, wg = cu(t0), cu(w0)
        af.runIntegrateWarpedTSDFFromFrameKernel(tg, wg, gv, gcoll, gc, cu(d), (mm.shape[1], mm.shape[0]), 0.016, vs,
                                                 size, dims, np.eye(3), c, K)
        assert np.array_equal(host(tg), t1)
        assert np.array_equal(host(wg), w1)


def _sort_dev(pts, fn, *extra):
    import ctypes as C

    from volumefusion_gb300._lib import check, lib
    n = len(pts)
    p = torch.from_numpy(np.ascontiguousarray(pts, np.float32).ravel()).cuda()
    cnt = torch.tensor([n], dtype=torch.int32, device="cuda")
    if fn == "general":
        wsb = lib().afx_sort_unique_points_workspace_size(n)
    else:
        wsb = lib().afx_sort_unique_volume_points_workspace_size(n, extra[0])
    ws = torch.empty(int(wsb), dtype=torch.uint8, device="cuda")
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    if fn == "general":
        check(lib().afx_sort_unique_points(C.c_void_p(p.data_ptr()), C.c_void_p(cnt.data_ptr()), n,
                                           C.c_void_p(ws.data_ptr()), int(wsb), st), "sort")
    else:
        check(lib().afx_sort_unique_volume_points(C.c_void_p(p.data_ptr()), C.c_void_p(cnt.data_ptr()), n, *extra,
                                                  C.c_void_p(ws.data_ptr()), int(wsb), st), "sort")
    m = int(cnt.item())
    return p[:3 * m].view(-1, 3).cpu().numpy()


def test_volume_sort_equals_general_sort():
    """The column-bucket sort + unique of a marching-cubes cloud gives the general sort's result bit
    for bit: on a real cloud, with +0/-0 twins, and with columns too large for shared memory (their
    CTA sorts runs of 8192 and merges them: 2 runs, and 5 runs over three merge rounds)."""
    import ctypes as C

    from volumefusion_gb300 import configs
    cfg, [mm] = configs.rigid_sphere_128()
    depth, _, _, cen = O.frame_prep(mm, cfg["K"])
    vs = configs.voxel_size(cfg)
    S = int(np.prod(cfg["dims"]))
    t = np.full(S, -1.0, np.float32)
    w = np.zeros(S, np.float32)
    O.integrate_rigid(t, w, depth, cfg["delta"], cfg["dims"], vs, cfg["volume_size"], np.eye(3), cen, cfg["K"])
    raw = O.mc_pointcloud(t, w, cfg["dims"], vs, cfg["volume_size"])
    rng = np.random.default_rng(4)
    twins = raw[rng.integers(0, len(raw), 200)].copy()
    twins[:, 0] = 0.0
    neg = twins.copy()
    neg[:, 0] = -0.0
    half = np.float32(cfg["volume_size"][0]) / 2
    column = np.stack([np.full(12000, -half + np.float32(40.5) * vs[0], np.float32),
                       (rng.integers(0, 100, 12000) * vs[1] - half).astype(np.float32),
                       (rng.integers(0, 100, 12000) * vs[2] - half).astype(np.float32)], axis=1)
    dims = (C.c_int * 3)(*cfg["dims"])
    f3 = lambda a: (C.c_float * 3)(*[float(x) for x in a])  # noqa: E731
    extra = (dims, f3(vs), f3(cfg["volume_size"]))
    big = np.stack([np.full(40000, -half + np.float32(60.25) * vs[0], np.float32),
                    (rng.integers(0, 150, 40000) * vs[1] - half).astype(np.float32),
                    (rng.integers(0, 150, 40000) * vs[2] - half).astype(np.float32)], axis=1)
    for case in (raw, np.concatenate([raw, neg, twins, raw[:500]]), np.concatenate([raw, column]),
                 np.concatenate([raw, column, big, big[:7000]])):
        case = case[rng.permutation(len(case))]
        a = _sort_dev(case, "general")
        b = _sort_dev(case, "volume", *extra)
        assert a.shape == b.shape and len(a) > 0
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert np.array_equal(_sort_dev(raw, "volume", *extra), O.sort_unique(raw))


def test_knn_large_graph(af):
    """KNN over a graph of several node tiles (4332 nodes) gives the oracle's lists (the K smallest
    (distance, index) pairs) bit for bit: nodes on a jittered lattice with duplicates and equidistant
    pairs, queries inside and outside the node cloud, K = 4 and 6, and the graph's own 8-NN excluding
    the closest."""
    rng = np.random.default_rng(12)
    g = np.stack(np.meshgrid(np.arange(18), np.arange(16), np.arange(14), indexing="ij"), -1).reshape(-1, 3)
    nodes = (g * 0.01 + rng.normal(0, 0.002, g.shape)).astype(np.float32)
    nodes = nodes[rng.permutation(len(nodes))]
    nodes[100:140] = nodes[:40]  # duplicates: equal distances, resolved by index
    nodes = np.concatenate([nodes, (g[:300] * 0.01).astype(np.float32)])  # exact lattice points (ties)
    n = len(nodes)
    assert n > 2048
    pts = np.concatenate([(rng.random((6000, 3)) * [0.19, 0.17, 0.15] - 0.01),
                          (rng.random((500, 3)) * 0.6 - 0.2),  # many far outside the cloud
                          (g[:300] * 0.01 + 0.005)]).astype(np.float32)  # equidistant to lattice neighbours
    nodes_g, n_g = cu(nodes), cu(np.array([n], np.int32))
    for k in (4, 6):
        idx = torch.empty((len(pts), k), dtype=torch.int32, device="cuda")
        dist = torch.empty((len(pts), k), dtype=torch.float32, device="cuda")
        af.getKnnData(idx, dist, nodes_g, n_g, cu(pts))
        io, do = O.knn(nodes, pts, k)
        assert np.array_equal(host(idx).view(np.uint32), io), k
        assert np.array_equal(host(dist), do), k
    gi = torch.empty((n, 8), dtype=torch.int32, device="cuda")
    gd = torch.empty((n, 8), dtype=torch.float32, device="cuda")
    af.getKnnData(gi, gd, nodes_g, n_g, nodes_g, excludeClosest=True)
    gio, gdo = O.knn(nodes, nodes, 8, exclude_closest=True)
    assert np.array_equal(host(gi).view(np.uint32), gio)
    assert np.array_equal(host(gd), gdo)
