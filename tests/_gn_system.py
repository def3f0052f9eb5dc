"""One Gauss-Newton system of the small non-rigid case, built with the CPU oracle only (numpy):
frame 12 integrated into an empty volume, its point cloud, the deformation graph and its skinning,
transforms moved by a seeded 3 mm jitter, correspondences against frame `frame`, and the
regularisation neighbours.  Shared by the GPU operator tests and the CPU solver-sensitivity test."""
import numpy as np

from oracle import pyoracle as O


def gn_system(k, kreg, frame=14):
    from volumefusion_gb300 import configs, synth
    cfg = configs.small_nonrigid(n_frames=30)
    cam = dict(width=cfg["width"], height=cfg["height"], fx=float(cfg["K"][0, 0]), fy=float(cfg["K"][1, 1]),
               cx=float(cfg["K"][0, 2]), cy=float(cfg["K"][1, 2]))
    mm0, K = synth.capsule_pair_frame(12, **cam)
    mm1, _ = synth.capsule_pair_frame(frame, **cam)
    d0, v0, n0, c = O.frame_prep(mm0, K)
    dims = np.asarray(cfg["dims"], np.int32)
    size = np.asarray(cfg["volume_size"], np.float32)
    vs = size / dims.astype(np.float32)
    S = int(np.prod(dims))
    t0, w0 = np.full(S, -1, np.float32), np.zeros(S, np.float32)
    O.integrate_rigid(t0, w0, d0, cfg["delta"], dims, vs, size, np.eye(3), c, K)
    mesh = O.translate(O.sort_unique(O.mc_pointcloud(t0, w0, dims, vs, size)), c)
    nodes, radii, T = O.build_graph(mesh, k, cfg["graph_radius"])
    rng = np.random.default_rng(11)
    T = T.copy()
    T[:, 12:15] += rng.normal(0, 0.003, (len(T), 3)).astype(np.float32)
    midx, mdist = O.knn(nodes, mesh, k)
    mw = O.warp_weights(radii, midx, mdist)
    warped = O.warp(mesh, T, midx, mw)
    d1, v1, n1, _ = O.frame_prep(mm1, K)
    corr = O.correspondences(warped, K, d1, v1, cfg["corr_thresh"])
    gidx, gdist = O.knn(nodes, nodes, kreg, exclude_closest=True)
    gidx, gdist = O.filter_disconnected(gidx, gdist, radii)
    return dict(mesh=mesh, nodes=nodes, T=T, midx=midx, mw=mw, warped=warped, v1=v1, n1=n1, corr=corr, gidx=gidx,
                lam_d=np.float32(cfg["lambda_depth"]), lam_r=np.float32(cfg["lambda_reg"]))


def assembled(s):
    """J^T J and J^T r of the system (the oracle's block assembly), binary32."""
    rd = O.residual_depth(s["corr"], s["warped"], s["v1"], s["n1"], s["lam_d"])
    rr = O.residual_reg(s["nodes"], s["T"], s["gidx"], s["lam_r"])
    A, b, _ = O.assemble(s["corr"], s["mesh"], s["midx"], s["mw"], s["n1"], s["lam_d"], s["nodes"], s["gidx"],
                         s["lam_r"], rd, rr)
    return A, b
