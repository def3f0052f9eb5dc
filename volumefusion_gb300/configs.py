"""Workload configurations, expressed in the reference's af::Settings terms.

Each maps a named workload onto the parameters af::runVolumeFusion reads
(src/Settings.cpp:8-39, src/VolumeFusion.cu:223-741).  Deviations from the reference's
defaults are stated beside the field.
"""
import math

import numpy as np

from . import synth


def _base():
    return dict(
        depth_threshold=1.2,       # dataPresets.json:13 (af::Settings default is 1.0)
        bilateral=1,
        bilateral_r=2,             # 5x5 window (bilateralD is the radius, src/VolumeFusion.cu:204)
        sigma_i=0.030,             # range sigma 30 mm
        sigma_s=2.0,               # spatial sigma 2 px
        bilateral_thr=0.09,        # 3 * sigma_r; the workloads name no hard threshold
        angle_lo=1.3, angle_hi=2.1,  # normExclAngleRange default (src/Settings.cpp:15)
        energy_min_step=1e-4,      # src/Settings.cpp:29
        lambda_depth=1.0,          # energyWeightDepth
        corr_thresh=0.01,          # correspThreshDist default (src/Settings.cpp:36)
        update_graph=1,            # src/Settings.cpp:20
        integrate=1,
        solver=1,                  # 1 = block-Jacobi PCG, 0 = dense direct solve
        pcg_iterations=10,
        pcg_tol=0.0,
        node_cap=16384,
        mesh_cap=4_000_000,
    )


def rigid_sphere_128():
    """One 320x288 sphere frame (r=150 mm at 600 mm), 128^3 FP32 volume, 4 mm voxels,
    16 mm truncation, identity warp, marching cubes at iso 0."""
    mm, K = synth.sphere_frame()
    cfg = _base()
    cfg.update(name="rigid_sphere_128", width=320, height=288, K=K, dims=(128, 128, 128),
               volume_size=(0.512, 0.512, 0.512), delta=0.016, graph_radius=0.025, knn=4, kreg=8,
               icp_iterations=1, gn_iterations=5, lambda_reg=math.sqrt(200.0))
    return cfg, [mm]


def nonrigid_capsules_256(n_frames=30, dims=(256, 256, 256), voxel=0.004):
    """30-frame 640x576 articulated capsule pair (r=60 mm, L=300 mm, bending 0->45 deg),
    256^3 FP32 volume at 4 mm, 25 mm motion-graph radius, K=4 skinning, 8-NN
    regularisation with lambda=200 (energyWeightMReg = sqrt(200), since the weight scales
    both residual and Jacobian), 1 ICP iteration x 5 Gauss-Newton x 10 PCG."""
    cfg = _base()
    size = tuple(d * voxel for d in dims)
    K = synth.intrinsics(504.0, 504.0, 320.0, 288.0)
    cfg.update(name="nonrigid_capsules_%d" % dims[0], width=640, height=576, K=K, dims=tuple(dims),
               volume_size=size, delta=0.016, graph_radius=0.025, knn=4, kreg=8, icp_iterations=1,
               gn_iterations=5, lambda_reg=math.sqrt(200.0), n_frames=n_frames)
    return cfg


def capsule_frames(cfg, frames=None):
    n = cfg.get("n_frames", 30)
    frames = range(n) if frames is None else frames
    return [synth.capsule_pair_frame(f, n_frames=n, width=cfg["width"], height=cfg["height"],
                                     fx=float(cfg["K"][0, 0]), fy=float(cfg["K"][1, 1]),
                                     cx=float(cfg["K"][0, 2]), cy=float(cfg["K"][1, 2]))[0] for f in frames]


def small_nonrigid(n_frames=6, dims=(64, 64, 64), voxel=0.008, width=160, height=144):
    """Reduced non-rigid case the CPU oracle finishes in seconds (parity tests)."""
    cfg = _base()
    size = tuple(d * voxel for d in dims)
    f = 126.0 * width / 160.0
    K = synth.intrinsics(f, f, width / 2.0, height / 2.0)
    cfg.update(name="small_nonrigid", width=width, height=height, K=K, dims=tuple(dims), volume_size=size,
               delta=0.032, graph_radius=0.05, knn=4, kreg=8, icp_iterations=1, gn_iterations=5,
               lambda_reg=math.sqrt(200.0), n_frames=n_frames, corr_thresh=0.02)
    return cfg


def small_frames(cfg, frames=None):
    n = cfg["n_frames"]
    frames = range(n) if frames is None else frames
    K = cfg["K"]
    return [synth.capsule_pair_frame(f, n_frames=n, width=cfg["width"], height=cfg["height"], fx=float(K[0, 0]),
                                     fy=float(K[1, 1]), cx=float(K[0, 2]), cy=float(K[1, 2]), max_bend_deg=15.0)[0]
            for f in frames]


def voxel_size(cfg):
    return np.array(cfg["volume_size"], np.float32) / np.array(cfg["dims"], np.float32)
