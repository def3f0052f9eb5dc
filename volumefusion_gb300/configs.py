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


def precision_capsules_512(n_frames=30, graph_radius=0.009):
    """The capsule sequence in the precision form: 512^3 at 2 mm (the same 1.024 m cube) with FP16
    TSDF values and uint16 weights (4 B/voxel, 537 MB), FP32 Jacobian/J^T J, PCG dot products in
    double-binary32 (about 48 bits) and FP64 6x6 block inverses.  A 9 mm graph radius gives a graph that grows to ~6000 nodes over the
    sequence (measured on the GPU: 11630 nodes at 6.5 mm, and node count goes as 1/r^2)."""
    cfg = nonrigid_capsules_256(n_frames=n_frames, dims=(512, 512, 512), voxel=0.002)
    cfg.update(name="precision_capsules_512", graph_radius=graph_radius, precision="fp16")
    return cfg


def capsule_frames(cfg, frames=None):
    n = cfg.get("n_frames", 30)
    frames = range(n) if frames is None else frames
    return [synth.capsule_pair_frame(f, n_frames=n, width=cfg["width"], height=cfg["height"],
                                     fx=float(cfg["K"][0, 0]), fy=float(cfg["K"][1, 1]),
                                     cx=float(cfg["K"][0, 2]), cy=float(cfg["K"][1, 2]),
                                     distortion=cfg.get("distortion"))[0] for f in frames]


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


# ---- many concurrent sessions (the batched and served workloads) ----

_VOLUMES = ((128, 0.008), (192, 0.006), (256, 0.004), (384, 0.003))  # cube edge ~1.0-1.15 m
_CAMERAS = ((320, 288, 252.0), (640, 576, 504.0))
SCENES = ("sphere", "torus", "capsule")


def session_config(dims, voxel, width, height, focal, graph_radius, scene, seed):
    """One served session: a seeded scene at one of the workload's volume and camera sizes."""
    cfg = _base()
    K = synth.intrinsics(focal, focal, width / 2.0, height / 2.0)
    cfg.update(name="%s_%d" % (scene, dims), width=width, height=height, K=K, dims=(dims, dims, dims),
               volume_size=(dims * voxel,) * 3, delta=max(0.016, 4 * voxel), graph_radius=graph_radius, knn=4, kreg=8,
               icp_iterations=1, gn_iterations=5, lambda_reg=math.sqrt(200.0), n_frames=30, scene=scene, seed=seed,
               node_cap=8192, mesh_cap=1_000_000, triangle_cap=1_000_000)
    return cfg


def session_mix(count, seed=0):
    """`count` session configurations drawn from the batched/served workload: volumes from
    {128, 192, 256, 384}^3, 320x288 or 640x576 depth, sphere / torus / bending capsules, graph
    radius 20-35 mm (a few hundred to a few thousand nodes), each with its own seed."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        dims, voxel = _VOLUMES[rng.integers(len(_VOLUMES))]
        w, h, f = _CAMERAS[rng.integers(len(_CAMERAS))]
        scene = SCENES[rng.integers(len(SCENES))]
        if scene == "torus":  # traced scene: the small camera keeps frame synthesis cheap
            w, h, f = _CAMERAS[0]
        out.append(session_config(dims, voxel, w, h, f, float(rng.uniform(0.020, 0.035)), scene, int(rng.integers(1 << 30))))
    return out


_FRAME_CACHE = {}


def scene_frames(cfg, n_unique=None):
    """Frames of a session's scene (cached per scene and camera).  Torus sequences have 10 unique
    frames, played forward and back by scene_frame()."""
    key = (cfg["scene"], cfg["width"], cfg["height"])
    if key not in _FRAME_CACHE:
        n = cfg.get("n_frames", 30)
        K = cfg["K"]
        kw = dict(width=cfg["width"], height=cfg["height"], fx=float(K[0, 0]), fy=float(K[1, 1]), cx=float(K[0, 2]),
                  cy=float(K[1, 2]))
        if cfg["scene"] == "sphere":
            frames = [synth.moving_sphere_frame(i, n_frames=n, **kw)[0] for i in range(n)]
        elif cfg["scene"] == "torus":
            frames = [synth.torus_frame(i, n_frames=10, **kw)[0] for i in range(n_unique or 10)]
        else:
            frames = [synth.capsule_pair_frame(i, n_frames=n, **kw)[0] for i in range(n)]
        _FRAME_CACHE[key] = frames
    return _FRAME_CACHE[key]


def scene_frame(cfg, i):
    frames = scene_frames(cfg)
    m = len(frames)
    period = max(2 * (m - 1), 1)
    r = i % period
    return frames[r if r < m else period - r]
