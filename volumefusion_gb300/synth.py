"""Seeded synthetic depth scenes standing in for the reference's recorded sequences.

The reference reads private 16-bit depth PNGs (millimetres) from disk
(src/dataset.cpp:168-189).  These renderers produce the same kind of frame --
uint16 millimetres, 0 where a pixel sees nothing -- from analytic scenes, ray-cast in
float64 through a pinhole camera with pixel (u, v) on the ray ((u-cx)/fx, (v-cy)/fy, 1).

Noise is N(0, (1 mm * (z / 1 m)^2)^2) per pixel.  It is drawn from a counter-based
generator (splitmix64 of seed and pixel index, Box-Muller), written here in numpy
integer arithmetic, so that a frame is bit-identical on every machine and numpy version.
"""
import math

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix64(x):
    x = (x + np.uint64(0x9E3779B97F4A7C15)) & _M64
    z = x
    z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _M64
    z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _M64
    return z ^ (z >> np.uint64(31))


def gaussian_noise(seed, n, stream=0):
    """n standard normal samples for (seed, stream), identical on every platform."""
    with np.errstate(over="ignore"):
        base = np.uint64((seed * 0x100000001B3 + stream * 0x9E3779B1) & 0xFFFFFFFFFFFFFFFF)
        idx = np.arange(n, dtype=np.uint64)
        a = _splitmix64(base ^ (idx * np.uint64(2)))
        b = _splitmix64(base ^ (idx * np.uint64(2) + np.uint64(1)))
    u1 = ((a >> np.uint64(11)).astype(np.float64) + 0.5) / float(1 << 53)
    u2 = ((b >> np.uint64(11)).astype(np.float64) + 0.5) / float(1 << 53)
    return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * math.pi * u2)


def intrinsics(fx, fy, cx, cy):
    """3x3 pinhole matrix (row-major numpy; column-major float[9] via .T.ravel())."""
    return np.array([[fx, 0.0, cx], [0.0, fy, cy], [0.0, 0.0, 1.0]], dtype=np.float64)


def _rays(width, height, K):
    u, v = np.meshgrid(np.arange(width, dtype=np.float64), np.arange(height, dtype=np.float64))
    dx = (u - K[0, 2]) / K[0, 0]
    dy = (v - K[1, 2]) / K[1, 1]
    return np.stack([dx, dy, np.ones_like(dx)], axis=-1)


def _distorted_rays(width, height, K, dist):
    """Rays of a camera whose lens follows OpenCV's rational + tangential model (k1..k6, p1, p2): pixel
    (u, v) sees the normalised point (x, y) that the model maps to ((u - cx) / fx, (v - cy) / fy),
    found by the fixed-point iteration cv::undistortPoints uses (40 passes in binary64)."""
    g = {k: float(dist.get(k, 0.0)) for k in ("k1", "k2", "k3", "k4", "k5", "k6", "p1", "p2")}
    u, v = np.meshgrid(np.arange(width, dtype=np.float64), np.arange(height, dtype=np.float64))
    xd = (u - K[0, 2]) / K[0, 0]
    yd = (v - K[1, 2]) / K[1, 1]
    x, y = xd.copy(), yd.copy()
    for _ in range(40):
        r2 = x * x + y * y
        kr = (1 + ((g["k3"] * r2 + g["k2"]) * r2 + g["k1"]) * r2) / (1 + ((g["k6"] * r2 + g["k5"]) * r2 + g["k4"]) * r2)
        tx = 2 * g["p1"] * x * y + g["p2"] * (r2 + 2 * x * x)
        ty = g["p1"] * (r2 + 2 * y * y) + 2 * g["p2"] * x * y
        x, y = (xd - tx) / kr, (yd - ty) / kr
    return np.stack([x, y, np.ones_like(x)], axis=-1)


def _hit_sphere(d, c, r):
    dd = np.einsum("...i,...i->...", d, d)
    dc = d @ c
    disc = dc * dc - dd * (c @ c - r * r)
    t = np.full(dd.shape, np.inf)
    ok = disc >= 0
    t[ok] = (dc[ok] - np.sqrt(disc[ok])) / dd[ok]
    t[t <= 0] = np.inf
    return t


def _hit_capsule(d, a, b, r):
    """Nearest positive ray parameter for a capsule (segment a-b, radius r), inf on a miss."""
    ab = b - a
    L2 = ab @ ab
    ax = ab / math.sqrt(L2)
    dd = np.einsum("...i,...i->...", d, d)
    # infinite cylinder around the axis through a: |(t d - a) x ax|^2 = r^2
    dpar = d @ ax
    dperp = d - dpar[..., None] * ax
    apar = -a @ ax
    aperp = -a - apar * ax
    A = np.einsum("...i,...i->...", dperp, dperp)
    B = 2.0 * (dperp @ aperp)
    C = aperp @ aperp - r * r
    disc = B * B - 4 * A * C
    t = np.full(dd.shape, np.inf)
    ok = (disc >= 0) & (A > 1e-15)
    tc = np.full(dd.shape, np.inf)
    tc[ok] = (-B[ok] - np.sqrt(disc[ok])) / (2 * A[ok])
    s = np.full(dd.shape, np.nan)
    s[ok] = tc[ok] * dpar[ok] + apar  # axial coordinate of the hit relative to a
    body = ok & (tc > 0) & (s >= 0) & (s <= math.sqrt(L2))
    t[body] = tc[body]
    t = np.minimum(t, _hit_sphere(d, a, r))
    t = np.minimum(t, _hit_sphere(d, b, r))
    return t


def _to_mm(z, seed, frame):
    noise = gaussian_noise(seed, z.size, stream=frame).reshape(z.shape)
    valid = np.isfinite(z)
    zz = np.where(valid, z, 0.0)
    sigma = 0.001 * zz * zz
    mm = np.rint((zz + sigma * noise) * 1000.0)
    mm = np.where(valid, np.clip(mm, 0, 65535), 0)
    return mm.astype(np.uint16)


def sphere_frame(width=320, height=288, fx=252.0, fy=252.0, cx=160.0, cy=144.0, radius=0.150,
                 center=(0.0, 0.0, 0.600), seed=0):
    """Single depth frame of a sphere (rigid single-frame workload: 320x288, r=150 mm at 600 mm)."""
    K = intrinsics(fx, fy, cx, cy)
    d = _rays(width, height, K)
    t = _hit_sphere(d, np.asarray(center, dtype=np.float64), radius)
    return _to_mm(t, seed, 0), K


def capsule_pair_frame(frame, n_frames=30, width=640, height=576, fx=504.0, fy=504.0, cx=320.0, cy=288.0,
                       radius=0.060, length=0.300, joint=(0.0, 0.0, 0.800), max_bend_deg=45.0, seed=0,
                       distortion=None):
    """Frame `frame` of the articulated capsule pair: two capsules of the given radius and length
    meeting at `joint`; the second one bends linearly from 0 to max_bend_deg about the camera y
    axis (its free end swings toward the camera) over n_frames frames.  With `distortion` (OpenCV
    coefficients) the frame is what a camera with that lens sees."""
    K = intrinsics(fx, fy, cx, cy)
    d = _distorted_rays(width, height, K, distortion) if distortion else _rays(width, height, K)
    j = np.asarray(joint, dtype=np.float64)
    theta = math.radians(max_bend_deg) * (frame / max(n_frames - 1, 1))
    a_end = j + length * np.array([-1.0, 0.0, 0.0])
    b_end = j + length * np.array([math.cos(theta), 0.0, -math.sin(theta)])
    t = np.minimum(_hit_capsule(d, a_end, j, radius), _hit_capsule(d, j, b_end, radius))
    return _to_mm(t, seed, frame), K


def capsule_pair_sequence(n_frames=30, **kw):
    frames = []
    K = None
    for f in range(n_frames):
        mm, K = capsule_pair_frame(f, n_frames=n_frames, **kw)
        frames.append(mm)
    return np.stack(frames), K


def _rot(axis, angle):
    axis = np.asarray(axis, dtype=np.float64)
    axis = axis / np.linalg.norm(axis)
    x, y, z = axis
    c, s = math.cos(angle), math.sin(angle)
    C1 = 1.0 - c
    return np.array([[c + x * x * C1, x * y * C1 - z * s, x * z * C1 + y * s],
                     [y * x * C1 + z * s, c + y * y * C1, y * z * C1 - x * s],
                     [z * x * C1 - y * s, z * y * C1 + x * s, c + z * z * C1]])


def _hit_torus(d, center, R_world, R, r, t0=0.2, t1=2.0, iters=96):
    """Nearest ray parameter on a torus (major R, minor r; axis = R_world[:, 2]) by sphere tracing
    its distance function; inf on a miss."""
    n = d.shape[:-1]
    dn = d / np.linalg.norm(d, axis=-1, keepdims=True)
    t = np.full(n, t0)
    alive = np.ones(n, dtype=bool)
    for _ in range(iters):
        p = dn * t[..., None] - center
        q = p @ R_world  # torus frame
        k = np.sqrt(q[..., 0] ** 2 + q[..., 1] ** 2) - R
        dist = np.sqrt(k * k + q[..., 2] ** 2) - r
        t = np.where(alive, t + dist, t)
        alive &= (dist > 1e-6) & (t < t1)
    hit = ~alive & (t < t1)
    scale = np.linalg.norm(d, axis=-1)
    return np.where(hit, t / scale, np.inf)


def torus_frame(frame, n_frames=30, width=320, height=288, fx=252.0, fy=252.0, cx=160.0, cy=144.0, major=0.16,
                minor=0.05, center=(0.0, 0.0, 0.8), tilt_deg=55.0, spin_deg=40.0, seed=0):
    """Frame `frame` of a torus tilted towards the camera and spinning about its axis."""
    K = intrinsics(fx, fy, cx, cy)
    d = _rays(width, height, K)
    a = math.radians(spin_deg) * (frame / max(n_frames - 1, 1))
    Rw = _rot((1.0, 0.0, 0.0), math.radians(tilt_deg)) @ _rot((0.0, 0.0, 1.0), a)
    t = _hit_torus(d, np.asarray(center, dtype=np.float64), Rw, major, minor)
    return _to_mm(t, seed, frame), K


def moving_sphere_frame(frame, n_frames=30, width=320, height=288, fx=252.0, fy=252.0, cx=160.0, cy=144.0,
                        radius=0.15, start=(-0.05, 0.0, 0.75), stop=(0.05, 0.02, 0.8), seed=0):
    """Frame `frame` of a sphere translating from `start` to `stop` over the sequence."""
    K = intrinsics(fx, fy, cx, cy)
    d = _rays(width, height, K)
    u = frame / max(n_frames - 1, 1)
    c = (1.0 - u) * np.asarray(start, dtype=np.float64) + u * np.asarray(stop, dtype=np.float64)
    return _to_mm(_hit_sphere(d, c, radius), seed, frame), K
