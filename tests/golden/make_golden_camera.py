"""Generate tests/golden/camera_calibration.npz by running the reference's own Brown-Conrady code.

Runs af::create_xy_lookup_table, af::transformation_unproject and af::transformation_project
(src/CameraCalibration.cpp, compiled into oracle/_ref/libvfref.so by ``make -C oracle -f Makefile.ref``)
on seeded synthetic cameras and points, and stores inputs and outputs.  The intrinsics are given as
the af::CameraIntrinsics fields {cx, cy, fx, fy}; the distortion as {k1..k6, codx, cody, p1, p2}.

    python tests/golden/make_golden_camera.py
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from make_golden import ref_lib  # noqa: E402

f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")

# (intrinsics cx cy fx fy, distortion k1..k6 codx cody p1 p2, width, height)
CAMERAS = [
    ([32.5, 24.25, 50.0, 50.5], [0.5, -0.1, 0.01, 0.8, -0.05, 0.02, 0.0, 0.0, 1e-3, -5e-4], 64, 48),
    ([40.0, 30.0, 60.0, 61.0], [-0.3, 0.1, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 2e-3, 1e-3], 80, 60),
    ([20.0, 15.0, 25.0, 25.0], [0.02, -0.01, 0.0, 0.0, 0.0, 0.0, 0.01, -0.02, 0.0, 0.0], 40, 30),
]


def main():
    R = ref_lib()
    R.ref_xy_lookup_table.argtypes = [f32p, C.c_int, C.c_int, f32p, f32p]
    R.ref_xy_lookup_table.restype = C.c_int
    R.ref_bc_unproject.argtypes = [f32p, i32p, f32p, f32p, C.c_long, f32p, f32p]
    R.ref_bc_project.argtypes = [f32p, i32p, f32p, C.c_long, f32p, f32p]
    out = {}
    rng = np.random.default_rng(11)
    for i, (intr, dist, W, H) in enumerate(CAMERAS):
        intr = np.asarray(intr, np.float32)
        dist = np.asarray(dist, np.float32)
        table = np.full((H, W, 2), np.nan, np.float32)
        assert R.ref_xy_lookup_table(table.ravel(), W, H, intr, dist) == 1
        px = (rng.random((400, 2)) * [3 * W, 3 * H] - [W, H]).astype(np.float32)
        depth = (rng.random(400) * 3).astype(np.float32)
        depth[::13] = 0
        pts = np.empty((400, 3), np.float32)
        valid_u = np.empty(400, np.int32)
        R.ref_bc_unproject(pts.ravel(), valid_u, px.ravel(), depth, 400, intr, dist)
        pts_in = (rng.random((400, 3)) * [2, 2, 3] - [1, 1, 0.5]).astype(np.float32)
        proj = np.full((400, 2), -7.0, np.float32)  # the reference leaves a pixel beyond the radius as passed in
        valid_p = np.empty(400, np.int32)
        R.ref_bc_project(proj.ravel(), valid_p, pts_in.ravel(), 400, intr, dist)
        out.update({"intr%d" % i: intr, "dist%d" % i: dist, "size%d" % i: np.array([W, H], np.int32),
                    "table%d" % i: table, "px%d" % i: px, "depth%d" % i: depth, "unproj%d" % i: pts,
                    "unproj_valid%d" % i: valid_u, "pts%d" % i: pts_in, "proj%d" % i: proj, "proj_valid%d" % i: valid_p})
    out["n"] = np.int32(len(CAMERAS))
    np.savez_compressed(os.path.join(HERE, "camera_calibration.npz"), **out)


if __name__ == "__main__":
    main()
