"""Runs the reference's own per-frame GPU loop (oracle/_ref/libvfref_gpu.so, built by
oracle/ref_gpu/build.py) on the headline sequence and prints its per-frame wall times as JSON.

Baseline infrastructure only.  bench.py starts this in a child process with a time limit, so the
reference's code runs in its own CUDA context and a stall there cannot hold up the benchmark.

    python oracle/ref_gpu/run.py [--frames N] [--runs R]
"""
import argparse
import ctypes as C
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
LIB = os.path.join(ROOT, "oracle", "_ref", "libvfref_gpu.so")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--frames", type=int, default=30)
    ap.add_argument("--runs", type=int, default=2, help="the last run is reported; earlier ones warm up")
    args = ap.parse_args()
    from volumefusion_gb300 import configs
    cfg = configs.nonrigid_capsules_256(n_frames=args.frames)
    frames = np.ascontiguousarray(np.stack(configs.capsule_frames(cfg)[:args.frames]).astype(np.uint16))
    n = len(frames)
    R = C.CDLL(LIB)
    R.ref_gpu_fusion.restype = C.c_int
    K = np.ascontiguousarray(np.asarray(cfg["K"], np.float32).T).ravel()
    size = np.asarray(cfg["volume_size"], np.float32)
    f32 = C.c_float
    out = {"runs": []}
    for _ in range(args.runs):
        ms = np.zeros(n, np.float64)
        nodes = C.c_int(0)
        err = C.create_string_buffer(4096)
        rc = R.ref_gpu_fusion(frames.ctypes.data_as(C.c_void_p), n, int(cfg["width"]), int(cfg["height"]),
                              K.ctypes.data_as(C.c_void_p), size.ctypes.data_as(C.c_void_p), f32(cfg["delta"]),
                              f32(cfg["depth_threshold"]), int(cfg["bilateral"]), int(cfg["bilateral_r"]),
                              f32(cfg["sigma_i"]), f32(cfg["sigma_s"]), f32(cfg["bilateral_thr"]),
                              f32(cfg["angle_lo"]), f32(cfg["angle_hi"]), f32(cfg["graph_radius"]),
                              int(cfg["update_graph"]), int(cfg["icp_iterations"]), f32(cfg["lambda_depth"]),
                              f32(cfg["lambda_reg"]), f32(cfg["energy_min_step"]), f32(cfg["corr_thresh"]),
                              ms.ctypes.data_as(C.c_void_p), C.byref(nodes), err, 4096)
        out["runs"].append({"rc": rc, "error": err.value.decode(errors="replace"), "frame_ms": ms.tolist(),
                            "nodes": nodes.value})
        if rc:
            break
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
