"""Benchmark: non-rigid fusion frames/s on the 256^3 articulated-capsule sequence.

A step is one non-rigid frame of the 30-frame 640x576 capsule-pair sequence (256^3 FP32
TSDF at 4 mm, 25 mm motion graph, K=4, 8-NN regularisation, 1 ICP x 5 Gauss-Newton x 10
PCG), played forward and back so that any number of steps sees continuous motion.

  value : frames/s with the depth frames already resident in HBM (afx_fusion_process)
  e2e   : frames/s through the C ABI with host depth buffers (afx_fusion_process_host from
          pinned memory + a device-to-host read of the frame statistics every frame)
  p50/p99 frame latency from the e2e loop.

--impl reference times the reference's CPU path (the oracle port of it: this box has no
build of the reference) with all host threads.  Under torchrun each rank runs an
independent replica (the path does not shard); value is the sum over ranks.
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_FRAMES = 30


def seq_index(f):
    """Forward-backward play of the 30-frame sequence: 0..29, 28..1, 0..29, ..."""
    period = 2 * (N_FRAMES - 1)
    r = f % period
    return r if r < N_FRAMES else period - r


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-frames", type=int, default=3)
    return ap.parse_args()


class ClockSampler(threading.Thread):
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""

    def __init__(self, gpu):
        super().__init__(daemon=True)
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def run(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            for line in self.proc.stdout:
                self.lines.append(line.strip())
        except Exception:
            pass

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(n):
    if n <= 1 or "RANK" not in os.environ:
        return None
    import torch.distributed as dist
    dist.init_process_group("nccl")
    return dist


def cpu_baseline(cfg, frames_np, n_frames):
    """Oracle port of the reference path on the host cores (all threads)."""
    from oracle import pyoracle as O
    ocfg = dict(cfg)
    ocfg["solver"] = 1
    o = O.Fusion(ocfg)
    o.process(frames_np[0])
    t0 = time.perf_counter()
    for f in range(1, n_frames + 1):
        o.process(frames_np[seq_index(f)])
    dt = time.perf_counter() - t0
    o.close()
    return n_frames / dt, dt


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from volumefusion_gb300 import configs
    cfg = configs.nonrigid_capsules_256(n_frames=N_FRAMES)
    frames_np = configs.capsule_frames(cfg)
    from oracle import pyoracle as O
    o = O.Fusion(dict(cfg))
    o.process(frames_np[0])
    for f in range(1, 1 + args.warmup):
        o.process(frames_np[seq_index(f)])
    t0 = time.perf_counter()
    for f in range(1 + args.warmup, 1 + args.warmup + args.steps):
        o.process(frames_np[seq_index(f)])
    dt = time.perf_counter() - t0
    fps = args.steps / dt
    cores = os.cpu_count()
    line = {
        "impl": "reference", "metric": "nonrigid_frames_per_s_256", "value": fps, "unit": "frames/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": cfg["name"], "frames": "640x576 capsule pair, 30-frame sequence played back and forth",
                   "volume": "256^3 FP32 @ 4 mm", "parallelism": "replicas"},
        "cpu_baseline": {"value": fps, "unit": "frames/s", "cores": cores, "kind": "port",
                         "sample": "%d frames of the workload after %d warm-up frames" % (args.steps, args.warmup)},
        "e2e": {"value": fps, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    import torch
    from volumefusion_gb300 import configs
    from volumefusion_gb300.fusion import FusionSession

    dist = dist_setup(args.gpus)
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    world = dist.get_world_size() if dist else 1
    torch.cuda.set_device(local)
    cfg = configs.nonrigid_capsules_256(n_frames=N_FRAMES)
    frames_np = configs.capsule_frames(cfg)
    frames_dev = [torch.from_numpy(f.astype(np.int16)).cuda() for f in frames_np]
    pinned = [torch.from_numpy(f.astype(np.int16)).pin_memory() for f in frames_np]
    stream = torch.cuda.Stream()

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    # ---- device-resident arm ----
    s = FusionSession(cfg, stream=stream)
    with torch.cuda.stream(stream):
        s.process(frames_dev[0])
        for f in range(1, 1 + args.warmup):
            s.process(frames_dev[seq_index(f)])
    s.stats()
    barrier()
    sampler = ClockSampler(local)
    sampler.start()
    l0 = s.kernel_launches()
    s.set_timing(True)
    s.stage_times(reset=True)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    with torch.cuda.stream(stream):
        for f in range(1 + args.warmup, 1 + args.warmup + args.steps):
            s.process(frames_dev[seq_index(f)])
    ev1.record(stream)
    barrier()
    sampler.stop()
    launches = s.kernel_launches() - l0
    ms = ev0.elapsed_time(ev1)
    stage_ms = s.stage_times(reset=True)
    s.set_timing(False)
    st = s.stats(check_errors=False)
    tmax = torch.tensor([ms], dtype=torch.float64, device="cuda")
    if dist:
        dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
    ms = float(tmax.item())
    fps = world * args.steps / (ms / 1000.0)
    s.close()

    # ---- end-to-end arm: host buffers through the C ABI, per-frame latency ----
    s2 = FusionSession(cfg, stream=stream)
    s2.process_host_ptr(pinned[0].data_ptr())
    s2.stats()
    for f in range(1, 1 + args.warmup):
        s2.process_host_ptr(pinned[seq_index(f)].data_ptr())
        s2.stats()
    barrier()
    lat = []
    t0 = time.perf_counter()
    for f in range(1 + args.warmup, 1 + args.warmup + args.steps):
        a = time.perf_counter()
        s2.process_host_ptr(pinned[seq_index(f)].data_ptr())
        s2.stats(check_errors=False)  # device-to-host read of the frame result
        lat.append(time.perf_counter() - a)
    barrier()
    e2e_s = time.perf_counter() - t0
    te = torch.tensor([e2e_s], dtype=torch.float64, device="cuda")
    if dist:
        dist.all_reduce(te, op=dist.ReduceOp.MAX)
    e2e_fps = world * args.steps / float(te.item())
    s2.close()

    # ---- roofline of the dominant stage ----
    S = int(np.prod(cfg["dims"]))
    dom = max(stage_ms, key=stage_ms.get)
    per_frame = {k: v / args.steps for k, v in stage_ms.items()}
    peaks = {}
    pk_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk_path):
        peaks = json.load(open(pk_path))
    hbm = peaks.get("hbm_gbs", 6800.0)
    # algorithmic bytes per launch of the stages we can state exactly
    tri = st["mesh_faces"]
    algo = {
        "marching_cubes": 8.0 * S + 12.0 * st["mesh_points"] * 4 + 48.0 * tri,
    }
    roof = None
    if dom in algo:
        achieved = algo[dom] / (per_frame[dom] / 1000.0) / 1e9
        roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "traffic": None, "peak_source": "measured" if peaks else "fallback"}
    else:
        mc = per_frame.get("marching_cubes", 0)
        if mc > 0:
            achieved = algo["marching_cubes"] / (mc / 1000.0) / 1e9
            roof = {"bound": "hbm", "kernel": "marching_cubes", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                    "frac": achieved / hbm, "traffic": None, "peak_source": "measured" if peaks else "fallback",
                    "note": "dominant stage is %s (%.3f ms/frame), latency-bound" % (dom, per_frame[dom])}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline and args.cpu_frames > 0:
        v, dt = cpu_baseline(cfg, frames_np, args.cpu_frames)
        cpu = {"value": v, "unit": "frames/s", "cores": os.cpu_count(), "kind": "port",
               "sample": "%d non-rigid frames of the workload (%.1f s) on all host threads" % (args.cpu_frames, dt)}

    if rank == 0:
        line = {
            "metric": "nonrigid_frames_per_s_256", "value": fps, "unit": "frames/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": cfg["name"],
                       "frames": "640x576 capsule pair, 30-frame sequence played back and forth",
                       "volume": "256^3 FP32 TSDF @ 4 mm (134 MB tsdf+weights, larger than L2)",
                       "graph_radius_mm": 25, "knn": 4, "kreg": 8, "gn": "1 ICP x 5 GN x 10 PCG",
                       "parallelism": "replicas" if world > 1 else "single", "l2": "working set larger than L2"},
            "e2e": {"value": e2e_fps, "unit": "frames/s", "h2d_bytes_per_step": int(frames_np[0].nbytes),
                    "d2h_bytes_per_step": int(C.sizeof(__import__("volumefusion_gb300._lib", fromlist=["x"]).FrameStats)),
                    "latency_ms_p50": 1000 * float(np.percentile(lat, 50)),
                    "latency_ms_p99": 1000 * float(np.percentile(lat, 99))},
            "gpu_launches": int(launches),
            "stage_ms_per_frame": per_frame,
            "frame_stats": {k: st[k] for k in ("n_nodes", "mesh_points", "correspondences", "gn_iterations_done",
                                                "mesh_faces", "error")},
            "roofline": roof,
            "cpu_baseline": cpu,
            "clocks": sampler.summary(),
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
