"""Benchmark: non-rigid fusion frames/s on the 256^3 articulated-capsule sequence.

A step fuses the 30-frame 640x576 capsule-pair sequence from an empty volume (256^3 FP32
TSDF at 4 mm, 25 mm motion graph, K=4, 8-NN regularisation, 1 ICP x 5 Gauss-Newton x 10
PCG): afx_fusion_reset, then frames 0..29 (frame 0 rigid, 29 non-rigid).  Every step is the
same work.  L2 is flushed (a 256 MiB write) between steps.

  value : frames/s with the depth frames already resident in HBM (afx_fusion_process)
  e2e   : frames/s through the C ABI with host depth buffers (afx_fusion_process_host from
          pinned memory + a device-to-host read of the frame statistics every frame, frames
          submitted back to back so that a frame's copy in overlaps the frame before it)
  p50/p99 frame latency from a second e2e pass that waits for every frame's statistics.
  dense_graph : the same sequence with the graph radius lowered to 7 mm (about 1500 nodes),
          device-resident, for the solver at the stated graph size.

--impl reference times the reference's CPU path (the oracle port of it, with all host threads:
the reference's own CPU code covers only rigid integration, marching cubes and the graph build,
its warp, solve and warped integration being GPU code; those three of its own functions are
timed single-threaded in cpu_baseline.reference_stages).  Under torchrun each rank runs an
independent replica (the path does not shard); value is the sum over ranks.
"""
import argparse
import ctypes as C
import json
import os
import platform
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_FRAMES = 30


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--clip", type=int, default=N_FRAMES, help="frames of the sequence per step")
    ap.add_argument("--no-dense-graph", action="store_true")
    ap.add_argument("--no-precision", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-rigid-stream", action="store_true")
    ap.add_argument("--no-served", action="store_true")
    ap.add_argument("--no-ingest", action="store_true")
    ap.add_argument("--profile-ingest", action="store_true",
                    help="run the depth-ingest kernels once at the headline size (for an ncu capture)")
    ap.add_argument("--served-streams", type=int, default=64)
    ap.add_argument("--served-seconds", type=float, default=4.0)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-reference-gpu", action="store_true", help="skip the reference's own GPU loop")
    ap.add_argument("--cpu-frames", type=int, default=3)
    ap.add_argument("--profile-step", action="store_true",
                    help="for ncu: the headline session, two warm steps, then one step with the marching-cubes tile "
                         "--mc-tile; prints the library kernel launches before that step and in it, and exits")
    ap.add_argument("--mc-tile", type=int, default=6, help="marching-cubes tile of --profile-step (6, the persistent "
                                                            "grid of 4-deep bricks: the one the autotuner picks on "
                                                            "this workload)")
    return ap.parse_args()


def profile_step(args):
    """The headline workload as ncu should see it: reset + frames 0..29 twice to warm up (frame graphs
    captured), the marching-cubes tile fixed (the autotuner would time tiles under the profiler), then one
    more step.  Prints "<launches before the step> <launches in the step>" for ncu's -s / -c."""
    import torch
    from volumefusion_gb300 import configs
    from volumefusion_gb300.fusion import FusionSession
    cfg = configs.nonrigid_capsules_256(n_frames=N_FRAMES)
    frames = [torch.from_numpy(f.astype(np.int16)).cuda() for f in configs.capsule_frames(cfg)]
    stream = torch.cuda.Stream()
    s = FusionSession(cfg, stream=stream)
    with torch.cuda.stream(stream):
        for step in range(3):
            if step == 1:
                torch.cuda.synchronize()
                s.set_tile(args.mc_tile)
            l0 = s.kernel_launches()
            s.reset()
            for f in frames:
                s.process(f)
            torch.cuda.synchronize()
    print(l0, s.kernel_launches() - l0, flush=True)
    s.close()


def profile_ingest(args):
    """The depth-ingest kernels as ncu should see them, at the headline size: a session with a distorted
    camera (map built at create) over frames 0..3 of the sequence seen through that lens (frame
    preparation samples through the cv::undistort map), then the stand-alone remap in both modes."""
    import torch
    from volumefusion_gb300 import configs, ingest
    from volumefusion_gb300.fusion import FusionSession
    cfg = dict(configs.nonrigid_capsules_256(n_frames=N_FRAMES), distortion=INGEST_DISTORTION)
    frames = [torch.from_numpy(f.astype(np.int16)).cuda() for f in configs.capsule_frames(cfg, frames=range(4))]
    s = FusionSession(cfg)
    for f in frames:
        s.process(f)
    torch.cuda.synchronize()
    K = np.asarray(cfg["K"], np.float32)
    src = frames[1].float() * 0.001
    for mode in (ingest.LINEAR, ingest.NEAREST):
        u = ingest.Undistorter(K, INGEST_DISTORTION, cfg["width"], cfg["height"], mode=mode)
        u(src)
    torch.cuda.synchronize()
    print("ok", s.stats()["error"], flush=True)
    s.close()


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


def dist_setup(n, backend="nccl"):
    """The process group of an N-replica run launched by torchrun (one rank per GPU), or None."""
    if n <= 1 or "RANK" not in os.environ:
        return None
    import torch.distributed as dist
    dist.init_process_group(backend)
    return dist


def max_over_ranks(x, dist, device):
    """The largest x over the ranks, on every rank (x itself without a process group): the timed
    region of an N-replica run is the slowest rank's."""
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    if dist:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, world, max_seconds):
    """Units per second of the whole job: every replica processes units_per_rank in the timed
    region, which lasts as long as the slowest rank (weak scaling)."""
    return world * units_per_rank / max_seconds


def headline_config(cfg, clip, world):
    """The workload description both arms report (the reference arm times the same steps)."""
    return {"workload": cfg["name"],
            "frames": "640x576 capsule pair, 30-frame sequence",
            "step": "reset + frames 0..%d (frame 0 rigid)" % (clip - 1),
            "volume": "256^3 FP32 TSDF @ 4 mm (134 MB tsdf+weights, larger than L2)",
            "graph_radius_mm": 25, "knn": 4, "kreg": 8, "gn": "1 ICP x 5 GN x 10 PCG",
            "parallelism": "replicas" if world > 1 else "single",
            "l2": "GPU arm: L2 flushed between steps (256 MiB write)"}


def cpu_model():
    """The host CPU's model name and logical core count."""
    name = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.split(":")[0].strip() == "Model name":
                name = line.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    if not name:
        try:
            for line in open("/proc/cpuinfo"):
                if line.lower().startswith("model name"):
                    name = line.split(":", 1)[1].strip()
                    break
        except OSError:
            pass
    return {"model": name or platform.processor() or platform.machine(), "nproc": os.cpu_count()}


def cpu_baseline(cfg, frames_np, n_frames):
    """Oracle port of the reference path on the host cores (all threads)."""
    from oracle import pyoracle as O
    O.set_threads(os.cpu_count() or 1)
    o = O.Fusion(dict(cfg))
    o.process(frames_np[0])
    t0 = time.perf_counter()
    for f in range(1, min(n_frames, N_FRAMES - 1) + 1):
        o.process(frames_np[f])
    dt = time.perf_counter() - t0
    o.close()
    return n_frames / dt, dt


def reference_cpu_stages(cfg, frames_np):
    """The reference's own CPU code for three stages of the path (oracle/_ref/libvfref.so, built from
    its unchanged sources for this host), each timed once, single-threaded as it is written, on the
    headline frame: TSDFVolume::integrate of frame 0 into an empty 256^3 volume (src/TSDFVolume.cpp:55),
    MarchingCubes::computeIsoSurface of that volume (src/MarchingCubes.cpp:297), and af::buildGraph +
    af::getKnnData<4> on its sorted, de-duplicated point cloud (src/GraphBuilder.cpp:12,
    include/af/GraphBuilder.h:20)."""
    path = os.path.join(ROOT, "oracle", "_ref", "libvfref.so")
    if not os.path.exists(path):
        return {"unavailable": "oracle/_ref/libvfref.so was not built (reference sources not staged)"}
    from oracle import pyoracle as O
    R = C.CDLL(path)
    R.ref_marching_cubes.restype = C.c_long

    def ptr(a):
        return a.ctypes.data_as(C.c_void_p)

    K = np.asarray(cfg["K"], np.float32)
    dims = np.asarray(cfg["dims"], np.int32)
    size = np.asarray(cfg["volume_size"], np.float32)
    vs = size / dims.astype(np.float32)
    S = int(np.prod(dims))
    depth = O.depth_from_mm(frames_np[0])  # the CPU class reads 0 as "no depth"
    _, _, _, c = O.frame_prep(frames_np[0], K)
    pose = np.eye(4, dtype=np.float32)
    pose[:3, 3] = c
    t, w = np.empty(S, np.float32), np.empty(S, np.float32)
    h, wd = depth.shape
    a = time.perf_counter()
    R.ref_integrate(ptr(t), ptr(w), ptr(np.ascontiguousarray(depth, np.float32)), wd, h, ptr(O.kcol(K)), ptr(dims),
                    ptr(size), C.c_float(cfg["delta"]), ptr(np.ascontiguousarray(pose.T).ravel()))
    t_int = time.perf_counter() - a
    cap = 4_000_000
    v = np.empty((cap, 3), np.float32)
    f = np.empty((cap, 3), np.int32)
    nf = C.c_long(0)
    a = time.perf_counter()
    nv = R.ref_marching_cubes(ptr(t), ptr(w), ptr(dims), ptr(size), C.c_float(0.0), 0, ptr(v), C.c_long(cap), ptr(f),
                              C.c_long(cap), C.byref(nf))
    t_mc = time.perf_counter() - a
    mesh = O.translate(O.sort_unique(O.mc_pointcloud(t, w, dims, vs, size)), c)
    ncap = 20000
    nn, rr, TT = np.zeros((ncap, 3), np.float32), np.zeros(ncap, np.float32), np.zeros((ncap, 16), np.float32)
    a = time.perf_counter()
    n = R.ref_build_graph(ptr(nn), ptr(rr), ptr(TT), 0, ncap, ptr(mesh), C.c_long(len(mesh)), int(cfg["knn"]),
                          C.c_float(cfg["graph_radius"]))
    t_graph = time.perf_counter() - a
    k = int(cfg["knn"])
    idx, dist = np.empty((len(mesh), k), np.uint32), np.empty((len(mesh), k), np.float32)
    a = time.perf_counter()
    R.ref_knn(ptr(nn), ptr(rr), int(n), ptr(mesh), C.c_long(len(mesh)), k, 0, ptr(idx), ptr(dist))
    t_knn = time.perf_counter() - a
    return {"kind": "reference", "cores": 1, "cpu": cpu_model(),
            "sample": "one call of each on frame 0 of the sequence (%dx%d depth, %d^3 volume)" % (wd, h, dims[0]),
            "integrate_ms": 1000 * t_int, "marching_cubes_ms": 1000 * t_mc, "triangles": int(nf.value),
            "vertices": int(nv), "build_graph_ms": 1000 * t_graph, "nodes": int(n), "points": len(mesh),
            "knn_ms": 1000 * t_knn}


def reference_gpu_arm(cfg, frames_np, stream, timeout_s=600):
    """The reference's own per-frame loop on this GPU: af::runVolumeFusion (src/VolumeFusion.cu:223-783)
    and every kernel, thrust call and cuSOLVER LU it makes, compiled unchanged for sm_103a
    (oracle/ref_gpu/build.py -> oracle/_ref/libvfref_gpu.so), fed the headline sequence from memory in a
    child process with a time limit (oracle/ref_gpu/run.py).  Its compile-time constants stay its own
    (256^3, K = 6 skinning, K_reg = 4, up to 20 Gauss-Newton iterations per ICP iteration with its
    energy-step break), so this library runs the same sequence with those settings beside it
    (device-resident frames, same ICP count, radius and weights)."""
    import torch
    from volumefusion_gb300.fusion import FusionSession
    lib_path = os.path.join(ROOT, "oracle", "_ref", "libvfref_gpu.so")
    build_s = 0.0
    if not os.path.exists(lib_path):
        sys.path.insert(0, os.path.join(ROOT, "oracle", "ref_gpu"))
        try:
            import build as ref_build
            t0 = time.perf_counter()
            ref_build.build()
            build_s = time.perf_counter() - t0
        except Exception as e:  # no staged sources, or the compile failed
            return {"unavailable": "reference GPU build: %s" % str(e).splitlines()[0][:200]}
    n = len(frames_np)
    try:
        p = subprocess.run([sys.executable, os.path.join(ROOT, "oracle", "ref_gpu", "run.py"), "--frames", str(n),
                            "--runs", "2"], capture_output=True, text=True, timeout=timeout_s)
    except subprocess.TimeoutExpired:
        return {"unavailable": "the reference loop did not finish within %d s" % timeout_s}
    if p.returncode != 0:
        return {"unavailable": "the reference loop exited with %d: %s" % (p.returncode, p.stderr.strip()[-300:])}
    runs = json.loads(p.stdout.strip().splitlines()[-1])["runs"]
    last = runs[-1]
    if last["rc"] != 0:
        return {"unavailable": "the reference loop stopped at frame %d: %s %s" % (
            int(np.count_nonzero(np.asarray(last["frame_ms"]))), last["error"], p.stderr.strip()[-200:])}
    ms = np.asarray(last["frame_ms"])
    ref_fps = (n - 1) / (ms[1:].sum() / 1000.0)
    # this library on the reference's constants, the same frames
    same = dict(cfg, knn=6, kreg=4, gn_iterations=20, name=cfg["name"] + "_reference_constants")
    frames_dev = [torch.from_numpy(f.astype(np.int16)).cuda() for f in frames_np]
    s = FusionSession(same, stream=stream)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        for step in range(3):
            s.reset()
            s.process(frames_dev[0])
            if step == 2:
                ev0.record(stream)
            for f in range(1, n):
                s.process(frames_dev[f])
        ev1.record(stream)
    torch.cuda.synchronize()
    ours_ms = ev0.elapsed_time(ev1)
    st = s.stats()
    s.close()
    ours_fps = (n - 1) / (ours_ms / 1000.0)
    return {"kind": "reference GPU loop (af::runVolumeFusion, unchanged, sm_103a)",
            "frames": "1..%d of the headline sequence (non-rigid), second of two runs" % (n - 1),
            "frames_per_s": ref_fps, "nodes_last_frame": last.get("nodes"),
            "ms_per_frame_median": float(np.median(ms[1:])),
            "ms_per_frame_max": float(ms[1:].max()), "ms_frame0": float(ms[0]), "build_s": build_s,
            "constants": "256^3, K=6, K_reg=4, <=20 GN iterations per ICP iteration (energy-step break), "
                         "dense J + cuSOLVER LU, graph build and KNN on the host",
            "ours_same_constants": {"frames_per_s": ours_fps, "nodes_last_frame": st["n_nodes"],
                                    "gn_iterations_last_frame": st["gn_iterations_done"]},
            "ratio_ours_over_reference": ours_fps / ref_fps}


def run_reference(args):
    """The reference's CPU path (the oracle's restatement of it) on the host cores, on the GPU
    arm's workload: a step is the same reset + frames 0..clip-1 of the sequence (frame 0 rigid,
    then non-rigid frames), all host threads."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from volumefusion_gb300 import configs
    cfg = configs.nonrigid_capsules_256(n_frames=N_FRAMES)
    frames_np = configs.capsule_frames(cfg)
    from oracle import pyoracle as O
    O.set_threads(os.cpu_count() or 1)  # every host thread, whatever the launcher set

    clip = max(1, min(args.clip, N_FRAMES))

    def step():
        t0 = time.perf_counter()
        o = O.Fusion(dict(cfg))  # the reset: an empty volume and graph
        for f in range(clip):
            o.process(frames_np[f])
        dt = time.perf_counter() - t0
        o.close()
        return dt

    for _ in range(args.warmup):
        step()
    dt = sum(step() for _ in range(args.steps))
    n = args.steps * clip
    fps = n / dt
    cores = O.threads()
    host = cpu_model()
    line = {
        "impl": "reference", "metric": "nonrigid_frames_per_s_256", "value": fps, "unit": "frames/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": headline_config(cfg, clip, args.gpus),
        "cpu_baseline": {"value": fps, "unit": "frames/s", "cores": cores, "kind": "port", "cpu": host,
                         "sample": "%d steps of reset + frames 0..%d (the GPU arm's step), after %d warm-up steps, "
                                   "all host threads (OpenMP)" % (args.steps, clip - 1, args.warmup)},
        "e2e": {"value": fps, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def ncu_traffic(stage):
    """DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of the stage's kernel from
    the committed ncu summary of the same workload, or None."""
    files = {"marching_cubes": "mc_pipe_kernel_capsules256.md"}
    if stage not in files:
        return None
    path = os.path.join(ROOT, "profiles", files[stage])
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("traffic_bytes_per_launch:"):
            return float(line.split(":", 1)[1])
    return None


def stage_bytes(cfg, st):
    """Algorithmic bytes per frame of the stages with an exact HBM figure."""
    S = int(np.prod(cfg["dims"]))
    P = cfg["width"] * cfg["height"]
    A = st.get("active_voxels", 0)
    return {
        "prep": P * (2.0 + 4.0 + 24.0),
        # the reference's kernel reads every voxel (8 B); this one reads the 8^3 bricks that hold a
        # weighted voxel (the rest cannot contain a cube with all eight weights set), then writes
        # 12 B per point (with the four edge copies) and 48 B per triangle
        "marching_cubes": 8.0 * 512 * st.get("occupied_bricks", S // 512) + 12.0 * st["mesh_points"] * 4
                          + 48.0 * st["mesh_faces"],
        # 16 B per supported voxel (value + weight read and written) + the collision word (4 B)
        "warped_integrate": 20.0 * A if A else None,
    }


def rigid_integration_arm(stream, barrier, hbm, frame_mm):
    """runIntegrateTSDFFromFrameKernel (afx_integrate_tsdf) alone at 256^3 / 4 mm on the sequence's first
    frame, into an initialised volume (268 MB of values + weights, larger than L2).  achieved uses the
    algorithmic bytes of the step, 16 B per voxel (values and weights read and written); the kernel
    itself only loads and stores the 4-voxel groups a frame updates."""
    import ctypes as C

    import torch
    from volumefusion_gb300 import configs
    from volumefusion_gb300._lib import check, lib
    cfg = configs.nonrigid_capsules_256(n_frames=N_FRAMES)
    dims, size = cfg["dims"], cfg["volume_size"]
    S = int(np.prod(dims))
    mm = torch.as_tensor(frame_mm).cuda().to(torch.int32)
    depth = (mm.float() * 0.001).contiguous()
    valid = mm > 0
    K = np.asarray(cfg["K"], np.float64)
    vv, uu = torch.nonzero(valid, as_tuple=True)
    z = depth[valid].double()
    cen = [float((((uu.double() - K[0, 2]) * z) / K[0, 0]).mean()), float((((vv.double() - K[1, 2]) * z) / K[1, 1]).mean()),
           float(z.mean())]
    tsdf = torch.full((S,), -1.0, device="cuda")
    weights = torch.zeros(S, device="cuda")
    f = lambda a: (C.c_float * len(a))(*[float(x) for x in a])  # noqa: E731
    col = lambda m: f(np.asarray(m, np.float64).T.ravel())  # noqa: E731
    vs = [s_ / d for s_, d in zip(size, dims)]
    args_c = (C.c_void_p(tsdf.data_ptr()), C.c_void_p(weights.data_ptr()), C.c_void_p(depth.data_ptr()),
              cfg["width"], cfg["height"], C.c_float(cfg["delta"]), (C.c_int * 3)(*dims), f(vs), f(size),
              col(np.eye(3)), f(cen), col(K), C.c_void_p(stream.cuda_stream))
    for _ in range(3):
        check(lib().afx_integrate_tsdf(*args_c), "afx_integrate_tsdf")
    reps = 20
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        check(lib().afx_integrate_tsdf(*args_c), "afx_integrate_tsdf")
    e1.record(stream)
    barrier()
    ms = e0.elapsed_time(e1) / reps
    updated = int((weights > 0).sum())
    gbs = 16.0 * S / (ms / 1000.0) / 1e9
    del tsdf, weights
    return {"kernel": "integrate_rigid_x4_kernel", "volume": "256^3 FP32 @ 4 mm", "ms": ms, "algorithmic_bytes": 16 * S,
            "achieved_gbs": gbs, "peak_gbs": hbm, "frac": gbs / hbm, "voxels_updated": updated,
            "note": "16 B per voxel is the reference kernel's traffic; this kernel loads and stores only the 4-voxel "
                    "groups the frame updates (%.1f%% of voxels updated)" % (100.0 * updated / S)}


def rigid_stream_arm(args, stream, barrier, reduce_max, world, hbm):
    """The rigid multi-camera stream at the reference's default volume (400^3 over 1 m, rotated
    45/-45/0 degrees): 3 cameras of 640x576 capsule frames, 30 frames per step; and the fused
    initialise + integrate kernel timed alone on that volume (8 B per voxel written)."""
    import ctypes as C

    import torch
    from volumefusion_gb300 import configs
    from volumefusion_gb300._lib import check, lib
    from volumefusion_gb300.rigid_stream import RigidStream

    cfg = configs.nonrigid_capsules_256(n_frames=N_FRAMES)
    frames = [torch.from_numpy(f.astype(np.int16)).cuda() for f in configs.capsule_frames(cfg)]
    K = np.asarray(cfg["K"], np.float32)

    def rot(axis, deg):
        a = np.radians(deg)
        c, s_ = np.cos(a), np.sin(a)
        return {"x": np.array([[1, 0, 0], [0, c, -s_], [0, s_, c]]), "y": np.array([[c, 0, s_], [0, 1, 0], [-s_, 0, c]]),
                "z": np.array([[c, -s_, 0], [s_, c, 0], [0, 0, 1]])}[axis]

    def pose(R, t):
        T = np.eye(4)
        T[:3, :3], T[:3, 3] = R, t
        return T

    c2w = [np.eye(4), pose(rot("y", 20), [0.15, 0.0, 0.05]), pose(rot("x", -15), [0.0, -0.1, 0.02])]
    mm0 = frames[0].cpu().numpy().astype(np.float64)
    v, u = np.nonzero(mm0 > 0)
    z = mm0[v, u] / 1000.0
    center = [float(np.mean((u - K[0, 2]) * z / K[0, 0])), float(np.mean((v - K[1, 2]) * z / K[1, 1])), float(np.mean(z))]
    R = (rot("x", 45) @ rot("y", -45)).astype(np.float32)  # settings.tsdfRotation default (45, -45, 0)
    dims, size = (400, 400, 400), (1.0, 1.0, 1.0)
    rs = RigidStream([K] * 3, c2w, cfg["width"], cfg["height"], dims, size, 0.016, center, R, stream=stream)
    nf = N_FRAMES

    def run(steps):
        with torch.cuda.stream(stream):
            for _ in range(steps):
                for i in range(nf):
                    rs.process([frames[i], frames[(i + 10) % nf], frames[(i + 20) % nf]])

    run(1)
    barrier()
    steps = max(1, min(3, args.steps))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    run(steps)
    e1.record(stream)
    barrier()
    fps = world * steps * nf / (reduce_max(e0.elapsed_time(e1)) / 1000.0)
    _, verts, _, _, _ = rs.outputs()
    rs.close()
    # the fused initialise + integrate kernel alone, on a volume of the same size
    S = int(np.prod(dims))
    tsdf = torch.empty(S, device="cuda")
    weights = torch.empty(S, device="cuda")
    depth = (frames[0].float() * 0.001).contiguous()
    f = lambda a: (C.c_float * len(a))(*[float(x) for x in a])  # noqa: E731
    col = lambda m: f(np.asarray(m, np.float64).T.ravel())  # noqa: E731
    args_c = (C.c_void_p(tsdf.data_ptr()), C.c_void_p(weights.data_ptr()), C.c_void_p(depth.data_ptr()),
              cfg["width"], cfg["height"], C.c_float(0.016), (C.c_int * 3)(*dims), f([s_ / d for s_, d in zip(size, dims)]),
              f(size), col(R), f(center), col(K), C.c_void_p(stream.cuda_stream))
    for _ in range(3):
        check(lib().afx_integrate_tsdf_fresh(*args_c), "afx_integrate_tsdf_fresh")
    reps = 20
    barrier()
    e0.record(stream)
    for _ in range(reps):
        check(lib().afx_integrate_tsdf_fresh(*args_c), "afx_integrate_tsdf_fresh")
    e1.record(stream)
    barrier()
    ms = e0.elapsed_time(e1) / reps
    gbs = 8.0 * S / (ms / 1000.0) / 1e9
    del tsdf, weights
    torch.cuda.empty_cache()
    return {"cameras": 3, "volume": "400^3 over 1 m, rotated (45, -45, 0) deg", "frames_per_s": fps,
            "mesh_vertices_last_frame": int(verts.shape[0]),
            "fresh_integration": {"ms": ms, "bytes": 8 * S, "achieved_gbs": gbs, "peak_gbs": hbm, "frac": gbs / hbm,
                                  "note": "write-only: 8 B per voxel; outputs (512 MB) larger than L2"}}


def encode_depth_png(img, level=1):
    """16-bit greyscale PNG of a depth frame the way libpng writes it by default: per scanline the
    filter whose bytes have the smallest sum of absolute values (as signed bytes), zlib at `level`
    (cv::imwrite's default PNG compression is 1).  Synthetic input for the ingest measurement."""
    import struct
    import zlib
    x = np.ascontiguousarray(img.astype(">u2")).view(np.uint8).reshape(img.shape[0], -1).astype(np.int16)
    a = np.zeros_like(x)
    a[:, 2:] = x[:, :-2]
    b = np.zeros_like(x)
    b[1:] = x[:-1]
    c = np.zeros_like(x)
    c[1:, 2:] = x[:-1, :-2]
    p = a + b - c
    pa, pb, pc = np.abs(p - a), np.abs(p - b), np.abs(p - c)
    paeth = np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))
    cand = np.stack([x, x - a, x - b, x - (a + b) // 2, x - paeth]) & 0xFF
    cost = np.minimum(cand, 256 - cand).sum(axis=2)
    pick = cost.argmin(axis=0)
    rows = cand[pick, np.arange(x.shape[0])].astype(np.uint8)
    raw = np.concatenate([pick.astype(np.uint8)[:, None], rows], axis=1).tobytes()

    def chunk(kind, data):
        return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data) & 0xFFFFFFFF)

    h, w = img.shape
    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 16, 0, 0, 0, 0)) +
            chunk(b"IDAT", zlib.compress(raw, level)) + chunk(b"IEND", b""))


# A depth camera's distortion for the ingest measurement (rational model, as depthDistortion.txt holds it)
INGEST_DISTORTION = dict(k1=0.45, k2=-0.05, p1=4e-5, p2=-6e-5, k3=0.003, k4=0.78, k5=0.01, k6=0.0)


def ingest_arm(args, cfg, frames_np, stream, barrier):
    """Depth ingest on the headline frames: host decoding of their PNG files (one thread and all host
    threads), the cost of undistorting every frame inside the session (cv::undistort before the
    filter; the undistorted session fuses the same scene seen through a lens with INGEST_DISTORTION),
    and frames/s from PNG bytes in host memory through decode + fusion."""
    import concurrent.futures as cf
    import torch
    from volumefusion_gb300 import configs, ingest
    from volumefusion_gb300.fusion import FusionSession
    clip = max(1, min(args.clip, N_FRAMES))
    blobs = [encode_depth_png(f) for f in frames_np[:clip]]
    raw_bytes = int(frames_np[0].nbytes)
    # one thread
    for b in blobs[:3]:
        ingest.decode_depth(b)
    t0 = time.perf_counter()
    reps = 3
    for _ in range(reps):
        for b in blobs:
            ingest.decode_depth(b)
    one = reps * len(blobs) / (time.perf_counter() - t0)
    # every host thread, batches of the sequence
    threads = os.cpu_count() or 1
    outs = [np.empty(frames_np[0].shape, np.uint16) for _ in blobs]
    batch = blobs * 4
    outs4 = outs * 4
    ingest.decode_depth_many(batch, threads=threads, outs=outs4)
    t0 = time.perf_counter()
    for _ in range(reps):
        ingest.decode_depth_many(batch, threads=threads, outs=outs4)
    many = reps * len(batch) / (time.perf_counter() - t0)
    assert all(np.array_equal(o, f) for o, f in zip(outs, frames_np[:clip]))
    res = {"workload": "the %d headline frames (640x576 uint16) as 16-bit PNG, libpng's default per-row filter "
                       "choice, zlib level 1; %.0f kB per file" % (clip, np.mean([len(b) for b in blobs]) / 1e3),
           "decode_one_thread": {"frames_per_s": one, "mb_per_s": one * raw_bytes / 1e6},
           "decode_all_threads": {"frames_per_s": many, "threads": threads, "mb_per_s": many * raw_bytes / 1e6}}
    # undistortion inside the session: device-resident frames, with and without a distorted camera
    dcfg = dict(cfg, distortion=INGEST_DISTORTION)
    seq = {"plain": frames_np[:clip], "undistorted": configs.capsule_frames(dcfg)[:clip]}
    per = {}
    for name, c in (("plain", cfg), ("undistorted", dcfg)):
        frames_dev = [torch.from_numpy(f.astype(np.int16)).cuda() for f in seq[name]]
        t_create = time.perf_counter()
        s = FusionSession(c, stream=stream)
        create_ms = 1000 * (time.perf_counter() - t_create)
        with torch.cuda.stream(stream):
            for _ in range(2):
                s.reset()
                for f in frames_dev:
                    s.process(f)
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        steps = max(1, min(3, args.steps))
        with torch.cuda.stream(stream):
            e0.record(stream)
            for _ in range(steps):
                s.reset()
                for f in frames_dev:
                    s.process(f)
            e1.record(stream)
        barrier()
        s.set_timing(True)
        s.stage_times(reset=True)
        with torch.cuda.stream(stream):
            s.reset()
            for f in frames_dev:
                s.process(f)
        barrier()
        stages = {k: v / clip for k, v in s.stage_times(reset=True).items()}
        s.set_timing(False)
        st = s.stats(check_errors=False)
        per[name] = {"frames_per_s": steps * clip / (e0.elapsed_time(e1) / 1000.0),
                     "prep_ms_per_frame": stages.get("prep", 0.0), "stage_ms_per_frame": stages,
                     "create_ms": create_ms, "error": st["error"],
                     "last_frame": {k: st[k] for k in ("n_nodes", "mesh_points", "correspondences")}}
        s.close()
    res["session"] = per
    # the stand-alone undistortion kernel on one frame (map built once), both modes
    K = np.asarray(cfg["K"], np.float32)
    src = torch.from_numpy(frames_np[1].astype(np.float32) * np.float32(0.001)).cuda()
    H, W = frames_np[0].shape
    kern = {}
    for mode, name in ((ingest.LINEAR, "linear"), (ingest.NEAREST, "nearest")):
        u = ingest.Undistorter(K, INGEST_DISTORTION, W, H, mode=mode)
        out = torch.empty_like(src)
        for _ in range(10):
            u(src, out=out)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        n = 200
        cur = torch.cuda.current_stream()
        e0.record(cur)
        for _ in range(n):
            u(src, out=out)
        e1.record(cur)
        torch.cuda.synchronize()
        us = 1000 * e0.elapsed_time(e1) / n
        kern[name] = {"us_per_launch": us, "algorithmic_bytes": W * H * 16,
                      "achieved_gbs": W * H * 16 / (us * 1e-6) / 1e9}
    res["undistort_kernel"] = kern
    # PNG bytes in host memory -> decode on a thread pool into pinned buffers -> the session (e2e)
    ring = 8
    pinned = [torch.empty(frames_np[0].shape, dtype=torch.int16).pin_memory() for _ in range(ring)]
    views = [p.numpy().view(np.uint16) for p in pinned]
    s = FusionSession(cfg, stream=stream)
    pool = cf.ThreadPoolExecutor(max_workers=min(threads, ring))

    def decode_into(i):
        ingest.decode_depth_many([blobs[i % clip]], threads=1, outs=[views[i % ring]])
        return i

    from volumefusion_gb300._lib import FrameStats, lib as _afx_lib
    stats_host = torch.empty(clip * C.sizeof(FrameStats), dtype=torch.uint8).pin_memory()
    slot_done = [None] * ring  # event after the frame that last read each pinned slot

    def run(steps):
        total = steps * clip
        futs = {i: pool.submit(decode_into, i) for i in range(min(ring - 1, total))}
        for i in range(total):
            if i % clip == 0:
                s.reset()
            futs.pop(i).result()
            s.process_host_ptr(pinned[i % ring].data_ptr())
            rc = _afx_lib().afx_fusion_stats_async(s.h, C.c_void_p(stats_host.data_ptr() + (i % clip) * C.sizeof(FrameStats)),
                                                   C.c_void_p(stream.cuda_stream))
            if rc:
                raise RuntimeError("afx_fusion_stats_async failed: %d" % rc)
            ev = torch.cuda.Event()
            ev.record(stream)
            slot_done[i % ring] = ev
            j = i + ring - 1
            if j < total:
                prev = slot_done[j % ring]  # the frame that last read slot j % ring
                if prev is not None:
                    prev.synchronize()
                futs[j] = pool.submit(decode_into, j)
        stream.synchronize()
        return total

    run(1)
    barrier()
    t0 = time.perf_counter()
    n = run(max(1, min(3, args.steps)))
    barrier()
    res["e2e_from_png"] = {"frames_per_s": n / (time.perf_counter() - t0), "decode_threads": min(threads, ring),
                           "note": "PNG bytes in host memory decoded on host threads ahead of the session into a ring "
                                   "of pinned buffers (a buffer is refilled once the frame that read it has run); "
                                   "frames submitted back to back through afx_fusion_process_host, each frame's "
                                   "statistics read into pinned memory"}
    pool.shutdown()
    s.close()
    return res


def batched_arm(args, stream, barrier, reduce_max, world):
    """16 sessions of uneven size (the config-4 mix: volumes 128^3-384^3, 320x288 or 640x576,
    sphere / torus / capsule) fusing 30-frame sequences: one afx_batch_process per frame of all
    sessions (frames 3.. as one graph launch) against the plain drop-in running the same sessions
    one after another; marching-cubes tiles chosen per session by the autotuner first."""
    import torch
    from volumefusion_gb300 import configs
    from volumefusion_gb300.batch import Batch
    from volumefusion_gb300.fusion import FusionSession

    pool = configs.session_mix(16, seed=3)
    nf = 30
    frames = [[torch.from_numpy(configs.scene_frame(c, i).astype(np.int16)).cuda() for i in range(nf)] for c in pool]
    sessions = [FusionSession(c, stream=stream) for c in pool]
    batch = Batch(sessions)

    def run_batch(steps):
        with torch.cuda.stream(stream):
            for _ in range(steps):
                for s in sessions:
                    s.reset()
                for i in range(nf):
                    batch.process([frames[k][i] for k in range(len(sessions))], stream)

    def run_plain(steps):
        with torch.cuda.stream(stream):
            for _ in range(steps):
                for k, s in enumerate(sessions):
                    s.reset()
                    for i in range(nf):
                        s.process(frames[k][i])

    run_batch(1)
    barrier()
    tiles = [s.autotune()[0] for s in sessions]  # on each session's last volume
    run_batch(1)  # graphs captured again with the chosen tiles
    barrier()
    steps = max(1, min(3, args.steps))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g0 = batch.graph_launches()
    e0.record(stream)
    run_batch(steps)
    e1.record(stream)
    barrier()
    bms = reduce_max(e0.elapsed_time(e1))
    glaunch = batch.graph_launches() - g0
    st = batch.stats(stream)
    run_plain(1)
    barrier()
    e0.record(stream)
    run_plain(steps)
    e1.record(stream)
    barrier()
    pms = reduce_max(e0.elapsed_time(e1))
    total = steps * nf * len(sessions)
    out = {"sessions": len(sessions), "volumes": sorted(int(c["dims"][0]) for c in pool),
           "frames_per_session_step": nf, "frames_per_s": world * total / (bms / 1000.0),
           "plain_frames_per_s": world * total / (pms / 1000.0), "graph_launches_per_step": glaunch // steps,
           "mc_tiles": tiles, "errors": sum(int(x["error"] != 0) for x in st),
           "nodes": [int(x["n_nodes"]) for x in st]}
    out["batched_over_plain"] = out["frames_per_s"] / out["plain_frames_per_s"]
    batch.close()
    for s in sessions:
        s.close()
    torch.cuda.empty_cache()
    return out


def served_arm(args, rank):
    """Many depth streams through afx_server: (1) the offered load -- N streams at 30 fps with
    exponential inter-arrival times (mean 33 ms), sessions drawn from the mixed workload, each
    stream closing its session after its 30-frame sequence and opening a new one (admission by a
    150 GB budget); (2) capacity -- the same sessions with frames submitted as fast as their
    four slots allow; (3) the plain per-stream drop-in -- those sessions' frames one session at
    a time through FusionSession, nothing overlapping."""
    import heapq

    import torch
    from volumefusion_gb300 import configs
    from volumefusion_gb300.fusion import FusionSession
    from volumefusion_gb300.serve import Server

    n = args.served_streams
    pool = configs.session_mix(4 * n, seed=7 + rank)
    for c in pool:
        configs.scene_frames(c)  # synthesise outside the timed regions
    budget = 150 << 30
    rng = np.random.default_rng(11 + rank)
    # (1) offered load
    srv = Server(budget, max_sessions=4 * n)
    next_cfg = 0
    streams = []  # [session id, cfg, frames submitted, frames done]
    for _ in range(n):
        cfg = pool[next_cfg % len(pool)]
        next_cfg += 1
        streams.append([srv.open(cfg), cfg, 0, 0])
    t0 = time.perf_counter()
    due = [(t0 + float(rng.exponential(1 / 30.0)), k) for k in range(n)]
    heapq.heapify(due)
    lat, done, denied_reopen, peak, errors = [], 0, 0, 0, 0
    t_end = t0 + args.served_seconds
    while True:
        now = time.perf_counter()
        if now >= t_end and not due:
            break
        while due and due[0][0] <= now:
            t_arr, k = heapq.heappop(due)
            sid, cfg, sent, _ = streams[k]
            if sid is None:  # not admitted yet: retry the open
                sid = streams[k][0] = srv.open(cfg)
            # a frame that finds the session's sequence complete or its slots full is dropped
            if sid is not None and sent < 30 and srv.submit(sid, configs.scene_frame(cfg, sent), tag=sent):
                streams[k][2] += 1
            if now < t_end:
                heapq.heappush(due, (t_arr + float(rng.exponential(1 / 30.0)), k))
        for sid_r, tag, ms, st in srv.poll():
            lat.append(ms)
            done += 1
            errors += st["error"] != 0
            for k, x in enumerate(streams):
                if x[0] == sid_r:
                    x[3] += 1
                    if x[3] == 30:  # sequence finished: close, open the next session
                        srv.close_session(sid_r)
                        cfg = pool[next_cfg % len(pool)]
                        next_cfg += 1
                        nsid = srv.open(cfg)
                        denied_reopen += nsid is None
                        streams[k] = [nsid, cfg, 0, 0]
                    break
        peak = max(peak, srv.usage()["used_bytes"])
        if not due or due[0][0] > time.perf_counter():
            time.sleep(0.0002)
    torch.cuda.synchronize()  # drain: every frame in flight completes
    while True:
        r = srv.poll()
        if not r:
            break
        lat += [x[2] for x in r]
        done += len(r)
    wall = time.perf_counter() - t0
    usage = srv.usage()
    offered_counters = srv.counters()
    srv.close()
    offered = {"streams": n, "seconds": round(wall, 3), "frames": done, "frames_per_s": done / wall,
               "latency_ms_p50": float(np.percentile(lat, 50)) if lat else None,
               "latency_ms_p99": float(np.percentile(lat, 99)) if lat else None,
               "peak_bytes": int(peak), "denied_opens": int(usage["denied"]), "frames_with_error_flags": int(errors)}
    # (2) capacity and (3) plain drop-in on the same sessions and frames
    cap_cfgs = pool[:n]
    frames_per = 30
    srv = Server(budget, max_sessions=n)

    def capacity():
        """All sessions' sequences submitted as fast as their slots allow; (frames, seconds, host s)."""
        sids = [srv.open(c) for c in cap_cfgs]
        sent = [0] * n
        got = 0
        want = frames_per * sum(s is not None for s in sids)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        host_s = 0.0  # time the submitting loop spends inside submit and poll (host work per frame)
        while got < want and time.perf_counter() - t0 < 120.0:
            for k, sid in enumerate(sids):
                while sid is not None and sent[k] < frames_per:
                    h0 = time.perf_counter()
                    ok = srv.submit(sid, configs.scene_frame(cap_cfgs[k], sent[k]))
                    host_s += time.perf_counter() - h0
                    if not ok:
                        break
                    sent[k] += 1
            h0 = time.perf_counter()
            got += len(srv.poll())
            host_s += time.perf_counter() - h0
        wall = time.perf_counter() - t0
        for sid in sids:
            if sid is not None:
                srv.close_session(sid)
        srv.poll()
        return got, wall, host_s, int(sum(s is not None for s in sids))

    def counter_delta(a, b):
        return {k: b[k] - a[k] if k not in ("idle_sessions", "idle_bytes") else b[k] for k in b}

    c0 = srv.counters()
    got, cap_s, host_s, n_sessions = capacity()  # fresh sessions: allocation and graph capture inside
    c1 = srv.counters()
    got_w, cap_w, host_w, _ = capacity()  # the same sessions reopened: reused, graphs kept
    c2 = srv.counters()
    srv.close()
    per_frame = lambda c, frames: {"staging_us": 1000 * c["staging_ms"] / max(frames, 1),  # noqa: E731
                                   "enqueue_us": 1000 * c["enqueue_ms"] / max(frames, 1),
                                   "poll_us": 1000 * c["poll_ms"] / max(frames, 1),
                                   "open_ms_total": c["open_ms"], "opens_fresh": c["opens_fresh"],
                                   "opens_reused": c["opens_reused"]}
    warm = {"frames": got_w, "frames_per_s": got_w / cap_w, "host_busy_frac": host_w / cap_w,
            "host_per_frame": per_frame(counter_delta(c1, c2), got_w)}
    served_fps = got / cap_s
    plain_frames, plain_s = 0, 0.0
    for c in cap_cfgs:  # creation and teardown outside the timed part
        s = FusionSession(c)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i in range(frames_per):
            s.process(configs.scene_frame(c, i))
            s.stats()  # the per-frame result the plain drop-in hands back
            plain_frames += 1
        plain_s += time.perf_counter() - t0
        s.close()
    plain_fps = plain_frames / plain_s
    offered["server_counters"] = {k: offered_counters[k] for k in ("opens_fresh", "opens_reused", "evictions")}
    return {"offered_load": offered,
            "capacity": {"sessions": n_sessions, "frames": got, "frames_per_s": served_fps,
                         "host_busy_frac": host_s / cap_s, "host_per_frame": per_frame(counter_delta(c0, c1), got),
                         "reused_sessions": warm},
            "plain_per_stream": {"frames": plain_frames, "frames_per_s": plain_fps,
                                 "note": "same sessions and frames, one session at a time, host frames"},
            "capacity_over_plain": served_fps / plain_fps,
            "reused_capacity_over_plain": warm["frames_per_s"] / plain_fps}


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.profile_step:
        return profile_step(args)
    if args.profile_ingest:
        return profile_ingest(args)
    import torch
    from volumefusion_gb300 import configs
    from volumefusion_gb300._lib import FrameStats
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
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    clip = max(1, min(args.clip, N_FRAMES))

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    def reduce_max(x):
        return max_over_ranks(x, dist, "cuda")

    def run_device(session, steps):
        """`steps` passes over the sequence, each from an empty volume."""
        with torch.cuda.stream(stream):
            for step in range(steps):
                if step:
                    flush.fill_(step & 0xFF)  # L2 flush between steps
                session.reset()
                for f in range(clip):
                    session.process(frames_dev[f])

    # ---- device-resident arm ----
    s = FusionSession(cfg, stream=stream)
    run_device(s, args.warmup)
    s.stats()
    barrier()
    # marching-cubes tile for this session (the library's autotuner, on the warmed-up volume), then
    # one more warm-up step so that the frame graphs are captured with it
    tile, tile_ms = s.autotune()
    run_device(s, 1)
    s.stats()
    barrier()
    sampler = ClockSampler(local)
    sampler.start()
    l0 = s.kernel_launches()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    run_device(s, args.steps)
    ev1.record(stream)
    barrier()
    sampler.stop()
    launches = s.kernel_launches() - l0
    ms = reduce_max(ev0.elapsed_time(ev1))
    frames = args.steps * clip
    fps = whole_job_rate(frames, world, ms / 1000.0)
    # per-stage breakdown: the same number of steps again, with CUDA events around each stage
    s.set_timing(True)
    s.stage_times(reset=True)
    run_device(s, args.steps)
    barrier()
    stage_ms = s.stage_times(reset=True)
    s.set_timing(False)
    st = s.stats(check_errors=False)
    st["active_bricks"], st["active_voxels"] = s.support_size()
    st["occupied_bricks"], st["bricks"] = s.occupied_bricks()
    s.close()

    # ---- end-to-end arm: host buffers through the C ABI ----
    # Throughput: every frame's pinned host buffer goes in through afx_fusion_process_host and its
    # statistics come back to pinned host memory (afx_fusion_stats_async), frames submitted back to
    # back, so a frame's copy in overlaps the frame before it; the step ends when the last statistics
    # have arrived.  Latency: the same calls with the host waiting for each frame's statistics.
    from volumefusion_gb300._lib import lib as _afx_lib
    s2 = FusionSession(cfg, stream=stream)
    stats_host = torch.empty(clip * C.sizeof(FrameStats), dtype=torch.uint8).pin_memory()

    def run_e2e(steps, lat=None):
        for _ in range(steps):
            s2.reset()
            for f in range(clip):
                a = time.perf_counter()
                s2.process_host_ptr(pinned[f].data_ptr())
                if lat is not None:
                    s2.stats(check_errors=False)  # device-to-host read of the frame result, waited for
                    lat.append(time.perf_counter() - a)
                else:
                    rc = _afx_lib().afx_fusion_stats_async(s2.h, C.c_void_p(stats_host.data_ptr() + f * C.sizeof(FrameStats)),
                                                           C.c_void_p(stream.cuda_stream))
                    if rc:
                        raise RuntimeError("afx_fusion_stats_async failed: %d" % rc)
            stream.synchronize()

    run_e2e(args.warmup)
    barrier()
    t0 = time.perf_counter()
    run_e2e(args.steps)
    barrier()
    e2e_fps = whole_job_rate(frames, world, reduce_max(time.perf_counter() - t0))
    last = FrameStats.from_buffer_copy(bytes(stats_host[(clip - 1) * C.sizeof(FrameStats):].numpy()))
    if last.error:
        raise RuntimeError("frame error flags in the end-to-end run: %d" % last.error)
    # Gauss-Newton iterations (each with one PCG solve) over the step's frames
    fsz = C.sizeof(FrameStats)
    raw_stats = bytes(stats_host.numpy())
    gn_step = sum(FrameStats.from_buffer_copy(raw_stats[f * fsz:(f + 1) * fsz]).gn_iterations_done for f in range(clip))
    lat = []
    run_e2e(args.steps, lat)
    barrier()
    s2.close()

    # ---- the same sequence with a ~1500-node graph (device-resident) ----
    dense = None
    if not args.no_dense_graph:
        dcfg = dict(cfg)
        dcfg["graph_radius"] = 0.007
        sd = FusionSession(dcfg, stream=stream)
        run_device(sd, 1)
        barrier()
        dsteps = max(1, args.steps // 2)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        run_device(sd, dsteps)
        e1.record(stream)
        barrier()
        dms = reduce_max(e0.elapsed_time(e1))
        sd.set_timing(True)
        sd.stage_times(reset=True)
        run_device(sd, 1)
        barrier()
        dstage = {k: v / clip for k, v in sd.stage_times(reset=True).items()}
        sd.set_timing(False)
        dst = sd.stats(check_errors=False)
        sd.close()
        dense = {"graph_radius_mm": 7, "value": world * dsteps * clip / (dms / 1000.0), "unit": "frames/s",
                 "n_nodes_last_frame": dst["n_nodes"], "correspondences_last_frame": dst["correspondences"],
                 "stage_ms_per_frame": dstage}

    # ---- precision form: the sequence at 512^3 / 2 mm, FP16 values + uint16 weights vs FP32 ----
    precision = None
    if not args.no_precision:
        from volumefusion_gb300.serve import session_bytes
        precision = {"workload": "capsule pair, 30 frames, 512^3 @ 2 mm, 9 mm graph radius"}
        for prec in ("fp16", "fp32"):
            pcfg = dict(configs.precision_capsules_512(n_frames=N_FRAMES), precision=prec)
            sp = FusionSession(pcfg, stream=stream)
            run_device(sp, 1)
            barrier()
            ptile, ptile_ms = sp.autotune()
            run_device(sp, 1)
            barrier()
            psteps = max(1, min(2, args.steps))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            run_device(sp, psteps)
            e1.record(stream)
            barrier()
            pms = reduce_max(e0.elapsed_time(e1))
            sp.set_timing(True)
            sp.stage_times(reset=True)
            run_device(sp, 1)
            barrier()
            pstage = {k: v / clip for k, v in sp.stage_times(reset=True).items()}
            sp.set_timing(False)
            pst = sp.stats(check_errors=False)
            sp.close()
            torch.cuda.empty_cache()
            precision[prec] = {"value": world * psteps * clip / (pms / 1000.0), "unit": "frames/s",
                               "session_bytes": session_bytes(pcfg), "n_nodes_last_frame": pst["n_nodes"],
                               "mesh_points_last_frame": pst["mesh_points"],
                               "error": pst["error"], "stage_ms_per_frame": pstage,
                               "mc_tile": ptile, "mc_tile_ms": [round(x, 4) for x in ptile_ms]}

    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    hbm_peak = json.load(open(peaks_path)).get("hbm_gbs", 6800.0) if os.path.exists(peaks_path) else 6800.0
    rigid_int = rigid_integration_arm(stream, barrier, hbm_peak, frames_np[0])
    rigid = None
    if not args.no_rigid_stream:
        rigid = rigid_stream_arm(args, stream, barrier, reduce_max, world, hbm_peak)

    batched = None
    if not args.no_batched:
        batched = batched_arm(args, stream, barrier, reduce_max, world)

    served = None
    if not args.no_served:
        served = served_arm(args, rank)

    ingest_res = None
    if not args.no_ingest and rank == 0:
        ingest_res = ingest_arm(args, cfg, frames_np, stream, barrier)

    # ---- roofline of the dominant stage ----
    per_frame = {k: v / frames for k, v in stage_ms.items()}
    dom = max(per_frame, key=per_frame.get)
    peaks = {}
    pk_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk_path):
        peaks = json.load(open(pk_path))
    hbm = peaks.get("hbm_gbs", 6800.0)
    algo = {k: v for k, v in stage_bytes(cfg, st).items() if v}
    pick = dom if dom in algo else max(algo, key=lambda k: per_frame.get(k, 0.0))
    achieved = algo[pick] / (per_frame[pick] / 1000.0) / 1e9
    roof = {"bound": "hbm", "kernel": pick, "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": achieved / hbm, "traffic": ncu_traffic(pick),
            "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if peaks else "fallback"}
    if pick != dom:
        roof["note"] = "dominant stage is %s (%.3f ms/frame), latency-bound" % (dom, per_frame[dom])
    # the dominant kernel, which no bandwidth roofline describes: one cluster launch per frame running
    # every Gauss-Newton iteration (up to 5) with its PCG (10 iterations, two cluster barriers each)
    pcg_mean = max(1e-9, 10.0 * gn_step / clip)
    roof["dominant_kernel"] = {
        "kernel": "gn_loop_kernel", "ms_per_frame": per_frame.get("gn_loop", 0.0),
        "bound": "latency: cluster barriers and the dot products' reduction chains (1.6 MB of DRAM traffic per launch)",
        "gn_iterations_last_frame": int(st["gn_iterations_done"]), "gn_iterations_per_step": gn_step,
        "pcg_iterations_per_frame_mean": pcg_mean,
        "us_per_pcg_iteration_upper_bound": 1000.0 * per_frame.get("gn_loop", 0.0) / pcg_mean,
        "cluster_barriers_per_pcg_iteration": 2}
    # every stage with an exact byte count, against the same peak
    roof["stages"] = {k: {"ms_per_frame": per_frame.get(k, 0.0), "algorithmic_bytes": v,
                          "achieved_gbs": v / (per_frame[k] / 1000.0) / 1e9 if per_frame.get(k) else None}
                      for k, v in algo.items()}

    ref_gpu = None
    if rank == 0 and world == 1 and not args.no_reference_gpu:
        ref_gpu = reference_gpu_arm(cfg, frames_np, stream)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline and args.cpu_frames > 0:
        v, dt = cpu_baseline(cfg, frames_np, args.cpu_frames)
        from oracle import pyoracle as O
        cpu = {"value": v, "unit": "frames/s", "cores": O.threads(), "kind": "port", "cpu": cpu_model(),
               "sample": "frames 1..%d of the sequence after the rigid frame 0 (%.1f s), all host threads"
                         % (args.cpu_frames, dt)}
        ref_stages = reference_cpu_stages(cfg, frames_np)
        if "unavailable" not in ref_stages:
            # the same stages on the GPU: the rigid integration kernel alone, and per-frame stage times
            ref_stages["gpu_ms"] = {"integrate": rigid_int["ms"] if rigid_int else None,
                                    "marching_cubes": per_frame.get("marching_cubes"),
                                    "build_graph": per_frame.get("graph"), "knn": per_frame.get("knn")}
        cpu["reference_stages"] = ref_stages

    if rank == 0:
        line = {
            "metric": "nonrigid_frames_per_s_256", "value": fps, "unit": "frames/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": headline_config(cfg, clip, world),
            "e2e": {"value": e2e_fps, "unit": "frames/s", "h2d_bytes_per_step": int(frames_np[0].nbytes) * clip,
                    "d2h_bytes_per_step": int(C.sizeof(FrameStats)) * clip,
                    "latency_ms_p50": 1000 * float(np.percentile(lat, 50)),
                    "latency_ms_p99": 1000 * float(np.percentile(lat, 99)),
                    "submission": "frames submitted back to back with each frame's statistics read into pinned "
                                  "memory; latency from a pass that waits for each frame's statistics"},
            "gpu_launches": int(launches),
            "stage_ms_per_frame": per_frame,
            "last_frame_stats": {k: st[k] for k in ("n_nodes", "mesh_points", "correspondences", "gn_iterations_done",
                                                "mesh_faces", "error")},
            "mc_tile": {"chosen": tile, "ms_per_tile": [round(x, 4) for x in tile_ms],
                        "tiles": ["tma16", "tma8", "tma32", "column", "pipe8", "pipe16", "pipe4"]},
            "dense_graph": dense,
            "precision": precision,
            "batched": batched,
            "rigid_stream": rigid,
            "rigid_integration": rigid_int,
            "served": served,
            "ingest": ingest_res,
            "reference_gpu": ref_gpu,
            "roofline": roof,
            "cpu_baseline": cpu,
            "clocks": sampler.summary(),
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
