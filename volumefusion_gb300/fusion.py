"""Device-resident non-rigid fusion session (af::runVolumeFusion's per-frame loop,
src/VolumeFusion.cu:223-769) over the C ABI."""
import ctypes as C

import numpy as np
import torch

from ._lib import FrameStats, FusionParams, check, lib

_KEYS_F = ("delta", "depth_threshold", "sigma_i", "sigma_s", "bilateral_thr", "graph_radius", "lambda_depth",
           "lambda_reg", "energy_min_step", "corr_thresh")
_KEYS_I = ("bilateral", "bilateral_r", "knn", "kreg", "update_graph", "icp_iterations", "gn_iterations", "solver",
           "pcg_iterations", "integrate", "node_cap", "mesh_cap")


def params_from_config(cfg, extract_mesh=True, triangle_capacity=None):
    p = FusionParams()
    lib().afx_fusion_default_params(C.byref(p))
    p.width, p.height = int(cfg["width"]), int(cfg["height"])
    p.K[:] = [float(v) for v in np.asarray(cfg["K"], dtype=np.float64).T.ravel()]
    p.dims[:] = [int(v) for v in cfg["dims"]]
    p.volume_size[:] = [float(v) for v in cfg["volume_size"]]
    for k in _KEYS_F:
        setattr(p, k, float(cfg[k]))
    p.excl_angle_lo = float(cfg["angle_lo"])
    p.excl_angle_hi = float(cfg["angle_hi"])
    for k in _KEYS_I:
        if k == "node_cap":
            p.node_capacity = int(cfg[k])
        elif k == "mesh_cap":
            p.mesh_capacity = int(cfg[k])
        else:
            setattr(p, k, int(cfg[k]))
    p.pcg_tol = float(cfg.get("pcg_tol", 0.0))
    p.extract_mesh = int(extract_mesh)
    p.triangle_capacity = int(triangle_capacity or cfg.get("triangle_cap", 4_000_000))
    p.precision = {"fp32": 0, "fp16": 1}[cfg.get("precision", "fp32")]
    p.warp_mesh = int(bool(cfg.get("warp_mesh", False)))
    p.blend = {"lbs": 0, "dqb": 1}[cfg.get("blend", "lbs")]
    if cfg.get("distortion"):
        from .ingest import distortion
        p.distortion = distortion(cfg["distortion"])
    return p


class FusionSession:
    """One depth stream: TSDF volume, motion graph and solver state live on the GPU."""

    def __init__(self, cfg, extract_mesh=True, stream=None):
        self.cfg = cfg
        self.params = params_from_config(cfg, extract_mesh=extract_mesh)
        h = C.c_void_p()
        check(lib().afx_fusion_create(C.byref(self.params), C.byref(h)), "afx_fusion_create")
        self.h = h
        self.stream = stream
        self.S = int(np.prod(cfg["dims"]))

    @classmethod
    def attach(cls, handle, cfg, stream=None):
        """View of a session owned elsewhere (e.g. by a Server); close() leaves it alone."""
        obj = cls.__new__(cls)
        obj.cfg = cfg
        obj.params = params_from_config(cfg)
        obj.h = C.c_void_p(handle)
        obj.stream = stream
        obj.S = int(np.prod(cfg["dims"]))
        obj._owned = False
        return obj

    def close(self):
        if getattr(self, "h", None):
            if getattr(self, "_owned", True):
                lib().afx_fusion_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _st(self):
        s = self.stream if self.stream is not None else torch.cuda.current_stream()
        return C.c_void_p(s.cuda_stream)

    def reset(self):
        """Start a new sequence: empty volume and graph (stream-ordered, no allocation)."""
        check(lib().afx_fusion_reset(self.h, self._st()), "afx_fusion_reset")

    def process(self, depth_mm):
        """depth_mm: uint16/int16 CUDA tensor (H, W) or host numpy uint16 array."""
        if isinstance(depth_mm, np.ndarray):
            arr = np.ascontiguousarray(depth_mm, dtype=np.uint16)
            check(lib().afx_fusion_process_host(self.h, arr.ctypes.data_as(C.c_void_p), self._st()),
                  "afx_fusion_process_host")
        else:
            assert depth_mm.is_cuda and depth_mm.is_contiguous()
            check(lib().afx_fusion_process(self.h, C.c_void_p(depth_mm.data_ptr()), self._st()), "afx_fusion_process")

    def process_host_ptr(self, ptr):
        check(lib().afx_fusion_process_host(self.h, C.c_void_p(ptr), self._st()), "afx_fusion_process_host")

    def stats(self, check_errors=True):
        s = FrameStats()
        st = lib().afx_fusion_stats(self.h, C.byref(s), self._st())
        if check_errors:
            check(st, "afx_fusion_stats")
        return {f[0]: getattr(s, f[0]) for f in FrameStats._fields_}

    def tsdf(self):
        """Copies of the volume as FP32 tensors (values, weights), whatever the storage format."""
        t, w, prec = C.c_void_p(), C.c_void_p(), C.c_int(0)
        check(lib().afx_fusion_volume(self.h, C.byref(t), C.byref(w), C.byref(prec)), "afx_fusion_volume")
        if prec.value == 0:
            return _wrap_device(t.value, self.S, torch.float32), _wrap_device(w.value, self.S, torch.float32)
        # precision form: FP16 values widen exactly; uint16 weights are counts <= 15
        return (_wrap_device(t.value, self.S, torch.float16).float(),
                _wrap_device(w.value, self.S, torch.int16).float())

    def volume_raw(self):
        """The stored arrays as they are: (values, weights, precision) with FP16 / int16 (bit
        pattern of uint16) tensors in the precision form."""
        t, w, prec = C.c_void_p(), C.c_void_p(), C.c_int(0)
        check(lib().afx_fusion_volume(self.h, C.byref(t), C.byref(w), C.byref(prec)), "afx_fusion_volume")
        if prec.value == 0:
            return _wrap_device(t.value, self.S, torch.float32), _wrap_device(w.value, self.S, torch.float32), "fp32"
        return _wrap_device(t.value, self.S, torch.float16), _wrap_device(w.value, self.S, torch.int16), "fp16"

    def graph(self):
        nodes, radii, T, n = C.c_void_p(), C.c_void_p(), C.c_void_p(), C.c_void_p()
        lib().afx_fusion_graph(self.h, C.byref(nodes), C.byref(radii), C.byref(T), C.byref(n))
        nn = int(_wrap_device(n.value, 1, torch.int32).item())
        return (_wrap_device(nodes.value, 3 * nn, torch.float32).view(-1, 3),
                _wrap_device(radii.value, nn, torch.float32),
                _wrap_device(T.value, 16 * nn, torch.float32).view(-1, 16))

    def centroid(self):
        c = C.c_void_p()
        lib().afx_fusion_centroid(self.h, C.byref(c))
        return _wrap_device(c.value, 3, torch.float32)

    def point_cloud(self):
        p, n = C.c_void_p(), C.c_void_p()
        lib().afx_fusion_point_cloud(self.h, C.byref(p), C.byref(n))
        cnt = int(_wrap_device(n.value, 1, torch.int32).item())
        return _wrap_device(p.value, 3 * cnt, torch.float32).view(-1, 3)

    def mesh(self):
        v, nv, f, nf = C.c_void_p(), C.c_void_p(), C.c_void_p(), C.c_void_p()
        lib().afx_fusion_mesh(self.h, C.byref(v), C.byref(nv), C.byref(f), C.byref(nf))
        nfc = int(_wrap_device(nf.value, 1, torch.int32).item())
        return (_wrap_device(v.value, 9 * nfc, torch.float32).view(-1, 3),
                _wrap_device(f.value, 3 * nfc, torch.int32).view(-1, 3))

    def frame_views(self):
        d, v, n = C.c_void_p(), C.c_void_p(), C.c_void_p()
        lib().afx_fusion_frame_views(self.h, C.byref(d), C.byref(v), C.byref(n))
        P = int(self.cfg["width"]) * int(self.cfg["height"])
        return (_wrap_device(d.value, P, torch.float32), _wrap_device(v.value, 3 * P, torch.float32).view(-1, 3),
                _wrap_device(n.value, 3 * P, torch.float32).view(-1, 3))

    def support_size(self):
        """(active bricks, supported voxels) of the last non-rigid frame's voxel support."""
        nb, nv = C.c_uint(0), C.c_ulonglong(0)
        check(lib().afx_fusion_support_size(self.h, C.byref(nb), C.byref(nv), self._st()), "afx_fusion_support_size")
        return nb.value, nv.value

    def occupied_bricks(self):
        """(8^3 bricks holding a weighted voxel, bricks in the volume): what marching cubes reads."""
        nb, tot = C.c_ulonglong(0), C.c_ulonglong(0)
        check(lib().afx_fusion_occupied_bricks(self.h, C.byref(nb), C.byref(tot), self._st()),
              "afx_fusion_occupied_bricks")
        return nb.value, tot.value

    def set_transforms(self, T):
        arr = np.ascontiguousarray(T, dtype=np.float32)
        check(lib().afx_fusion_set_transforms(self.h, arr.ctypes.data_as(C.c_void_p), arr.shape[0], self._st()),
              "afx_fusion_set_transforms")
        torch.cuda.synchronize()

    STAGES = ("prep", "rigid_integrate", "sort_unique", "graph", "knn", "gn_setup", "gn_loop", "voxel_support",
              "voxel_warp", "warped_integrate", "marching_cubes")

    def set_graphs(self, on=True):
        """Replay non-rigid frames from CUDA graphs (default) or launch kernels one by one."""
        check(lib().afx_fusion_set_graphs(self.h, int(bool(on))), "afx_fusion_set_graphs")

    def graph_count(self):
        return lib().afx_fusion_graph_count(self.h)

    def save_volume(self, path):
        """The volume in TSDFVolume::save's file format (FP16 sessions are widened)."""
        check(lib().afx_fusion_save_volume(self.h, str(path).encode(), self._st()), "afx_fusion_save_volume")

    def load_volume(self, path):
        """Replace the volume with a TSDFVolume file of the same dims."""
        check(lib().afx_fusion_load_volume(self.h, str(path).encode(), self._st()), "afx_fusion_load_volume")

    def save_mesh_ply(self, path):
        """The frame's output mesh as Mesh::savePly writes it."""
        check(lib().afx_fusion_save_mesh_ply(self.h, str(path).encode(), self._st()), "afx_fusion_save_mesh_ply")

    def set_tile(self, tile):
        """Marching-cubes tile: 0 TMA 16 cubes along z (default), 1 TMA 8, 2 TMA 32, 3 column march,
        4 / 5 persistent two-stage TMA 8 / 16."""
        check(lib().afx_fusion_set_tile(self.h, int(tile)), "afx_fusion_set_tile")

    def tile(self):
        return lib().afx_fusion_get_tile(self.h)

    def autotune(self):
        """Time every marching-cubes tile on the current volume and keep the fastest: (tile, ms per tile)."""
        t, ms = C.c_int(0), (C.c_float * 7)()
        check(lib().afx_fusion_autotune(self.h, C.byref(t), ms, self._st()), "afx_fusion_autotune")
        return t.value, list(ms)

    def set_timing(self, on=True):
        check(lib().afx_fusion_set_timing(self.h, int(on)), "afx_fusion_set_timing")

    def stage_times(self, reset=True):
        """Milliseconds per stage accumulated since timing was enabled or last reset."""
        arr = (C.c_double * len(self.STAGES))()
        n = lib().afx_fusion_stage_times(self.h, arr, len(self.STAGES), int(reset))
        return {self.STAGES[i]: arr[i] for i in range(min(n, len(self.STAGES)))}

    def kernel_launches(self):
        return lib().afx_fusion_kernel_launches(self.h)


def _wrap_device(ptr, n, dtype):
    """Copy n elements of device memory at ptr into a new CUDA tensor."""
    out = torch.empty(n, dtype=dtype, device="cuda")
    if n:
        nbytes = n * out.element_size()
        st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        check(lib().afx_copy_device(C.c_void_p(out.data_ptr()), C.c_void_p(ptr), nbytes, st), "afx_copy_device")
        torch.cuda.current_stream().synchronize()
    return out
