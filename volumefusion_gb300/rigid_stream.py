"""Rigid multi-camera reconstruction stream (af::startMeshReconstructionStream) over the C ABI
(afx_rigid_stream_*): per frame, every camera's depth is filtered and back-projected into one world
point cloud, camera 0's depth is integrated into a fresh volume, and the mesh is extracted."""
import ctypes as C

import numpy as np
import torch

from ._lib import MAX_CAMERAS, RigidStreamParams, check, lib
from .fusion import _wrap_device


def _colmajor(m):
    return [float(v) for v in np.asarray(m, np.float64).T.ravel()]


class RigidStream:
    def __init__(self, Ks, camera_to_world, width, height, dims, volume_size, delta, center, rotation,
                 depth_threshold=1.2, bilateral=True, bilateral_r=2, sigma_i=0.03, sigma_s=2.0, bilateral_thr=0.09,
                 triangle_capacity=4_000_000, distortions=None, stream=None):
        """Ks: per-camera 3x3 intrinsics; camera_to_world: per-camera 4x4 (inverse of world2camera);
        center, rotation: the volume pose (settings.tsdfCenter and the rotation settings.tsdfRotation gives);
        distortions: per camera None or the distortion coefficients (dict of k1..k6, p1, p2)."""
        n = len(Ks)
        assert 1 <= n <= MAX_CAMERAS and len(camera_to_world) == n
        p = RigidStreamParams()
        lib().afx_rigid_stream_default_params(C.byref(p))
        p.n_cameras, p.width, p.height = n, int(width), int(height)
        for c in range(n):
            p.K[c][:] = _colmajor(Ks[c])
            p.camera_to_world[c][:] = _colmajor(camera_to_world[c])
        p.dims[:] = [int(v) for v in dims]
        p.volume_size[:] = [float(v) for v in volume_size]
        p.delta = float(delta)
        p.center[:] = [float(v) for v in center]
        p.rotation[:] = _colmajor(rotation)
        p.depth_threshold = float(depth_threshold)
        p.bilateral, p.bilateral_r = int(bool(bilateral)), int(bilateral_r)
        p.sigma_i, p.sigma_s, p.bilateral_thr = float(sigma_i), float(sigma_s), float(bilateral_thr)
        p.triangle_capacity = int(triangle_capacity)
        if distortions:
            from .ingest import distortion
            for c, d in enumerate(distortions):
                if d:
                    p.distortion[c] = distortion(d)
        h = C.c_void_p()
        check(lib().afx_rigid_stream_create(C.byref(p), C.byref(h)), "afx_rigid_stream_create")
        self.h, self.params, self.stream, self.n = h, p, stream, n
        self.S = int(np.prod(dims))
        self._ptrs = (C.c_void_p * n)()

    def close(self):
        if getattr(self, "h", None):
            lib().afx_rigid_stream_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def process(self, frames):
        """frames: per-camera uint16/int16 CUDA tensors (height, width) of depth in mm."""
        assert len(frames) == self.n
        for c, f in enumerate(frames):
            assert f.is_cuda and f.is_contiguous() and f.element_size() == 2
            self._ptrs[c] = f.data_ptr()
        s = self.stream if self.stream is not None else torch.cuda.current_stream()
        check(lib().afx_rigid_stream_process(self.h, self._ptrs, C.c_void_p(s.cuda_stream)), "afx_rigid_stream_process")

    def outputs(self):
        """(cloud (n*H*W, 3), mesh vertices (3F, 3), faces (F, 3), tsdf, weights) as new CUDA tensors."""
        cl, n, v, nv, f, nf, t, w = (C.c_void_p(), C.c_long(0), C.c_void_p(), C.c_void_p(), C.c_void_p(),
                                     C.c_void_p(), C.c_void_p(), C.c_void_p())
        check(lib().afx_rigid_stream_outputs(self.h, C.byref(cl), C.byref(n), C.byref(v), C.byref(nv), C.byref(f),
                                             C.byref(nf), C.byref(t), C.byref(w)), "afx_rigid_stream_outputs")
        faces = int(_wrap_device(nf.value, 1, torch.int32).item())
        return (_wrap_device(cl.value, 3 * n.value, torch.float32).view(-1, 3),
                _wrap_device(v.value, 9 * faces, torch.float32).view(-1, 3),
                _wrap_device(f.value, 3 * faces, torch.int32).view(-1, 3),
                _wrap_device(t.value, self.S, torch.float32), _wrap_device(w.value, self.S, torch.float32))


__all__ = ["RigidStream"]
