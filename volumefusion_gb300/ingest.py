"""Depth ingest over the C ABI: decoding of depth images on the host and undistortion on the device.

The reference reads every depth frame with cv::imread(IMREAD_ANYDEPTH | IMREAD_ANYCOLOR) and converts
it to metres (src/dataset.cpp:168-189, src/KinectReader.cpp:9-21, src/AzureReader.cpp:10-22); with a
depthDistortion.txt present it undistorts the frame with OpenCV -- cv::undistort in the non-rigid loop
(src/VolumeFusion.cu:162-180), initUndistortRectifyMap + remap(INTER_NEAREST) in the stream readers
(src/MeshRecontructionStream.cu:94-101) -- and the point-cloud stream builds a Brown-Conrady ray table
(src/CameraCalibration.cpp:261-295).  Here decoding returns the uint16 millimetre image (the sessions
convert to metres on the device), the undistortion maps are built once per camera on the device, and
sessions take the distortion as a parameter (cfg["distortion"]).
"""
import ctypes as C
import os

import numpy as np
import torch

from ._lib import CameraDistortion, check, lib

LINEAR = 0    # AFX_UNDISTORT_LINEAR: cv::undistort
NEAREST = 1   # AFX_UNDISTORT_NEAREST: initUndistortRectifyMap(CV_32FC1) + remap(INTER_NEAREST)

_DIST_KEYS = ("k1", "k2", "k3", "k4", "k5", "k6", "codx", "cody", "p1", "p2")


def distortion(d=None, **coeffs):
    """af::CameraDistortion from a dict (or keywords) of k1..k6, p1, p2 (codx, cody): distorted unless
    d is None and no coefficient is given."""
    if isinstance(d, CameraDistortion):
        return d
    vals = dict(d or {})
    vals.update(coeffs)
    out = CameraDistortion()
    for k in _DIST_KEYS:
        setattr(out, k, float(vals.get(k, 0.0)))
    out.is_distorted = int(bool(vals.get("is_distorted", bool(vals))))
    return out


def load_camera_distortion(path):
    """af::loadCameraDistortion (src/dataset.cpp:44-79): 8 numbers k1 k2 p1 p2 k3 k4 k5 k6; None when the
    file cannot be opened (the reference then leaves the camera undistorted)."""
    try:
        with open(path) as f:
            v = [float(x) for x in f.read().split()[:8]]
    except OSError:
        return None
    v += [0.0] * (8 - len(v))
    return distortion(dict(k1=v[0], k2=v[1], p1=v[2], p2=v[3], k3=v[4], k4=v[5], k5=v[6], k6=v[7]))


def load_intrinsics(path):
    """af::loadIntrinsics (src/dataset.cpp:22-42): nine numbers, row by row."""
    with open(path) as f:
        v = [float(x) for x in f.read().split()[:9]]
    if len(v) < 9:
        raise ValueError("%s: expected 9 intrinsics values" % path)
    return np.asarray(v, np.float32).reshape(3, 3)


def _status(rc, what):
    check(rc, what)


def decode_depth(data):
    """One PNG or TIFF depth image (bytes) -> uint16 array (height, width) in millimetres."""
    buf = np.frombuffer(data, np.uint8)
    w, h = C.c_int(), C.c_int()
    _status(lib().afx_decode_depth_image(buf.ctypes.data, buf.size, None, 0, C.byref(w), C.byref(h)),
            "afx_decode_depth_image")
    out = np.empty((h.value, w.value), np.uint16)
    _status(lib().afx_decode_depth_image(buf.ctypes.data, buf.size, out.ctypes.data, out.size, C.byref(w),
                                         C.byref(h)), "afx_decode_depth_image")
    return out


def decode_depth_many(blobs, threads=None, outs=None):
    """Several images decoded on host threads; returns the arrays (or fills `outs`, preallocated
    uint16 arrays, e.g. pinned host tensors' numpy views)."""
    n = len(blobs)
    bufs = [np.frombuffer(b, np.uint8) for b in blobs]
    if outs is None:
        outs = []
        for b in bufs:
            w, h = C.c_int(), C.c_int()
            _status(lib().afx_decode_depth_image(b.ctypes.data, b.size, None, 0, C.byref(w), C.byref(h)),
                    "afx_decode_depth_image")
            outs.append(np.empty((h.value, w.value), np.uint16))
    data = (C.c_void_p * n)(*[b.ctypes.data for b in bufs])
    lens = (C.c_size_t * n)(*[b.size for b in bufs])
    ptrs = (C.c_void_p * n)(*[o.ctypes.data for o in outs])
    caps = (C.c_long * n)(*[o.size for o in outs])
    status = (C.c_int * n)()
    threads = threads or min(n, os.cpu_count() or 1)
    rc = lib().afx_decode_depth_images(n, data, lens, ptrs, caps, None, None, status, int(threads))
    _status(rc, "afx_decode_depth_images")
    return outs


def depth_file_name(pattern, index):
    """af::insertIntoPattern (src/dataset.cpp:131-150)."""
    out = C.create_string_buffer(len(pattern) + 64)
    _status(lib().afx_depth_file_name(pattern.encode(), int(index), out, len(out)), "afx_depth_file_name")
    return out.value.decode()


def read_depth_frame(pattern, index):
    """af::loadDepthFrame without the conversion to metres: the uint16 millimetre image."""
    with open(depth_file_name(pattern, index), "rb") as f:
        return decode_depth(f.read())


def _kcol(K):
    return np.ascontiguousarray(np.asarray(K, np.float64).T.ravel(), dtype=np.float32)


def _cur_stream(stream):
    return (stream or torch.cuda.current_stream()).cuda_stream


class Undistorter:
    """The undistortion map of one camera on the device (built once) and its application to float
    depth images (metres)."""

    def __init__(self, K, dist, width, height, mode=LINEAR, stream=None):
        self.width, self.height, self.mode = int(width), int(height), int(mode)
        self.dist = distortion(dist)
        self.K = _kcol(K)
        self.map = torch.empty(2 * self.width * self.height, dtype=torch.int32, device="cuda")
        _status(lib().afx_undistort_map(self.map.data_ptr(), self.width, self.height, self.K.ctypes.data,
                                        C.byref(self.dist), self.mode, _cur_stream(stream)), "afx_undistort_map")

    def __call__(self, depth, out=None, stream=None):
        depth = depth.contiguous()
        out = torch.empty_like(depth) if out is None else out
        _status(lib().afx_undistort_depth(out.data_ptr(), depth.data_ptr(), self.width, self.height,
                                          self.map.data_ptr(), self.mode, _cur_stream(stream)), "afx_undistort_depth")
        return out


def _intr(intrinsics):
    return np.ascontiguousarray(np.asarray(intrinsics, np.float32).ravel()[:4])


def xy_lookup_table(intrinsics, dist, width, height, stream=None):
    """af::create_xy_lookup_table: (height, width, 2) float32 CUDA tensor; intrinsics = the
    af::CameraIntrinsics fields (cx, cy, fx, fy) as the caller filled them."""
    d = distortion(dist)
    intr = _intr(intrinsics)
    out = torch.empty((int(height), int(width), 2), dtype=torch.float32, device="cuda")
    _status(lib().afx_xy_lookup_table(out.data_ptr(), int(width), int(height), intr.ctypes.data, C.byref(d),
                                      _cur_stream(stream)), "afx_xy_lookup_table")
    return out


def unproject_points(pixels, depths, intrinsics, dist, stream=None):
    """af::transformation_unproject over CUDA tensors: pixels (n, 2), depths (n,) -> points (n, 3), valid (n,)."""
    d = distortion(dist)
    intr = _intr(intrinsics)
    pixels, depths = pixels.contiguous(), depths.contiguous()
    n = depths.numel()
    pts = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    valid = torch.empty(n, dtype=torch.int32, device="cuda")
    _status(lib().afx_unproject_points(pts.data_ptr(), valid.data_ptr(), pixels.data_ptr(), depths.data_ptr(), n,
                                       intr.ctypes.data, C.byref(d), _cur_stream(stream)), "afx_unproject_points")
    return pts, valid


def project_points(points, intrinsics, dist, out=None, stream=None):
    """af::transformation_project over CUDA tensors: points (n, 3) -> pixels (n, 2), valid (n,).  A point
    beyond the projection radius leaves its pixel as it was in `out`."""
    d = distortion(dist)
    intr = _intr(intrinsics)
    points = points.contiguous()
    n = points.shape[0]
    px = torch.zeros((n, 2), dtype=torch.float32, device="cuda") if out is None else out
    valid = torch.empty(n, dtype=torch.int32, device="cuda")
    _status(lib().afx_project_points(px.data_ptr(), valid.data_ptr(), points.data_ptr(), n, intr.ctypes.data,
                                     C.byref(d), _cur_stream(stream)), "afx_project_points")
    return px, valid
