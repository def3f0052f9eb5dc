"""afx_correspondences_static (scratch in a fixed device array, no allocation) against
afx_correspondences (caller workspace), both called through the C ABI.

Two static calls run back to back on different inputs -- the larger one first -- so a
result that depended on scratch left over from the previous call would differ from the
workspace entry point's.  The file is named to be collected last, after every other test
has used the library on the same device."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import pyoracle as O  # noqa: E402


def _lib():
    from volumefusion_gb300 import _lib as L
    return L.lib()


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _k9(K):
    return (C.c_float * 9)(*np.asarray(K, np.float64).T.ravel().astype(np.float32))


def _case(frame_index, stride, offset):
    from volumefusion_gb300 import synth
    mm, K = synth.capsule_pair_frame(frame_index, width=640, height=576, fx=504.0, fy=504.0, cx=320.0, cy=288.0)
    d, v, _, _ = O.frame_prep(mm, K)
    pts = v.reshape(-1, 3)
    pts = pts[pts[:, 2] > 0][::stride] + np.asarray(offset, np.float32)
    return d, v, np.ascontiguousarray(pts, np.float32), K


def _run(L, static, d, v, pts, K, device_count=None):
    dev = torch.device("cuda")
    n = len(pts)
    gd = torch.from_numpy(d).to(dev)
    gv = torch.from_numpy(v).to(dev)
    gp = torch.from_numpy(pts).to(dev)
    corr = torch.full((n, 2), -7, dtype=torch.int32, device=dev)
    cnt = torch.full((1,), 12345, dtype=torch.int32, device=dev)
    cnt_dev = None
    if device_count is not None:
        cnt_dev = torch.tensor([device_count], dtype=torch.int32, device=dev)
    count_ptr = _ptr(cnt_dev) if cnt_dev is not None else None
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rows, cols = d.shape
    if static:
        rc = L.afx_correspondences_static(_ptr(corr), _ptr(cnt), n, _ptr(gp), count_ptr, n, _k9(K), _ptr(gd), rows,
                                          cols, _ptr(gv), C.c_float(0.01), stream)
    else:
        ws_bytes = L.afx_correspondences_workspace_size(n)
        ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device=dev)
        rc = L.afx_correspondences(_ptr(corr), _ptr(cnt), n, _ptr(gp), count_ptr, n, _k9(K), _ptr(gd), rows, cols,
                                   _ptr(gv), C.c_float(0.01), _ptr(ws), ws_bytes, stream)
    assert rc == 0, L.afx_status_string(rc)
    torch.cuda.synchronize()
    m = int(cnt.item())
    return m, corr.cpu().numpy()[:m]


@pytest.mark.gpu
def test_static_scratch_matches_workspace_entry_point_twice_in_a_row():
    L = _lib()
    big = _case(12, 3, (0.002, -0.001, 0.003))
    small = _case(21, 11, (-0.001, 0.002, 0.001))
    assert len(big[2]) > len(small[2])
    m_big_s, c_big_s = _run(L, True, *big)
    m_small_s, c_small_s = _run(L, True, *small)
    m_big_w, c_big_w = _run(L, False, *big)
    m_small_w, c_small_w = _run(L, False, *small)
    assert m_big_s == m_big_w and m_big_s > 1000
    assert np.array_equal(c_big_s, c_big_w)
    assert m_small_s == m_small_w and m_small_s > 100
    assert np.array_equal(c_small_s, c_small_w)
    # and the CPU oracle agrees with both
    d, v, pts, K = small
    assert np.array_equal(c_small_s, O.correspondences(pts, K, d, v, 0.01))


@pytest.mark.gpu
def test_static_scratch_with_device_vertex_count():
    L = _lib()
    d, v, pts, K = _case(5, 4, (0.001, 0.001, -0.002))
    live = len(pts) // 2
    m_s, c_s = _run(L, True, d, v, pts, K, device_count=live)
    m_w, c_w = _run(L, False, d, v, pts, K, device_count=live)
    assert m_s == m_w and m_s > 100
    assert np.array_equal(c_s, c_w)
    assert c_s[:, 0].max() < live


def test_static_scratch_rejects_oversize_before_any_work():
    """The size check precedes every CUDA call, so it runs without a GPU too."""
    from volumefusion_gb300 import build
    lib = C.CDLL(build.build())
    lib.afx_correspondences_static.restype = C.c_int
    lib.afx_correspondences_static.argtypes = [C.c_void_p] * 2 + [C.c_long] + [C.c_void_p] * 2 + [C.c_long] + \
        [C.c_void_p] * 2 + [C.c_int] * 2 + [C.c_void_p, C.c_float, C.c_void_p]
    dummy = C.c_void_p(256)
    k9 = (C.c_float * 9)()
    too_many = 262144 + 1
    rc = lib.afx_correspondences_static(dummy, dummy, too_many, dummy, None, too_many, k9, dummy, 576, 640, dummy,
                                        C.c_float(0.01), None)
    assert rc == 2  # AFX_ERR_CAPACITY
