"""The reference's file formats: PLY meshes (Mesh::savePly) and TSDF volumes (TSDFVolume::save /
load), written and read by libafx on the host.  Pinned byte for byte against the reference's own
code (oracle/_ref/libvfref.so, built from the reference sources where they are present)."""
import ctypes as C
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libvfref.so")


def _ref():
    if not os.path.exists(REF_LIB):
        pytest.skip("reference CPU library not built here")
    L = C.CDLL(REF_LIB)
    vp = C.c_void_p
    L.ref_save_ply.restype = C.c_int
    L.ref_save_ply.argtypes = [C.c_char_p, vp, C.c_long, vp, vp, C.c_long]
    L.ref_tsdf_save.restype = C.c_int
    L.ref_tsdf_save.argtypes = [C.c_char_p, vp, vp, C.c_float, vp, vp]
    L.ref_tsdf_load.restype = C.c_long
    L.ref_tsdf_load.argtypes = [C.c_char_p, vp, vp, vp, vp, vp, vp, C.c_long]
    return L


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _mesh(seed=0, n=500):
    rng = np.random.default_rng(seed)
    v = (rng.standard_normal((n, 3)) * np.array([0.3, 1e-3, 250.0])).astype(np.float32)
    v[:5] = [[0, 0, 0], [1e-7, -2.5e-5, 1.0], [123456.7, -0.1, 3.0], [1e20, -1e-20, 0.5], [-0.0, 7.0, 8.25]]
    f = rng.integers(0, n, size=(n // 2, 3)).astype(np.int32)
    c = rng.integers(0, 256, size=(n, 3)).astype(np.uint8)
    return v, f, c


def test_ply_matches_reference_saveply(tmp_path):
    from volumefusion_gb300 import formats
    L = _ref()
    v, f, c = _mesh()
    for colors in (c, None):
        ours, theirs = tmp_path / "ours.ply", tmp_path / "ref.ply"
        formats.save_ply(ours, v, f, colors)
        cc = np.zeros_like(c) if colors is None else colors
        assert L.ref_save_ply(str(theirs).encode(), _p(v), len(v), _p(cc), _p(f), len(f)) == 0
        assert ours.read_bytes() == theirs.read_bytes()


def test_tsdf_file_matches_reference_save_and_load(tmp_path):
    from volumefusion_gb300 import formats
    L = _ref()
    rng = np.random.default_rng(1)
    dims = np.array([12, 10, 7], np.int32)
    size = np.array([0.48, 0.4, 0.28], np.float32)
    t = rng.uniform(-1, 1, size=dims[::-1]).astype(np.float32)
    w = rng.integers(0, 16, size=dims[::-1]).astype(np.float32)
    vs = (size / dims.astype(np.float32)).astype(np.float32)
    ours, theirs = tmp_path / "ours.tsdf", tmp_path / "ref.tsdf"
    formats.save_tsdf(ours, t, w, size, vs, 0.016)
    assert L.ref_tsdf_save(str(theirs).encode(), _p(dims), _p(size), C.c_float(0.016), _p(t), _p(w)) == 0
    assert ours.read_bytes() == theirs.read_bytes()
    # the reference reads what we wrote ...
    d2, s2, v2, de = np.zeros(3, np.int32), np.zeros(3, np.float32), np.zeros(3, np.float32), np.zeros(1, np.float32)
    t2, w2 = np.zeros(t.size, np.float32), np.zeros(t.size, np.float32)
    assert L.ref_tsdf_load(str(ours).encode(), _p(d2), _p(s2), _p(v2), _p(de), _p(t2), _p(w2), t.size) == t.size
    assert np.array_equal(d2, dims) and np.array_equal(s2, size) and np.array_equal(v2, vs) and de[0] == np.float32(0.016)
    assert np.array_equal(t2, t.ravel()) and np.array_equal(w2, w.ravel())
    # ... and we read what the reference wrote
    t3, w3, d3, s3, v3, de3 = formats.load_tsdf(theirs)
    assert np.array_equal(t3, t) and np.array_equal(w3, w) and np.array_equal(d3, dims)
    assert np.array_equal(s3, size) and np.array_equal(v3, vs) and de3 == np.float32(0.016)


def test_formats_refuse_bad_input(tmp_path):
    from volumefusion_gb300 import formats
    from volumefusion_gb300._lib import AfxError
    with pytest.raises(AfxError):
        formats.save_ply(tmp_path / "empty.ply", np.zeros((0, 3), np.float32), np.zeros((0, 3), np.int32))
    with pytest.raises(AfxError):
        formats.load_tsdf(tmp_path / "missing.tsdf")
    (tmp_path / "short.tsdf").write_bytes(b"\x01\x00")
    with pytest.raises(AfxError):
        formats.load_tsdf(tmp_path / "short.tsdf")
