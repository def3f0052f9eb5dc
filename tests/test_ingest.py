"""Depth ingest on the host: the decoder of 16-bit PNG / TIFF depth frames (what the reference reads
with cv::imread(IMREAD_ANYDEPTH | IMREAD_ANYCOLOR), src/dataset.cpp:168-189), the frame-name pattern
(af::insertIntoPattern, src/dataset.cpp:131-150), the calibration file readers, and the oracle's
Brown-Conrady restatement pinned to the reference's own src/CameraCalibration.cpp (golden fixture).

The decoder's expected output is the image the test encoded: PNG and TIFF are lossless, so the
specification fixes every decoded value.  These run without a GPU (decoding is host code)."""
import os
import struct
import zlib

import numpy as np
import pytest

import _depth_codecs as D

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _ingest():
    from volumefusion_gb300 import ingest
    return ingest


def _afx():
    from volumefusion_gb300._lib import AfxError
    return AfxError


def _status(data, cap=None):
    import ctypes as C
    from volumefusion_gb300._lib import lib
    buf = np.frombuffer(data, np.uint8)
    w, h = C.c_int(), C.c_int()
    out = np.zeros(cap if cap is not None else 1 << 16, np.uint16)
    return lib().afx_decode_depth_image(buf.ctypes.data, buf.size, out.ctypes.data, out.size, C.byref(w), C.byref(h))


def _img(rng, shape, depth, smooth):
    if smooth:
        return ((np.cumsum(rng.integers(0, 4, shape), axis=1) * 7) % (1 << depth)).astype(np.uint16)
    return rng.integers(0, 1 << depth, shape).astype(np.uint16)


@pytest.mark.parametrize("interlace", [False, True])
@pytest.mark.parametrize("ftype", [-1, 0, 1, 2, 3, 4])
def test_png_filters_and_interlace(interlace, ftype):
    ingest = _ingest()
    rng = np.random.default_rng(ftype + 1 + 10 * interlace)
    for shape in ((1, 1), (1, 17), (17, 1), (13, 29), (48, 64)):
        for depth in (8, 16):
            img = _img(rng, shape, depth, smooth=shape[0] > 20)
            data = D.png(img, depth, ftype, level=6, interlace=interlace)
            out = ingest.decode_depth(data)
            assert out.dtype == np.uint16 and np.array_equal(out, img), (shape, depth)


@pytest.mark.parametrize("level,strategy,idat", [(0, None, None), (1, None, 61), (9, None, None),
                                                  (6, zlib.Z_FIXED, 200), (6, zlib.Z_HUFFMAN_ONLY, None),
                                                  (6, zlib.Z_RLE, 1000)])
def test_png_deflate_block_kinds(level, strategy, idat):
    """Stored, fixed- and dynamic-Huffman blocks, split over several IDAT chunks."""
    ingest = _ingest()
    rng = np.random.default_rng(level)
    img = _img(rng, (90, 70), 16, smooth=True)
    img[20:40, 10:50] = 0  # long runs: distance-1 matches
    data = D.png(img, 16, -1, level=level, strategy=strategy, idat_size=idat)
    assert np.array_equal(ingest.decode_depth(data), img)


def test_png_depth_frame_sized():
    ingest = _ingest()
    from volumefusion_gb300 import configs
    cfg = configs.small_nonrigid(n_frames=2)
    mm = configs.small_frames(cfg)[1]
    for ft in (0, 2, 4):
        assert np.array_equal(ingest.decode_depth(D.png(mm, 16, ft)), mm)


def test_png_errors():
    AFX_ERR_INVALID, AFX_ERR_CAPACITY, AFX_ERR_UNSUPPORTED = 1, 2, 6
    img = np.arange(12 * 10, dtype=np.uint16).reshape(12, 10) * 300
    good = D.png(img, 16, 1)
    assert _status(good) == 0
    assert _status(good, cap=119) == AFX_ERR_CAPACITY
    # a flipped bit in the IDAT payload breaks the chunk CRC
    i = good.index(b"IDAT") + 10
    assert _status(good[:i] + bytes([good[i] ^ 4]) + good[i + 1:]) == AFX_ERR_INVALID
    # truncated file
    assert _status(good[:len(good) - 20]) == AFX_ERR_INVALID
    # a zlib stream whose Adler-32 is wrong (chunk CRC recomputed, so only the Adler check sees it)
    raw = D._filter_rows(D._rows(img, 16), 0, 2)
    z = zlib.compress(raw)
    z = z[:-1] + bytes([z[-1] ^ 1])
    bad = (D.PNG_SIG + D.png_chunk(b"IHDR", struct.pack(">IIBBBBB", 10, 12, 16, 0, 0, 0, 0)) +
           D.png_chunk(b"IDAT", z) + D.png_chunk(b"IEND", b""))
    assert _status(bad) == AFX_ERR_INVALID
    # more image data than the header's size holds
    extra = zlib.compress(raw + b"\x00" * 21)
    bad = (D.PNG_SIG + D.png_chunk(b"IHDR", struct.pack(">IIBBBBB", 10, 12, 16, 0, 0, 0, 0)) +
           D.png_chunk(b"IDAT", extra) + D.png_chunk(b"IEND", b""))
    assert _status(bad) == AFX_ERR_INVALID
    # colour and other bit depths are not depth frames
    assert _status(D.png(np.zeros((4, 4)), 16, color=2)) == AFX_ERR_UNSUPPORTED
    # an unknown critical chunk; an ancillary chunk with a bad CRC is skipped
    crit = D.png(img, 16, 0, extra_chunks=[D.png_chunk(b"ABCD", b"xy")])
    assert _status(crit) == AFX_ERR_UNSUPPORTED
    anc = D.png(img, 16, 0, extra_chunks=[D.png_chunk(b"tEXt", b"key\x00value", crc=1234)])
    assert _status(anc) == 0
    assert _status(b"not an image at all") == AFX_ERR_UNSUPPORTED


@pytest.mark.parametrize("compression", [1, 5, 8, 32946, 32773])
@pytest.mark.parametrize("predictor", [1, 2])
def test_tiff_strips(compression, predictor):
    ingest = _ingest()
    rng = np.random.default_rng(compression + predictor)
    for big_endian in (False, True):
        for depth in (8, 16):
            for shape in ((1, 1), (9, 23), (70, 50)):
                img = _img(rng, shape, depth, smooth=shape[0] > 20)
                data = D.tiff(img, depth, compression, predictor, rows_per_strip=max(1, shape[0] // 3),
                              big_endian=big_endian)
                assert np.array_equal(ingest.decode_depth(data), img), (big_endian, depth, shape)


def test_tiff_lzw_table_resets():
    """Random 16-bit data fills the 4096-entry LZW table several times (Clear codes mid-strip)."""
    ingest = _ingest()
    img = np.random.default_rng(5).integers(0, 65536, (64, 96)).astype(np.uint16)
    assert np.array_equal(ingest.decode_depth(D.tiff(img, 16, 5)), img)


def test_decode_many_threads_and_files(tmp_path):
    ingest = _ingest()
    rng = np.random.default_rng(9)
    imgs = [_img(rng, (30 + i, 40 + 2 * i), 16, smooth=True) for i in range(9)]
    blobs = [D.png(im, 16, i % 5) if i % 2 else D.tiff(im, 16, 8, 2) for i, im in enumerate(imgs)]
    for threads in (1, 4):
        outs = ingest.decode_depth_many(blobs, threads=threads)
        assert all(np.array_equal(o, im) for o, im in zip(outs, imgs))
    # af::insertIntoPattern and reading by index
    assert ingest.depth_file_name("frame-******.depth.png", 12) == "frame-000012.depth.png"
    assert ingest.depth_file_name("d/**.png", 1234) == "d/1234ng"  # a longer index overwrites what follows
    with pytest.raises(_afx()):
        ingest.depth_file_name("no-placeholder.png", 3)
    with pytest.raises(_afx()):
        ingest.depth_file_name("x**", 12345)  # past the end of the pattern
    pattern = str(tmp_path / "frame-******.depth.png")
    for i, b in enumerate(blobs[:3]):
        with open(ingest.depth_file_name(pattern, i), "wb") as f:
            f.write(b)
    for i in range(3):
        assert np.array_equal(ingest.read_depth_frame(pattern, i), imgs[i])
    with pytest.raises(FileNotFoundError):
        ingest.read_depth_frame(pattern, 7)


def test_calibration_files(tmp_path):
    ingest = _ingest()
    p = tmp_path / "depthIntrinsics.txt"
    p.write_text("504 0 320.5\n0 505 288\n0 0 1\n")
    K = ingest.load_intrinsics(str(p))
    assert K[0, 0] == 504 and K[0, 2] == np.float32(320.5) and K[1, 1] == 505 and K[2, 2] == 1
    d = tmp_path / "depthDistortion.txt"
    d.write_text("0.1 -0.2 0.001 0.002 0.3 0.4 0.5 0.6")
    dist = ingest.load_camera_distortion(str(d))
    vals = {k: getattr(dist, k) for k in ("k1", "k2", "p1", "p2", "k3", "k4", "k5", "k6")}
    assert vals == {k: float(np.float32(v)) for k, v in zip(vals, (0.1, -0.2, 0.001, 0.002, 0.3, 0.4, 0.5, 0.6))}
    assert dist.is_distorted == 1
    assert ingest.load_camera_distortion(str(tmp_path / "missing.txt")) is None


def test_oracle_brown_conrady_matches_reference_cpu():
    """The oracle's restatement of src/CameraCalibration.cpp against the reference's own code
    (tests/golden/make_golden_camera.py): ray table, unprojection and projection, bit for bit."""
    from oracle import pyoracle as O
    g = np.load(os.path.join(G, "camera_calibration.npz"))
    names = ("k1", "k2", "k3", "k4", "k5", "k6", "codx", "cody", "p1", "p2")
    for i in range(int(g["n"])):
        intr, dist = g["intr%d" % i], dict(zip(names, g["dist%d" % i].tolist()))
        W, H = g["size%d" % i]
        assert np.array_equal(O.xy_lookup_table(intr, dist, int(W), int(H)).view(np.uint32),
                              g["table%d" % i].view(np.uint32))
        pts, valid = O.bc_unproject(g["px%d" % i], g["depth%d" % i], intr, dist)
        assert np.array_equal(pts.view(np.uint32), g["unproj%d" % i].view(np.uint32))
        assert np.array_equal(valid, g["unproj_valid%d" % i])
        px, valid = O.bc_project(g["pts%d" % i], intr, dist, out=np.full((len(valid), 2), -7.0, np.float32))
        assert np.array_equal(px.view(np.uint32), g["proj%d" % i].view(np.uint32))
        assert np.array_equal(valid, g["proj_valid%d" % i])
        assert 0 < valid.sum() < len(valid)  # both branches exercised


def test_oracle_undistort_maps_identity_without_distortion():
    """With every coefficient zero both OpenCV maps are the identity (sub-pixel index 0), so the
    remap returns the image unchanged."""
    from oracle import pyoracle as O
    K = np.array([[50.0, 0, 31.5], [0, 51.0, 23.5], [0, 0, 1]], np.float32)
    for mode in (0, 1):
        m = O.undistort_map(K, {}, 64, 48, mode).reshape(48, 64, 2)
        sx = (m[..., 0] & 0xFFFF).astype(np.int16)
        sy = (m[..., 0] >> 16).astype(np.int16)
        yy, xx = np.mgrid[0:48, 0:64]
        assert np.array_equal(sx, xx) and np.array_equal(sy, yy) and not m[..., 1].any()
        img = np.random.default_rng(1).random((48, 64)).astype(np.float32)
        assert np.array_equal(O.undistort_depth(img, m.ravel(), mode), img)


def test_oracle_undistort_linear_is_a_convex_blend():
    """cv::undistort's bilinear taps: inside the image the result lies between the four source
    values it blends (weights sum to 1), and a constant image stays constant away from the border."""
    from oracle import pyoracle as O
    K = np.array([[60.0, 0, 40.0], [0, 60.0, 30.0], [0, 0, 1]], np.float32)
    d = dict(k1=-0.25, k2=0.08, p1=1e-3, p2=-2e-3)
    m = O.undistort_map(K, d, 80, 60, 0).reshape(60, 80, 2)
    sx = (m[..., 0] & 0xFFFF).astype(np.int16).astype(int)
    sy = (m[..., 0] >> 16).astype(np.int16).astype(int)
    inside = (sx >= 0) & (sx < 79) & (sy >= 0) & (sy < 59)
    assert inside.mean() > 0.9
    out = O.undistort_depth(np.full((60, 80), 1.5, np.float32), m.ravel(), 0)
    assert np.all(out[inside] == np.float32(1.5))
    assert np.all(out[~inside] <= 1.5)


def test_decoder_survives_corrupt_files():
    """Random byte changes and truncations of valid PNG / TIFF files (PNG chunk CRCs recomputed for most,
    so the damage reaches the inflater and the filters): every call returns a status, and a file that
    still decodes gives an image of the size its header states."""
    import ctypes as C
    from volumefusion_gb300._lib import lib
    rng = np.random.default_rng(21)
    img = ((np.cumsum(rng.integers(0, 4, (30, 40)), axis=1) * 7) % 65536).astype(np.uint16)
    bases = [D.png(img, 16, -1), D.png(img, 16, 4, level=0), D.png(img, 16, 2, interlace=True),
             D.tiff(img, 16, 5, 2, rows_per_strip=7), D.tiff(img, 16, 8, 1, rows_per_strip=13, big_endian=True),
             D.tiff(img, 16, 32773)]

    def fix_crcs(b):
        b, pos = bytearray(b), 8
        while pos + 12 <= len(b):
            ln = struct.unpack(">I", bytes(b[pos:pos + 4]))[0]
            if pos + 12 + ln > len(b):
                break
            b[pos + 8 + ln:pos + 12 + ln] = struct.pack(">I", zlib.crc32(bytes(b[pos + 4:pos + 8 + ln])) & 0xFFFFFFFF)
            pos += 12 + ln
        return bytes(b)

    out = np.zeros(1 << 20, np.uint16)
    w, h = C.c_int(), C.c_int()
    seen = set()
    for it in range(3000):
        b = bytearray(bases[it % len(bases)])
        for _ in range(int(rng.integers(1, 6))):
            b[int(rng.integers(0, len(b)))] = int(rng.integers(0, 256))
        if rng.random() < 0.3:
            b = b[:int(rng.integers(1, len(b)))]
        b = bytes(b)
        if b[:4] == b"\x89PNG" and rng.random() < 0.7:
            b = fix_crcs(b)
        buf = np.frombuffer(b, np.uint8)
        rc = lib().afx_decode_depth_image(buf.ctypes.data, buf.size, out.ctypes.data, out.size, C.byref(w), C.byref(h))
        assert rc in (0, 1, 2, 6), rc
        if rc == 0:
            assert 0 < w.value * h.value <= out.size
        seen.add(rc)
    assert {0, 1} <= seen
