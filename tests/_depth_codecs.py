"""Writers of greyscale PNG and TIFF depth images for the decoder tests (test infrastructure).

Built from the format specifications with Python's zlib as the DEFLATE compressor: PNG (ISO/IEC
15948) with a chosen filter per scanline and optional Adam7 interlacing, and TIFF 6.0 strips with no
compression, LZW (MSB-first codes, the code width growing as libtiff's encoder grows it), Deflate or
PackBits, optionally with horizontal differencing.
"""
import struct
import zlib

import numpy as np

PNG_SIG = b"\x89PNG\r\n\x1a\n"
ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]


def png_chunk(kind, data, crc=None):
    c = zlib.crc32(kind + data) & 0xFFFFFFFF if crc is None else crc
    return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", c)


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def _filter_rows(rows, ftype, bpp):
    """rows: list of bytes; ftype 0-4, or -1 to cycle through all five."""
    out = bytearray()
    prev = bytes(len(rows[0])) if rows else b""
    for y, r in enumerate(rows):
        ft = ftype if ftype >= 0 else y % 5
        line = bytearray([ft])
        for i in range(len(r)):
            a = r[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            pred = (0, a, b, (a + b) // 2, _paeth(a, b, c))[ft]
            line.append((r[i] - pred) & 0xFF)
        out += line
        prev = r
    return bytes(out)


def _rows(img, depth):
    if depth == 16:
        return [img[y].astype(">u2").tobytes() for y in range(img.shape[0])]
    return [img[y].astype(np.uint8).tobytes() for y in range(img.shape[0])]


def png(img, depth=16, ftype=0, level=6, interlace=False, strategy=None, idat_size=None, extra_chunks=(),
        color=0):
    """Encode a (h, w) integer image as greyscale PNG."""
    img = np.asarray(img)
    h, w = img.shape
    bpp = depth // 8
    if interlace:
        raw = b""
        for x0, y0, dx, dy in ADAM7:
            sub = img[y0::dy, x0::dx]
            if sub.size:
                raw += _filter_rows(_rows(sub, depth), ftype, bpp)
    else:
        raw = _filter_rows(_rows(img, depth), ftype, bpp)
    if strategy is None:
        z = zlib.compress(raw, level)
    else:
        co = zlib.compressobj(level, zlib.DEFLATED, 15, 9, strategy)
        z = co.compress(raw) + co.flush()
    idat = [z] if not idat_size else [z[i:i + idat_size] for i in range(0, len(z), idat_size)]
    out = PNG_SIG + png_chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, color, 0, 0, int(interlace)))
    for c in extra_chunks:
        out += c
    for part in idat:
        out += png_chunk(b"IDAT", part)
    return out + png_chunk(b"IEND", b"")


def lzw_encode(data):
    """TIFF LZW: Clear first, codes of 9-12 bits MSB-first, the width growing after the entry that
    fills it (as libtiff's encoder does), Clear when the table reaches 4094 entries, EOI last."""
    bits = []

    def emit(code, width):
        bits.append((code, width))

    def reset():
        return {bytes([i]): i for i in range(256)}, 258, 9

    table, nxt, width = reset()
    emit(256, width)
    w = b""
    for c in data:
        wc = w + bytes([c])
        if wc in table:
            w = wc
            continue
        emit(table[w], width)
        table[wc] = nxt
        nxt += 1
        if nxt == 4094:
            emit(256, width)
            table, nxt, width = reset()
        elif nxt > (1 << width) - 1:
            width += 1
        w = bytes([c])
    if w:
        emit(table[w], width)
        nxt += 1
        if nxt > (1 << width) - 1 and width < 12:
            width += 1
    emit(257, width)
    acc, n, out = 0, 0, bytearray()
    for code, wd in bits:
        acc = (acc << wd) | code
        n += wd
        while n >= 8:
            out.append((acc >> (n - 8)) & 0xFF)
            n -= 8
    if n:
        out.append((acc << (8 - n)) & 0xFF)
    return bytes(out)


def packbits_encode(data):
    out, i, n = bytearray(), 0, len(data)
    while i < n:
        j = i
        while j + 1 < n and data[j + 1] == data[i] and j - i < 127:
            j += 1
        if j - i >= 2:
            out += bytes([(257 - (j - i + 1)) & 0xFF, data[i]])
            i = j + 1
            continue
        j = i
        while j < n and j - i < 128 and not (j + 2 < n and data[j] == data[j + 1] == data[j + 2]):
            j += 1
        out.append(j - i - 1)
        out += data[i:j]
        i = j
    return bytes(out)


def tiff(img, depth=16, compression=1, predictor=1, rows_per_strip=None, big_endian=False):
    """Encode a (h, w) integer image as a greyscale TIFF with strips."""
    img = np.asarray(img)
    h, w = img.shape
    rps = rows_per_strip or h
    e = ">" if big_endian else "<"
    dt = np.dtype(e + ("u2" if depth == 16 else "u1"))
    strips = []
    for y0 in range(0, h, rps):
        block = img[y0:y0 + rps].astype(np.int64)
        if predictor == 2:
            d = block.copy()
            d[:, 1:] = block[:, 1:] - block[:, :-1]
            block = d % (1 << depth)
        raw = block.astype(dt).tobytes()
        if compression == 5:
            raw = lzw_encode(raw)
        elif compression in (8, 32946):
            raw = zlib.compress(raw)
        elif compression == 32773:
            raw = packbits_encode(raw)
        strips.append(raw)
    head = (b"MM\x00\x2a" if big_endian else b"II\x2a\x00")
    offsets, pos, body = [], 8, b""
    for s in strips:
        offsets.append(pos + len(body))
        body += s
        if len(body) % 2:
            body += b"\x00"
    extra = b""
    extra_pos = 8 + len(body)

    def longs(vals):
        nonlocal extra
        if len(vals) == 1:
            return struct.pack(e + "HII", 4, 1, vals[0])
        at = extra_pos + len(extra)
        extra += struct.pack(e + "%dI" % len(vals), *vals)
        return struct.pack(e + "HII", 4, len(vals), at)

    def short(v):
        return struct.pack(e + "HIHH", 3, 1, v, 0)

    entries = [(256, struct.pack(e + "HII", 4, 1, w)), (257, struct.pack(e + "HII", 4, 1, h)),
               (258, short(depth)), (259, short(compression)), (262, short(1)), (273, longs(offsets)),
               (277, short(1)), (278, struct.pack(e + "HII", 4, 1, rps)), (279, longs([len(s) for s in strips]))]
    if predictor != 1:
        entries.append((317, short(predictor)))
    ifd_pos = extra_pos + len(extra)
    ifd = struct.pack(e + "H", len(entries))
    for tag, rest in sorted(entries):
        ifd += struct.pack(e + "H", tag) + rest
    ifd += struct.pack(e + "I", 0)
    return head + struct.pack(e + "I", ifd_pos) + body + extra + ifd
