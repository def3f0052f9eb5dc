// afx_decode.cu -- host decoding of depth frames: greyscale 8/16-bit PNG and TIFF, the images the
// reference's depth readers load with cv::imread(file, IMREAD_ANYDEPTH | IMREAD_ANYCOLOR)
// (src/dataset.cpp:168-189, src/KinectReader.cpp:9-21, src/AzureReader.cpp:10-22), and the reference's
// frame-name pattern (af::insertIntoPattern, src/dataset.cpp:131-150).  The decoded frame is the
// uint16 image in millimetres; the conversion to metres (convertTo(CV_32FC1, 1/1000)) happens on the
// device in the frame preparation.
//
// Everything here is host code written from the format specifications:
//   - zlib stream (RFC 1950) and DEFLATE (RFC 1951): stored, fixed- and dynamic-Huffman blocks,
//     Adler-32 checked;
//   - PNG (ISO/IEC 15948): chunk CRC-32 checked for critical chunks, filters 0-4 per scanline,
//     non-interlaced and Adam7, big-endian 16-bit samples;
//   - TIFF 6.0 baseline strips: uncompressed, LZW (with horizontal differencing), Deflate, PackBits.
// Decoding is serial per image (every DEFLATE symbol depends on the bits before it), so the batch
// entry point decodes several frames at once on host threads.
#include <atomic>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/afx/afx.h"

namespace {

// ------------------------------------------------------------------------------------
// Checksums
// ------------------------------------------------------------------------------------

struct Crc32Tables {
    uint32_t t[8][256];
    Crc32Tables() {
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t c = i;
            for (int k = 0; k < 8; ++k) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            t[0][i] = c;
        }
        for (int s = 1; s < 8; ++s)
            for (uint32_t i = 0; i < 256; ++i) t[s][i] = (t[s - 1][i] >> 8) ^ t[0][t[s - 1][i] & 0xFF];
    }
};

const Crc32Tables& crc_tables() {
    static const Crc32Tables tables;
    return tables;
}

// CRC-32 (ISO 3309 / ITU-T V.42, the PNG chunk CRC), eight bytes per step.
uint32_t crc32(const uint8_t* p, size_t n, uint32_t crc = 0) {
    const Crc32Tables& T = crc_tables();
    crc = ~crc;
    while (n >= 8) {
        const uint32_t a = crc ^ ((uint32_t)p[0] | (uint32_t)p[1] << 8 | (uint32_t)p[2] << 16 | (uint32_t)p[3] << 24);
        const uint32_t b = (uint32_t)p[4] | (uint32_t)p[5] << 8 | (uint32_t)p[6] << 16 | (uint32_t)p[7] << 24;
        crc = T.t[7][a & 0xFF] ^ T.t[6][(a >> 8) & 0xFF] ^ T.t[5][(a >> 16) & 0xFF] ^ T.t[4][a >> 24] ^
              T.t[3][b & 0xFF] ^ T.t[2][(b >> 8) & 0xFF] ^ T.t[1][(b >> 16) & 0xFF] ^ T.t[0][b >> 24];
        p += 8;
        n -= 8;
    }
    while (n--) crc = T.t[0][(crc ^ *p++) & 0xFF] ^ (crc >> 8);
    return ~crc;
}

// Adler-32 (RFC 1950 section 8.2); 5552 is the longest run whose sums cannot overflow 32 bits.
uint32_t adler32(const uint8_t* p, size_t n) {
    uint32_t a = 1, b = 0;
    while (n) {
        size_t k = n < 5552 ? n : 5552;
        n -= k;
        while (k--) {
            a += *p++;
            b += a;
        }
        a %= 65521u;
        b %= 65521u;
    }
    return (b << 16) | a;
}

uint32_t be32(const uint8_t* p) { return (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | p[3]; }

// ------------------------------------------------------------------------------------
// DEFLATE (RFC 1951)
// ------------------------------------------------------------------------------------

constexpr int kFastBits = 10;

// Canonical Huffman code: a table indexed by the next kFastBits input bits for codes of at most
// kFastBits bits (entry = symbol << 4 | length, 0 for a longer code), plus the per-length counts
// and the symbols in canonical order for the longer ones.
struct Huffman {
    uint16_t fast[1 << kFastBits];
    uint16_t count[16];
    uint16_t symbol[320];

    // lens[0..n): code length of each symbol (0 = unused).  False for an over-subscribed set.
    bool build(const uint8_t* lens, int n) {
        std::memset(count, 0, sizeof(count));
        for (int s = 0; s < n; ++s) count[lens[s]]++;
        count[0] = 0;
        int left = 1;
        for (int l = 1; l < 16; ++l) {
            left <<= 1;
            left -= count[l];
            if (left < 0) return false;
        }
        uint16_t offs[16];
        offs[1] = 0;
        for (int l = 1; l < 15; ++l) offs[l + 1] = (uint16_t)(offs[l] + count[l]);
        for (int s = 0; s < n; ++s)
            if (lens[s]) symbol[offs[lens[s]]++] = (uint16_t)s;
        std::memset(fast, 0, sizeof(fast));
        int code = 0, k = 0;
        for (int l = 1; l <= kFastBits; ++l) {
            for (int i = 0; i < count[l]; ++i, ++k, ++code) {
                int rev = 0;
                for (int b = 0; b < l; ++b) rev |= ((code >> b) & 1) << (l - 1 - b);
                const uint16_t e = (uint16_t)(symbol[k] << 4 | l);
                for (int j = rev; j < (1 << kFastBits); j += 1 << l) fast[j] = e;
            }
            code <<= 1;
        }
        return true;
    }
};

struct Bits {
    const uint8_t* p;
    const uint8_t* end;
    uint64_t buf = 0;
    int cnt = 0;
    int pad = 0;  // zero bytes supplied past the end of the input

    Bits(const uint8_t* b, const uint8_t* e) : p(b), end(e) {}

    // Tops the bit buffer up to at least 56 bits.  Bits above `cnt` are either zero or the true
    // bits of the bytes at p (a whole-word load claims only the bytes it fully covers), so OR-ing
    // a later load over them is exact.
    inline void refill() {
        if (end - p >= 8) {
            uint64_t w;
            std::memcpy(&w, p, 8);
#if defined(__BYTE_ORDER__) && __BYTE_ORDER__ == __ORDER_BIG_ENDIAN__
            w = __builtin_bswap64(w);
#endif
            buf |= w << cnt;
            p += (63 - cnt) >> 3;
            cnt |= 56;
        } else {
            while (cnt <= 56) {
                uint64_t b = 0;
                if (p < end)
                    b = *p++;
                else
                    ++pad;
                buf |= b << cnt;
                cnt += 8;
            }
        }
    }
    inline uint32_t get(int n) {  // n <= 32
        if (cnt < n) refill();
        const uint32_t v = (uint32_t)(buf & ((1ull << n) - 1));
        buf >>= n;
        cnt -= n;
        return v;
    }
    inline int decode(const Huffman& h) {
        if (cnt < 15) refill();
        const uint16_t e = h.fast[buf & ((1u << kFastBits) - 1)];
        if (e) {
            const int l = e & 15;
            buf >>= l;
            cnt -= l;
            return e >> 4;
        }
        // a code longer than kFastBits: canonical decode one bit at a time
        uint64_t b = buf;
        int code = 0, first = 0, index = 0;
        for (int l = 1; l < 16; ++l) {
            code |= (int)(b & 1);
            b >>= 1;
            const int c = h.count[l];
            if (code - c < first) {
                buf >>= l;
                cnt -= l;
                return h.symbol[index + (code - first)];
            }
            index += c;
            first = (first + c) << 1;
            code <<= 1;
        }
        return -1;
    }
    bool overrun() const { return pad * 8 > cnt; }
};

const uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31,
                               35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

struct FixedCodes {
    Huffman lit, dist;
    FixedCodes() {
        uint8_t l[288];
        for (int i = 0; i < 144; ++i) l[i] = 8;
        for (int i = 144; i < 256; ++i) l[i] = 9;
        for (int i = 256; i < 280; ++i) l[i] = 7;
        for (int i = 280; i < 288; ++i) l[i] = 8;
        lit.build(l, 288);
        uint8_t d[30];
        for (int i = 0; i < 30; ++i) d[i] = 5;
        dist.build(d, 30);
    }
};

const FixedCodes& fixed_codes() {
    static const FixedCodes codes;
    return codes;
}

// Inflates one Huffman-coded block into out[o..cap).  `cap` is the logical capacity; the
// buffer behind it has at least 8 bytes of slack for the word-wise match copy.
int inflate_codes(Bits& in, const Huffman& lit, const Huffman& dist, uint8_t* out, size_t& o, size_t cap) {
    for (;;) {
        const int sym = in.decode(lit);
        if (sym < 256) {
            if (sym < 0) return AFX_ERR_INVALID_ARGUMENT;
            if (o >= cap) return AFX_ERR_CAPACITY;
            out[o++] = (uint8_t)sym;
            continue;
        }
        if (sym == 256) return in.overrun() ? AFX_ERR_INVALID_ARGUMENT : AFX_OK;
        const int ls = sym - 257;
        if (ls >= 29) return AFX_ERR_INVALID_ARGUMENT;
        const size_t len = kLenBase[ls] + in.get(kLenExtra[ls]);
        const int ds = in.decode(dist);
        if (ds < 0 || ds >= 30) return AFX_ERR_INVALID_ARGUMENT;
        const size_t d = kDistBase[ds] + in.get(kDistExtra[ds]);
        if (d > o) return AFX_ERR_INVALID_ARGUMENT;
        if (len > cap - o) return AFX_ERR_CAPACITY;
        if (in.overrun()) return AFX_ERR_INVALID_ARGUMENT;
        uint8_t* dst = out + o;
        const uint8_t* src = dst - d;
        if (d >= 8) {  // chunks of 8 never overlap their own source; the last may run into the slack
            for (size_t k = 0; k < len; k += 8) std::memcpy(dst + k, src + k, 8);
        } else if (d == 1) {
            std::memset(dst, *src, len);
        } else {
            for (size_t k = 0; k < len; ++k) dst[k] = src[k];
        }
        o += len;
    }
}

// Decodes a raw DEFLATE stream; *used receives the input bytes consumed (rounded up to a byte).
int inflate_raw(const uint8_t* src, size_t n, uint8_t* out, size_t cap, size_t* out_len, size_t* used) {
    Bits in(src, src + n);
    size_t o = 0;
    Huffman lit, dist;
    for (;;) {
        const uint32_t final_block = in.get(1);
        const uint32_t type = in.get(2);
        int rc = AFX_OK;
        if (type == 0) {  // stored
            const int drop = in.cnt & 7;
            in.buf >>= drop;
            in.cnt -= drop;
            const uint32_t len = in.get(16), nlen = in.get(16);
            if (in.overrun() || (len ^ 0xFFFFu) != nlen) return AFX_ERR_INVALID_ARGUMENT;
            if (len > cap - o) return AFX_ERR_CAPACITY;
            uint32_t k = 0;
            while (k < len && in.cnt >= 8) {
                out[o++] = (uint8_t)in.buf;
                in.buf >>= 8;
                in.cnt -= 8;
                ++k;
            }
            if (k < len) {
                if (in.pad || (size_t)(in.end - in.p) < len - k) return AFX_ERR_INVALID_ARGUMENT;
                std::memcpy(out + o, in.p, len - k);
                in.p += len - k;
                o += len - k;
                in.buf = 0;
                in.cnt = 0;
            }
        } else if (type == 1) {
            rc = inflate_codes(in, fixed_codes().lit, fixed_codes().dist, out, o, cap);
        } else if (type == 2) {
            const int hlit = (int)in.get(5) + 257, hdist = (int)in.get(5) + 1, hclen = (int)in.get(4) + 4;
            static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19] = {};
            for (int i = 0; i < hclen; ++i) cl[order[i]] = (uint8_t)in.get(3);
            Huffman clh;
            if (!clh.build(cl, 19)) return AFX_ERR_INVALID_ARGUMENT;
            uint8_t lens[320];
            int k = 0;
            while (k < hlit + hdist) {
                const int s = in.decode(clh);
                if (s < 0) return AFX_ERR_INVALID_ARGUMENT;
                if (s < 16) {
                    lens[k++] = (uint8_t)s;
                    continue;
                }
                int rep;
                uint8_t v = 0;
                if (s == 16) {
                    if (k == 0) return AFX_ERR_INVALID_ARGUMENT;
                    v = lens[k - 1];
                    rep = 3 + (int)in.get(2);
                } else if (s == 17) {
                    rep = 3 + (int)in.get(3);
                } else {
                    rep = 11 + (int)in.get(7);
                }
                if (k + rep > hlit + hdist) return AFX_ERR_INVALID_ARGUMENT;
                while (rep--) lens[k++] = v;
            }
            if (in.overrun() || lens[256] == 0) return AFX_ERR_INVALID_ARGUMENT;
            if (!lit.build(lens, hlit) || !dist.build(lens + hlit, hdist)) return AFX_ERR_INVALID_ARGUMENT;
            rc = inflate_codes(in, lit, dist, out, o, cap);
        } else {
            return AFX_ERR_INVALID_ARGUMENT;
        }
        if (rc) return rc;
        if (final_block) break;
    }
    if (in.overrun()) return AFX_ERR_INVALID_ARGUMENT;
    // bytes consumed: those loaded into the buffer less the whole bytes still unread in it
    const size_t loaded = (size_t)(in.p - src) + (size_t)in.pad;
    *used = loaded - (size_t)(in.cnt / 8);
    *out_len = o;
    return AFX_OK;
}

// zlib stream (RFC 1950): header, DEFLATE data, Adler-32 of the output (big-endian).
int inflate_zlib(const uint8_t* src, size_t n, uint8_t* out, size_t cap, size_t* out_len) {
    if (n < 6) return AFX_ERR_INVALID_ARGUMENT;
    const unsigned cmf = src[0], flg = src[1];
    if ((cmf & 15) != 8 || (cmf >> 4) > 7 || ((cmf << 8) | flg) % 31 != 0 || (flg & 0x20)) return AFX_ERR_INVALID_ARGUMENT;
    size_t used = 0;
    const int rc = inflate_raw(src + 2, n - 2, out, cap, out_len, &used);
    if (rc) return rc;
    if (2 + used + 4 > n) return AFX_ERR_INVALID_ARGUMENT;
    if (be32(src + 2 + used) != adler32(out, *out_len)) return AFX_ERR_INVALID_ARGUMENT;
    return AFX_OK;
}

// ------------------------------------------------------------------------------------
// PNG (ISO/IEC 15948)
// ------------------------------------------------------------------------------------

const uint8_t kPngSig[8] = {0x89, 'P', 'N', 'G', 0x0D, 0x0A, 0x1A, 0x0A};

struct PngHeader {
    uint32_t width = 0, height = 0;
    int depth = 0, color = 0, interlace = 0;
};

int png_header(const uint8_t* d, size_t n, PngHeader* h) {
    if (n < 8 + 25 || std::memcmp(d, kPngSig, 8) != 0) return AFX_ERR_INVALID_ARGUMENT;
    if (be32(d + 8) != 13 || std::memcmp(d + 12, "IHDR", 4) != 0) return AFX_ERR_INVALID_ARGUMENT;
    if (crc32(d + 12, 17) != be32(d + 29)) return AFX_ERR_INVALID_ARGUMENT;
    const uint8_t* p = d + 16;
    h->width = be32(p);
    h->height = be32(p + 4);
    h->depth = p[8];
    h->color = p[9];
    h->interlace = p[12];
    if (h->width == 0 || h->height == 0 || h->width > 0x7FFFFFFFu || h->height > 0x7FFFFFFFu) return AFX_ERR_INVALID_ARGUMENT;
    if (p[10] != 0 || p[11] != 0 || h->interlace > 1) return AFX_ERR_INVALID_ARGUMENT;
    if (h->color != 0 || (h->depth != 8 && h->depth != 16)) return AFX_ERR_UNSUPPORTED;  // greyscale depth only
    if ((uint64_t)h->width * h->height > (1ull << 30)) return AFX_ERR_UNSUPPORTED;
    return AFX_OK;
}

// Paeth predictor (ISO/IEC 15948 section 9.4): a, b or c, whichever is closest to a + b - c, ties
// resolved in the order a, b, c; written as two strict-less updates so that it compiles to selects.
inline int paeth(int a, int b, int c) {
    const int pa = b > c ? b - c : c - b, pb = a > c ? a - c : c - a;
    const int s = a + b - 2 * c, pc = s < 0 ? -s : s;
    int pred = a, best = pa;
    pred = pb < best ? b : pred;
    best = pb < best ? pb : best;
    pred = pc < best ? c : pred;
    return pred;
}

// Reverses the filter of one scanline in place (prev = the previous reconstructed line, or null).
// BPP bytes per pixel; the left neighbours are carried in registers, so the serial dependence along
// the line is a register chain rather than a store and a reload.
template <int BPP>
bool unfilter_line(int type, uint8_t* cur, const uint8_t* prev, size_t rb) {
    if (rb < (size_t)BPP) return type >= 0 && type <= 4;
    uint8_t a[BPP], c[BPP];
    switch (type) {
        case 0: return true;
        case 1:
            for (int k = 0; k < BPP; ++k) a[k] = cur[k];
            for (size_t i = BPP; i + BPP <= rb; i += BPP)
                for (int k = 0; k < BPP; ++k) cur[i + k] = a[k] = (uint8_t)(cur[i + k] + a[k]);
            return true;
        case 2:
            if (prev)
                for (size_t i = 0; i < rb; ++i) cur[i] = (uint8_t)(cur[i] + prev[i]);
            return true;
        case 3:
            for (int k = 0; k < BPP; ++k) a[k] = cur[k] = (uint8_t)(cur[k] + (prev ? prev[k] >> 1 : 0));
            for (size_t i = BPP; i + BPP <= rb; i += BPP)
                for (int k = 0; k < BPP; ++k)
                    cur[i + k] = a[k] = (uint8_t)(cur[i + k] + ((a[k] + (prev ? prev[i + k] : 0)) >> 1));
            return true;
        case 4:
            if (!prev) {  // b = c = 0: the predictor is a (the Sub filter)
                for (int k = 0; k < BPP; ++k) a[k] = cur[k];
                for (size_t i = BPP; i + BPP <= rb; i += BPP)
                    for (int k = 0; k < BPP; ++k) cur[i + k] = a[k] = (uint8_t)(cur[i + k] + a[k]);
                return true;
            }
            for (int k = 0; k < BPP; ++k) {  // first pixel: a = c = 0, the predictor is b
                a[k] = cur[k] = (uint8_t)(cur[k] + prev[k]);
                c[k] = prev[k];
            }
            for (size_t i = BPP; i + BPP <= rb; i += BPP)
                for (int k = 0; k < BPP; ++k) {
                    const uint8_t b = prev[i + k];
                    cur[i + k] = a[k] = (uint8_t)(cur[i + k] + paeth(a[k], b, c[k]));
                    c[k] = b;
                }
            return true;
    }
    return false;
}

bool unfilter(int type, uint8_t* cur, const uint8_t* prev, size_t rb, int bpp) {
    return bpp == 2 ? unfilter_line<2>(type, cur, prev, rb) : unfilter_line<1>(type, cur, prev, rb);
}

struct Scratch {
    std::vector<uint8_t> a, b;
};

Scratch& scratch() {
    thread_local Scratch s;
    return s;
}

int png_decode(const uint8_t* d, size_t n, uint16_t* out, long cap, int* width, int* height) {
    PngHeader h;
    int rc = png_header(d, n, &h);
    if (rc) return rc;
    if (width) *width = (int)h.width;
    if (height) *height = (int)h.height;
    if (!out) return AFX_OK;
    const uint64_t W = h.width, H = h.height;
    if (cap < 0 || (uint64_t)cap < W * H) return AFX_ERR_CAPACITY;
    const int bpp = h.depth / 8;
    // pass geometry (Adam7, or one pass covering the image)
    struct Pass {
        int x0, y0, dx, dy;
    };
    static const Pass adam7[7] = {{0, 0, 8, 8}, {4, 0, 8, 8}, {0, 4, 4, 8}, {2, 0, 4, 4},
                                  {0, 2, 2, 4}, {1, 0, 2, 2}, {0, 1, 1, 2}};
    static const Pass whole = {0, 0, 1, 1};
    const Pass* passes = h.interlace ? adam7 : &whole;
    const int n_pass = h.interlace ? 7 : 1;
    uint64_t raw_size = 0;
    for (int k = 0; k < n_pass; ++k) {
        const uint64_t pw = (W - passes[k].x0 + passes[k].dx - 1) / passes[k].dx;
        const uint64_t ph = (H - passes[k].y0 + passes[k].dy - 1) / passes[k].dy;
        if (pw && ph) raw_size += ph * (1 + pw * bpp);
    }
    // gather the IDAT chunks (CRC-checked) into one zlib stream
    Scratch& s = scratch();
    s.a.clear();
    size_t pos = 8;
    bool seen_iend = false;
    while (pos + 12 <= n) {
        const uint32_t len = be32(d + pos);
        const uint8_t* type = d + pos + 4;
        if (len > 0x7FFFFFFFu || pos + 12 + (size_t)len > n) return AFX_ERR_INVALID_ARGUMENT;
        const bool critical = (type[0] & 0x20) == 0;
        if (critical && crc32(type, 4 + (size_t)len) != be32(d + pos + 8 + len)) return AFX_ERR_INVALID_ARGUMENT;
        if (std::memcmp(type, "IDAT", 4) == 0) {
            s.a.insert(s.a.end(), d + pos + 8, d + pos + 8 + len);
        } else if (std::memcmp(type, "IEND", 4) == 0) {
            seen_iend = true;
            break;
        } else if (critical && std::memcmp(type, "IHDR", 4) != 0 && std::memcmp(type, "PLTE", 4) != 0) {
            return AFX_ERR_UNSUPPORTED;  // an unknown critical chunk
        }
        pos += 12 + (size_t)len;
    }
    if (!seen_iend || s.a.empty()) return AFX_ERR_INVALID_ARGUMENT;
    s.b.resize(raw_size + 16);
    size_t got = 0;
    rc = inflate_zlib(s.a.data(), s.a.size(), s.b.data(), raw_size, &got);
    if (rc == AFX_ERR_CAPACITY) return AFX_ERR_INVALID_ARGUMENT;  // more data than the image holds
    if (rc) return rc;
    if (got != raw_size) return AFX_ERR_INVALID_ARGUMENT;
    uint8_t* raw = s.b.data();
    for (int k = 0; k < n_pass; ++k) {
        const Pass& P = passes[k];
        const uint64_t pw = (W - P.x0 + P.dx - 1) / P.dx, ph = (H - P.y0 + P.dy - 1) / P.dy;
        if (!pw || !ph) continue;
        const size_t rb = (size_t)pw * bpp;
        const uint8_t* prev = nullptr;
        for (uint64_t y = 0; y < ph; ++y) {
            uint8_t* line = raw + 1;
            if (!unfilter(raw[0], line, prev, rb, bpp)) return AFX_ERR_INVALID_ARGUMENT;
            uint16_t* o = out + (P.y0 + y * P.dy) * W + P.x0;
            if (bpp == 2) {
                for (uint64_t x = 0; x < pw; ++x) o[x * P.dx] = (uint16_t)(line[2 * x] << 8 | line[2 * x + 1]);
            } else {
                for (uint64_t x = 0; x < pw; ++x) o[x * P.dx] = line[x];
            }
            prev = line;
            raw += 1 + rb;
        }
    }
    return AFX_OK;
}

// ------------------------------------------------------------------------------------
// TIFF 6.0 baseline strips
// ------------------------------------------------------------------------------------

struct Tiff {
    bool le = true;
    const uint8_t* d = nullptr;
    size_t n = 0;
    uint32_t u16(size_t o) const { return le ? (uint32_t)(d[o] | d[o + 1] << 8) : (uint32_t)(d[o] << 8 | d[o + 1]); }
    uint32_t u32(size_t o) const {
        return le ? (uint32_t)d[o] | (uint32_t)d[o + 1] << 8 | (uint32_t)d[o + 2] << 16 | (uint32_t)d[o + 3] << 24
                  : be32(d + o);
    }
};

struct TiffImage {
    uint32_t width = 0, height = 0, bits = 1, compression = 1, samples = 1, rows_per_strip = 0xFFFFFFFFu;
    uint32_t predictor = 1, planar = 1, sample_format = 1, photometric = 1;
    bool tiled = false;
    std::vector<uint32_t> offsets, counts;
};

// Reads one IFD entry's values (SHORT or LONG) into v.
bool tiff_values(const Tiff& t, size_t e, std::vector<uint32_t>& v) {
    const uint32_t type = t.u16(e + 2), count = t.u32(e + 4);
    const uint32_t size = type == 3 ? 2 : type == 4 ? 4 : 0;
    if (!size || count == 0 || count > (1u << 24)) return false;
    size_t at = e + 8;
    if ((uint64_t)size * count > 4) {
        at = t.u32(e + 8);
        if ((uint64_t)at + (uint64_t)size * count > t.n) return false;
    }
    v.resize(count);
    for (uint32_t i = 0; i < count; ++i) v[i] = size == 2 ? t.u16(at + 2 * i) : t.u32(at + 4 * i);
    return true;
}

int tiff_parse(const uint8_t* d, size_t n, Tiff* t, TiffImage* im) {
    if (n < 8) return AFX_ERR_INVALID_ARGUMENT;
    if (d[0] == 'I' && d[1] == 'I')
        t->le = true;
    else if (d[0] == 'M' && d[1] == 'M')
        t->le = false;
    else
        return AFX_ERR_INVALID_ARGUMENT;
    t->d = d;
    t->n = n;
    if (t->u16(2) != 42) return AFX_ERR_UNSUPPORTED;  // BigTIFF and others
    const uint32_t ifd = t->u32(4);
    if ((uint64_t)ifd + 2 > n) return AFX_ERR_INVALID_ARGUMENT;
    const uint32_t entries = t->u16(ifd);
    if ((uint64_t)ifd + 2 + 12ull * entries > n) return AFX_ERR_INVALID_ARGUMENT;
    std::vector<uint32_t> v;
    for (uint32_t i = 0; i < entries; ++i) {
        const size_t e = ifd + 2 + 12 * (size_t)i;
        const uint32_t tag = t->u16(e);
        if (tag == 322 || tag == 323 || tag == 324 || tag == 325) {
            im->tiled = true;
            continue;
        }
        if (tag != 256 && tag != 257 && tag != 258 && tag != 259 && tag != 262 && tag != 273 && tag != 277 &&
            tag != 278 && tag != 279 && tag != 284 && tag != 317 && tag != 339)
            continue;
        if (!tiff_values(*t, e, v)) return AFX_ERR_INVALID_ARGUMENT;
        switch (tag) {
            case 256: im->width = v[0]; break;
            case 257: im->height = v[0]; break;
            case 258: im->bits = v[0]; break;
            case 259: im->compression = v[0]; break;
            case 262: im->photometric = v[0]; break;
            case 273: im->offsets = v; break;
            case 277: im->samples = v[0]; break;
            case 278: im->rows_per_strip = v[0]; break;
            case 279: im->counts = v; break;
            case 284: im->planar = v[0]; break;
            case 317: im->predictor = v[0]; break;
            case 339: im->sample_format = v[0]; break;
        }
    }
    if (im->width == 0 || im->height == 0 || im->width > 0x7FFFFFFFu || im->height > 0x7FFFFFFFu) return AFX_ERR_INVALID_ARGUMENT;
    if ((uint64_t)im->width * im->height > (1ull << 30)) return AFX_ERR_UNSUPPORTED;
    if (im->tiled || im->samples != 1 || (im->bits != 8 && im->bits != 16) || im->sample_format != 1 ||
        im->photometric > 1 || (im->predictor != 1 && im->predictor != 2))
        return AFX_ERR_UNSUPPORTED;
    if (im->compression != 1 && im->compression != 5 && im->compression != 8 && im->compression != 32946 &&
        im->compression != 32773)
        return AFX_ERR_UNSUPPORTED;
    if (im->offsets.empty() || im->offsets.size() != im->counts.size()) return AFX_ERR_INVALID_ARGUMENT;
    return AFX_OK;
}

// TIFF LZW (TIFF 6.0 section 13): MSB-first codes of 9-12 bits, Clear = 256, EOI = 257, the code
// width growing one code early.
int lzw_decode(const uint8_t* src, size_t n, uint8_t* out, size_t cap, size_t* out_len) {
    std::vector<uint16_t> prefix(4096);
    std::vector<uint8_t> suffix(4096), first(4096);
    std::vector<uint16_t> length(4096);
    for (int i = 0; i < 256; ++i) {
        prefix[i] = 0xFFFF;
        suffix[i] = first[i] = (uint8_t)i;
        length[i] = 1;
    }
    size_t o = 0;
    uint64_t buf = 0;
    int cnt = 0;
    size_t p = 0;
    int width = 9, next = 258, old = -1;
    for (;;) {
        while (cnt < width) {
            if (p >= n) {  // ran out without EOI: accept what was decoded (writers may omit it)
                *out_len = o;
                return AFX_OK;
            }
            buf = (buf << 8) | src[p++];
            cnt += 8;
        }
        const int code = (int)((buf >> (cnt - width)) & ((1u << width) - 1));
        cnt -= width;
        if (code == 257) break;
        if (code == 256) {
            width = 9;
            next = 258;
            old = -1;
            continue;
        }
        int emit;
        if (old < 0) {
            if (code > 255) return AFX_ERR_INVALID_ARGUMENT;
            emit = code;
        } else {
            if (code > next || (code == next && next >= 4096)) return AFX_ERR_INVALID_ARGUMENT;
            if (next < 4096) {  // a full table takes no entry until the next Clear
                const uint8_t f = code < next ? first[code] : first[old];
                prefix[next] = (uint16_t)old;
                suffix[next] = f;
                first[next] = first[old];
                length[next] = (uint16_t)(length[old] + 1);
                ++next;
            }
            emit = code;
        }
        const size_t len = length[emit];
        if (len > cap - o) return AFX_ERR_CAPACITY;
        for (int c = emit, k = (int)len - 1; k >= 0; --k) {
            out[o + k] = suffix[c];
            c = prefix[c];
        }
        o += len;
        old = code;
        if (next + 1 >= (1 << width) && width < 12) ++width;
    }
    *out_len = o;
    return AFX_OK;
}

int packbits_decode(const uint8_t* src, size_t n, uint8_t* out, size_t cap, size_t* out_len) {
    size_t o = 0, p = 0;
    while (p < n && o < cap) {
        const int c = (int8_t)src[p++];
        if (c >= 0) {
            const size_t k = (size_t)c + 1;
            if (p + k > n || k > cap - o) return AFX_ERR_INVALID_ARGUMENT;
            std::memcpy(out + o, src + p, k);
            p += k;
            o += k;
        } else if (c != -128) {
            const size_t k = (size_t)(1 - c);
            if (p >= n || k > cap - o) return AFX_ERR_INVALID_ARGUMENT;
            std::memset(out + o, src[p++], k);
            o += k;
        }
    }
    *out_len = o;
    return AFX_OK;
}

int tiff_decode(const uint8_t* d, size_t n, uint16_t* out, long cap, int* width, int* height) {
    Tiff t;
    TiffImage im;
    int rc = tiff_parse(d, n, &t, &im);
    if (rc) return rc;
    if (width) *width = (int)im.width;
    if (height) *height = (int)im.height;
    if (!out) return AFX_OK;
    const uint64_t W = im.width, H = im.height;
    if (cap < 0 || (uint64_t)cap < W * H) return AFX_ERR_CAPACITY;
    const int bpp = (int)im.bits / 8;
    const uint64_t rps = im.rows_per_strip == 0 ? H : (im.rows_per_strip > H ? H : im.rows_per_strip);
    const uint64_t strips = (H + rps - 1) / rps;
    if (im.offsets.size() < strips) return AFX_ERR_INVALID_ARGUMENT;
    const size_t row_bytes = (size_t)W * bpp;
    Scratch& s = scratch();
    s.b.resize(rps * row_bytes + 16);
    for (uint64_t k = 0; k < strips; ++k) {
        const uint64_t rows = (k + 1) * rps <= H ? rps : H - k * rps;
        const size_t want = (size_t)rows * row_bytes;
        const uint64_t off = im.offsets[k], cnt = im.counts[k];
        if (off + cnt > n) return AFX_ERR_INVALID_ARGUMENT;
        const uint8_t* src = d + off;
        size_t got = 0;
        uint8_t* buf = s.b.data();
        switch (im.compression) {
            case 1:
                if (cnt < want) return AFX_ERR_INVALID_ARGUMENT;
                std::memcpy(buf, src, want);
                got = want;
                break;
            case 5: rc = lzw_decode(src, cnt, buf, want, &got); break;
            case 8:
            case 32946: rc = inflate_zlib(src, cnt, buf, want, &got); break;
            case 32773: rc = packbits_decode(src, cnt, buf, want, &got); break;
        }
        if (rc == AFX_ERR_CAPACITY) return AFX_ERR_INVALID_ARGUMENT;
        if (rc) return rc;
        if (got != want) return AFX_ERR_INVALID_ARGUMENT;
        for (uint64_t r = 0; r < rows; ++r) {
            const uint8_t* line = buf + r * row_bytes;
            uint16_t* o = out + (k * rps + r) * W;
            if (bpp == 2) {
                for (uint64_t x = 0; x < W; ++x)
                    o[x] = t.le ? (uint16_t)(line[2 * x] | line[2 * x + 1] << 8) : (uint16_t)(line[2 * x] << 8 | line[2 * x + 1]);
            } else {
                for (uint64_t x = 0; x < W; ++x) o[x] = line[x];
            }
            if (im.predictor == 2)  // horizontal differencing, per sample, modulo the sample size
                for (uint64_t x = 1; x < W; ++x)
                    o[x] = bpp == 2 ? (uint16_t)(o[x] + o[x - 1]) : (uint16_t)((o[x] + o[x - 1]) & 0xFF);
        }
    }
    return AFX_OK;
}

int decode_any(const uint8_t* d, size_t n, uint16_t* out, long cap, int* width, int* height) {
    if (!d) return AFX_ERR_INVALID_ARGUMENT;
    if (n >= 8 && std::memcmp(d, kPngSig, 8) == 0) return png_decode(d, n, out, cap, width, height);
    if (n >= 4 && ((d[0] == 'I' && d[1] == 'I') || (d[0] == 'M' && d[1] == 'M'))) return tiff_decode(d, n, out, cap, width, height);
    return AFX_ERR_UNSUPPORTED;
}

int read_file(const char* path, std::vector<uint8_t>& data) {
    FILE* f = std::fopen(path, "rb");
    if (!f) return AFX_ERR_IO;
    int rc = AFX_OK;
    if (std::fseek(f, 0, SEEK_END) != 0) rc = AFX_ERR_IO;
    const long size = rc ? -1 : std::ftell(f);
    if (size < 0 || std::fseek(f, 0, SEEK_SET) != 0) rc = AFX_ERR_IO;
    if (!rc) {
        data.resize((size_t)size);
        if (size && std::fread(data.data(), 1, (size_t)size, f) != (size_t)size) rc = AFX_ERR_IO;
    }
    std::fclose(f);
    return rc;
}

}  // namespace

extern "C" {

int afx_decode_depth_image(const uint8_t* data, size_t len, uint16_t* out, long capacity, int* width, int* height) {
    try {
        return decode_any(data, len, out, capacity, width, height);
    } catch (...) {
        return AFX_ERR_NO_MEMORY;
    }
}

int afx_decode_depth_images(int n, const uint8_t* const* data, const size_t* lens, uint16_t* const* outs,
                            const long* capacities, int* widths, int* heights, int* status, int threads) {
    if (n < 0 || (n > 0 && (!data || !lens || !outs || !capacities || !status))) return AFX_ERR_INVALID_ARGUMENT;
    if (threads < 1) threads = 1;
    if (threads > n) threads = n;
    std::atomic<int> next(0);
    auto work = [&]() {
        for (int i = next.fetch_add(1); i < n; i = next.fetch_add(1)) {
            int w = 0, h = 0;
            status[i] = afx_decode_depth_image(data[i], lens[i], outs[i], capacities[i], &w, &h);
            if (widths) widths[i] = w;
            if (heights) heights[i] = h;
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; ++t) {
        try {
            pool.emplace_back(work);
        } catch (...) {
            break;  // fewer threads: the remaining ones take the work
        }
    }
    work();
    for (auto& th : pool) th.join();
    int rc = AFX_OK;
    for (int i = 0; i < n && !rc; ++i) rc = status[i];
    return rc;
}

int afx_depth_file_name(const char* pattern, long index, char* out, size_t capacity) {
    if (!pattern || !out || capacity == 0 || index < 0) return AFX_ERR_INVALID_ARGUMENT;
    std::string s(pattern);
    size_t stars = 0;
    for (char c : s) stars += c == '*';
    const size_t at = s.find(std::string(stars, '*'));
    if (stars == 0 || at == std::string::npos) return AFX_ERR_INVALID_ARGUMENT;
    std::string digits = std::to_string(index);
    if (digits.size() < stars) digits.insert(0, stars - digits.size(), '0');
    const size_t nd = digits.size();
    if (at + nd > s.size()) return AFX_ERR_INVALID_ARGUMENT;  // the index runs past the end of the pattern
    s.replace(at, nd, digits);  // overwrites nd characters, as the reference's std::copy does
    if (s.size() + 1 > capacity) return AFX_ERR_CAPACITY;
    std::memcpy(out, s.c_str(), s.size() + 1);
    return AFX_OK;
}

int afx_read_depth_frame(const char* pattern, long index, uint16_t* out, long capacity, int* width, int* height) {
    char path[4096];
    int rc = afx_depth_file_name(pattern, index, path, sizeof(path));
    if (rc) return rc;
    try {
        std::vector<uint8_t> data;
        rc = read_file(path, data);
        if (rc) return rc;
        return decode_any(data.data(), data.size(), out, capacity, width, height);
    } catch (...) {
        return AFX_ERR_NO_MEMORY;
    }
}

}  // extern "C"
