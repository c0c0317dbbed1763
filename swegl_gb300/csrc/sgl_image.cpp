// sgl_image.cpp — host image decoders (BMP, PNG with its own inflater,
// baseline JPEG) for texture upload.  The reference reads images with its
// own BMP reader and with libpng / libjpeg (src/misc/image.cpp:20-265); the
// PNG path is lossless, so any correct decoder gives libpng's texels.
#include "sgl_image.h"

#include <algorithm>
#include <cctype>
#include <cstring>

namespace sgl {

static uint32_t rd32le(const uint8_t *p) { return p[0] | (p[1] << 8) | (p[2] << 16) | ((uint32_t)p[3] << 24); }
static uint16_t rd16le(const uint8_t *p) { return (uint16_t)(p[0] | (p[1] << 8)); }
static uint32_t rd32be(const uint8_t *p) { return ((uint32_t)p[0] << 24) | (p[1] << 16) | (p[2] << 8) | p[3]; }

static bool fail(std::string &err, const char *msg)
{
    err = msg;
    return false;
}

// ------------------------------------------------------------------- BMP --

bool decode_bmp(const uint8_t *d, size_t size, Image &out, std::string &err)
{
    if (size < 54)
        return fail(err, "BMP: file shorter than its 54-byte header");
    const int w = (int)rd32le(d + 18), h = (int)rd32le(d + 22);
    if (w <= 0 || h <= 0 || (int64_t)w * h > (1ll << 28))
        return fail(err, "BMP: width and height must be positive (bottom-up 24-bit images)");
    const size_t pad = (size_t)((w * 3) % 4); // the reference skips (width*3)%4 bytes per row
    const size_t need = 54 + (size_t)h * ((size_t)w * 3 + pad);
    if (size < need)
        return fail(err, "BMP: pixel data shorter than width x height x 3");
    out.width = w;
    out.height = h;
    out.texels.assign((size_t)w * h, 0u);
    const uint8_t *p = d + 54; // rows follow the header directly (the data offset is not used)
    for (int row = h - 1; row >= 0; row--) {
        uint32_t *dst = out.texels.data() + (size_t)row * w;
        for (int i = 0; i < w; i++, p += 3)
            dst[i] = 0xFF000000u | ((uint32_t)p[2] << 16) | ((uint32_t)p[1] << 8) | p[0];
        p += pad;
    }
    return true;
}

// --------------------------------------------------------------- inflate --
//
// RFC 1951 with canonical Huffman codes decoded a bit at a time against the
// per-length code counts; RFC 1950 framing (the Adler-32 is checked).

namespace {

struct Bits {
    const uint8_t *p;
    size_t n, pos = 0;
    uint64_t buf = 0;
    int cnt = 0;
    bool bad = false;

    uint32_t get(int k)
    {
        while (cnt < k) {
            if (pos >= n) {
                bad = true;
                return 0;
            }
            buf |= (uint64_t)p[pos++] << cnt;
            cnt += 8;
        }
        const uint32_t v = (uint32_t)(buf & ((1ull << k) - 1));
        buf >>= k;
        cnt -= k;
        return v;
    }
    void align()
    {
        buf >>= cnt & 7;
        cnt -= cnt & 7;
    }
};

struct Huff {
    uint16_t count[16];
    uint16_t symbol[320];
};

// Code counts per length and the symbols in code order; false for an
// over-subscribed set of lengths.
bool huff_build(Huff &h, const uint8_t *len, int n)
{
    std::memset(h.count, 0, sizeof h.count);
    for (int s = 0; s < n; s++)
        h.count[len[s]]++;
    h.count[0] = 0;
    int left = 1;
    for (int l = 1; l < 16; l++) {
        left <<= 1;
        left -= h.count[l];
        if (left < 0)
            return false;
    }
    uint16_t offs[16];
    offs[1] = 0;
    for (int l = 1; l < 15; l++)
        offs[l + 1] = (uint16_t)(offs[l] + h.count[l]);
    for (int s = 0; s < n; s++)
        if (len[s])
            h.symbol[offs[len[s]]++] = (uint16_t)s;
    return true;
}

int huff_decode(Bits &b, const Huff &h)
{
    int code = 0, first = 0, index = 0;
    for (int l = 1; l < 16; l++) {
        code |= (int)b.get(1);
        if (b.bad)
            return -1;
        const int c = h.count[l];
        if (code - c < first)
            return h.symbol[index + (code - first)];
        index += c;
        first += c;
        first <<= 1;
        code <<= 1;
    }
    return -1; // ran out of codes
}

// RFC 1951 section 3.2.5
const uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31,
                               35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129, 193,
                                257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

bool inflate_codes(Bits &b, std::vector<uint8_t> &out, const Huff &lit, const Huff &dist, std::string &err)
{
    for (;;) {
        int s = huff_decode(b, lit);
        if (s < 0)
            return fail(err, "inflate: bad literal/length code");
        if (s < 256) {
            out.push_back((uint8_t)s);
            continue;
        }
        if (s == 256)
            return true;
        s -= 257;
        if (s >= 29)
            return fail(err, "inflate: bad length symbol");
        const size_t len = kLenBase[s] + b.get(kLenExtra[s]);
        const int ds = huff_decode(b, dist);
        if (ds < 0 || ds >= 30)
            return fail(err, "inflate: bad distance code");
        const size_t d = kDistBase[ds] + b.get(kDistExtra[ds]);
        if (b.bad)
            return fail(err, "inflate: stream ends inside a block");
        if (d > out.size())
            return fail(err, "inflate: distance before the start of the output");
        const size_t from = out.size() - d;
        for (size_t k = 0; k < len; k++)
            out.push_back(out[from + k]);
    }
}

} // namespace

bool zlib_inflate(const uint8_t *d, size_t size, std::vector<uint8_t> &out, std::string &err)
{
    if (size < 6)
        return fail(err, "zlib: stream too short");
    if ((d[0] & 0x0F) != 8 || ((d[0] << 8) | d[1]) % 31 != 0 || (d[1] & 0x20))
        return fail(err, "zlib: bad header (deflate without a preset dictionary expected)");
    Bits b{d + 2, size - 2};
    out.clear();
    int last = 0;
    while (!last) {
        last = (int)b.get(1);
        const int type = (int)b.get(2);
        if (b.bad)
            return fail(err, "inflate: truncated block header");
        if (type == 0) {
            b.align();
            b.buf = 0;
            b.cnt = 0;
            if (b.pos + 4 > b.n)
                return fail(err, "inflate: truncated stored block");
            const uint16_t len = rd16le(b.p + b.pos), nlen = rd16le(b.p + b.pos + 2);
            if ((uint16_t)~nlen != len)
                return fail(err, "inflate: stored block length check failed");
            b.pos += 4;
            if (b.pos + len > b.n)
                return fail(err, "inflate: truncated stored block");
            out.insert(out.end(), b.p + b.pos, b.p + b.pos + len);
            b.pos += len;
        } else if (type == 1) {
            struct Fixed {
                Huff lit, dist;
                Fixed()
                {
                    uint8_t l[288];
                    int s = 0;
                    for (; s < 144; s++) l[s] = 8;
                    for (; s < 256; s++) l[s] = 9;
                    for (; s < 280; s++) l[s] = 7;
                    for (; s < 288; s++) l[s] = 8;
                    huff_build(lit, l, 288);
                    uint8_t dl[30];
                    for (int k = 0; k < 30; k++) dl[k] = 5;
                    huff_build(dist, dl, 30);
                }
            };
            static const Fixed fixed; // the fixed codes of RFC 1951 section 3.2.6
            if (!inflate_codes(b, out, fixed.lit, fixed.dist, err))
                return false;
        } else if (type == 2) {
            const int hlit = (int)b.get(5) + 257, hdist = (int)b.get(5) + 1, hclen = (int)b.get(4) + 4;
            static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19] = {0};
            for (int k = 0; k < hclen; k++)
                cl[order[k]] = (uint8_t)b.get(3);
            Huff clh;
            if (b.bad || hlit > 286 || hdist > 30 || !huff_build(clh, cl, 19))
                return fail(err, "inflate: bad dynamic block header");
            uint8_t lens[320] = {0};
            int k = 0;
            while (k < hlit + hdist) {
                const int sym = huff_decode(b, clh);
                if (sym < 0)
                    return fail(err, "inflate: bad code-length code");
                if (sym < 16) {
                    lens[k++] = (uint8_t)sym;
                    continue;
                }
                int rep = 0;
                uint8_t v = 0;
                if (sym == 16) {
                    if (k == 0)
                        return fail(err, "inflate: repeat with no previous length");
                    v = lens[k - 1];
                    rep = 3 + (int)b.get(2);
                } else if (sym == 17) {
                    rep = 3 + (int)b.get(3);
                } else {
                    rep = 11 + (int)b.get(7);
                }
                if (k + rep > hlit + hdist)
                    return fail(err, "inflate: code lengths overrun");
                while (rep--)
                    lens[k++] = v;
            }
            if (lens[256] == 0)
                return fail(err, "inflate: no end-of-block code");
            Huff lit, dist;
            if (!huff_build(lit, lens, hlit) || !huff_build(dist, lens + hlit, hdist))
                return fail(err, "inflate: over-subscribed code lengths");
            if (!inflate_codes(b, out, lit, dist, err))
                return false;
        } else {
            return fail(err, "inflate: reserved block type");
        }
    }
    // Adler-32 of the output, big-endian after the byte-aligned end
    b.align();
    size_t at = b.pos - (size_t)(b.cnt / 8);
    if (at + 4 > b.n)
        return fail(err, "zlib: missing Adler-32");
    uint32_t a = 1, s2 = 0;
    for (uint8_t c : out) {
        a = (a + c) % 65521u;
        s2 = (s2 + a) % 65521u;
    }
    if (rd32be(b.p + at) != ((s2 << 16) | a))
        return fail(err, "zlib: Adler-32 mismatch");
    return true;
}

// ------------------------------------------------------------------- PNG --

static int paeth(int a, int b, int c)
{
    const int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
    if (pa <= pb && pa <= pc)
        return a;
    return pb <= pc ? b : c;
}

// Reverse the per-row filters of one (sub)image in place; rows are 1 + rb bytes.
static bool unfilter(uint8_t *rows, int h, size_t rb, int bpp, std::string &err)
{
    uint8_t *prev = nullptr;
    for (int y = 0; y < h; y++) {
        uint8_t *r = rows + (size_t)y * (rb + 1);
        const int f = r[0];
        uint8_t *x = r + 1;
        for (size_t i = 0; i < rb; i++) {
            const int a = i >= (size_t)bpp ? x[i - bpp] : 0;
            const int b = prev ? prev[i] : 0;
            const int c = (prev && i >= (size_t)bpp) ? prev[i - bpp] : 0;
            int v;
            switch (f) {
            case 0: v = 0; break;
            case 1: v = a; break;
            case 2: v = b; break;
            case 3: v = (a + b) >> 1; break;
            case 4: v = paeth(a, b, c); break;
            default: return fail(err, "PNG: unknown row filter");
            }
            x[i] = (uint8_t)(x[i] + v);
        }
        prev = x;
    }
    return true;
}

bool decode_png(const uint8_t *d, size_t size, Image &out, std::string &err)
{
    static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    if (size < 8 || std::memcmp(d, sig, 8) != 0)
        return fail(err, "PNG: bad signature");
    uint32_t w = 0, h = 0;
    int depth = 0, ctype = -1, interlace = 0;
    std::vector<uint8_t> idat, plte, trns;
    bool have_hdr = false;
    for (size_t p = 8; p + 12 <= size;) {
        const uint32_t len = rd32be(d + p);
        const uint8_t *type = d + p + 4, *body = d + p + 8;
        if (len > size - p - 12)
            return fail(err, "PNG: chunk overruns the file");
        if (!std::memcmp(type, "IHDR", 4)) {
            if (len < 13)
                return fail(err, "PNG: short IHDR");
            w = rd32be(body);
            h = rd32be(body + 4);
            depth = body[8];
            ctype = body[9];
            interlace = body[12];
            if (body[10] != 0 || body[11] != 0)
                return fail(err, "PNG: unknown compression or filter method");
            have_hdr = true;
        } else if (!std::memcmp(type, "PLTE", 4)) {
            plte.assign(body, body + len);
        } else if (!std::memcmp(type, "tRNS", 4)) {
            trns.assign(body, body + len);
        } else if (!std::memcmp(type, "IDAT", 4)) {
            idat.insert(idat.end(), body, body + len);
        } else if (!std::memcmp(type, "IEND", 4)) {
            break;
        }
        p += 12 + (size_t)len;
    }
    if (!have_hdr || w == 0 || h == 0 || (uint64_t)w * h > (1ull << 28))
        return fail(err, "PNG: missing or bad IHDR");
    int channels;
    switch (ctype) {
    case 0: channels = 1; break;
    case 2: channels = 3; break;
    case 3: channels = 1; break;
    case 4: channels = 2; break;
    case 6: channels = 4; break;
    default: return fail(err, "PNG: unknown colour type");
    }
    const bool depth_ok = (ctype == 0 && (depth == 1 || depth == 2 || depth == 4 || depth == 8 || depth == 16)) ||
                          (ctype == 3 && (depth == 1 || depth == 2 || depth == 4 || depth == 8)) ||
                          ((ctype == 2 || ctype == 4 || ctype == 6) && (depth == 8 || depth == 16));
    if (!depth_ok)
        return fail(err, "PNG: bit depth not allowed for the colour type");
    if (ctype == 3 && (plte.empty() || plte.size() % 3))
        return fail(err, "PNG: palette image without a valid PLTE");
    if (interlace > 1)
        return fail(err, "PNG: unknown interlace method");
    std::vector<uint8_t> raw;
    if (!zlib_inflate(idat.data(), idat.size(), raw, err))
        return false;
    const int bits_px = channels * depth;
    const int bpp = std::max(1, bits_px / 8);
    out.width = (int)w;
    out.height = (int)h;
    out.texels.assign((size_t)w * h, 0u);
    // tRNS of grey / RGB images: the transparent sample value(s) at the image depth
    const bool key = !trns.empty() && (ctype == 0 || ctype == 2);
    uint16_t kg = 0, kr = 0, kgg = 0, kb = 0;
    if (key) {
        if (ctype == 0 && trns.size() >= 2)
            kg = (uint16_t)((trns[0] << 8) | trns[1]);
        if (ctype == 2 && trns.size() >= 6) {
            kr = (uint16_t)((trns[0] << 8) | trns[1]);
            kgg = (uint16_t)((trns[2] << 8) | trns[3]);
            kb = (uint16_t)((trns[4] << 8) | trns[5]);
        }
    }
    auto sample = [&](const uint8_t *row, uint32_t x, int c) -> uint32_t {
        const uint64_t bit = ((uint64_t)x * channels + c) * depth;
        if (depth == 16)
            return (uint32_t)((row[bit / 8] << 8) | row[bit / 8 + 1]);
        if (depth == 8)
            return row[bit / 8];
        const int shift = 8 - depth - (int)(bit % 8);
        return (uint32_t)((row[bit / 8] >> shift) & ((1 << depth) - 1));
    };
    auto to8 = [&](uint32_t v) -> uint32_t {
        switch (depth) {
        case 1: return v * 255u;
        case 2: return v * 85u;
        case 4: return v * 17u;
        case 16: return v >> 8;
        default: return v;
        }
    };
    // passes: Adam7 or the whole image
    static const int ax0[7] = {0, 4, 0, 2, 0, 1, 0}, ay0[7] = {0, 0, 4, 0, 2, 0, 1};
    static const int adx[7] = {8, 8, 4, 4, 2, 2, 1}, ady[7] = {8, 8, 8, 4, 4, 2, 2};
    const int n_pass = interlace ? 7 : 1;
    size_t at = 0;
    for (int pass = 0; pass < n_pass; pass++) {
        const uint32_t x0 = interlace ? ax0[pass] : 0, y0 = interlace ? ay0[pass] : 0;
        const uint32_t dx = interlace ? adx[pass] : 1, dy = interlace ? ady[pass] : 1;
        if (x0 >= w || y0 >= h)
            continue;
        const uint32_t pw = (w - x0 + dx - 1) / dx, ph = (h - y0 + dy - 1) / dy;
        const size_t rb = ((size_t)pw * bits_px + 7) / 8;
        const size_t need = (size_t)ph * (rb + 1);
        if (raw.size() - at < need)
            return fail(err, "PNG: image data shorter than the image");
        uint8_t *rows = raw.data() + at;
        if (!unfilter(rows, (int)ph, rb, bpp, err))
            return false;
        for (uint32_t py = 0; py < ph; py++) {
            const uint8_t *row = rows + (size_t)py * (rb + 1) + 1;
            uint32_t *dst = out.texels.data() + (size_t)(y0 + py * dy) * w;
            for (uint32_t px = 0; px < pw; px++) {
                uint32_t r, g, b, a = 255;
                if (ctype == 3) {
                    const uint32_t idx = sample(row, px, 0);
                    if (idx * 3 + 2 >= plte.size())
                        return fail(err, "PNG: palette index outside PLTE");
                    r = plte[idx * 3];
                    g = plte[idx * 3 + 1];
                    b = plte[idx * 3 + 2];
                    if (idx < trns.size())
                        a = trns[idx];
                } else if (ctype == 0 || ctype == 4) {
                    const uint32_t v = sample(row, px, 0);
                    r = g = b = to8(v);
                    if (ctype == 4)
                        a = to8(sample(row, px, 1));
                    else if (key && v == kg)
                        a = 0;
                } else {
                    const uint32_t vr = sample(row, px, 0), vg = sample(row, px, 1), vb = sample(row, px, 2);
                    r = to8(vr);
                    g = to8(vg);
                    b = to8(vb);
                    if (ctype == 6)
                        a = to8(sample(row, px, 3));
                    else if (key && vr == kr && vg == kgg && vb == kb)
                        a = 0;
                }
                dst[x0 + px * dx] = (a << 24) | (r << 16) | (g << 8) | b;
            }
        }
        at += need;
    }
    return true;
}

// ------------------------------------------------------------------ JPEG --
//
// Baseline, extended sequential and progressive Huffman JPEG (ITU T.81 /
// JFIF), decoded the way libjpeg's default decompression (which
// read_jpeg_file uses) does it: the accurate integer IDCT (the
// Loeffler-Ligtenberg-Moschytz flow graph in 13-bit fixed point, two passes,
// columns then rows), "fancy" triangle upsampling of subsampled chroma, and
// fixed-point YCbCr -> RGB with 16 fraction bits.  A progressive file's scans
// (spectral selection and successive approximation, T.81 Annex G) fill the
// same coefficient store that a sequential scan fills at once; the pixels
// are then made the same way.  Lossless, hierarchical and arithmetic-coded
// files are errors.

namespace {

const uint8_t kZigzag[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,
                             12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6,  7,  14, 21, 28,
                             35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51,
                             58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};

struct JHuff {
    bool present = false;
    uint8_t val[256];
    int mincode[17], maxcode[18], valptr[17];
};

void jhuff_build(JHuff &h, const uint8_t *counts, const uint8_t *vals, int nvals)
{
    std::memcpy(h.val, vals, (size_t)nvals);
    int code = 0, k = 0;
    for (int l = 1; l <= 16; l++) {
        h.valptr[l] = k;
        h.mincode[l] = code;
        code += counts[l - 1];
        k += counts[l - 1];
        h.maxcode[l] = counts[l - 1] ? code - 1 : -1;
        code <<= 1;
    }
    h.maxcode[17] = 0x7FFFFFFF;
    h.present = true;
}

struct JBits {
    const uint8_t *p, *end;
    uint32_t buf = 0;
    int cnt = 0;
    bool marker = false; // a marker was reached: further bits are zeros

    void fill()
    {
        while (cnt <= 24) {
            uint32_t byte = 0;
            if (!marker && p < end) {
                byte = *p;
                if (byte == 0xFF) {
                    if (p + 1 < end && p[1] == 0x00) {
                        p += 2;
                    } else {
                        marker = true;
                        byte = 0;
                    }
                } else {
                    p++;
                }
            }
            buf |= byte << (24 - cnt);
            cnt += 8;
        }
    }
    int bit()
    {
        if (cnt < 1)
            fill();
        const int b = (int)(buf >> 31);
        buf <<= 1;
        cnt--;
        return b;
    }
    int bits(int n)
    {
        if (n == 0)
            return 0;
        if (cnt < n)
            fill();
        const int v = (int)(buf >> (32 - n));
        buf <<= n;
        cnt -= n;
        return v;
    }
    // a restart marker: byte-align and skip it
    bool restart()
    {
        buf = 0;
        cnt = 0;
        marker = false;
        while (p + 1 < end && !(p[0] == 0xFF && p[1] >= 0xD0 && p[1] <= 0xD7))
            p++;
        if (p + 1 >= end)
            return false;
        p += 2;
        return true;
    }
};

int jdecode(JBits &b, const JHuff &h)
{
    int code = b.bit();
    int l = 1;
    while (code > h.maxcode[l]) {
        code = (code << 1) | b.bit();
        if (++l > 16)
            return -1;
    }
    return h.val[(h.valptr[l] + code - h.mincode[l]) & 0xFF];
}

int jextend(int v, int s) { return v < (1 << (s - 1)) ? v - (1 << s) + 1 : v; }

struct JComp {
    int id = 0, h = 1, v = 1, tq = 0;
    int td = 0, ta = 0, pred = 0;
    int bw = 0, bh = 0;          // blocks across and down in the coefficient store
    int dw = 0, dh = 0;          // downsampled width and height
    std::vector<int16_t> coef;   // bw * bh blocks of 64 (natural order)
    std::vector<uint8_t> plane;  // (8 bw) x (8 bh) samples after the IDCT
};

// The accurate integer inverse DCT of one block: dequantised coefficients,
// columns with 2 extra fraction bits, then rows; output level-shifted by 128
// and clamped (out-of-range values wrap mod 1024 first, as a masked table
// lookup does).  64-bit intermediates, like libjpeg's on LP64 hosts.
void idct_islow(const int16_t *in, const uint16_t *q, uint8_t *out, int stride)
{
    constexpr int CB = 13, P1 = 2;
    constexpr int64_t F0298 = 2446, F0390 = 3196, F0541 = 4433, F0765 = 6270, F0899 = 7373, F1175 = 9633,
                      F1501 = 12299, F1847 = 15137, F1961 = 16069, F2053 = 16819, F2562 = 20995, F3072 = 25172;
    auto descale = [](int64_t x, int n) { return (x + ((int64_t)1 << (n - 1))) >> n; };
    auto clamp = [](int64_t x) {
        x &= 1023; // the low bits of the descaled value, as the masked table lookup sees them
        if (x >= 512)
            x -= 1024;
        x += 128;
        return (uint8_t)(x < 0 ? 0 : (x > 255 ? 255 : x));
    };
    int64_t ws[64];
    for (int c = 0; c < 8; c++) {
        const int16_t *i = in + c;
        const uint16_t *qq = q + c;
        if (!i[8] && !i[16] && !i[24] && !i[32] && !i[40] && !i[48] && !i[56]) {
            const int64_t dc = ((int64_t)i[0] * qq[0]) * (1 << P1);
            for (int r = 0; r < 8; r++)
                ws[c + 8 * r] = dc;
            continue;
        }
        int64_t z2 = i[16] * qq[16], z3 = i[48] * qq[48];
        int64_t z1 = (z2 + z3) * F0541;
        int64_t t2 = z1 + z3 * (-F1847), t3 = z1 + z2 * F0765;
        z2 = i[0] * qq[0];
        z3 = i[32] * qq[32];
        int64_t t0 = (z2 + z3) * (1 << CB), t1 = (z2 - z3) * (1 << CB);
        const int64_t t10 = t0 + t3, t13 = t0 - t3, t11 = t1 + t2, t12 = t1 - t2;
        t0 = i[56] * qq[56];
        t1 = i[40] * qq[40];
        t2 = i[24] * qq[24];
        t3 = i[8] * qq[8];
        z1 = t0 + t3;
        z2 = t1 + t2;
        z3 = t0 + t2;
        int64_t z4 = t1 + t3;
        const int64_t z5 = (z3 + z4) * F1175;
        t0 *= F0298;
        t1 *= F2053;
        t2 *= F3072;
        t3 *= F1501;
        z1 *= -F0899;
        z2 *= -F2562;
        z3 *= -F1961;
        z4 *= -F0390;
        z3 += z5;
        z4 += z5;
        t0 += z1 + z3;
        t1 += z2 + z4;
        t2 += z2 + z3;
        t3 += z1 + z4;
        ws[c + 0] = descale(t10 + t3, CB - P1);
        ws[c + 56] = descale(t10 - t3, CB - P1);
        ws[c + 8] = descale(t11 + t2, CB - P1);
        ws[c + 48] = descale(t11 - t2, CB - P1);
        ws[c + 16] = descale(t12 + t1, CB - P1);
        ws[c + 40] = descale(t12 - t1, CB - P1);
        ws[c + 24] = descale(t13 + t0, CB - P1);
        ws[c + 32] = descale(t13 - t0, CB - P1);
    }
    for (int r = 0; r < 8; r++) {
        const int64_t *w = ws + 8 * r;
        uint8_t *o = out + (size_t)r * stride;
        if (!w[1] && !w[2] && !w[3] && !w[4] && !w[5] && !w[6] && !w[7]) {
            const uint8_t v = clamp(descale(w[0], P1 + 3));
            for (int k = 0; k < 8; k++)
                o[k] = v;
            continue;
        }
        int64_t z2 = w[2], z3 = w[6];
        int64_t z1 = (z2 + z3) * F0541;
        int64_t t2 = z1 + z3 * (-F1847), t3 = z1 + z2 * F0765;
        int64_t t0 = (w[0] + w[4]) * (1 << CB), t1 = (w[0] - w[4]) * (1 << CB);
        const int64_t t10 = t0 + t3, t13 = t0 - t3, t11 = t1 + t2, t12 = t1 - t2;
        t0 = w[7];
        t1 = w[5];
        t2 = w[3];
        t3 = w[1];
        z1 = t0 + t3;
        z2 = t1 + t2;
        z3 = t0 + t2;
        int64_t z4 = t1 + t3;
        const int64_t z5 = (z3 + z4) * F1175;
        t0 *= F0298;
        t1 *= F2053;
        t2 *= F3072;
        t3 *= F1501;
        z1 *= -F0899;
        z2 *= -F2562;
        z3 *= -F1961;
        z4 *= -F0390;
        z3 += z5;
        z4 += z5;
        t0 += z1 + z3;
        t1 += z2 + z4;
        t2 += z2 + z3;
        t3 += z1 + z4;
        constexpr int S = CB + P1 + 3;
        o[0] = clamp(descale(t10 + t3, S));
        o[7] = clamp(descale(t10 - t3, S));
        o[1] = clamp(descale(t11 + t2, S));
        o[6] = clamp(descale(t11 - t2, S));
        o[2] = clamp(descale(t12 + t1, S));
        o[5] = clamp(descale(t12 - t1, S));
        o[3] = clamp(descale(t13 + t0, S));
        o[4] = clamp(descale(t13 - t0, S));
    }
}

// One component plane upsampled to hmax/h x vmax/v: triangle ("fancy")
// filters for 2x1, 2x2 and 1x2 (edge samples repeated), replication
// otherwise.  Output rows of width 2*dw (or dw*hx) for dh*vx rows.
bool upsample(const JComp &c, int hx, int vx, std::vector<uint8_t> &out, int &ow, int &oh)
{
    const int w = c.dw, h = c.dh, st = 8 * c.bw;
    ow = w * hx;
    oh = h * vx;
    out.assign((size_t)ow * oh, 0);
    auto in = [&](int y, int x) -> int { return c.plane[(size_t)y * st + x]; };
    if (hx == 1 && vx == 1) {
        for (int y = 0; y < h; y++)
            std::memcpy(&out[(size_t)y * ow], &c.plane[(size_t)y * st], (size_t)w);
        return true;
    }
    const bool fancy = w > 2;
    if (hx == 2 && vx == 1 && fancy) {
        for (int y = 0; y < h; y++) {
            uint8_t *o = &out[(size_t)y * ow];
            int v = in(y, 0);
            o[0] = (uint8_t)v;
            o[1] = (uint8_t)((v * 3 + in(y, 1) + 2) >> 2);
            for (int x = 1; x < w - 1; x++) {
                v = in(y, x) * 3;
                o[2 * x] = (uint8_t)((v + in(y, x - 1) + 1) >> 2);
                o[2 * x + 1] = (uint8_t)((v + in(y, x + 1) + 2) >> 2);
            }
            v = in(y, w - 1);
            o[2 * w - 2] = (uint8_t)((v * 3 + in(y, w - 2) + 1) >> 2);
            o[2 * w - 1] = (uint8_t)v;
        }
        return true;
    }
    if (hx == 2 && vx == 2 && fancy) {
        for (int y = 0; y < h; y++)
            for (int half = 0; half < 2; half++) {
                const int y1 = half == 0 ? (y > 0 ? y - 1 : 0) : (y < h - 1 ? y + 1 : h - 1);
                uint8_t *o = &out[(size_t)(2 * y + half) * ow];
                auto col = [&](int x) { return in(y, x) * 3 + in(y1, x); };
                int this_s = col(0), next_s = col(1), last_s;
                o[0] = (uint8_t)((this_s * 4 + 8) >> 4);
                o[1] = (uint8_t)((this_s * 3 + next_s + 7) >> 4);
                last_s = this_s;
                this_s = next_s;
                for (int x = 1; x < w - 1; x++) {
                    next_s = col(x + 1);
                    o[2 * x] = (uint8_t)((this_s * 3 + last_s + 8) >> 4);
                    o[2 * x + 1] = (uint8_t)((this_s * 3 + next_s + 7) >> 4);
                    last_s = this_s;
                    this_s = next_s;
                }
                o[2 * w - 2] = (uint8_t)((this_s * 3 + last_s + 8) >> 4);
                o[2 * w - 1] = (uint8_t)((this_s * 4 + 7) >> 4);
            }
        return true;
    }
    if (hx == 1 && vx == 2) {
        for (int y = 0; y < h; y++)
            for (int half = 0; half < 2; half++) {
                const int y1 = half == 0 ? (y > 0 ? y - 1 : 0) : (y < h - 1 ? y + 1 : h - 1);
                const int bias = half == 0 ? 1 : 2;
                uint8_t *o = &out[(size_t)(2 * y + half) * ow];
                for (int x = 0; x < w; x++)
                    o[x] = (uint8_t)((in(y, x) * 3 + in(y1, x) + bias) >> 2);
            }
        return true;
    }
    for (int y = 0; y < oh; y++)
        for (int x = 0; x < ow; x++)
            out[(size_t)y * ow + x] = (uint8_t)in(y / vx, x / hx);
    return true;
}

} // namespace

bool decode_jpeg(const uint8_t *d, size_t size, Image &out, std::string &err)
{
    if (size < 4 || d[0] != 0xFF || d[1] != 0xD8)
        return fail(err, "JPEG: missing SOI marker");
    uint16_t qt[4][64] = {{0}};
    bool have_qt[4] = {false, false, false, false};
    JHuff dc[4], ac[4];
    std::vector<JComp> comps;
    int width = 0, height = 0, hmax = 1, vmax = 1, restart = 0;
    bool frame = false, adobe = false, jfif = false, scanned = false, progressive = false;
    int adobe_transform = -1;
    size_t p = 2;
    while (p + 4 <= size) {
        if (d[p] != 0xFF) {
            p++;
            continue;
        }
        const int m = d[p + 1];
        if (m == 0xFF || m == 0x01 || (m >= 0xD0 && m <= 0xD7)) {
            p++;
            continue;
        }
        if (m == 0xD9)
            break; // EOI
        const size_t len = (size_t)((d[p + 2] << 8) | d[p + 3]);
        const uint8_t *b = d + p + 4;
        if (len < 2 || p + 2 + len > size)
            return fail(err, "JPEG: segment overruns the file");
        const size_t n = len - 2;
        if (m == 0xDB) { // DQT
            for (size_t k = 0; k < n;) {
                const int pq = b[k] >> 4, tq = b[k] & 15;
                if (tq > 3 || k + 1 + 64 * (pq + 1) > n)
                    return fail(err, "JPEG: bad DQT");
                for (int i = 0; i < 64; i++)
                    qt[tq][kZigzag[i]] = pq ? (uint16_t)((b[k + 1 + 2 * i] << 8) | b[k + 2 + 2 * i]) : b[k + 1 + i];
                have_qt[tq] = true;
                k += 1 + 64 * (pq + 1);
            }
        } else if (m == 0xC4) { // DHT
            for (size_t k = 0; k < n;) {
                if (k + 17 > n)
                    return fail(err, "JPEG: bad DHT");
                const int tc = b[k] >> 4, th = b[k] & 15;
                int total = 0;
                for (int i = 0; i < 16; i++)
                    total += b[k + 1 + i];
                if (tc > 1 || th > 3 || total > 256 || k + 17 + total > n)
                    return fail(err, "JPEG: bad DHT");
                jhuff_build(tc ? ac[th] : dc[th], b + k + 1, b + k + 17, total);
                k += 17 + (size_t)total;
            }
        } else if (m == 0xC0 || m == 0xC1 || m == 0xC2) { // SOF0 / SOF1 / SOF2: sequential or progressive, Huffman
            if (frame)
                return fail(err, "JPEG: second frame header");
            progressive = m == 0xC2;
            if (n < 6 || b[0] != 8)
                return fail(err, "JPEG: only 8-bit samples are decoded");
            height = (b[1] << 8) | b[2];
            width = (b[3] << 8) | b[4];
            const int nc = b[5];
            if (width <= 0 || height <= 0 || (nc != 1 && nc != 3) || n < 6 + 3 * (size_t)nc ||
                (int64_t)width * height > (1ll << 28))
                return fail(err, "JPEG: unsupported frame (1 or 3 components, known size expected)");
            comps.resize((size_t)nc);
            for (int c = 0; c < nc; c++) {
                comps[c].id = b[6 + 3 * c];
                comps[c].h = b[7 + 3 * c] >> 4;
                comps[c].v = b[7 + 3 * c] & 15;
                comps[c].tq = b[8 + 3 * c] & 3;
                if (comps[c].h < 1 || comps[c].h > 4 || comps[c].v < 1 || comps[c].v > 4)
                    return fail(err, "JPEG: bad sampling factors");
                hmax = std::max(hmax, comps[c].h);
                vmax = std::max(vmax, comps[c].v);
            }
            const int mcux = (width + 8 * hmax - 1) / (8 * hmax), mcuy = (height + 8 * vmax - 1) / (8 * vmax);
            for (JComp &c : comps) {
                if (hmax % c.h || vmax % c.v)
                    return fail(err, "JPEG: non-integral sampling ratios");
                c.bw = mcux * c.h;
                c.bh = mcuy * c.v;
                c.dw = (width * c.h + hmax - 1) / hmax;
                c.dh = (height * c.v + vmax - 1) / vmax;
                c.coef.assign((size_t)c.bw * c.bh * 64, 0);
            }
            frame = true;
        } else if (m >= 0xC3 && m <= 0xCF && m != 0xC4 && m != 0xC8 && m != 0xCC) {
            return fail(err, "JPEG: lossless, hierarchical or arithmetic-coded files are not decoded");
        } else if (m == 0xDD) { // DRI
            if (n < 2)
                return fail(err, "JPEG: bad DRI");
            restart = (b[0] << 8) | b[1];
        } else if (m == 0xE0 && n >= 5 && !std::memcmp(b, "JFIF", 4)) {
            jfif = true;
        } else if (m == 0xEE && n >= 12 && !std::memcmp(b, "Adobe", 5)) {
            adobe = true;
            adobe_transform = b[11];
        } else if (m == 0xDA) { // SOS
            if (!frame)
                return fail(err, "JPEG: scan before the frame header");
            const int ns = b[0];
            if (ns < 1 || ns > 4 || n < 1 + 2 * (size_t)ns + 3)
                return fail(err, "JPEG: bad scan header");
            // spectral selection and successive approximation (sequential: 0, 63, 0, 0)
            const int ss = b[1 + 2 * ns], se = b[2 + 2 * ns], ah = b[3 + 2 * ns] >> 4, al = b[3 + 2 * ns] & 15;
            if (progressive) {
                // a DC scan has Ss = Se = 0; an AC scan holds one component and a band within 1..63
                const bool ok = ss == 0 ? se == 0 : (ns == 1 && ss <= se && se <= 63);
                if (!ok || al > 13 || ah > 13 || (ah && ah != al + 1))
                    return fail(err, "JPEG: bad progressive scan parameters");
            } else if (ss != 0 || se != 63 || ah != 0 || al != 0) {
                return fail(err, "JPEG: bad scan parameters for a sequential frame");
            }
            std::vector<JComp *> sc;
            for (int k = 0; k < ns; k++) {
                const int cid = b[1 + 2 * k];
                JComp *c = nullptr;
                for (JComp &cc : comps)
                    if (cc.id == cid)
                        c = &cc;
                if (!c)
                    return fail(err, "JPEG: scan names an unknown component");
                c->td = b[2 + 2 * k] >> 4;
                c->ta = b[2 + 2 * k] & 15;
                // the Huffman tables a scan codes with: DC for a first DC scan, AC
                // for an AC scan, both for a sequential one (a DC refinement scan
                // sends raw bits only)
                const bool need_dc = !progressive || (ss == 0 && ah == 0), need_ac = !progressive || ss > 0;
                if (c->td > 3 || c->ta > 3 || (need_dc && !dc[c->td].present) || (need_ac && !ac[c->ta].present) ||
                    !have_qt[c->tq])
                    return fail(err, "JPEG: scan uses a missing table");
                c->pred = 0;
                sc.push_back(c);
            }
            JBits bits{d + p + 2 + len, d + size};
            auto block = [&](JComp &c, int bx, int by) {
                int16_t *co = &c.coef[((size_t)by * c.bw + bx) * 64];
                const int t = jdecode(bits, dc[c.td]);
                if (t < 0 || t > 11)
                    return false;
                c.pred += t ? jextend(bits.bits(t), t) : 0;
                co[0] = (int16_t)c.pred;
                for (int k = 1; k < 64;) {
                    const int rs = jdecode(bits, ac[c.ta]);
                    if (rs < 0)
                        return false;
                    const int r = rs >> 4, s2 = rs & 15;
                    if (s2) {
                        k += r;
                        if (k > 63)
                            return false;
                        co[kZigzag[k]] = (int16_t)jextend(bits.bits(s2), s2);
                        k++;
                    } else if (r == 15) {
                        k += 16;
                    } else {
                        break;
                    }
                }
                return true;
            };
            // progressive scans (T.81 G.1.2): the end-of-band run carries over
            // from block to block within a scan
            int eobrun = 0;
            const int p1 = 1 << al, m1 = -(1 << al);
            auto refine = [&](int16_t &coefv) { // a correction bit for a coefficient already nonzero
                if (bits.bit() && (coefv & p1) == 0)
                    coefv = (int16_t)(coefv + (coefv >= 0 ? p1 : m1));
            };
            auto pblock = [&](JComp &c, int bx, int by) {
                int16_t *co = &c.coef[((size_t)by * c.bw + bx) * 64];
                if (ss == 0) {
                    if (ah == 0) { // DC, first pass: the difference of the point-transformed values
                        const int t = jdecode(bits, dc[c.td]);
                        if (t < 0 || t > 11)
                            return false;
                        c.pred += t ? jextend(bits.bits(t), t) : 0;
                        co[0] = (int16_t)(c.pred * (1 << al));
                    } else if (bits.bit()) { // DC, refinement: one more bit
                        co[0] = (int16_t)(co[0] | p1);
                    }
                    return true;
                }
                if (ah == 0) { // AC, first pass over the band
                    if (eobrun > 0) {
                        eobrun--;
                        return true;
                    }
                    for (int k = ss; k <= se;) {
                        const int rs = jdecode(bits, ac[c.ta]);
                        if (rs < 0)
                            return false;
                        const int r = rs >> 4, s2 = rs & 15;
                        if (s2) {
                            k += r;
                            if (k > se)
                                return false;
                            co[kZigzag[k]] = (int16_t)(jextend(bits.bits(s2), s2) * (1 << al));
                            k++;
                        } else if (r == 15) {
                            k += 16;
                        } else { // an end-of-band run of 2^r + r more bits blocks, this one included
                            eobrun = (1 << r) - 1;
                            if (r)
                                eobrun += bits.bits(r);
                            break;
                        }
                    }
                    return true;
                }
                // AC, refinement: newly nonzero coefficients (magnitude 1 at bit
                // al) and a correction bit for every coefficient of the band that
                // was already nonzero, sent where the decoder passes over it
                int k = ss;
                if (eobrun == 0) {
                    for (; k <= se; k++) {
                        const int rs = jdecode(bits, ac[c.ta]);
                        if (rs < 0)
                            return false;
                        int r = rs >> 4;
                        const int s2 = rs & 15;
                        int val = 0;
                        if (s2) {
                            if (s2 != 1)
                                return false;
                            val = bits.bit() ? p1 : m1;
                        } else if (r != 15) { // end of band here and in the run's next blocks
                            eobrun = 1 << r;
                            if (r)
                                eobrun += bits.bits(r);
                            break;
                        }
                        // skip r zero coefficients (refining the nonzero ones on the way),
                        // then place the new one; a zero run of 16 places nothing
                        for (; k <= se; k++) {
                            int16_t &cv = co[kZigzag[k]];
                            if (cv != 0) {
                                refine(cv);
                            } else {
                                if (r == 0)
                                    break;
                                r--;
                            }
                        }
                        if (val) {
                            if (k > se)
                                return false;
                            co[kZigzag[k]] = (int16_t)val;
                        }
                    }
                }
                if (eobrun > 0) { // the rest of the band: correction bits only
                    for (; k <= se; k++) {
                        int16_t &cv = co[kZigzag[k]];
                        if (cv != 0)
                            refine(cv);
                    }
                    eobrun--;
                }
                return true;
            };
            auto unit = [&](JComp &c, int bx, int by) { return progressive ? pblock(c, bx, by) : block(c, bx, by); };
            int units_x, units_y;
            if (ns == 1) {
                units_x = (sc[0]->dw + 7) / 8;
                units_y = (sc[0]->dh + 7) / 8;
            } else {
                units_x = (width + 8 * hmax - 1) / (8 * hmax);
                units_y = (height + 8 * vmax - 1) / (8 * vmax);
            }
            int todo = restart;
            for (int my = 0; my < units_y; my++)
                for (int mx = 0; mx < units_x; mx++) {
                    if (restart && todo == 0) {
                        if (!bits.restart())
                            return fail(err, "JPEG: missing restart marker");
                        for (JComp *c : sc)
                            c->pred = 0;
                        eobrun = 0;
                        todo = restart;
                    }
                    if (ns == 1) {
                        if (!unit(*sc[0], mx, my))
                            return fail(err, "JPEG: corrupt entropy-coded data");
                    } else {
                        for (JComp *c : sc)
                            for (int v = 0; v < c->v; v++)
                                for (int h = 0; h < c->h; h++)
                                    if (!unit(*c, mx * c->h + h, my * c->v + v))
                                        return fail(err, "JPEG: corrupt entropy-coded data");
                    }
                    todo--;
                }
            scanned = true;
            // continue after the entropy-coded data: the next marker
            p = (size_t)(bits.p - d);
            while (p + 1 < size && !(d[p] == 0xFF && d[p + 1] != 0 && !(d[p + 1] >= 0xD0 && d[p + 1] <= 0xD7)))
                p++;
            continue;
        }
        p += 2 + len;
    }
    if (!frame || !scanned)
        return fail(err, "JPEG: no frame or no scan");
    for (JComp &c : comps) {
        c.plane.assign((size_t)c.bw * 8 * c.bh * 8, 0);
        for (int by = 0; by < c.bh; by++)
            for (int bx = 0; bx < c.bw; bx++)
                idct_islow(&c.coef[((size_t)by * c.bw + bx) * 64], qt[c.tq],
                           &c.plane[(size_t)by * 8 * (8 * c.bw) + (size_t)bx * 8], 8 * c.bw);
    }
    std::vector<std::vector<uint8_t>> full(comps.size());
    std::vector<int> fw(comps.size());
    for (size_t k = 0; k < comps.size(); k++) {
        int ow, oh;
        upsample(comps[k], hmax / comps[k].h, vmax / comps[k].v, full[k], ow, oh);
        if (ow < width || oh < height)
            return fail(err, "JPEG: component smaller than the image");
        fw[k] = ow;
    }
    out.width = width;
    out.height = height;
    out.texels.assign((size_t)width * height, 0u);
    if (comps.size() == 1) {
        // grey to grey RGB (the reference would read a one-channel buffer as RGB)
        for (int y = 0; y < height; y++)
            for (int x = 0; x < width; x++) {
                const uint32_t g = full[0][(size_t)y * fw[0] + x];
                out.texels[(size_t)y * width + x] = 0xFF000000u | (g << 16) | (g << 8) | g;
            }
        return true;
    }
    // colour space as libjpeg guesses it: a JFIF marker means YCbCr, else an
    // Adobe marker's transform flag, else component ids 'R', 'G', 'B'
    const bool rgb = !jfif && (adobe ? adobe_transform == 0
                                     : (comps[0].id == 'R' && comps[1].id == 'G' && comps[2].id == 'B'));
    // YCbCr -> RGB with 16 fraction bits (JFIF coefficients 1.402, 0.34414, 0.71414, 1.772)
    auto fix = [](double x) { return (int32_t)(x * 65536.0 + 0.5); };
    int32_t cr_r[256], cb_b[256], cr_g[256], cb_g[256];
    for (int i = 0; i < 256; i++) {
        const int32_t x = i - 128;
        cr_r[i] = (fix(1.40200) * x + (1 << 15)) >> 16;
        cb_b[i] = (fix(1.77200) * x + (1 << 15)) >> 16;
        cr_g[i] = -fix(0.71414) * x;
        cb_g[i] = -fix(0.34414) * x + (1 << 15);
    }
    auto lim = [](int32_t v) { return (uint32_t)(v < 0 ? 0 : (v > 255 ? 255 : v)); };
    for (int y = 0; y < height; y++)
        for (int x = 0; x < width; x++) {
            const int c0 = full[0][(size_t)y * fw[0] + x], c1 = full[1][(size_t)y * fw[1] + x],
                      c2 = full[2][(size_t)y * fw[2] + x];
            uint32_t r, g, b;
            if (rgb) {
                r = (uint32_t)c0;
                g = (uint32_t)c1;
                b = (uint32_t)c2;
            } else {
                r = lim(c0 + cr_r[c2]);
                g = lim(c0 + ((cb_g[c1] + cr_g[c2]) >> 16));
                b = lim(c0 + cb_b[c1]);
            }
            out.texels[(size_t)y * width + x] = 0xFF000000u | (r << 16) | (g << 8) | b;
        }
    return true;
}

// ---------------------------------------------------------- by file name --

bool decode_by_name(const std::string &name, const uint8_t *data, size_t size, Image &out, std::string &err)
{
    std::string n = name;
    for (char &c : n)
        c = (char)std::tolower((unsigned char)c);
    auto ends = [&](const char *s) {
        const size_t k = std::strlen(s);
        return n.size() >= k && n.compare(n.size() - k, k, s) == 0;
    };
    if (ends("png"))
        return decode_png(data, size, out, err);
    if (ends("jpg") || ends("jpeg"))
        return decode_jpeg(data, size, out, err);
    if (ends("bmp"))
        return decode_bmp(data, size, out, err);
    return fail(err, "image: unknown file extension (png, jpg, jpeg or bmp expected)");
}

} // namespace sgl
