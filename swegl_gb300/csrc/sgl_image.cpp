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

bool decode_jpeg(const uint8_t *, size_t, Image &, std::string &err)
{
    return fail(err, "JPEG: decoding is not built (PNG and BMP textures are)");
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
