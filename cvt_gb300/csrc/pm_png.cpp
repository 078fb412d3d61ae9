/*
 * pm_png.cpp — PNG files for real stereo pairs and for saved maps (host
 * code): the reference's loader and saver (plugins/iloader/PNG/PNGLoader.cpp,
 * plugins/isaver/PNG/PNGSaver.cpp, both over libpng) without libpng or zlib.
 * The zlib stream (RFC 1950) and DEFLATE (RFC 1951) are implemented here;
 * the file layout, filters and Adam7 interlacing follow the PNG
 * specification (ISO/IEC 15948).
 *
 * Loading applies the transformations the reference asks libpng for:
 *   gray 1/2/4/8 bit      -> GRAY_UINT8 (low depths scaled to 0..255)
 *   gray 16 bit           -> GRAY_UINT16
 *   gray + alpha 8/16     -> GRAYALPHA_UINT8/16
 *   RGB 8, palette        -> RGBA_UINT8, alpha 255 (png_set_add_alpha 0xff)
 *   RGB 16                -> RGBA_UINT16, alpha 255 (the 16-bit filler is
 *                            the same 0x00ff value)
 *   RGBA 8/16             -> RGBA_UINT8/16
 * A tRNS chunk becomes the alpha channel (png_set_expand): palette alpha
 * from its entries; gray and RGB alpha 0 where the sample equals the tRNS
 * colour, else the maximum.  16-bit samples are stored in host order
 * (png_set_swap on little-endian hosts).
 *
 * Saving writes GRAY, GRAYALPHA, RGBA and BGRA images of 8 or 16 bits (BGRA
 * in RGBA order, as png_set_bgr); float images are first converted to their
 * 8-bit equivalent as the reference's Image::convert does
 * (cvt/gfx/IConvert.cpp, cvt/util/SIMD.cpp): colour channels through the
 * 8192-step float-to-sRGB table (F_TO_SRGB_U8, the sRGB transfer function
 * rounded), alpha and gray-alpha channels linearly, (uint8)(clamp(v * 255 +
 * 0.5)) (Conv_f_to_u8, Conv_XXXAf_to_XXXAu8).  Rows are filtered with the
 * per-row minimum-sum-of-absolute-differences choice and compressed with
 * fixed-Huffman DEFLATE blocks over a greedy LZ77 match search.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <new>
#include <string>
#include <vector>

#include "cvtpm.h"

void pm_set_free_error(const std::string& m);   /* pm_image.cu */

namespace {

cvtpm_status fail(cvtpm_status s, const std::string& m) {
    pm_set_free_error(m);
    return s;
}

/* a host allocation sized by the file or image failed: no exception leaves
 * the C ABI */
cvtpm_status pm_out_of_memory() { return fail(CVTPM_ERR_ALLOC, "host memory exhausted"); }

bool host_little_endian() {
    const uint16_t v = 1;
    unsigned char b;
    memcpy(&b, &v, 1);
    return b == 1;
}

uint32_t be32(const uint8_t* p) { return (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | p[3]; }

void put_be32(std::vector<uint8_t>* o, uint32_t v) {
    o->push_back((uint8_t)(v >> 24));
    o->push_back((uint8_t)(v >> 16));
    o->push_back((uint8_t)(v >> 8));
    o->push_back((uint8_t)v);
}

/* ---------------------------------------------------------- checks -- */
/* CRC-32 of the chunks: reflected polynomial 0xEDB88320, initial and final
 * value all ones.  Eight bytes per step ("slicing by 8"): t[k][b] is the CRC
 * contribution of byte b followed by k zero bytes, so the eight table
 * lookups of one step are independent. */
struct CrcTable {
    uint32_t t[8][256];
    CrcTable() {
        for (uint32_t n = 0; n < 256; ++n) {
            uint32_t c = n;
            for (int k = 0; k < 8; ++k) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            t[0][n] = c;
        }
        for (int k = 1; k < 8; ++k)
            for (uint32_t n = 0; n < 256; ++n) t[k][n] = (t[k - 1][n] >> 8) ^ t[0][t[k - 1][n] & 0xff];
    }
};

uint32_t crc32(const uint8_t* p, size_t n, uint32_t crc = 0) {
    static const CrcTable tab;
    crc = ~crc;
    size_t i = 0;
    for (; i + 8 <= n; i += 8) {
        const uint32_t lo = crc ^ ((uint32_t)p[i] | (uint32_t)p[i + 1] << 8 | (uint32_t)p[i + 2] << 16 | (uint32_t)p[i + 3] << 24);
        crc = tab.t[7][lo & 0xff] ^ tab.t[6][(lo >> 8) & 0xff] ^ tab.t[5][(lo >> 16) & 0xff] ^ tab.t[4][lo >> 24] ^
              tab.t[3][p[i + 4]] ^ tab.t[2][p[i + 5]] ^ tab.t[1][p[i + 6]] ^ tab.t[0][p[i + 7]];
    }
    for (; i < n; ++i) crc = tab.t[0][(crc ^ p[i]) & 0xff] ^ (crc >> 8);
    return ~crc;
}

/* Adler-32 of the zlib stream (RFC 1950 section 8.2) */
uint32_t adler32(const uint8_t* p, size_t n) {
    uint32_t a = 1, b = 0;
    while (n) {
        const size_t k = n < 5552 ? n : 5552;   /* no overflow before the reduction */
        for (size_t i = 0; i < k; ++i) {
            a += p[i];
            b += a;
        }
        a %= 65521;
        b %= 65521;
        p += k;
        n -= k;
    }
    return b << 16 | a;
}

/* --------------------------------------------------------- inflate -- */
/* RFC 1951 section 3.2.5: base values and extra bits of the length codes
 * 257..285 and the distance codes 0..29. */
const uint16_t LEN_BASE[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t LEN_EXTRA[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t DIST_BASE[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t DIST_EXTRA[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
/* order of the code-length code lengths in a dynamic block header */
const uint8_t CLEN_ORDER[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

/* LSB-first bit reader over the deflate data */
struct BitReader {
    const uint8_t* p;
    size_t n, pos = 0;
    uint64_t buf = 0;
    int cnt = 0;
    bool overrun = false;   /* a read went past the end */

    BitReader(const uint8_t* data, size_t size) : p(data), n(size) {}
    void fill() {
        while (cnt <= 56) {
            uint64_t b = 0;
            if (pos < n) b = p[pos];
            else if (pos >= n + 8) break;   /* zero padding past the end, counted */
            ++pos;
            buf |= b << cnt;
            cnt += 8;
        }
    }
    uint32_t peek(int k) {
        if (cnt < k) fill();
        return (uint32_t)(buf & ((1ull << k) - 1));
    }
    void drop(int k) {
        buf >>= k;
        cnt -= k;
        if (pos > n && (size_t)cnt < (pos - n) * 8) overrun = true;
    }
    uint32_t bits(int k) {
        if (!k) return 0;
        const uint32_t v = peek(k);
        drop(k);
        return v;
    }
    void align() { drop(cnt & 7); }
};

/* Canonical Huffman code (RFC 1951 section 3.2.2), decoded through a table
 * of the next FAST_BITS bits and, for longer codes, code by code. */
const int FAST_BITS = 10;
struct Huffman {
    uint16_t count[16];        /* codes of each length */
    uint16_t symbol[320];      /* symbols ordered by (length, value) */
    uint16_t fast[1 << FAST_BITS];   /* (symbol << 4) | length, 0 = longer code */
    bool ok = false;
};

uint32_t reverse_bits(uint32_t v, int k) {
    uint32_t r = 0;
    for (int i = 0; i < k; ++i) r = r << 1 | ((v >> i) & 1);
    return r;
}

/* Builds the code from n code lengths; false if the lengths over-subscribe
 * the code space.  Incomplete codes are allowed (a single distance code). */
bool build(Huffman* h, const uint8_t* len, int n) {
    memset(h->count, 0, sizeof h->count);
    for (int i = 0; i < n; ++i) h->count[len[i]]++;
    h->count[0] = 0;
    int left = 1;
    for (int l = 1; l < 16; ++l) {
        left <<= 1;
        left -= h->count[l];
        if (left < 0) return false;
    }
    uint16_t offs[16];
    offs[1] = 0;
    for (int l = 1; l < 15; ++l) offs[l + 1] = offs[l] + h->count[l];
    for (int i = 0; i < n; ++i)
        if (len[i]) h->symbol[offs[len[i]]++] = (uint16_t)i;
    memset(h->fast, 0, sizeof h->fast);
    uint32_t code = 0;
    int idx = 0;
    for (int l = 1; l < 16; ++l) {
        for (int k = 0; k < h->count[l]; ++k, ++code, ++idx) {
            if (l > FAST_BITS) continue;
            const uint32_t r = reverse_bits(code, l);
            for (uint32_t f = r; f < (1u << FAST_BITS); f += 1u << l)
                h->fast[f] = (uint16_t)(h->symbol[idx] << 4 | l);
        }
        code <<= 1;
    }
    h->ok = true;
    return true;
}

/* the next symbol, or -1 for a code not in the table */
int decode(BitReader* br, const Huffman* h) {
    const uint32_t look = br->peek(FAST_BITS);
    const uint16_t e = h->fast[look];
    if (e) {
        br->drop(e & 15);
        return e >> 4;
    }
    /* canonical decoding, one bit at a time: codes of length l occupy
     * [first, first + count[l]) */
    int code = 0, first = 0, index = 0;
    for (int l = 1; l < 16; ++l) {
        code |= (int)br->bits(1);
        const int c = h->count[l];
        if (code - first < c) return h->symbol[index + code - first];
        index += c;
        first = (first + c) << 1;
        code <<= 1;
    }
    return -1;
}

/* the fixed codes of RFC 1951 section 3.2.6, built once (function-local
 * statics are initialised once, thread-safely) */
const Huffman& fixed_lit() {
    static const Huffman h = [] {
        Huffman t;
        uint8_t l[288];
        for (int i = 0; i < 288; ++i) l[i] = i < 144 ? 8 : (i < 256 ? 9 : (i < 280 ? 7 : 8));
        build(&t, l, 288);
        return t;
    }();
    return h;
}

const Huffman& fixed_dist() {
    static const Huffman h = [] {
        Huffman t;
        uint8_t l[30];
        for (int i = 0; i < 30; ++i) l[i] = 5;
        build(&t, l, 30);
        return t;
    }();
    return h;
}

/* Inflates a zlib stream into out, which must come to exactly `expect`
 * bytes.  Returns an error message or an empty string. */
std::string inflate_zlib(const uint8_t* z, size_t n, size_t expect, std::vector<uint8_t>* out) {
    if (n < 6) return "zlib stream too short";
    const int cmf = z[0], flg = z[1];
    if ((cmf & 15) != 8 || (cmf >> 4) > 7 || (cmf * 256 + flg) % 31) return "bad zlib header";
    if (flg & 32) return "zlib preset dictionary not allowed";
    out->assign(expect, 0);
    uint8_t* const o = out->data();
    size_t on = 0;                                   /* bytes written */
    BitReader br(z + 2, n - 2);
    for (int last = 0; !last;) {
        last = (int)br.bits(1);
        const int type = (int)br.bits(2);
        if (type == 0) {
            br.align();
            const uint32_t len = br.bits(16), nlen = br.bits(16);
            if ((len ^ 0xffff) != nlen) return "stored block length check failed";
            for (uint32_t i = 0; i < len; ++i) {
                if (on >= expect) return "more image data than the header describes";
                o[on++] = (uint8_t)br.bits(8);
            }
            if (br.overrun) return "truncated stored block";
            continue;
        }
        Huffman dl, dd;
        const Huffman *lit = &fixed_lit(), *dist = &fixed_dist();
        if (type == 2) {
            const int nlen = (int)br.bits(5) + 257, ndist = (int)br.bits(5) + 1, ncode = (int)br.bits(4) + 4;
            if (nlen > 286 || ndist > 30) return "bad dynamic block counts";
            uint8_t cl[19] = {0};
            for (int i = 0; i < ncode; ++i) cl[CLEN_ORDER[i]] = (uint8_t)br.bits(3);
            Huffman ch;
            if (!build(&ch, cl, 19)) return "bad code-length code";
            uint8_t lens[320] = {0};
            for (int i = 0; i < nlen + ndist;) {
                const int s = decode(&br, &ch);
                if (s < 0 || br.overrun) return "bad code length";
                if (s < 16) {
                    lens[i++] = (uint8_t)s;
                    continue;
                }
                int rep, val = 0;
                if (s == 16) {
                    if (!i) return "repeat with no previous length";
                    val = lens[i - 1];
                    rep = 3 + (int)br.bits(2);
                } else if (s == 17) {
                    rep = 3 + (int)br.bits(3);
                } else {
                    rep = 11 + (int)br.bits(7);
                }
                if (i + rep > nlen + ndist) return "code lengths overrun";
                while (rep--) lens[i++] = (uint8_t)val;
            }
            if (!lens[256]) return "no end-of-block code";
            if (!build(&dl, lens, nlen) || !build(&dd, lens + nlen, ndist)) return "bad literal or distance code";
            lit = &dl;
            dist = &dd;
        } else if (type != 1) {
            return "bad block type";
        }
        for (;;) {
            const int s = decode(&br, lit);
            if (s < 0 || br.overrun) return "bad literal/length code";
            if (s < 256) {
                if (on >= expect) return "more image data than the header describes";
                o[on++] = (uint8_t)s;
                continue;
            }
            if (s == 256) break;
            if (s > 285) return "bad length symbol";
            const size_t len = LEN_BASE[s - 257] + br.bits(LEN_EXTRA[s - 257]);
            const int ds = decode(&br, dist);
            if (ds < 0 || ds > 29) return "bad distance symbol";
            const size_t d = DIST_BASE[ds] + br.bits(DIST_EXTRA[ds]);
            if (br.overrun) return "truncated compressed data";
            if (d > on) return "distance before the start of the data";
            if (on + len > expect) return "more image data than the header describes";
            const uint8_t* from = o + on - d;
            for (size_t i = 0; i < len; ++i) o[on + i] = from[i];   /* byte by byte: overlapping copies repeat */
            on += len;
        }
        if (br.overrun) return "truncated compressed data";
    }
    if (on != expect) return "less image data than the header describes";
    br.align();
    uint8_t a[4];
    for (int i = 0; i < 4; ++i) a[i] = (uint8_t)br.bits(8);
    if (br.overrun) return "missing Adler-32";
    if (be32(a) != adler32(out->data(), out->size())) return "Adler-32 mismatch";
    return "";
}

/* --------------------------------------------------------- deflate -- */
struct BitWriter {
    std::vector<uint8_t>* o;
    uint64_t buf = 0;
    int cnt = 0;
    void put(uint32_t v, int k) {
        buf |= (uint64_t)v << cnt;
        cnt += k;
        while (cnt >= 8) {
            o->push_back((uint8_t)buf);
            buf >>= 8;
            cnt -= 8;
        }
    }
    void flush() {
        if (cnt) o->push_back((uint8_t)buf);
        buf = 0;
        cnt = 0;
    }
};

/* a fixed-Huffman code, MSB-first, written into the LSB-first stream */
void put_code(BitWriter* bw, uint32_t code, int len) { bw->put(reverse_bits(code, len), len); }

void put_lit(BitWriter* bw, int s) {
    if (s < 144) put_code(bw, 0x30 + s, 8);
    else if (s < 256) put_code(bw, 0x190 + (s - 144), 9);
    else if (s < 280) put_code(bw, s - 256, 7);
    else put_code(bw, 0xc0 + (s - 280), 8);
}

void put_match(BitWriter* bw, int len, int dist) {
    int c = 28;
    while (LEN_BASE[c] > len) --c;
    put_lit(bw, 257 + c);
    bw->put((uint32_t)(len - LEN_BASE[c]), LEN_EXTRA[c]);
    int d = 29;
    while (DIST_BASE[d] > dist) --d;
    put_code(bw, (uint32_t)d, 5);
    bw->put((uint32_t)(dist - DIST_BASE[d]), DIST_EXTRA[d]);
}

/* zlib stream of one fixed-Huffman block: greedy LZ77 over a 32 KB window,
 * 3-byte hash chains searched up to 32 deep. */
void deflate_zlib(const uint8_t* p, size_t n, std::vector<uint8_t>* o) {
    o->push_back(0x78);
    o->push_back(0x01);
    BitWriter bw{o};
    bw.put(1, 1);   /* final */
    bw.put(1, 2);   /* fixed Huffman */
    const int HBITS = 15, WIN = 32768, DEPTH = 32;
    std::vector<int32_t> head(1 << HBITS, -1), prev(n ? n : 1, -1);
    auto hash = [&](size_t i) { return ((uint32_t)p[i] << 10 ^ (uint32_t)p[i + 1] << 5 ^ p[i + 2]) & ((1u << HBITS) - 1); };
    size_t i = 0;
    while (i < n) {
        int best = 0, bdist = 0;
        if (i + 3 <= n) {
            const uint32_t h = hash(i);
            int32_t c = head[h];
            const size_t maxlen = n - i < 258 ? n - i : 258;
            for (int k = 0; k < DEPTH && c >= 0 && i - (size_t)c <= (size_t)WIN; ++k, c = prev[c]) {
                size_t l = 0;
                while (l < maxlen && p[c + l] == p[i + l]) ++l;
                if ((int)l > best) {
                    best = (int)l;
                    bdist = (int)(i - c);
                    if (l == maxlen) break;
                }
            }
        }
        const size_t adv = best >= 3 ? (size_t)best : 1;
        if (best >= 3) put_match(&bw, best, bdist);
        else put_lit(&bw, p[i]);
        for (size_t k = 0; k < adv; ++k, ++i) {
            if (i + 3 <= n) {
                const uint32_t h = hash(i);
                prev[i] = head[h];
                head[h] = (int32_t)i;
            }
        }
    }
    put_lit(&bw, 256);
    bw.flush();
    put_be32(o, adler32(p, n));
}

/* ---------------------------------------------------------- filters -- */
uint8_t paeth(int a, int b, int c) {
    const int p = a + b - c, pa = p > a ? p - a : a - p, pb = p > b ? p - b : b - p, pc = p > c ? p - c : c - p;
    return (uint8_t)(pa <= pb && pa <= pc ? a : (pb <= pc ? b : c));
}

/* undoes the filter of one row in place; prior is the previous unfiltered
 * row of the pass (zeros for its first) */
bool unfilter(int type, uint8_t* row, const uint8_t* prior, size_t len, size_t bpp) {
    switch (type) {
    case 0: return true;
    case 1: for (size_t i = bpp; i < len; ++i) row[i] = (uint8_t)(row[i] + row[i - bpp]); return true;
    case 2: for (size_t i = 0; i < len; ++i) row[i] = (uint8_t)(row[i] + prior[i]); return true;
    case 3:
        for (size_t i = 0; i < len; ++i) row[i] = (uint8_t)(row[i] + (((i >= bpp ? row[i - bpp] : 0) + prior[i]) >> 1));
        return true;
    case 4:
        for (size_t i = 0; i < len; ++i)
            row[i] = (uint8_t)(row[i] + paeth(i >= bpp ? row[i - bpp] : 0, prior[i], i >= bpp ? prior[i - bpp] : 0));
        return true;
    default: return false;
    }
}

/* ------------------------------------------------------------- read -- */
struct Png {
    uint32_t w = 0, h = 0;
    int depth = 0, ctype = 0, interlace = 0;
    std::vector<uint8_t> plte, trns, idat;
    bool has_trns = false;
    int channels() const { return ctype == 0 ? 1 : ctype == 2 ? 3 : ctype == 3 ? 1 : ctype == 4 ? 2 : 4; }
    int out_format() const {
        const bool d16 = depth == 16;
        switch (ctype) {
        case 0: return has_trns ? (d16 ? CVTPM_IFORMAT_GRAYALPHA_UINT16 : CVTPM_IFORMAT_GRAYALPHA_UINT8)
                                : (d16 ? CVTPM_IFORMAT_GRAY_UINT16 : CVTPM_IFORMAT_GRAY_UINT8);
        case 4: return d16 ? CVTPM_IFORMAT_GRAYALPHA_UINT16 : CVTPM_IFORMAT_GRAYALPHA_UINT8;
        case 3: return CVTPM_IFORMAT_RGBA_UINT8;
        default: return d16 ? CVTPM_IFORMAT_RGBA_UINT16 : CVTPM_IFORMAT_RGBA_UINT8;
        }
    }
};

const int ADAM7[7][4] = {{0, 0, 8, 8}, {4, 0, 8, 8}, {0, 4, 4, 8}, {2, 0, 4, 4}, {0, 2, 2, 4}, {1, 0, 2, 2}, {0, 1, 1, 2}};

/* The chunks of a PNG file; with header_only, parsing stops at the first
 * IDAT (IHDR, PLTE and tRNS precede it), which is all the format needs. */
std::string parse(const std::vector<uint8_t>& d, Png* png, bool header_only = false) {
    static const uint8_t SIG[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    if (d.size() < 8 || memcmp(d.data(), SIG, 8)) return "Invalid PNG image header";
    size_t pos = 8;
    bool ihdr = false, iend = false;
    while (!iend) {
        if (d.size() - pos < 12) return "truncated chunk";
        const uint32_t len = be32(&d[pos]);
        if (len > 0x7fffffffu || d.size() - pos - 12 < len) return "truncated chunk";
        const uint8_t* type = &d[pos + 4];
        const uint8_t* data = type + 4;
        const std::string t((const char*)type, 4);
        if (!ihdr && t != "IHDR") return "IHDR is not the first chunk";
        if (header_only && t == "IDAT") break;
        if (crc32(type, 4 + (size_t)len) != be32(data + len)) return "chunk CRC mismatch";
        if (t == "IHDR") {
            if (ihdr || len != 13) return "bad IHDR";
            png->w = be32(data);
            png->h = be32(data + 4);
            png->depth = data[8];
            png->ctype = data[9];
            if (data[10] || data[11] || data[12] > 1) return "unknown compression, filter or interlace method";
            png->interlace = data[12];
            const int dp = png->depth, ct = png->ctype;
            const bool ok = (ct == 0 && (dp == 1 || dp == 2 || dp == 4 || dp == 8 || dp == 16)) ||
                            (ct == 3 && (dp == 1 || dp == 2 || dp == 4 || dp == 8)) ||
                            ((ct == 2 || ct == 4 || ct == 6) && (dp == 8 || dp == 16));
            if (!ok) return "Unsupported PNG format";
            if (!png->w || !png->h || png->w > (1u << 24) || png->h > (1u << 24) ||
                (uint64_t)png->w * png->h > (1ull << 30))
                return "bad image size";
            ihdr = true;
        } else if (t == "PLTE") {
            if (len % 3 || len == 0 || len > 768) return "bad PLTE";
            png->plte.assign(data, data + len);
        } else if (t == "tRNS") {
            png->trns.assign(data, data + len);
            png->has_trns = true;
        } else if (t == "IDAT") {
            png->idat.insert(png->idat.end(), data, data + len);
        } else if (t == "IEND") {
            iend = true;
        } else if (!(type[0] & 0x20)) {
            return "unknown critical chunk " + t;
        }
        pos += 12 + (size_t)len;
    }
    if (png->ctype == 3) {
        if (png->plte.empty()) return "palette image without PLTE";
        if (png->has_trns && png->trns.size() > png->plte.size() / 3) return "bad tRNS";
    }
    if (png->has_trns && ((png->ctype == 0 && png->trns.size() != 2) || (png->ctype == 2 && png->trns.size() != 6) ||
                          png->ctype == 4 || png->ctype == 6))
        return "bad tRNS";
    return "";
}

/* the filtered stream's size for the image (all passes) */
size_t stream_size(const Png& p) {
    const size_t bits = (size_t)p.depth * p.channels();
    size_t total = 0;
    for (int k = 0; k < (p.interlace ? 7 : 1); ++k) {
        const int* a = ADAM7[k];
        const size_t pw = p.interlace ? (p.w + a[2] - 1 - a[0]) / a[2] : p.w;
        const size_t ph = p.interlace ? (p.h + a[3] - 1 - a[1]) / a[3] : p.h;
        if (p.w <= (uint32_t)(p.interlace ? a[0] : 0) || p.h <= (uint32_t)(p.interlace ? a[1] : 0)) continue;
        total += ph * (1 + (pw * bits + 7) / 8);
    }
    return total;
}

uint32_t sample(const uint8_t* row, size_t x, int depth, int ch, int nch) {
    if (depth == 8) return row[x * nch + ch];
    if (depth == 16) return (uint32_t)row[(x * nch + ch) * 2] << 8 | row[(x * nch + ch) * 2 + 1];
    const size_t bit = x * depth;   /* low depths: one channel, MSB first */
    return (row[bit >> 3] >> (8 - depth - (bit & 7))) & ((1u << depth) - 1);
}

/* writes pixel (x, y) of the output image from the unfiltered row */
void emit(const Png& p, const uint8_t* row, size_t sx, uint8_t* out, size_t stride, size_t x, size_t y, bool le) {
    const int nch = p.channels(), dp = p.depth;
    uint32_t v[4];
    int n;
    const uint32_t maxv = dp == 16 ? 65535u : 255u;
    if (p.ctype == 3) {
        const uint32_t idx = sample(row, sx, dp, 0, 1);
        const bool in = idx * 3 + 2 < p.plte.size();
        for (int c = 0; c < 3; ++c) v[c] = in ? p.plte[idx * 3 + c] : 0;   /* out-of-range index: black */
        v[3] = p.has_trns && idx < p.trns.size() ? p.trns[idx] : 255;
        n = 4;
    } else if (p.ctype == 0) {
        uint32_t g = sample(row, sx, dp, 0, 1);
        const uint32_t raw = g;
        if (dp < 8) g = g * (255u / ((1u << dp) - 1));   /* 1, 2, 4 bits: 255, 85, 17 per step */
        v[0] = g;
        n = 1;
        if (p.has_trns) {
            const uint32_t key = ((uint32_t)p.trns[0] << 8 | p.trns[1]) & (dp == 16 ? 0xffffu : (1u << dp) - 1);
            v[1] = raw == key ? 0 : maxv;
            n = 2;
        }
    } else if (p.ctype == 4) {
        v[0] = sample(row, sx, dp, 0, 2);
        v[1] = sample(row, sx, dp, 1, 2);
        n = 2;
    } else {
        for (int c = 0; c < nch; ++c) v[c] = sample(row, sx, dp, c, nch);
        if (nch == 3) {
            if (p.has_trns) {
                bool eq = true;
                for (int c = 0; c < 3; ++c) eq = eq && v[c] == ((uint32_t)p.trns[2 * c] << 8 | p.trns[2 * c + 1]);
                v[3] = eq ? 0 : maxv;
            } else {
                v[3] = 255;   /* png_set_add_alpha(0xff): 255 at 8 and at 16 bits */
            }
        }
        n = 4;
    }
    uint8_t* o = out + y * stride;
    if (dp == 16) {
        for (int c = 0; c < n; ++c) {
            const uint16_t s = (uint16_t)v[c];
            uint8_t* q = o + (x * n + c) * 2;
            q[le ? 0 : 1] = (uint8_t)s;
            q[le ? 1 : 0] = (uint8_t)(s >> 8);
        }
    } else {
        for (int c = 0; c < n; ++c) o[x * n + c] = (uint8_t)v[c];
    }
}

/* one unfiltered row of a pass into the output: 8-bit gray, gray + alpha,
 * RGB and RGBA without tRNS by plain byte loops, the rest through emit */
void emit_row(const Png& p, const uint8_t* row, size_t pw, uint8_t* out, size_t stride, size_t x0, size_t dx,
              size_t y, bool le) {
    uint8_t* o = out + y * stride;
    if (p.depth == 8 && !p.has_trns && p.ctype != 3) {
        switch (p.ctype) {
        case 0:
            for (size_t i = 0; i < pw; ++i) o[x0 + i * dx] = row[i];
            return;
        case 4:
            for (size_t i = 0; i < pw; ++i) {
                uint8_t* q = o + (x0 + i * dx) * 2;
                q[0] = row[2 * i];
                q[1] = row[2 * i + 1];
            }
            return;
        case 2:
            for (size_t i = 0; i < pw; ++i) {
                uint8_t* q = o + (x0 + i * dx) * 4;
                q[0] = row[3 * i];
                q[1] = row[3 * i + 1];
                q[2] = row[3 * i + 2];
                q[3] = 255;
            }
            return;
        default:
            if (dx == 1) {
                memcpy(o + x0 * 4, row, pw * 4);
                return;
            }
            for (size_t i = 0; i < pw; ++i) memcpy(o + (x0 + i * dx) * 4, row + 4 * i, 4);
            return;
        }
    }
    for (size_t i = 0; i < pw; ++i) emit(p, row, i, out, stride, x0 + i * dx, y, le);
}

std::string decode_pixels(const Png& p, uint8_t* out, size_t stride) {
    /* DEFLATE expands at most 1032:1 (258-byte matches in ~2-bit codes):
     * refuse a header that the compressed data cannot fill before
     * allocating for it */
    const size_t need = stream_size(p);
    if (need / 1032 > p.idat.size() + 64) return "less image data than the header describes";
    std::vector<uint8_t> raw;
    const std::string e = inflate_zlib(p.idat.data(), p.idat.size(), need, &raw);
    if (!e.empty()) return e;
    const size_t bits = (size_t)p.depth * p.channels(), bpp = bits >= 8 ? bits / 8 : 1;
    const bool le = host_little_endian();
    size_t pos = 0;
    for (int k = 0; k < (p.interlace ? 7 : 1); ++k) {
        const int x0 = p.interlace ? ADAM7[k][0] : 0, y0 = p.interlace ? ADAM7[k][1] : 0;
        const int dx = p.interlace ? ADAM7[k][2] : 1, dy = p.interlace ? ADAM7[k][3] : 1;
        if (p.w <= (uint32_t)x0 || p.h <= (uint32_t)y0) continue;
        const size_t pw = (p.w - x0 + dx - 1) / dx, ph = (p.h - y0 + dy - 1) / dy;
        const size_t len = (pw * bits + 7) / 8;
        std::vector<uint8_t> prior(len, 0);
        for (size_t r = 0; r < ph; ++r) {
            uint8_t* row = raw.data() + pos + 1;
            if (!unfilter(raw[pos], row, prior.data(), len, bpp)) return "bad filter type";
            emit_row(p, row, pw, out, stride, x0, dx, y0 + r * dy, le);
            memcpy(prior.data(), row, len);
            pos += 1 + len;
        }
    }
    return "";
}

bool read_file(const char* path, std::vector<uint8_t>* out) {
    FILE* f = fopen(path, "rb");
    if (!f) return false;
    out->clear();
    uint8_t buf[1 << 16];
    size_t n;
    while ((n = fread(buf, 1, sizeof buf, f)) > 0) out->insert(out->end(), buf, buf + n);
    const bool ok = !ferror(f);
    fclose(f);
    return ok;
}

/* ------------------------------------------------------------ write -- */
/* F_TO_SRGB_U8: the float scaled by 8192 and truncated indexes a table of
 * round(255 * sRGB(i / 8192)); below 0 gives 0, from 8192 on 255; NaN 0. */
struct SrgbTable {
    uint8_t t[8192];
    SrgbTable() {
        for (int i = 0; i < 8192; ++i) {
            const double l = i / 8192.0;
            const double s = l <= 0.0031308 ? 12.92 * l : 1.055 * pow(l, 1.0 / 2.4) - 0.055;
            t[i] = (uint8_t)floor(s * 255.0 + 0.5);
        }
    }
};

uint8_t f_to_srgb_u8(float v) {
    static const SrgbTable table;   /* built once, thread-safely */
    const float t = v * 8192.0f;
    if (!(t > -1.0f)) return 0;   /* NaN and negatives truncating below 0 */
    if (t >= 8192.0f) return 255;
    return table.t[(int)t];
}

/* Conv_f_to_u8 and the alpha of Conv_XXXAf_to_XXXAu8: (uint8)(clamp(v * 255
 * + 0.5, 0, 255)) and (uint8)(clamp(v, 0, 1) * 255 + 0.5); NaN 0 */
uint8_t f_to_u8_linear(float v) {
    const float t = v * 255.0f + 0.5f;
    if (!(t > 0.0f)) return 0;
    return t >= 255.0f ? 255 : (uint8_t)t;
}

uint8_t alpha_to_u8(float a) {
    if (!(a > 0.0f)) return 0;   /* clamp(a, 0, 1) = 0 gives (uint8)0.5 = 0; NaN as 0 */
    if (a > 1.0f) a = 1.0f;
    return (uint8_t)(a * 255.0f + 0.5f);
}

}  // namespace

extern "C" {

uint8_t cvtpm_float_to_srgb_u8(float v) { return f_to_srgb_u8(v); }

static cvtpm_status cvtpm_png_read_impl(const char* path, cvtpm_image* img) {
    if (!path || !img) return fail(CVTPM_ERR_INVALID_ARGUMENT, "png read: path or descriptor is NULL");
    std::vector<uint8_t> d;
    if (!read_file(path, &d)) return fail(CVTPM_ERR_IO, std::string("Cannot open PNG file: ") + path);
    Png p;
    std::string e = parse(d, &p, !img->data);
    if (!e.empty()) return fail(e == "Unsupported PNG format" ? CVTPM_ERR_NOT_SUPPORTED : CVTPM_ERR_IO, "png read: " + e);
    const int fmt = p.out_format();
    const size_t bpp = cvtpm_iformat_bpp(fmt), row = (size_t)p.w * bpp;
    if (!img->data) {
        img->format = fmt;
        img->width = (int)p.w;
        img->height = (int)p.h;
        img->stride = row;
        return CVTPM_OK;
    }
    if (img->format != fmt || img->width != (int)p.w || img->height != (int)p.h || img->stride < row)
        return fail(CVTPM_ERR_INVALID_ARGUMENT, "png read: descriptor does not match the file");
    e = decode_pixels(p, (uint8_t*)img->data, img->stride);
    if (!e.empty()) return fail(CVTPM_ERR_IO, "png read: " + e);
    return CVTPM_OK;
}

cvtpm_status cvtpm_png_read(const char* path, cvtpm_image* img) {
    try {
        return cvtpm_png_read_impl(path, img);
    } catch (const std::bad_alloc&) {
        return pm_out_of_memory();
    }
}

static cvtpm_status cvtpm_png_write_impl(const char* path, const cvtpm_image* img) {
    if (!path || !img || !img->data) return fail(CVTPM_ERR_INVALID_ARGUMENT, "png write: NULL argument");
    const int f = img->format;
    const int W = img->width, H = img->height;
    if (W < 1 || H < 1 || W > (1 << 24) || H > (1 << 24)) return fail(CVTPM_ERR_SIZE, "png write: bad image size");
    int ctype, nch, depth;
    switch (f) {
    case CVTPM_IFORMAT_GRAY_UINT8: case CVTPM_IFORMAT_GRAY_FLOAT: ctype = 0; nch = 1; depth = 8; break;
    case CVTPM_IFORMAT_GRAY_UINT16: ctype = 0; nch = 1; depth = 16; break;
    case CVTPM_IFORMAT_GRAYALPHA_UINT8: case CVTPM_IFORMAT_GRAYALPHA_FLOAT: ctype = 4; nch = 2; depth = 8; break;
    case CVTPM_IFORMAT_GRAYALPHA_UINT16: ctype = 4; nch = 2; depth = 16; break;
    case CVTPM_IFORMAT_RGBA_UINT8: case CVTPM_IFORMAT_RGBA_FLOAT:
    case CVTPM_IFORMAT_BGRA_UINT8: case CVTPM_IFORMAT_BGRA_FLOAT: ctype = 6; nch = 4; depth = 8; break;
    case CVTPM_IFORMAT_RGBA_UINT16: case CVTPM_IFORMAT_BGRA_UINT16: ctype = 6; nch = 4; depth = 16; break;
    default: return fail(CVTPM_ERR_NOT_SUPPORTED, "png write: Input channel format not supported for writing");
    }
    const size_t in_bpp = cvtpm_iformat_bpp(f);
    if (img->stride < (size_t)W * in_bpp) return fail(CVTPM_ERR_INVALID_ARGUMENT, "png write: stride below a row");
    const bool bgr = f == CVTPM_IFORMAT_BGRA_UINT8 || f == CVTPM_IFORMAT_BGRA_UINT16 || f == CVTPM_IFORMAT_BGRA_FLOAT;
    const bool isf = f == CVTPM_IFORMAT_GRAY_FLOAT || f == CVTPM_IFORMAT_GRAYALPHA_FLOAT ||
                     f == CVTPM_IFORMAT_RGBA_FLOAT || f == CVTPM_IFORMAT_BGRA_FLOAT;
    const size_t bpp = (size_t)nch * depth / 8, len = (size_t)W * bpp;
    /* rows in PNG byte order, channels in RGBA order */
    std::vector<uint8_t> rows((size_t)H * len);
    for (int y = 0; y < H; ++y) {
        const uint8_t* s = (const uint8_t*)img->data + (size_t)y * img->stride;
        uint8_t* o = rows.data() + (size_t)y * len;
        for (int x = 0; x < W; ++x)
            for (int c = 0; c < nch; ++c) {
                const int sc = bgr && c < 3 ? 2 - c : c;   /* png_set_bgr */
                if (isf) {
                    float v;
                    memcpy(&v, s + ((size_t)x * nch + sc) * 4, 4);
                    uint8_t q;
                    if (f == CVTPM_IFORMAT_GRAYALPHA_FLOAT) q = f_to_u8_linear(v);
                    else if (nch == 4 && c == 3) q = alpha_to_u8(v);
                    else q = f_to_srgb_u8(v);
                    o[(size_t)x * nch + c] = q;
                } else if (depth == 16) {
                    uint16_t v;
                    memcpy(&v, s + ((size_t)x * nch + sc) * 2, 2);
                    o[((size_t)x * nch + c) * 2] = (uint8_t)(v >> 8);
                    o[((size_t)x * nch + c) * 2 + 1] = (uint8_t)v;
                } else {
                    o[(size_t)x * nch + c] = s[(size_t)x * nch + sc];
                }
            }
    }
    /* filters: per row the type of the smallest sum of |signed bytes| */
    std::vector<uint8_t> filt((size_t)H * (len + 1)), cand(len), prior(len, 0);
    for (int y = 0; y < H; ++y) {
        const uint8_t* r = rows.data() + (size_t)y * len;
        uint64_t best = ~0ull;
        for (int t = 0; t < 5; ++t) {
            for (size_t i = 0; i < len; ++i) {
                const int a = i >= bpp ? r[i - bpp] : 0, b = prior[i], c = i >= bpp ? prior[i - bpp] : 0;
                const int pred = t == 0 ? 0 : t == 1 ? a : t == 2 ? b : t == 3 ? (a + b) >> 1 : paeth(a, b, c);
                cand[i] = (uint8_t)(r[i] - pred);
            }
            uint64_t sum = 0;
            for (size_t i = 0; i < len; ++i) sum += cand[i] < 128 ? cand[i] : 256 - cand[i];
            if (sum < best) {
                best = sum;
                filt[(size_t)y * (len + 1)] = (uint8_t)t;
                memcpy(&filt[(size_t)y * (len + 1) + 1], cand.data(), len);
            }
        }
        memcpy(prior.data(), r, len);
    }
    std::vector<uint8_t> z;
    deflate_zlib(filt.data(), filt.size(), &z);
    std::vector<uint8_t> out = {137, 80, 78, 71, 13, 10, 26, 10};
    auto chunk = [&](const char* type, const uint8_t* data, size_t n) {
        put_be32(&out, (uint32_t)n);
        const size_t at = out.size();
        out.insert(out.end(), type, type + 4);
        out.insert(out.end(), data, data + n);
        put_be32(&out, crc32(&out[at], 4 + n));
    };
    std::vector<uint8_t> ihdr;
    put_be32(&ihdr, (uint32_t)W);
    put_be32(&ihdr, (uint32_t)H);
    ihdr.push_back((uint8_t)depth);
    ihdr.push_back((uint8_t)ctype);
    ihdr.push_back(0);
    ihdr.push_back(0);
    ihdr.push_back(0);
    chunk("IHDR", ihdr.data(), ihdr.size());
    for (size_t at = 0; at < z.size(); at += 1 << 20) chunk("IDAT", z.data() + at, z.size() - at < (1u << 20) ? z.size() - at : 1u << 20);
    chunk("IEND", nullptr, 0);
    FILE* fp = fopen(path, "wb");
    if (!fp) return fail(CVTPM_ERR_IO, std::string("png write: Could not create file ") + path);
    const bool ok = fwrite(out.data(), 1, out.size(), fp) == out.size();
    if (fclose(fp) != 0 || !ok) return fail(CVTPM_ERR_IO, std::string("png write: cannot write ") + path);
    return CVTPM_OK;
}

cvtpm_status cvtpm_png_write(const char* path, const cvtpm_image* img) {
    try {
        return cvtpm_png_write_impl(path, img);
    } catch (const std::bad_alloc&) {
        return pm_out_of_memory();
    }
}

}  // extern "C"
