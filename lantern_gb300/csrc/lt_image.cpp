// lt_image.cpp -- PNG decoding for image textures.
//
// The reference loads image textures with stb_image (`stbi_load(path, &w, &h,
// &n, 0)`, image_cache.cpp:23-31): 8-bit samples with the file's own channel
// count. This decoder returns the same for PNG files: grey 1, grey+alpha 2,
// RGB 3, RGBA 4 channels; palette images expand to RGB (RGBA with a tRNS
// chunk); a tRNS key on grey/RGB adds an alpha channel; 1/2/4-bit grey scales
// to 0..255; 16-bit samples keep their high byte. Interlaced files are not
// supported. The zlib stream is inflated by the decoder below (RFC 1950/1951:
// stored, fixed-Huffman and dynamic-Huffman blocks, canonical codes decoded one
// bit at a time).
#include <stdint.h>
#include <string.h>

#include <cstdio>
#include <string>
#include <vector>

#include "lt_scene.h"

namespace lt {

namespace {

struct Bits {
    const uint8_t *p;
    size_t n, pos = 0;
    uint32_t buf = 0;
    int cnt = 0;
    bool bad = false;
    int bit() {
        if (cnt == 0) {
            if (pos >= n) {
                bad = true;
                return 0;
            }
            buf = p[pos++];
            cnt = 8;
        }
        int b = (int)(buf & 1u);
        buf >>= 1;
        --cnt;
        return b;
    }
    uint32_t take(int k) {  // k bits, least significant first
        uint32_t v = 0;
        for (int i = 0; i < k; ++i) v |= (uint32_t)bit() << i;
        return v;
    }
};

// Canonical Huffman code: number of codes per length and symbols in code order.
struct Code {
    uint16_t count[16];
    uint16_t sym[320];
};

bool make_code(Code &c, const uint8_t *len, int n) {
    memset(c.count, 0, sizeof c.count);
    for (int i = 0; i < n; ++i) c.count[len[i]]++;
    c.count[0] = 0;
    int left = 1;
    for (int l = 1; l < 16; ++l) {
        left = 2 * left - c.count[l];
        if (left < 0) return false;  // over-subscribed
    }
    uint16_t off[16];
    off[1] = 0;
    for (int l = 1; l < 15; ++l) off[l + 1] = (uint16_t)(off[l] + c.count[l]);
    for (int i = 0; i < n; ++i)
        if (len[i]) c.sym[off[len[i]]++] = (uint16_t)i;
    return true;
}

int decode(Bits &b, const Code &c) {
    int code = 0, first = 0, index = 0;
    for (int l = 1; l < 16; ++l) {
        code |= b.bit();
        int cnt = c.count[l];
        if (code - first < cnt) return c.sym[index + code - first];
        index += cnt;
        first = (first + cnt) << 1;
        code <<= 1;
        if (b.bad) return -1;
    }
    return -1;
}

const uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31,
                               35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6,
                                6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

bool inflate_block(Bits &b, const Code &lit, const Code &dist, std::vector<uint8_t> &out) {
    for (;;) {
        int s = decode(b, lit);
        if (s < 0) return false;
        if (s < 256) {
            out.push_back((uint8_t)s);
        } else if (s == 256) {
            return true;
        } else {
            s -= 257;
            if (s >= 29) return false;
            size_t len = kLenBase[s] + b.take(kLenExtra[s]);
            int d = decode(b, dist);
            if (d < 0 || d >= 30) return false;
            size_t back = kDistBase[d] + b.take(kDistExtra[d]);
            if (b.bad || back > out.size()) return false;
            size_t from = out.size() - back;
            for (size_t k = 0; k < len; ++k) out.push_back(out[from + k]);
        }
    }
}

// zlib stream (RFC 1950) -> bytes. Returns false on a malformed stream.
bool inflate_zlib(const uint8_t *p, size_t n, std::vector<uint8_t> &out) {
    if (n < 2 || (p[0] & 0x0F) != 8 || ((p[0] << 8) | p[1]) % 31 != 0 || (p[1] & 0x20)) return false;
    Bits b{p + 2, n - 2};
    int last = 0;
    do {
        last = b.bit();
        int type = (int)b.take(2);
        if (type == 0) {  // stored: byte-aligned LEN, NLEN, data
            b.cnt = 0;
            if (b.pos + 4 > b.n) return false;
            uint32_t len = b.p[b.pos] | (b.p[b.pos + 1] << 8), nlen = b.p[b.pos + 2] | (b.p[b.pos + 3] << 8);
            b.pos += 4;
            if ((len ^ 0xFFFFu) != nlen || b.pos + len > b.n) return false;
            out.insert(out.end(), b.p + b.pos, b.p + b.pos + len);
            b.pos += len;
        } else if (type == 1) {  // fixed codes
            uint8_t len[320];
            for (int i = 0; i < 288; ++i) len[i] = i < 144 ? 8 : i < 256 ? 9 : i < 280 ? 7 : 8;
            Code lit, dist;
            make_code(lit, len, 288);
            for (int i = 0; i < 30; ++i) len[i] = 5;
            make_code(dist, len, 30);
            if (!inflate_block(b, lit, dist, out)) return false;
        } else if (type == 2) {  // dynamic codes
            const int nlit = (int)b.take(5) + 257, ndist = (int)b.take(5) + 1, nclen = (int)b.take(4) + 4;
            static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            if (nlit > 286 || ndist > 30) return false;
            uint8_t len[320];
            memset(len, 0, sizeof len);
            for (int i = 0; i < nclen; ++i) len[order[i]] = (uint8_t)b.take(3);
            Code clc;
            if (!make_code(clc, len, 19)) return false;
            uint8_t ll[320];
            int i = 0;
            while (i < nlit + ndist) {
                int s = decode(b, clc);
                if (s < 0) return false;
                if (s < 16) {
                    ll[i++] = (uint8_t)s;
                    continue;
                }
                int rep = 0;
                uint8_t v = 0;
                if (s == 16) {
                    if (i == 0) return false;
                    v = ll[i - 1];
                    rep = 3 + (int)b.take(2);
                } else if (s == 17) {
                    rep = 3 + (int)b.take(3);
                } else {
                    rep = 11 + (int)b.take(7);
                }
                if (i + rep > nlit + ndist) return false;
                while (rep--) ll[i++] = v;
            }
            if (ll[256] == 0) return false;
            Code lit, dist;
            if (!make_code(lit, ll, nlit) || !make_code(dist, ll + nlit, ndist)) return false;
            if (!inflate_block(b, lit, dist, out)) return false;
        } else {
            return false;
        }
        if (b.bad) return false;
    } while (!last);
    return true;
}

uint32_t be32(const uint8_t *p) { return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3]; }

int paeth(int a, int b, int c) {
    int p = a + b - c, pa = p > a ? p - a : a - p, pb = p > b ? p - b : b - p, pc = p > c ? p - c : c - p;
    if (pa <= pb && pa <= pc) return a;
    return pb <= pc ? b : c;
}

}  // namespace

lt_status decode_png(const uint8_t *file, size_t size, std::vector<uint8_t> *data, uint32_t *w_out,
                     uint32_t *h_out, uint32_t *n_out, std::string *err) {
    static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
    if (size < 8 || memcmp(file, sig, 8) != 0) { *err = "not a PNG file"; return LT_ERR_PARSE; }
    uint32_t W = 0, H = 0, depth = 0, ctype = 0, interlace = 0;
    std::vector<uint8_t> idat, plte, trns;
    bool have_ihdr = false;
    size_t pos = 8;
    while (pos + 12 <= size) {
        const uint32_t len = be32(file + pos);
        const uint8_t *tag = file + pos + 4, *body = file + pos + 8;
        if (len > size - pos - 12) { *err = "truncated PNG chunk"; return LT_ERR_PARSE; }
        if (!memcmp(tag, "IHDR", 4) && len >= 13) {
            W = be32(body);
            H = be32(body + 4);
            depth = body[8];
            ctype = body[9];
            interlace = body[12];
            have_ihdr = true;
        } else if (!memcmp(tag, "PLTE", 4)) {
            plte.assign(body, body + len);
        } else if (!memcmp(tag, "tRNS", 4)) {
            trns.assign(body, body + len);
        } else if (!memcmp(tag, "IDAT", 4)) {
            idat.insert(idat.end(), body, body + len);
        } else if (!memcmp(tag, "IEND", 4)) {
            break;
        }
        pos += 12 + len;
    }
    if (!have_ihdr || W == 0 || H == 0 || W > 65536 || H > 65536) { *err = "bad PNG header"; return LT_ERR_PARSE; }
    if (interlace) { *err = "interlaced PNG files are not supported"; return LT_ERR_UNSUPPORTED; }
    int chans = 0;
    switch (ctype) {
        case 0: chans = 1; break;
        case 2: chans = 3; break;
        case 3: chans = 1; break;
        case 4: chans = 2; break;
        case 6: chans = 4; break;
        default: *err = "bad PNG colour type"; return LT_ERR_PARSE;
    }
    const bool depth_ok = depth == 8 || depth == 16 || ((ctype == 0 || ctype == 3) && (depth == 1 || depth == 2 || depth == 4));
    if (!depth_ok || (ctype == 3 && depth == 16)) { *err = "bad PNG bit depth"; return LT_ERR_PARSE; }
    if (ctype == 3 && (plte.empty() || plte.size() % 3)) { *err = "PNG palette missing"; return LT_ERR_PARSE; }
    // deflate expands at most 1032:1 (258-byte matches in 2-bit codes), so a
    // header whose filtered image cannot come out of this much data is
    // rejected before anything of its size is allocated
    const size_t raw_bytes = (size_t)H * (((size_t)W * chans * depth + 7) / 8 + 1);
    if (raw_bytes / 1032 > idat.size() + 1) { *err = "PNG image data too short"; return LT_ERR_PARSE; }
    std::vector<uint8_t> raw;
    raw.reserve(raw_bytes);
    if (!inflate_zlib(idat.data(), idat.size(), raw)) { *err = "corrupt PNG image data"; return LT_ERR_PARSE; }
    const size_t stride = ((size_t)W * chans * depth + 7) / 8;
    const size_t bpp = ((size_t)chans * depth + 7) / 8;  // filter unit, bytes
    if (raw.size() < H * (stride + 1)) { *err = "PNG image data too short"; return LT_ERR_PARSE; }
    std::vector<uint8_t> img(H * stride), prev(stride, 0);
    for (uint32_t y = 0; y < H; ++y) {
        const uint8_t f = raw[y * (stride + 1)];
        const uint8_t *src = &raw[y * (stride + 1) + 1];
        uint8_t *dst = &img[y * stride];
        for (size_t i = 0; i < stride; ++i) {
            const int a = i >= bpp ? dst[i - bpp] : 0, b = prev[i], c = i >= bpp ? prev[i - bpp] : 0;
            int v = src[i];
            switch (f) {
                case 0: break;
                case 1: v += a; break;
                case 2: v += b; break;
                case 3: v += (a + b) >> 1; break;
                case 4: v += paeth(a, b, c); break;
                default: *err = "bad PNG filter"; return LT_ERR_PARSE;
            }
            dst[i] = (uint8_t)v;
        }
        memcpy(prev.data(), dst, stride);
    }
    // samples -> 8-bit output channels
    const bool key_alpha = !trns.empty() && (ctype == 0 || ctype == 2);
    const int out_n = ctype == 3 ? (trns.empty() ? 3 : 4) : chans + (key_alpha ? 1 : 0);
    data->assign((size_t)W * H * out_n, 0);
    auto sample = [&](const uint8_t *row, size_t k) -> uint32_t {  // k-th sample of a row, raw value
        if (depth == 8) return row[k];
        if (depth == 16) return ((uint32_t)row[2 * k] << 8) | row[2 * k + 1];
        const size_t bit = k * depth;
        return (row[bit >> 3] >> (8 - depth - (bit & 7))) & ((1u << depth) - 1u);
    };
    for (uint32_t y = 0; y < H; ++y) {
        const uint8_t *row = &img[y * stride];
        uint8_t *o = &(*data)[(size_t)y * W * out_n];
        for (uint32_t x = 0; x < W; ++x, o += out_n) {
            if (ctype == 3) {
                const uint32_t i = sample(row, x);
                if (3 * (size_t)i + 2 < plte.size()) memcpy(o, &plte[3 * (size_t)i], 3);
                if (out_n == 4) o[3] = i < trns.size() ? trns[i] : 255;
                continue;
            }
            bool keyed = key_alpha;
            for (int c = 0; c < chans; ++c) {
                const uint32_t v = sample(row, (size_t)x * chans + c);
                if (key_alpha) {
                    const size_t t = 2 * (size_t)c;
                    uint32_t key = t + 1 < trns.size() ? ((uint32_t)trns[t] << 8 | trns[t + 1]) : 0xFFFFFFFFu;
                    if (depth <= 8 && key != 0xFFFFFFFFu) key &= 255u;  // stb keeps the low byte
                    keyed = keyed && v == key;
                }
                if (depth == 16) o[c] = (uint8_t)(v >> 8);
                else if (depth == 8) o[c] = (uint8_t)v;
                else o[c] = (uint8_t)(v * (255u / ((1u << depth) - 1u)));
            }
            if (key_alpha) o[chans] = keyed ? 0 : 255;
        }
    }
    *w_out = W;
    *h_out = H;
    *n_out = (uint32_t)out_n;
    return LT_OK;
}

lt_status load_png(const std::string &path, std::vector<uint8_t> *data, uint32_t *w, uint32_t *h, uint32_t *n,
                   std::string *err) {
    FILE *f = fopen(path.c_str(), "rb");
    if (!f) { *err = path + ": cannot open"; return LT_ERR_IO; }
    std::vector<uint8_t> bytes;
    uint8_t buf[65536];
    size_t k;
    while ((k = fread(buf, 1, sizeof buf, f)) > 0) bytes.insert(bytes.end(), buf, buf + k);
    fclose(f);
    lt_status st = decode_png(bytes.data(), bytes.size(), data, w, h, n, err);
    if (st != LT_OK) *err = path + ": " + *err;
    return st;
}

}  // namespace lt
