// png.cu -- image ingest (host): a PNG decoder and the reference's gray
// conversion, image_to_grid (main.cpp:29-109).
//
// The reference reads PNGs through libpng with these transforms: 16-bit
// samples stripped to their high byte, palettes expanded to RGB, gray of 1,
// 2 or 4 bits expanded to 8, tRNS turned into alpha, an 0xFF filler after RGB;
// then gray = 0.299 r + 0.587 g + 0.114 b on samples / 255.0 (main.cpp:91-99).
// libpng is not available here, so this file decodes PNG itself (RFC 2083:
// chunks with CRC check, zlib stream per RFC 1950/1951 with its Adler-32 check,
// the five scanline filters, Adam7 interlacing, all colour types and bit
// depths) into 8-bit RGBA with the same transforms.  One deliberate
// difference: for gray and gray+alpha images the reference indexes its rows as
// if they held 4 bytes per pixel (they hold 2 after the filler), reading
// across pixels and past the row end; here gray is taken as r = g = b.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"

namespace pcd {
namespace png {

namespace {

// ---- DEFLATE (RFC 1951) ----------------------------------------------------
struct Bits {
    const uint8_t *p;
    size_t n, pos = 0;
    uint32_t buf = 0;
    int cnt = 0;
    bool over = false;
    int bit()
    {
        if (cnt == 0) {
            if (pos >= n) {
                over = true;
                return 0;
            }
            buf = p[pos++];
            cnt = 8;
        }
        const int b = buf & 1;
        buf >>= 1;
        cnt--;
        return b;
    }
    int bits(int k)  // LSB first
    {
        int v = 0;
        for (int i = 0; i < k; i++) v |= bit() << i;
        return v;
    }
};

// Canonical Huffman code: count of codes per length and the symbols in code order.
struct Huff {
    int count[16] = {0};
    std::vector<int> symbol;
    bool build(const int *len, int n)
    {
        std::memset(count, 0, sizeof(count));
        for (int s = 0; s < n; s++) count[len[s]]++;
        count[0] = 0;
        int left = 1;
        for (int l = 1; l < 16; l++) {
            left <<= 1;
            left -= count[l];
            if (left < 0) return false;  // over-subscribed
        }
        int offs[16];
        offs[1] = 0;
        for (int l = 1; l < 15; l++) offs[l + 1] = offs[l] + count[l];
        symbol.assign(n, 0);
        for (int s = 0; s < n; s++)
            if (len[s]) symbol[offs[len[s]]++] = s;
        return true;
    }
    // codes are read MSB first within a code, one bit at a time
    int decode(Bits &b) const
    {
        int code = 0, first = 0, index = 0;
        for (int l = 1; l < 16; l++) {
            code |= b.bit();
            const int c = count[l];
            if (code - first < c) return symbol[index + (code - first)];
            index += c;
            first += c;
            first <<= 1;
            code <<= 1;
            if (b.over) return -1;
        }
        return -1;
    }
};

const int kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31,
                          35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const int kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const int kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129,
                           193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const int kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

bool inflate_block(Bits &b, const Huff &lit, const Huff &dist, std::vector<uint8_t> &out, std::string &err)
{
    for (;;) {
        int sym = lit.decode(b);
        if (sym < 0 || b.over) { err = "bad literal/length code"; return false; }
        if (sym < 256) {
            out.push_back((uint8_t)sym);
        } else if (sym == 256) {
            return true;
        } else {
            sym -= 257;
            if (sym >= 29) { err = "bad length symbol"; return false; }
            const int len = kLenBase[sym] + b.bits(kLenExtra[sym]);
            const int ds = dist.decode(b);
            if (ds < 0 || ds >= 30) { err = "bad distance code"; return false; }
            const size_t d = (size_t)kDistBase[ds] + b.bits(kDistExtra[ds]);
            if (d > out.size()) { err = "distance before the start"; return false; }
            const size_t from = out.size() - d;
            for (int k = 0; k < len; k++) out.push_back(out[from + k]);
        }
        if (b.over) { err = "truncated deflate stream"; return false; }
    }
}

bool inflate(const uint8_t *in, size_t n, std::vector<uint8_t> &out, std::string &err)
{
    Bits b{in, n};
    int last;
    do {
        last = b.bit();
        const int type = b.bits(2);
        if (type == 0) {  // stored
            b.cnt = 0;  // to a byte boundary
            if (b.pos + 4 > n) { err = "truncated stored block"; return false; }
            const unsigned len = in[b.pos] | (in[b.pos + 1] << 8), nlen = in[b.pos + 2] | (in[b.pos + 3] << 8);
            if ((len ^ 0xFFFFu) != nlen) { err = "stored block length check"; return false; }
            b.pos += 4;
            if (b.pos + len > n) { err = "truncated stored block"; return false; }
            out.insert(out.end(), in + b.pos, in + b.pos + len);
            b.pos += len;
        } else if (type == 1) {  // fixed codes
            int l[288], d[30];
            for (int s = 0; s < 144; s++) l[s] = 8;
            for (int s = 144; s < 256; s++) l[s] = 9;
            for (int s = 256; s < 280; s++) l[s] = 7;
            for (int s = 280; s < 288; s++) l[s] = 8;
            for (int s = 0; s < 30; s++) d[s] = 5;
            Huff lit, dist;
            lit.build(l, 288);
            dist.build(d, 30);
            if (!inflate_block(b, lit, dist, out, err)) return false;
        } else if (type == 2) {  // dynamic codes
            const int nlen = b.bits(5) + 257, ndist = b.bits(5) + 1, ncode = b.bits(4) + 4;
            if (nlen > 286 || ndist > 30) { err = "bad code counts"; return false; }
            static const int order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            int cl[19] = {0};
            for (int k = 0; k < ncode; k++) cl[order[k]] = b.bits(3);
            Huff clh;
            if (!clh.build(cl, 19)) { err = "bad code-length code"; return false; }
            int lens[320] = {0};
            int k = 0;
            while (k < nlen + ndist) {
                const int sym = clh.decode(b);
                if (sym < 0 || b.over) { err = "bad code-length symbol"; return false; }
                if (sym < 16) {
                    lens[k++] = sym;
                } else {
                    int rep, val = 0;
                    if (sym == 16) {
                        if (k == 0) { err = "repeat without a length"; return false; }
                        val = lens[k - 1];
                        rep = 3 + b.bits(2);
                    } else if (sym == 17) {
                        rep = 3 + b.bits(3);
                    } else {
                        rep = 11 + b.bits(7);
                    }
                    if (k + rep > nlen + ndist) { err = "too many code lengths"; return false; }
                    while (rep--) lens[k++] = val;
                }
            }
            if (lens[256] == 0) { err = "no end-of-block code"; return false; }
            Huff lit, dist;
            if (!lit.build(lens, nlen) || !dist.build(lens + nlen, ndist)) { err = "bad dynamic code"; return false; }
            if (!inflate_block(b, lit, dist, out, err)) return false;
        } else {
            err = "bad block type";
            return false;
        }
        if (b.over) { err = "truncated deflate stream"; return false; }
    } while (!last);
    return true;
}

uint32_t adler32(const uint8_t *p, size_t n)
{
    uint32_t a = 1, c = 0;
    for (size_t i = 0; i < n; i++) {
        a = (a + p[i]) % 65521u;
        c = (c + a) % 65521u;
    }
    return (c << 16) | a;
}

uint32_t crc32(const uint8_t *p, size_t n)
{
    static uint32_t table[256];
    static bool init = false;
    if (!init) {
        for (uint32_t k = 0; k < 256; k++) {
            uint32_t c = k;
            for (int j = 0; j < 8; j++) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            table[k] = c;
        }
        init = true;
    }
    uint32_t c = 0xFFFFFFFFu;
    for (size_t i = 0; i < n; i++) c = table[(c ^ p[i]) & 0xFF] ^ (c >> 8);
    return c ^ 0xFFFFFFFFu;
}

uint32_t be32(const uint8_t *p) { return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3]; }

int paeth(int a, int b, int c)
{
    const int p = a + b - c, pa = p > a ? p - a : a - p, pb = p > b ? p - b : b - p, pc = p > c ? p - c : c - p;
    if (pa <= pb && pa <= pc) return a;
    return pb <= pc ? b : c;
}

// Reverses the scanline filters of an image of w x h pixels in place; raw
// holds h rows of 1 filter byte + rowbytes; out gets h x rowbytes.
bool unfilter(const uint8_t *raw, int w, int h, int bitspp, std::vector<uint8_t> &out, std::string &err)
{
    const size_t rowbytes = ((size_t)w * bitspp + 7) / 8;
    const int bpp = bitspp >= 8 ? bitspp / 8 : 1;
    out.assign(rowbytes * h, 0);
    for (int y = 0; y < h; y++) {
        const uint8_t ft = raw[(size_t)y * (rowbytes + 1)];
        const uint8_t *src = raw + (size_t)y * (rowbytes + 1) + 1;
        uint8_t *dst = out.data() + (size_t)y * rowbytes;
        const uint8_t *prev = y ? dst - rowbytes : nullptr;
        for (size_t i = 0; i < rowbytes; i++) {
            const int a = i >= (size_t)bpp ? dst[i - bpp] : 0, b = prev ? prev[i] : 0;
            const int c = (prev && i >= (size_t)bpp) ? prev[i - bpp] : 0;
            int v;
            switch (ft) {
            case 0: v = src[i]; break;
            case 1: v = src[i] + a; break;
            case 2: v = src[i] + b; break;
            case 3: v = src[i] + ((a + b) >> 1); break;
            case 4: v = src[i] + paeth(a, b, c); break;
            default: err = "bad filter type"; return false;
            }
            dst[i] = (uint8_t)v;
        }
    }
    return true;
}

struct Header {
    int w, h, depth, ctype, interlace;
    int channels() const { return ctype == 0 ? 1 : ctype == 2 ? 3 : ctype == 3 ? 1 : ctype == 4 ? 2 : 4; }
};

// one sample (channel c of pixel x) of an unfiltered row, at its bit depth
int sample(const uint8_t *row, int x, int c, const Header &H)
{
    const int ch = H.channels();
    if (H.depth == 8) return row[(size_t)x * ch + c];
    if (H.depth == 16) return row[((size_t)x * ch + c) * 2];  // high byte (png_set_strip_16)
    const int per = 8 / H.depth, idx = x * ch + c;
    const int byte = row[idx / per], shift = 8 - H.depth * (idx % per + 1);
    return (byte >> shift) & ((1 << H.depth) - 1);
}

}  // namespace

int decode(const uint8_t *data, size_t size, int *width, int *height, std::vector<uint8_t> *rgba, std::string &err)
{
    static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    if (size < 8 || std::memcmp(data, sig, 8) != 0) { err = "not a PNG file"; return PCD_BAD_ARG; }
    Header H{};
    bool have_hdr = false;
    std::vector<uint8_t> idat, plte, trns;
    size_t pos = 8;
    bool end = false;
    while (!end) {
        if (pos + 12 > size) { err = "truncated chunk"; return PCD_BAD_ARG; }
        const uint32_t len = be32(data + pos);
        if (len > size - pos - 12) { err = "truncated chunk"; return PCD_BAD_ARG; }
        const uint8_t *type = data + pos + 4, *body = data + pos + 8;
        if (crc32(type, 4 + (size_t)len) != be32(body + len)) { err = "chunk CRC mismatch"; return PCD_BAD_ARG; }
        if (!std::memcmp(type, "IHDR", 4)) {
            if (len != 13) { err = "bad IHDR"; return PCD_BAD_ARG; }
            H.w = (int)be32(body);
            H.h = (int)be32(body + 4);
            H.depth = body[8];
            H.ctype = body[9];
            H.interlace = body[12];
            if (body[10] != 0 || body[11] != 0 || H.interlace > 1) { err = "unsupported PNG method"; return PCD_BAD_ARG; }
            const int d = H.depth, c = H.ctype;
            const bool ok = (c == 0 && (d == 1 || d == 2 || d == 4 || d == 8 || d == 16)) ||
                            (c == 3 && (d == 1 || d == 2 || d == 4 || d == 8)) ||
                            ((c == 2 || c == 4 || c == 6) && (d == 8 || d == 16));
            if (!ok || H.w <= 0 || H.h <= 0 || H.w > (1 << 16) || H.h > (1 << 16)) {
                err = "unsupported PNG header";
                return PCD_BAD_ARG;
            }
            have_hdr = true;
        } else if (!std::memcmp(type, "PLTE", 4)) {
            plte.assign(body, body + len);
        } else if (!std::memcmp(type, "tRNS", 4)) {
            trns.assign(body, body + len);
        } else if (!std::memcmp(type, "IDAT", 4)) {
            idat.insert(idat.end(), body, body + len);
        } else if (!std::memcmp(type, "IEND", 4)) {
            end = true;
        }
        pos += 12 + (size_t)len;
    }
    if (!have_hdr || idat.size() < 6) { err = "missing IHDR or IDAT"; return PCD_BAD_ARG; }
    if (H.ctype == 3 && (plte.empty() || plte.size() % 3)) { err = "missing palette"; return PCD_BAD_ARG; }
    // zlib wrapper (RFC 1950)
    const uint8_t cmf = idat[0], flg = idat[1];
    if ((cmf & 15) != 8 || ((cmf << 8) | flg) % 31 != 0 || (flg & 32)) { err = "bad zlib header"; return PCD_BAD_ARG; }
    std::vector<uint8_t> raw;
    if (!inflate(idat.data() + 2, idat.size() - 6, raw, err)) return PCD_BAD_ARG;
    if (adler32(raw.data(), raw.size()) != be32(idat.data() + idat.size() - 4)) {
        err = "zlib Adler-32 mismatch";
        return PCD_BAD_ARG;
    }
    *width = H.w;
    *height = H.h;
    if (!rgba) return PCD_OK;
    rgba->assign((size_t)H.w * H.h * 4, 0);
    const int bitspp = H.channels() * H.depth;
    const int gmax = (1 << H.depth) - 1;
    // pixel (x, y) of an unfiltered sub-image row -> RGBA
    auto put = [&](const uint8_t *row, int x, int X, int Y) {
        uint8_t *o = rgba->data() + ((size_t)Y * H.w + X) * 4;
        int r, g, b, a = 255;
        if (H.ctype == 3) {
            const int i = sample(row, x, 0, H);
            if ((size_t)(3 * i + 2) < plte.size()) {
                r = plte[3 * i]; g = plte[3 * i + 1]; b = plte[3 * i + 2];
            } else {
                r = g = b = 0;
            }
            if ((size_t)i < trns.size()) a = trns[i];
        } else if (H.ctype == 0 || H.ctype == 4) {
            const int v = sample(row, x, 0, H);
            const int v8 = H.depth < 8 ? v * 255 / gmax : v;
            r = g = b = v8;
            if (H.ctype == 4) a = sample(row, x, 1, H);
            else if (trns.size() >= 2) {
                const int key = (trns[0] << 8) | trns[1];
                const int full = H.depth == 16 ? ((row[(size_t)x * 2] << 8) | row[(size_t)x * 2 + 1]) : v;
                if (full == key) a = 0;
            }
        } else {
            r = sample(row, x, 0, H);
            g = sample(row, x, 1, H);
            b = sample(row, x, 2, H);
            if (H.ctype == 6) a = sample(row, x, 3, H);
            else if (trns.size() >= 6) {
                const int ch = 3;
                auto full = [&](int c) {
                    return H.depth == 16 ? ((row[((size_t)x * ch + c) * 2] << 8) | row[((size_t)x * ch + c) * 2 + 1])
                                         : row[(size_t)x * ch + c];
                };
                if (full(0) == ((trns[0] << 8) | trns[1]) && full(1) == ((trns[2] << 8) | trns[3]) &&
                    full(2) == ((trns[4] << 8) | trns[5]))
                    a = 0;
            }
        }
        o[0] = (uint8_t)r; o[1] = (uint8_t)g; o[2] = (uint8_t)b; o[3] = (uint8_t)a;
    };
    if (H.interlace == 0) {
        const size_t need = ((size_t)H.w * bitspp + 7) / 8 + 1;
        if (raw.size() < need * H.h) { err = "short image data"; return PCD_BAD_ARG; }
        std::vector<uint8_t> img;
        if (!unfilter(raw.data(), H.w, H.h, bitspp, img, err)) return PCD_BAD_ARG;
        const size_t rowbytes = need - 1;
        for (int y = 0; y < H.h; y++)
            for (int x = 0; x < H.w; x++) put(img.data() + (size_t)y * rowbytes, x, x, y);
    } else {  // Adam7
        static const int x0[7] = {0, 4, 0, 2, 0, 1, 0}, y0[7] = {0, 0, 4, 0, 2, 0, 1};
        static const int dx[7] = {8, 8, 4, 4, 2, 2, 1}, dy[7] = {8, 8, 8, 4, 4, 2, 2};
        size_t off = 0;
        for (int pass = 0; pass < 7; pass++) {
            const int pw = (H.w - x0[pass] + dx[pass] - 1) / dx[pass];
            const int ph = (H.h - y0[pass] + dy[pass] - 1) / dy[pass];
            if (pw <= 0 || ph <= 0) continue;
            const size_t rb = ((size_t)pw * bitspp + 7) / 8;
            if (raw.size() < off + (rb + 1) * ph) { err = "short interlaced data"; return PCD_BAD_ARG; }
            std::vector<uint8_t> img;
            if (!unfilter(raw.data() + off, pw, ph, bitspp, img, err)) return PCD_BAD_ARG;
            for (int y = 0; y < ph; y++)
                for (int x = 0; x < pw; x++)
                    put(img.data() + (size_t)y * rb, x, x0[pass] + x * dx[pass], y0[pass] + y * dy[pass]);
            off += (rb + 1) * ph;
        }
    }
    return PCD_OK;
}

}  // namespace png
}  // namespace pcd

using namespace pcd;

extern "C" {

int pcd_png_decode(const unsigned char *data, size_t size, int *width, int *height, unsigned char *rgba)
{
    if (!data || !width || !height) return PCD_BAD_ARG;
    std::string err;
    std::vector<uint8_t> out;
    const int st = png::decode(data, size, width, height, rgba ? &out : nullptr, err);
    if (st != PCD_OK) {
        set_error("png: " + err);
        return st;
    }
    if (rgba) std::memcpy(rgba, out.data(), out.size());
    return PCD_OK;
}

int pcd_image_to_grid(const char *filename, int *width, int *height, double *gray)
{
    if (!filename || !width || !height) return PCD_BAD_ARG;
    FILE *fp = std::fopen(filename, "rb");
    if (!fp) {
        set_error(std::string("Failed to open PNG file: ") + filename);  // main.cpp:32
        return PCD_BAD_ARG;
    }
    std::vector<uint8_t> bytes;
    uint8_t buf[1 << 16];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof(buf), fp)) > 0) bytes.insert(bytes.end(), buf, buf + n);
    std::fclose(fp);
    std::string err;
    std::vector<uint8_t> rgba;
    const int st = png::decode(bytes.data(), bytes.size(), width, height, gray ? &rgba : nullptr, err);
    if (st != PCD_OK) {
        set_error("png: " + err);
        return st;
    }
    if (!gray) return PCD_OK;
    const size_t px = (size_t)*width * *height;
    for (size_t i = 0; i < px; i++) {
        const double r = rgba[4 * i] / 255.0, g = rgba[4 * i + 1] / 255.0, b = rgba[4 * i + 2] / 255.0;
        gray[i] = (0.299 * r) + (0.587 * g) + (0.114 * b);  // main.cpp:91-99
    }
    return PCD_OK;
}

}  // extern "C"
