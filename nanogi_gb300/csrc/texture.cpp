// Texture decoding for TexR (see texture.hpp). The decoders follow the published formats:
// PNG (ISO/IEC 15948), zlib (RFC 1950) and deflate (RFC 1951), Windows BMP, netpbm PPM,
// Radiance RGBE and PFM.
#include "texture.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <fstream>
#include <iterator>

#include "image_io.hpp"

namespace ngi {

namespace {

[[noreturn]] void Bad(const std::string& path, const std::string& what) {
    throw ImageError(3, "Failed to load an image " + path + ": " + what);
}
[[noreturn]] void Unsupported(const std::string& path, const std::string& what) {
    throw ImageError(7, "Unsupported format: " + path + " (" + what + ")");
}

std::vector<uint8_t> ReadFile(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw ImageError(2, "Failed to load an image " + path);
    return std::vector<uint8_t>(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
}

uint32_t BE32(const uint8_t* p) { return (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | p[3]; }
uint32_t LE32(const uint8_t* p) { return (uint32_t)p[3] << 24 | (uint32_t)p[2] << 16 | (uint32_t)p[1] << 8 | p[0]; }
uint16_t LE16(const uint8_t* p) { return (uint16_t)(p[1] << 8 | p[0]); }

// ---- deflate ---------------------------------------------------------------------------------
struct Bits {
    const uint8_t* p;
    size_t n, pos = 0;
    uint32_t buf = 0;
    int cnt = 0;
    uint32_t get(int k) {
        while (cnt < k) {
            if (pos >= n) throw ImageError(3, "deflate stream ends early");
            buf |= (uint32_t)p[pos++] << cnt;
            cnt += 8;
        }
        const uint32_t v = buf & ((1u << k) - 1u);
        buf >>= k;
        cnt -= k;
        return v;
    }
    void align() {  // fewer than 8 bits are buffered: they belong to the current byte
        buf = 0;
        cnt = 0;
    }
};

// Canonical Huffman code: number of codes of each length, symbols ordered by (length, value).
struct Huffman {
    uint16_t count[16];
    uint16_t symbol[320];
    void build(const uint8_t* lengths, int n) {
        std::memset(count, 0, sizeof(count));
        for (int i = 0; i < n; i++) count[lengths[i]]++;
        count[0] = 0;
        uint16_t offs[16];
        offs[1] = 0;
        for (int l = 1; l < 15; l++) offs[l + 1] = (uint16_t)(offs[l] + count[l]);
        for (int i = 0; i < n; i++)
            if (lengths[i]) symbol[offs[lengths[i]]++] = (uint16_t)i;
    }
    int decode(Bits& b) const {
        int code = 0, first = 0, index = 0;
        for (int len = 1; len < 16; len++) {
            code |= (int)b.get(1);
            const int c = count[len];
            if (code - first < c) return symbol[index + code - first];
            index += c;
            first = (first + c) << 1;
            code <<= 1;
        }
        throw ImageError(3, "bad Huffman code in deflate stream");
    }
};

const uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6,
                                6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

void InflateBlock(Bits& b, std::vector<uint8_t>& out, const Huffman& lit, const Huffman& dist) {
    while (true) {
        const int sym = lit.decode(b);
        if (sym < 256) {
            out.push_back((uint8_t)sym);
        } else if (sym == 256) {
            return;
        } else {
            const int li = sym - 257;
            if (li >= 29) throw ImageError(3, "bad length code in deflate stream");
            const size_t len = kLenBase[li] + b.get(kLenExtra[li]);
            const int di = dist.decode(b);
            if (di >= 30) throw ImageError(3, "bad distance code in deflate stream");
            const size_t d = kDistBase[di] + b.get(kDistExtra[di]);
            if (d > out.size()) throw ImageError(3, "deflate distance beyond the output");
            const size_t from = out.size() - d;
            for (size_t k = 0; k < len; k++) out.push_back(out[from + k]);
        }
    }
}

}  // namespace

std::vector<uint8_t> Inflate(const uint8_t* data, size_t size) {
    if (size < 6) throw ImageError(3, "zlib stream too short");
    const int cmf = data[0], flg = data[1];
    if ((cmf & 0x0F) != 8 || ((cmf << 8) | flg) % 31 != 0 || (flg & 0x20))
        throw ImageError(3, "not a zlib deflate stream");
    Bits b{data + 2, size - 2};
    std::vector<uint8_t> out;
    bool last = false;
    while (!last) {
        last = b.get(1) != 0;
        const uint32_t type = b.get(2);
        if (type == 0) {
            b.align();
            if (b.pos + 4 > b.n) throw ImageError(3, "deflate stream ends early");
            const uint16_t len = LE16(b.p + b.pos), nlen = LE16(b.p + b.pos + 2);
            if ((uint16_t)~len != nlen) throw ImageError(3, "bad stored block length");
            b.pos += 4;
            if (b.pos + len > b.n) throw ImageError(3, "deflate stream ends early");
            out.insert(out.end(), b.p + b.pos, b.p + b.pos + len);
            b.pos += len;
        } else if (type == 1) {
            static Huffman lit, dist;
            static bool init = false;
            if (!init) {
                uint8_t l[288];
                for (int i = 0; i < 288; i++) l[i] = i < 144 ? 8 : (i < 256 ? 9 : (i < 280 ? 7 : 8));
                lit.build(l, 288);
                uint8_t d[30];
                std::fill(d, d + 30, 5);
                dist.build(d, 30);
                init = true;
            }
            InflateBlock(b, out, lit, dist);
        } else if (type == 2) {
            const int hlit = (int)b.get(5) + 257, hdist = (int)b.get(5) + 1, hclen = (int)b.get(4) + 4;
            static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19] = {0};
            for (int i = 0; i < hclen; i++) cl[order[i]] = (uint8_t)b.get(3);
            Huffman clh;
            clh.build(cl, 19);
            uint8_t lens[320] = {0};
            int k = 0;
            while (k < hlit + hdist) {
                const int sym = clh.decode(b);
                if (sym < 16) {
                    lens[k++] = (uint8_t)sym;
                } else {
                    int rep;
                    uint8_t val = 0;
                    if (sym == 16) {
                        if (k == 0) throw ImageError(3, "bad code-length repeat");
                        val = lens[k - 1];
                        rep = 3 + (int)b.get(2);
                    } else if (sym == 17) {
                        rep = 3 + (int)b.get(3);
                    } else {
                        rep = 11 + (int)b.get(7);
                    }
                    if (k + rep > hlit + hdist) throw ImageError(3, "bad code-length repeat");
                    while (rep--) lens[k++] = val;
                }
            }
            Huffman lit, dist;
            lit.build(lens, hlit);
            dist.build(lens + hlit, hdist);
            InflateBlock(b, out, lit, dist);
        } else {
            throw ImageError(3, "bad deflate block type");
        }
    }
    b.align();
    if (b.pos + 4 > b.n) throw ImageError(3, "zlib stream ends early");
    uint32_t a = 1, s = 0;
    for (uint8_t c : out) {
        a = (a + c) % 65521u;
        s = (s + a) % 65521u;
    }
    if (BE32(b.p + b.pos) != ((s << 16) | a)) throw ImageError(3, "zlib checksum mismatch");
    return out;
}

namespace {

// ---- PNG ----------------------------------------------------------------------------------
TextureImage LoadPng(const std::string& path, const std::vector<uint8_t>& f) {
    size_t pos = 8;
    uint32_t w = 0, h = 0;
    int depth = 0, ctype = -1, interlace = 0;
    std::vector<uint8_t> idat;
    while (pos + 12 <= f.size()) {
        const uint32_t len = BE32(&f[pos]);
        if (pos + 12 + (size_t)len > f.size()) Bad(path, "truncated chunk");
        const uint8_t* type = &f[pos + 4];
        const uint8_t* d = &f[pos + 8];
        if (!std::memcmp(type, "IHDR", 4)) {
            if (len < 13) Bad(path, "short IHDR");
            w = BE32(d);
            h = BE32(d + 4);
            depth = d[8];
            ctype = d[9];
            interlace = d[12];
        } else if (!std::memcmp(type, "IDAT", 4)) {
            idat.insert(idat.end(), d, d + len);
        } else if (!std::memcmp(type, "IEND", 4)) {
            break;
        }
        pos += 12 + len;
    }
    if (w == 0 || h == 0 || w > 65536 || h > 65536) Bad(path, "bad image size");
    // the reference keeps 24- and 32-bit bitmaps only (rt.hpp:205-212)
    if (depth != 8 || (ctype != 2 && ctype != 6)) Unsupported(path, "PNG must be 8-bit RGB or RGBA");
    if (interlace != 0) Unsupported(path, "interlaced PNG");
    const int bpp = ctype == 6 ? 4 : 3;
    const size_t stride = (size_t)w * bpp;
    const std::vector<uint8_t> raw = Inflate(idat.data(), idat.size());
    if (raw.size() < (size_t)h * (stride + 1)) Bad(path, "short image data");
    std::vector<uint8_t> cur(stride), prev(stride, 0);
    TextureImage t;
    t.width = (int)w;
    t.height = (int)h;
    t.rgb.resize(3 * (size_t)w * h);
    for (uint32_t y = 0; y < h; y++) {
        const uint8_t* row = &raw[(size_t)y * (stride + 1)];
        const int filter = row[0];
        for (size_t i = 0; i < stride; i++) {
            const int x = row[1 + i];
            const int a = i >= (size_t)bpp ? cur[i - bpp] : 0;
            const int b = prev[i];
            const int c = i >= (size_t)bpp ? prev[i - bpp] : 0;
            int v;
            switch (filter) {
                case 0: v = x; break;
                case 1: v = x + a; break;
                case 2: v = x + b; break;
                case 3: v = x + (a + b) / 2; break;
                case 4: {
                    const int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
                    v = x + ((pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c));
                    break;
                }
                default: Bad(path, "bad PNG filter");
            }
            cur[i] = (uint8_t)v;
        }
        for (uint32_t x = 0; x < w; x++)
            for (int k = 0; k < 3; k++) t.rgb[3 * ((size_t)y * w + x) + k] = (float)cur[(size_t)x * bpp + k] / 255.0f;
        std::swap(cur, prev);
    }
    return t;
}

// ---- BMP (uncompressed 24/32-bit) ------------------------------------------------------------
TextureImage LoadBmp(const std::string& path, const std::vector<uint8_t>& f) {
    if (f.size() < 54) Bad(path, "short BMP header");
    const uint32_t off = LE32(&f[10]);
    const int32_t w = (int32_t)LE32(&f[18]), hs = (int32_t)LE32(&f[22]);
    const int bits = LE16(&f[28]);
    const uint32_t comp = LE32(&f[30]);
    if (comp != 0 || (bits != 24 && bits != 32)) Unsupported(path, "BMP must be uncompressed 24- or 32-bit");
    const int h = hs < 0 ? -hs : hs;
    if (w <= 0 || h <= 0) Bad(path, "bad image size");
    const size_t bpp = (size_t)bits / 8, stride = ((size_t)w * bpp + 3) & ~(size_t)3;
    if (off + stride * h > f.size()) Bad(path, "short image data");
    TextureImage t;
    t.width = w;
    t.height = h;
    t.rgb.resize(3 * (size_t)w * h);
    for (int y = 0; y < h; y++) {
        const int file_row = hs > 0 ? h - 1 - y : y;  // positive height: bottom-up rows
        const uint8_t* row = &f[off + stride * (size_t)file_row];
        for (int x = 0; x < w; x++)
            for (int k = 0; k < 3; k++) t.rgb[3 * ((size_t)y * w + x) + k] = (float)row[(size_t)x * bpp + 2 - k] / 255.0f;
    }
    return t;
}

// ---- PPM (P6, maxval 255) / PFM ----------------------------------------------------------------
size_t NextToken(const std::vector<uint8_t>& f, size_t pos, std::string& tok) {
    while (pos < f.size()) {
        if (f[pos] == '#') {
            while (pos < f.size() && f[pos] != '\n') pos++;
        } else if (std::isspace(f[pos])) {
            pos++;
        } else {
            break;
        }
    }
    tok.clear();
    while (pos < f.size() && !std::isspace(f[pos])) tok.push_back((char)f[pos++]);
    return pos;
}

TextureImage LoadPnm(const std::string& path, const std::vector<uint8_t>& f) {
    std::string magic, sw, sh, sm;
    size_t pos = NextToken(f, 0, magic);
    pos = NextToken(f, pos, sw);
    pos = NextToken(f, pos, sh);
    pos = NextToken(f, pos, sm);
    pos++;  // the single whitespace before the raster
    const int w = std::atoi(sw.c_str()), h = std::atoi(sh.c_str());
    if (w <= 0 || h <= 0) Bad(path, "bad image size");
    TextureImage t;
    t.width = w;
    t.height = h;
    t.rgb.resize(3 * (size_t)w * h);
    if (magic == "P6") {
        if (std::atoi(sm.c_str()) != 255) Unsupported(path, "PPM must have maxval 255");
        if (pos + 3 * (size_t)w * h > f.size()) Bad(path, "short image data");
        for (size_t i = 0; i < t.rgb.size(); i++) t.rgb[i] = (float)f[pos + i] / 255.0f;
        return t;
    }
    if (magic == "PF") {
        const double scale = std::atof(sm.c_str());
        if (scale >= 0) Unsupported(path, "big-endian PFM");
        if (pos + 12 * (size_t)w * h > f.size()) Bad(path, "short image data");
        for (int y = 0; y < h; y++) {  // file rows run bottom to top
            const uint8_t* row = &f[pos + 12 * (size_t)(h - 1 - y) * w];
            std::memcpy(&t.rgb[3 * (size_t)y * w], row, 12 * (size_t)w);
        }
        return t;
    }
    Unsupported(path, "netpbm type " + magic);
}

}  // namespace

TextureImage LoadTexture(const std::string& path) {
    const std::vector<uint8_t> f = ReadFile(path);
    // format by signature first, then by extension (rt.hpp:171-184)
    if (f.size() >= 8 && !std::memcmp(f.data(), "\x89PNG\r\n\x1a\n", 8)) return LoadPng(path, f);
    if (f.size() >= 2 && f[0] == 'B' && f[1] == 'M') return LoadBmp(path, f);
    if (f.size() >= 2 && f[0] == 'P' && (f[1] == '6' || f[1] == 'F')) return LoadPnm(path, f);
    if (f.size() >= 2 && f[0] == '#' && f[1] == '?') {
        int w = 0, h = 0;
        std::vector<float> rgb;
        ReadHdr(path, w, h, rgb);
        TextureImage t;
        t.width = w;
        t.height = h;
        t.rgb = std::move(rgb);
        return t;
    }
    if (f.size() >= 3 && f[0] == 0xFF && f[1] == 0xD8 && f[2] == 0xFF) Unsupported(path, "JPEG textures");
    Unsupported(path, "unknown image type");
}

}  // namespace ngi
