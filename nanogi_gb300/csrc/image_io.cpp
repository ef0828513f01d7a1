// Film output: Radiance RGBE (.hdr), OpenEXR (.exr), 8-bit PNG (.png) and portable float
// map (.pfm).
//
// The reference saves films through FreeImage and tinyexr (include/nanogi/basic.hpp:506-659):
// the film's row 0 is the bottom scanline (FreeImage bitmaps are bottom-up; the EXR path
// flips y), so every saved image is upright. These writers produce the same upright images,
// with the film's top row (row H-1) first in the file:
//   .hdr  Ward's shared-exponent RGBE (Graphics Gems II, "Real Pixels"), flat scanlines;
//   .exr  scanline OpenEXR 2.0 file, float channels B, G, R; uncompressed where the
//         reference asks tinyexr for ZIP (every EXR reader decodes both);
//   .png  8-bit RGB, value = clamp(int(255 v^(1/2.2)), 0, 255) as the reference's tone map
//         (basic.hpp:625-634); the zlib stream uses stored deflate blocks (RFC 1950/1951).
// The output directory is created when missing, as the reference does (basic.hpp:509-521).
#include "image_io.hpp"

#include <sys/stat.h>

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <vector>

namespace ngi {

namespace {

void FloatToRgbe(float r, float g, float b, unsigned char out[4]) {
    float v = r;
    if (g > v) v = g;
    if (b > v) v = b;
    if (!(v >= 1e-32f)) {  // also maps NaN to black
        out[0] = out[1] = out[2] = out[3] = 0;
        return;
    }
    int e;
    const float m = std::frexp(v, &e);
    const float scale = m * 256.0f / v;
    out[0] = (unsigned char)(r > 0 ? r * scale : 0);
    out[1] = (unsigned char)(g > 0 ? g * scale : 0);
    out[2] = (unsigned char)(b > 0 ? b * scale : 0);
    out[3] = (unsigned char)(e + 128);
}

void RgbeToFloat(const unsigned char in[4], float& r, float& g, float& b) {
    if (in[3] == 0) {
        r = g = b = 0;
        return;
    }
    const float f = std::ldexp(1.0f, (int)in[3] - (128 + 8));
    r = (in[0] + 0.5f) * f;
    g = (in[1] + 0.5f) * f;
    b = (in[2] + 0.5f) * f;
}

std::string Extension(const std::string& path) {
    const size_t dot = path.find_last_of('.');
    const size_t slash = path.find_last_of('/');
    if (dot == std::string::npos || (slash != std::string::npos && dot < slash)) return "";
    return path.substr(dot);
}

// mkdir -p of the directory part of path.
void CreateParentDirs(const std::string& path) {
    const size_t slash = path.find_last_of('/');
    if (slash == std::string::npos || slash == 0) return;
    const std::string dir = path.substr(0, slash);
    for (size_t i = 1; i <= dir.size(); i++) {
        if (i < dir.size() && dir[i] != '/') continue;
        const std::string part = dir.substr(0, i);
        if (mkdir(part.c_str(), 0755) != 0 && errno != EEXIST)
            throw ImageError(2, "Failed to create output directory : " + part);
    }
}

template <typename T>
void Put(std::string& out, T v) {  // the value's bytes; both hosts (x86-64, aarch64) are little endian
    char b[sizeof(T)];
    std::memcpy(b, &v, sizeof(T));
    out.append(b, sizeof(T));
}
void PutBE32(std::string& out, uint32_t v) {
    for (int i = 3; i >= 0; i--) out.push_back((char)(v >> (8 * i) & 0xFF));
}
void PutAttr(std::string& out, const char* name, const char* type, const std::string& value) {
    out.append(name).push_back('\0');
    out.append(type).push_back('\0');
    Put<int32_t>(out, (int32_t)value.size());
    out.append(value);
}

std::string Exr(const double* film, int w, int h) {
    std::string out;
    Put<uint32_t>(out, 20000630u);  // magic 76 2f 31 01
    Put<uint32_t>(out, 2u);         // version 2, single-part scanline
    std::string ch;
    for (const char* name : {"B", "G", "R"}) {  // alphabetical, as the format requires
        ch.append(name).push_back('\0');
        Put<int32_t>(ch, 2);  // FLOAT
        Put<uint32_t>(ch, 0u);  // pLinear + reserved
        Put<int32_t>(ch, 1);
        Put<int32_t>(ch, 1);
    }
    ch.push_back('\0');
    PutAttr(out, "channels", "chlist", ch);
    PutAttr(out, "compression", "compression", std::string(1, '\0'));
    std::string box;
    Put<int32_t>(box, 0); Put<int32_t>(box, 0); Put<int32_t>(box, w - 1); Put<int32_t>(box, h - 1);
    PutAttr(out, "dataWindow", "box2i", box);
    PutAttr(out, "displayWindow", "box2i", box);
    PutAttr(out, "lineOrder", "lineOrder", std::string(1, '\0'));
    std::string one;
    Put<float>(one, 1.0f);
    PutAttr(out, "pixelAspectRatio", "float", one);
    std::string center;
    Put<float>(center, 0.0f); Put<float>(center, 0.0f);
    PutAttr(out, "screenWindowCenter", "v2f", center);
    PutAttr(out, "screenWindowWidth", "float", one);
    out.push_back('\0');
    const size_t block = 8 + 12 * (size_t)w;  // y, size, 3 channels of w floats
    const size_t table = out.size();
    for (int y = 0; y < h; y++) Put<uint64_t>(out, table + 8 * (size_t)h + block * (size_t)y);
    for (int y = 0; y < h; y++) {
        const double* row = film + 3 * (size_t)(h - 1 - y) * w;  // file row 0 = top = film row h-1
        Put<int32_t>(out, y);
        Put<int32_t>(out, (int32_t)(12 * (size_t)w));
        for (int c : {2, 1, 0})  // B, G, R
            for (int x = 0; x < w; x++) Put<float>(out, (float)row[3 * (size_t)x + c]);
    }
    return out;
}

uint32_t Crc32(const unsigned char* p, size_t n, uint32_t crc = 0) {
    static uint32_t table[256];
    static bool init = false;
    if (!init) {
        for (uint32_t i = 0; i < 256; i++) {
            uint32_t c = i;
            for (int k = 0; k < 8; k++) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            table[i] = c;
        }
        init = true;
    }
    crc = ~crc;
    for (size_t i = 0; i < n; i++) crc = table[(crc ^ p[i]) & 0xFF] ^ (crc >> 8);
    return ~crc;
}

void PngChunk(std::string& out, const char* type, const std::string& data) {
    PutBE32(out, (uint32_t)data.size());
    const std::string td = std::string(type, 4) + data;
    out.append(td);
    PutBE32(out, Crc32((const unsigned char*)td.data(), td.size()));
}

std::string Png(const double* film, int w, int h) {
    std::string raw;
    raw.reserve((size_t)h * (1 + 3 * (size_t)w));
    for (int y = h - 1; y >= 0; y--) {
        raw.push_back('\0');  // filter: none
        for (int x = 0; x < w; x++)
            for (int c = 0; c < 3; c++) {
                const double v = std::pow(film[3 * ((size_t)y * w + x) + c], 1.0 / 2.2) * 255.0;
                const int b = v >= 255.0 ? 255 : (v >= 0.0 ? (int)v : 0);  // NaN -> 0
                raw.push_back((char)b);
            }
    }
    std::string z;
    z.push_back((char)0x78);
    z.push_back((char)0x01);
    for (size_t pos = 0; pos < raw.size() || pos == 0;) {
        const size_t len = std::min<size_t>(65535, raw.size() - pos);
        const bool last = pos + len >= raw.size();
        z.push_back((char)(last ? 1 : 0));  // stored block
        Put<uint16_t>(z, (uint16_t)len);
        Put<uint16_t>(z, (uint16_t)~len);
        z.append(raw, pos, len);
        pos += len;
        if (last) break;
    }
    uint32_t a = 1, b = 0;  // Adler-32
    for (unsigned char c : raw) {
        a = (a + c) % 65521u;
        b = (b + a) % 65521u;
    }
    PutBE32(z, (b << 16) | a);
    std::string out("\x89PNG\r\n\x1a\n", 8);
    std::string ihdr;
    PutBE32(ihdr, (uint32_t)w);
    PutBE32(ihdr, (uint32_t)h);
    ihdr.append({(char)8, (char)2, (char)0, (char)0, (char)0});  // 8-bit RGB
    PngChunk(out, "IHDR", ihdr);
    PngChunk(out, "IDAT", z);
    PngChunk(out, "IEND", "");
    return out;
}

}  // namespace

void SaveImage(const std::string& path, const double* film, int w, int h) {
    if (w <= 0 || h <= 0) throw ImageError(1, "width and height must be positive");
    const std::string ext = Extension(path);
    if (ext != ".hdr" && ext != ".pfm" && ext != ".exr" && ext != ".png")
        throw ImageError(1, "Invalid extension: " + ext);
    CreateParentDirs(path);
    std::ofstream f(path, std::ios::binary);
    if (!f) throw ImageError(2, "Failed to save image : " + path);
    if (ext == ".exr" || ext == ".png") {
        const std::string data = ext == ".exr" ? Exr(film, w, h) : Png(film, w, h);
        f.write(data.data(), (std::streamsize)data.size());
        if (!f) throw ImageError(2, "Failed to save image : " + path);
        return;
    }
    if (ext == ".hdr") {
        std::ostringstream hdr;
        hdr << "#?RADIANCE\n# nanogi-gb300\nFORMAT=32-bit_rle_rgbe\n\n-Y " << h << " +X " << w << "\n";
        const std::string hs = hdr.str();
        f.write(hs.data(), (std::streamsize)hs.size());
        std::vector<unsigned char> line(4 * (size_t)w);
        for (int y = h - 1; y >= 0; y--) {
            for (int x = 0; x < w; x++) {
                const double* p = film + 3 * ((size_t)y * w + x);
                FloatToRgbe((float)p[0], (float)p[1], (float)p[2], &line[4 * (size_t)x]);
            }
            f.write((const char*)line.data(), (std::streamsize)line.size());
        }
    } else if (ext == ".pfm") {
        // PFM: bottom-to-top rows, negative scale = little endian
        std::ostringstream hdr;
        hdr << "PF\n" << w << " " << h << "\n-1.0\n";
        const std::string hs = hdr.str();
        f.write(hs.data(), (std::streamsize)hs.size());
        std::vector<float> row(3 * (size_t)w);
        for (int y = 0; y < h; y++) {
            for (int i = 0; i < 3 * w; i++) row[i] = (float)film[3 * (size_t)y * w + i];
            f.write((const char*)row.data(), (std::streamsize)(row.size() * sizeof(float)));
        }
    } else {
        throw ImageError(1, "Invalid extension: " + ext);
    }
    if (!f) throw ImageError(2, "Failed to save image : " + path);
}

void ReadHdr(const std::string& path, int& w, int& h, std::vector<float>& rgb) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw ImageError(2, "cannot open " + path);
    std::string line;
    bool magic = false;
    while (std::getline(f, line)) {
        if (line.rfind("#?", 0) == 0) magic = true;
        if (line.empty()) break;
    }
    if (!magic) throw ImageError(3, "not a Radiance file: " + path);
    if (!std::getline(f, line)) throw ImageError(3, "missing resolution line");
    int hh = 0, ww = 0;
    if (std::sscanf(line.c_str(), "-Y %d +X %d", &hh, &ww) != 2) throw ImageError(3, "unsupported resolution line: " + line);
    if (hh <= 0 || ww <= 0 || (size_t)hh * (size_t)ww > ((size_t)1 << 31)) throw ImageError(3, "bad image size");
    w = ww;
    h = hh;
    rgb.assign(3 * (size_t)w * h, 0.0f);
    std::vector<unsigned char> scan(4 * (size_t)w);
    for (int row = 0; row < h; row++) {
        unsigned char head[4];
        if (!f.read((char*)head, 4)) throw ImageError(3, "truncated file");
        if (head[0] == 2 && head[1] == 2 && ((head[2] << 8) | head[3]) == w && w >= 8 && w < 32768) {
            // new-style run-length encoded scanline: four planes
            for (int c = 0; c < 4; c++) {
                int x = 0;
                while (x < w) {
                    unsigned char cnt;
                    if (!f.read((char*)&cnt, 1)) throw ImageError(3, "truncated RLE data");
                    if (cnt > 128) {
                        unsigned char val;
                        f.read((char*)&val, 1);
                        cnt -= 128;
                        if (x + cnt > w) throw ImageError(3, "bad RLE run");
                        for (int k = 0; k < cnt; k++) scan[4 * (size_t)(x++) + c] = val;
                    } else {
                        if (cnt == 0 || x + cnt > w) throw ImageError(3, "bad RLE run");
                        for (int k = 0; k < cnt; k++) {
                            unsigned char val;
                            f.read((char*)&val, 1);
                            scan[4 * (size_t)(x++) + c] = val;
                        }
                    }
                }
            }
        } else {
            std::memcpy(scan.data(), head, 4);
            if (!f.read((char*)scan.data() + 4, (std::streamsize)(4 * (size_t)w - 4))) throw ImageError(3, "truncated file");
        }
        for (int x = 0; x < w; x++) {  // file rows run top to bottom
            float* p = &rgb[3 * ((size_t)row * w + x)];
            RgbeToFloat(&scan[4 * (size_t)x], p[0], p[1], p[2]);
        }
    }
}

void LoadHdr(const std::string& path, double* film, int w, int h) {
    int ww = 0, hh = 0;
    std::vector<float> rgb;
    ReadHdr(path, ww, hh, rgb);
    if (hh != h || ww != w) throw ImageError(1, "image is " + std::to_string(ww) + "x" + std::to_string(hh));
    for (int row = 0; row < h; row++)  // film row 0 is the bottom scanline
        for (size_t k = 0; k < 3 * (size_t)w; k++) film[3 * (size_t)(h - 1 - row) * w + k] = rgb[3 * (size_t)row * w + k];
}

}  // namespace ngi
