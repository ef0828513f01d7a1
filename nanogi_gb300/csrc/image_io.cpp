// Film output: Radiance RGBE (.hdr) and portable float map (.pfm).
//
// The reference saves films through FreeImage (include/nanogi/basic.hpp:531-565): the
// film's row 0 is the bottom scanline (FreeImage bitmaps are bottom-up), so the saved
// image is upright. This writer produces the same upright image: the Radiance header
// "-Y H +X W" lists scanlines top to bottom, so film row H-1 is written first. Pixels are
// encoded with Ward's shared-exponent RGBE (Graphics Gems II, "Real Pixels").
#include "image_io.hpp"

#include <cmath>
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

}  // namespace

void SaveImage(const std::string& path, const double* film, int w, int h) {
    if (w <= 0 || h <= 0) throw ImageError(1, "width and height must be positive");
    const std::string ext = Extension(path);
    std::ofstream f(path, std::ios::binary);
    if (!f) throw ImageError(2, "Failed to save image : " + path);
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

void LoadHdr(const std::string& path, double* film, int w, int h) {
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
    if (hh != h || ww != w) throw ImageError(1, "image is " + std::to_string(ww) + "x" + std::to_string(hh));
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
        const int y = h - 1 - row;
        for (int x = 0; x < w; x++) {
            float r, g, b;
            RgbeToFloat(&scan[4 * (size_t)x], r, g, b);
            double* p = film + 3 * ((size_t)y * w + x);
            p[0] = r; p[1] = g; p[2] = b;
        }
    }
}

}  // namespace ngi
