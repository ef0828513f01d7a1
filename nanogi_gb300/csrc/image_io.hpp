// Film I/O (SaveImage, include/nanogi/basic.hpp:506-672).
#pragma once

#include <stdexcept>
#include <string>
#include <vector>

namespace ngi {

struct ImageError : std::runtime_error {
    int code;  // ngi_status value
    ImageError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// film: w*h*3 doubles, row 0 = bottom scanline. Extension selects .hdr, .exr, .png or .pfm.
void SaveImage(const std::string& path, const double* film, int w, int h);
void LoadHdr(const std::string& path, double* film, int w, int h);
// Radiance RGBE file of any size: rgb holds 3 floats per pixel, row 0 = the top scanline.
void ReadHdr(const std::string& path, int& w, int& h, std::vector<float>& rgb);

}  // namespace ngi
