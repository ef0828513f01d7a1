// Film I/O (SaveImage, include/nanogi/basic.hpp:506-672).
#pragma once

#include <stdexcept>
#include <string>

namespace ngi {

struct ImageError : std::runtime_error {
    int code;  // ngi_status value
    ImageError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// film: w*h*3 doubles, row 0 = bottom scanline. Extension selects .hdr or .pfm.
void SaveImage(const std::string& path, const double* film, int w, int h);
void LoadHdr(const std::string& path, double* film, int w, int h);

}  // namespace ngi
