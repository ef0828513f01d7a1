// Texture images for textured albedo (TexR), the reference's Texture (include/nanogi/rt.hpp:157-270).
//
// The reference loads textures through FreeImage and accepts RGB/RGBA float images and 24/32-bit
// bitmaps (rt.hpp:205-212); 8-bit values become v/255 with no gamma. After its vertical flip
// the first stored row is the image's top row, and a lookup at uv reads the texel
// (clamp(int(fract(u) W), 0, W-1), clamp(int(fract(v) H), 0, H-1)) -- nearest, wrapped.
// This loader reads the same images from the formats it decodes itself: PNG (8-bit RGB or
// RGBA, not interlaced), binary PPM (P6, maxval 255), BMP (uncompressed 24/32-bit), Radiance
// .hdr and PFM. Other files fail with a message, as FreeImage's unsupported types do.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace ngi {

struct TextureImage {
    int width = 0, height = 0;
    std::vector<float> rgb;  // 3 floats per texel, row 0 = the image's top row
};

// Throws ImageError (image_io.hpp) on a missing, malformed or unsupported file.
TextureImage LoadTexture(const std::string& path);

// zlib stream (RFC 1950) holding deflate data (RFC 1951) -> bytes. Throws ImageError.
std::vector<uint8_t> Inflate(const uint8_t* data, size_t size);

}  // namespace ngi
