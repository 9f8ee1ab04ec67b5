// PNG decoding for 8-bit bitmap textures (own zlib / deflate decoder; see png_decode.cpp).
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

#include "image_io.h"

namespace illume {

// Decodes a whole PNG file into 8-bit RGBA texels stored as floats 0..255 (Image::hdr
// false), the texels stb_image would give the reference.
bool decode_png(const std::vector<uint8_t>& file, Image* out, std::string* err);

}  // namespace illume
