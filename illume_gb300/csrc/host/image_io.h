// Image files: texture input (Radiance .hdr, .pfm, binary .ppm / .pgm, .png, .bmp, .tga)
// and render output (8-bit RGB .png and .ppm, float .pfm). The PNG writer compresses with
// the library's own deflate encoder (deflate_encode.h), so it needs no zlib.
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

namespace illume {

struct Image {
  int width = 0, height = 0;
  bool hdr = false;             // float texels (bilinear) vs 8-bit texels (point sampled)
  std::vector<float> rgba;      // 4 floats per texel, row-major, top row first; 8-bit as 0..255
};

bool load_image(const std::string& path, Image* out, std::string* err);
bool save_png_rgb8(const std::string& path, const uint8_t* rgb, int width, int height, std::string* err);
bool save_ppm_rgb8(const std::string& path, const uint8_t* rgb, int width, int height, std::string* err);
bool save_pfm_rgb(const std::string& path, const float* rgb, int width, int height, std::string* err);

}  // namespace illume
