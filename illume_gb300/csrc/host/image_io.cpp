#include "image_io.h"

#include "deflate_encode.h"
#include "png_decode.h"

#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <fstream>
#include <sstream>
#include <thread>

namespace illume {

namespace {

std::string lower_ext(const std::string& p) {
  const size_t dot = p.find_last_of('.');
  std::string e = dot == std::string::npos ? "" : p.substr(dot + 1);
  for (char& c : e) c = (char)tolower(c);
  return e;
}

bool read_file(const std::string& path, std::vector<uint8_t>* data) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  data->assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
  return true;
}

// PFM: "PF" (RGB) or "Pf" (grey), width height, scale (< 0 little endian), rows bottom-up.
bool load_pfm(const std::vector<uint8_t>& d, Image* out, std::string* err) {
  std::string hdr;
  size_t pos = 0;
  int fields = 0;
  std::string tok[4];
  while (pos < d.size() && fields < 4) {
    while (pos < d.size() && isspace(d[pos])) ++pos;
    while (pos < d.size() && !isspace(d[pos])) tok[fields] += (char)d[pos++];
    ++fields;
  }
  ++pos;  // single whitespace after the scale
  if (fields < 4 || (tok[0] != "PF" && tok[0] != "Pf")) { *err = "not a PFM file"; return false; }
  const int ch = tok[0] == "PF" ? 3 : 1;
  const int w = atoi(tok[1].c_str()), h = atoi(tok[2].c_str());
  const double scale = atof(tok[3].c_str());
  if (w <= 0 || h <= 0 || d.size() < pos + (size_t)w * h * ch * 4) { *err = "truncated PFM file"; return false; }
  const bool little = scale < 0;
  out->width = w; out->height = h; out->hdr = true;
  out->rgba.assign((size_t)w * h * 4, 1.0f);
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x)
      for (int c = 0; c < ch; ++c) {
        const uint8_t* p = d.data() + pos + 4 * (((size_t)y * w + x) * ch + c);
        uint32_t u = little ? (p[0] | p[1] << 8 | p[2] << 16 | (uint32_t)p[3] << 24)
                            : (p[3] | p[2] << 8 | p[1] << 16 | (uint32_t)p[0] << 24);
        float f;
        memcpy(&f, &u, 4);
        const size_t o = 4 * ((size_t)(h - 1 - y) * w + x);
        if (ch == 3) out->rgba[o + c] = f;
        else out->rgba[o] = out->rgba[o + 1] = out->rgba[o + 2] = f;
      }
  return true;
}

// binary PPM (P6, maxval <= 255)
bool load_ppm(const std::vector<uint8_t>& d, Image* out, std::string* err) {
  size_t pos = 0;
  std::string tok[4];
  int fields = 0;
  while (pos < d.size() && fields < 4) {
    while (pos < d.size() && isspace(d[pos])) ++pos;
    if (pos < d.size() && d[pos] == '#') { while (pos < d.size() && d[pos] != '\n') ++pos; continue; }
    while (pos < d.size() && !isspace(d[pos])) tok[fields] += (char)d[pos++];
    ++fields;
  }
  ++pos;
  if (fields < 4 || tok[0] != "P6") { *err = "not a binary PPM file"; return false; }
  const int w = atoi(tok[1].c_str()), h = atoi(tok[2].c_str()), mx = atoi(tok[3].c_str());
  if (w <= 0 || h <= 0 || mx <= 0 || mx > 255 || d.size() < pos + (size_t)w * h * 3) { *err = "truncated PPM file"; return false; }
  out->width = w; out->height = h; out->hdr = false;
  out->rgba.assign((size_t)w * h * 4, 255.0f);
  for (size_t i = 0; i < (size_t)w * h; ++i)
    for (int c = 0; c < 3; ++c) out->rgba[4 * i + c] = (float)d[pos + 3 * i + c];
  return true;
}

// Radiance RGBE (.hdr): flat or new-style run-length scanlines, "-Y h +X w" orientation.
bool load_hdr(const std::vector<uint8_t>& d, Image* out, std::string* err) {
  size_t pos = 0;
  auto line = [&]() {
    std::string s;
    while (pos < d.size() && d[pos] != '\n') s += (char)d[pos++];
    ++pos;
    return s;
  };
  std::string l = line();
  if (l.rfind("#?", 0) != 0) { *err = "not a Radiance HDR file"; return false; }
  while (pos < d.size()) {
    l = line();
    if (l.empty()) break;
  }
  l = line();
  int w = 0, h = 0;
  char ya[4], xa[4];
  if (sscanf(l.c_str(), "%3s %d %3s %d", ya, &h, xa, &w) != 4 || strcmp(ya, "-Y") != 0 || strcmp(xa, "+X") != 0 ||
      w <= 0 || h <= 0) {
    *err = "unsupported HDR orientation";
    return false;
  }
  out->width = w; out->height = h; out->hdr = true;
  out->rgba.assign((size_t)w * h * 4, 1.0f);
  std::vector<uint8_t> scan((size_t)w * 4);
  for (int y = 0; y < h; ++y) {
    if (pos + 4 > d.size()) { *err = "truncated HDR file"; return false; }
    if (w >= 8 && w < 32768 && d[pos] == 2 && d[pos + 1] == 2 && (d[pos + 2] << 8 | d[pos + 3]) == w) {
      pos += 4;
      for (int c = 0; c < 4; ++c) {
        int x = 0;
        while (x < w) {
          if (pos >= d.size()) { *err = "truncated HDR file"; return false; }
          int n = d[pos++];
          if (n > 128) {
            n -= 128;
            if (pos >= d.size() || x + n > w) { *err = "bad HDR run"; return false; }
            const uint8_t v = d[pos++];
            for (int k = 0; k < n; ++k) scan[4 * (x++) + c] = v;
          } else {
            if (n == 0 || pos + n > d.size() || x + n > w) { *err = "bad HDR run"; return false; }
            for (int k = 0; k < n; ++k) scan[4 * (x++) + c] = d[pos++];
          }
        }
      }
    } else {
      if (pos + (size_t)w * 4 > d.size()) { *err = "truncated HDR file"; return false; }
      memcpy(scan.data(), d.data() + pos, (size_t)w * 4);
      pos += (size_t)w * 4;
    }
    for (int x = 0; x < w; ++x) {
      const uint8_t* p = &scan[4 * x];
      const float f = p[3] ? ldexpf(1.0f, (int)p[3] - (128 + 8)) : 0.0f;
      float* o = &out->rgba[4 * ((size_t)y * w + x)];
      o[0] = p[0] * f; o[1] = p[1] * f; o[2] = p[2] * f; o[3] = 1.0f;
    }
  }
  return true;
}

struct CrcTable {
  uint32_t t[256];
  CrcTable() {
    for (uint32_t i = 0; i < 256; ++i) {
      uint32_t v = i;
      for (int k = 0; k < 8; ++k) v = (v & 1) ? 0xedb88320u ^ (v >> 1) : v >> 1;
      t[i] = v;
    }
  }
};
uint32_t crc32(const uint8_t* p, size_t n, uint32_t c = 0xffffffffu) {
  static const CrcTable table;   // built once, thread-safe
  for (size_t i = 0; i < n; ++i) c = table.t[(c ^ p[i]) & 0xff] ^ (c >> 8);
  return c;
}

// The scanlines of an 8-bit RGB image, each behind the filter byte of the filter (none,
// sub, up, average, Paeth; ISO 15948 9.2) whose output has the least sum of absolute
// values read as signed bytes, the usual choice of PNG writers.
std::vector<uint8_t> filtered_scanlines(const uint8_t* rgb, int w, int h) {
  const size_t stride = (size_t)w * 3;
  std::vector<uint8_t> raw((size_t)h * (stride + 1));
  std::vector<uint8_t> zero(stride, 0);
  auto mag = [](int v) { const uint8_t u = (uint8_t)v; return u < 128 ? (int)u : 256 - (int)u; };
  auto paeth = [](int a, int b, int c) {
    const int p = a + b - c, pa = p > a ? p - a : a - p, pb = p > b ? p - b : b - p, pc = p > c ? p - c : c - p;
    return (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
  };
  auto row = [&](int y) {
    const uint8_t* cur = rgb + (size_t)y * stride;
    const uint8_t* up = y > 0 ? rgb + (size_t)(y - 1) * stride : zero.data();
    long s0 = 0, s1 = 0, s2 = 0, s3 = 0, s4 = 0;
    for (size_t i = 0; i < stride; ++i) {
      const int x = cur[i], a = i >= 3 ? cur[i - 3] : 0, b = up[i], c = i >= 3 ? up[i - 3] : 0;
      s0 += mag(x);
      s1 += mag(x - a);
      s2 += mag(x - b);
      s3 += mag(x - ((a + b) >> 1));
      s4 += mag(x - paeth(a, b, c));
    }
    const long sums[5] = {s0, s1, s2, s3, s4};
    int f = 0;
    for (int k = 1; k < 5; ++k)
      if (sums[k] < sums[f]) f = k;
    uint8_t* o = raw.data() + (size_t)y * (stride + 1);
    o[0] = (uint8_t)f;
    ++o;
    for (size_t i = 0; i < stride; ++i) {
      const int a = i >= 3 ? cur[i - 3] : 0, b = up[i], c = i >= 3 ? up[i - 3] : 0;
      const int pred = f == 0 ? 0 : f == 1 ? a : f == 2 ? b : f == 3 ? (a + b) >> 1 : paeth(a, b, c);
      o[i] = (uint8_t)(cur[i] - pred);
    }
  };
  // rows filter independently (each reads the image, not its neighbours' output): bands
  // of rows on the host threads
  const int threads = (int)std::max(1u, std::min({16u, std::thread::hardware_concurrency(), (unsigned)(h / 64 + 1)}));
  std::atomic<int> next{0};
  auto work = [&]() {
    for (int y0 = next.fetch_add(64); y0 < h; y0 = next.fetch_add(64))
      for (int y = y0; y < std::min(h, y0 + 64); ++y) row(y);
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < threads; ++t) pool.emplace_back(work);
  work();
  for (auto& th : pool) th.join();
  return raw;
}

void be32(std::vector<uint8_t>& v, uint32_t x) {
  v.push_back(x >> 24); v.push_back(x >> 16); v.push_back(x >> 8); v.push_back(x);
}

void chunk(std::vector<uint8_t>& out, const char* type, const std::vector<uint8_t>& data) {
  be32(out, (uint32_t)data.size());
  std::vector<uint8_t> td(type, type + 4);
  td.insert(td.end(), data.begin(), data.end());
  out.insert(out.end(), td.begin(), td.end());
  be32(out, crc32(td.data(), td.size()) ^ 0xffffffffu);
}

}  // namespace

bool load_image(const std::string& path, Image* out, std::string* err) {
  std::vector<uint8_t> d;
  if (!read_file(path, &d)) { *err = "cannot read image " + path; return false; }
  const std::string e = lower_ext(path);
  if (e == "pfm") return load_pfm(d, out, err);
  if (e == "ppm") return load_ppm(d, out, err);
  if (e == "hdr") return load_hdr(d, out, err);
  if (e == "png") return decode_png(d, out, err);
  *err = "unsupported image format ." + e + " (" + path + ")";
  return false;
}

bool save_png_rgb8(const std::string& path, const uint8_t* rgb, int w, int h, std::string* err) {
  const std::vector<uint8_t> raw = filtered_scanlines(rgb, w, h);
  const std::vector<uint8_t> z = zlib_compress(raw.data(), raw.size());
  std::vector<uint8_t> png{0x89, 'P', 'N', 'G', 0x0d, 0x0a, 0x1a, 0x0a};
  std::vector<uint8_t> ihdr;
  be32(ihdr, (uint32_t)w);
  be32(ihdr, (uint32_t)h);
  ihdr.insert(ihdr.end(), {8, 2, 0, 0, 0});
  chunk(png, "IHDR", ihdr);
  chunk(png, "IDAT", z);
  chunk(png, "IEND", {});
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) { *err = "cannot write " + path; return false; }
  const bool ok = fwrite(png.data(), 1, png.size(), f) == png.size();
  fclose(f);
  if (!ok) *err = "short write to " + path;
  return ok;
}

bool save_ppm_rgb8(const std::string& path, const uint8_t* rgb, int w, int h, std::string* err) {
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) { *err = "cannot write " + path; return false; }
  fprintf(f, "P6\n%d %d\n255\n", w, h);
  const bool ok = fwrite(rgb, 1, (size_t)w * h * 3, f) == (size_t)w * h * 3;
  fclose(f);
  if (!ok) *err = "short write to " + path;
  return ok;
}

bool save_pfm_rgb(const std::string& path, const float* rgb, int w, int h, std::string* err) {
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) { *err = "cannot write " + path; return false; }
  fprintf(f, "PF\n%d %d\n-1.0\n", w, h);
  bool ok = true;
  for (int y = h - 1; y >= 0 && ok; --y) ok = fwrite(rgb + (size_t)y * w * 3, 4, (size_t)w * 3, f) == (size_t)w * 3;
  fclose(f);
  if (!ok) *err = "short write to " + path;
  return ok;
}

}  // namespace illume
