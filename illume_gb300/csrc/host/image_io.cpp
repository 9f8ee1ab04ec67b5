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

uint32_t le16(const std::vector<uint8_t>& d, size_t p) { return d[p] | (uint32_t)d[p + 1] << 8; }
uint32_t le32(const std::vector<uint8_t>& d, size_t p) {
  return d[p] | (uint32_t)d[p + 1] << 8 | (uint32_t)d[p + 2] << 16 | (uint32_t)d[p + 3] << 24;
}

// Windows bitmap: uncompressed (BI_RGB) 4 and 8 bits per pixel through the palette, 24
// (B, G, R) and 32 bits (B, G, R, A; or BI_BITFIELDS with byte-aligned masks); rows padded
// to 4 bytes, bottom-up unless the height is negative. As stb_image 2.14 reads it (the
// reference's loader, texture.cu:36-65): 8-bit texels, alpha 255 where there is none;
// 1-bit files, which it refuses, are refused too (the texture becomes black in both).
bool load_bmp(const std::vector<uint8_t>& d, Image* out, std::string* err) {
  if (d.size() < 26 || d[0] != 'B' || d[1] != 'M') { *err = "not a BMP file"; return false; }
  const size_t offset = le32(d, 10), hsz = le32(d, 14);
  if (hsz != 12 && hsz != 40 && hsz != 56 && hsz != 108 && hsz != 124) { *err = "unsupported BMP header"; return false; }
  long w, h;
  int bpp, comp = 0, ncolors = 0;
  if (hsz == 12) {
    w = (int16_t)le16(d, 18);
    h = (int16_t)le16(d, 20);
    bpp = (int)le16(d, 24);
  } else {
    if (d.size() < 14 + hsz) { *err = "truncated BMP file"; return false; }
    w = (int32_t)le32(d, 18);
    h = (int32_t)le32(d, 22);
    bpp = (int)le16(d, 28);
    comp = (int)le32(d, 30);
    ncolors = (int)le32(d, 46);
  }
  const bool top_down = h < 0;
  if (h < 0) h = -h;
  if (w <= 0 || h <= 0 || w > (1 << 16) || h > (1 << 16) || (long long)w * h > (1LL << 28)) {
    *err = "bad BMP size";
    return false;
  }
  uint32_t mask[4] = {0x00ff0000u, 0x0000ff00u, 0x000000ffu, 0xff000000u};
  if (comp == 3) {
    if (bpp != 32) { *err = "unsupported BMP bit fields"; return false; }
    const size_t mp = 54;   // the masks follow a 40-byte header, or sit at the same place inside a longer one
    if (d.size() < mp + 12) { *err = "truncated BMP file"; return false; }
    mask[0] = le32(d, mp);
    mask[1] = le32(d, mp + 4);
    mask[2] = le32(d, mp + 8);
    mask[3] = hsz >= 56 && d.size() >= mp + 16 ? le32(d, mp + 12) : 0;
    for (int c = 0; c < 3; ++c) {
      uint32_t m = mask[c];
      int sh = 0;
      while (m && !(m & 1)) { m >>= 1; ++sh; }
      if (m != 0xff || sh % 8) { *err = "unsupported BMP bit fields"; return false; }
    }
  } else if (comp != 0) {
    *err = "unsupported BMP compression";
    return false;
  }
  if (bpp != 4 && bpp != 8 && bpp != 24 && bpp != 32) { *err = "unsupported BMP bit depth"; return false; }
  uint8_t pal[256][3] = {};
  if (bpp <= 8) {
    const int entry = hsz == 12 ? 3 : 4;
    const int n = ncolors > 0 && ncolors <= 256 ? ncolors : 1 << bpp;
    const size_t pp = 14 + hsz;
    if (d.size() < pp + (size_t)n * entry) { *err = "truncated BMP palette"; return false; }
    for (int i = 0; i < n; ++i)
      for (int c = 0; c < 3; ++c) pal[i][c] = d[pp + (size_t)i * entry + 2 - c];   // stored B, G, R
  }
  const size_t stride = (((size_t)w * bpp + 31) / 32) * 4;
  if (offset + stride * h > d.size()) { *err = "truncated BMP file"; return false; }
  out->width = (int)w;
  out->height = (int)h;
  out->hdr = false;
  out->rgba.assign((size_t)w * h * 4, 255.0f);
  auto shift_of = [](uint32_t m) { int s = 0; while (m && !(m & 1)) { m >>= 1; ++s; } return s; };
  const int sh[4] = {shift_of(mask[0]), shift_of(mask[1]), shift_of(mask[2]), shift_of(mask[3])};
  for (long y = 0; y < h; ++y) {
    const uint8_t* row = d.data() + offset + stride * (size_t)(top_down ? y : h - 1 - y);
    float* o = &out->rgba[(size_t)y * w * 4];
    for (long x = 0; x < w; ++x, o += 4) {
      if (bpp <= 8) {
        const int per = 8 / bpp;
        const int idx = (row[x / per] >> (8 - bpp * (x % per + 1))) & ((1 << bpp) - 1);
        for (int c = 0; c < 3; ++c) o[c] = pal[idx][c];
      } else if (bpp == 24) {
        for (int c = 0; c < 3; ++c) o[c] = row[3 * x + 2 - c];
      } else {
        const uint32_t v = row[4 * x] | (uint32_t)row[4 * x + 1] << 8 | (uint32_t)row[4 * x + 2] << 16 |
                           (uint32_t)row[4 * x + 3] << 24;
        for (int c = 0; c < 3; ++c) o[c] = (float)((v & mask[c]) >> sh[c]);
        if (mask[3]) o[3] = (float)((v & mask[3]) >> sh[3]);
      }
    }
  }
  return true;
}

// Truevision TGA: colour-mapped (1), true-colour (2) and grey (3) images, run-length coded
// or not (9, 10, 11), 8, 15/16 (5 bits a channel, scaled by 255 / 31 as integers), 24
// and 32 bits per pixel (B, G, R[, A]); bottom-up unless the descriptor's bit 5 is set.
// As stb_image 2.14 reads it (the reference's loader): 8-bit texels, grey replicated. One
// deviation: a colour map whose first entry index is not 0 is read as the format defines
// it (pixel index minus first entry); stb_image 2.14 skips that many bytes instead.
bool load_tga(const std::vector<uint8_t>& d, Image* out, std::string* err) {
  if (d.size() < 18) { *err = "not a TGA file"; return false; }
  const int idlen = d[0], cmtype = d[1], type = d[2];
  const int cm_first = (int)le16(d, 3), cm_len = (int)le16(d, 5), cm_bits = d[7];
  const int w = (int)le16(d, 12), h = (int)le16(d, 14), bpp = d[16], desc = d[17];
  const int base = type & 7;
  const bool rle = type & 8;
  if ((base != 1 && base != 2 && base != 3) || (type & ~11) || w <= 0 || h <= 0) { *err = "unsupported TGA type"; return false; }
  if ((long long)w * h > (1LL << 28)) { *err = "bad TGA size"; return false; }
  if ((base == 1 && (cmtype != 1 || bpp != 8)) || (base == 3 && bpp != 8) ||
      (base == 2 && bpp != 15 && bpp != 16 && bpp != 24 && bpp != 32)) {
    *err = "unsupported TGA bit depth";
    return false;
  }
  size_t pos = 18 + (size_t)idlen;
  // one pixel of `bits` at p as R, G, B, A
  auto decode = [](const uint8_t* p, int bits, uint8_t* rgba) {
    if (bits == 8) {
      rgba[0] = rgba[1] = rgba[2] = p[0];
      rgba[3] = 255;
    } else if (bits == 15 || bits == 16) {
      const uint32_t v = p[0] | (uint32_t)p[1] << 8;
      rgba[0] = (uint8_t)(((v >> 10) & 31) * 255 / 31);
      rgba[1] = (uint8_t)(((v >> 5) & 31) * 255 / 31);
      rgba[2] = (uint8_t)((v & 31) * 255 / 31);
      rgba[3] = 255;
    } else {
      rgba[0] = p[2];
      rgba[1] = p[1];
      rgba[2] = p[0];
      rgba[3] = bits == 32 ? p[3] : 255;
    }
  };
  std::vector<uint8_t> pal;
  if (cmtype == 1) {
    const int eb = (cm_bits + 7) / 8;
    if (pos + (size_t)cm_len * eb > d.size()) { *err = "truncated TGA palette"; return false; }
    if (base == 1) {
      if (cm_bits != 15 && cm_bits != 16 && cm_bits != 24 && cm_bits != 32) { *err = "unsupported TGA palette"; return false; }
      pal.resize((size_t)cm_len * 4);
      for (int i = 0; i < cm_len; ++i) decode(d.data() + pos + (size_t)i * eb, cm_bits, &pal[4 * (size_t)i]);
    }
    pos += (size_t)cm_len * eb;
  }
  const int pb = (bpp + 7) / 8;
  const size_t npx = (size_t)w * h;
  // no allocation beyond what the file can hold: raw pixels, or 128 per run-length packet
  if ((!rle && pos + npx * pb > d.size()) || (rle && npx > 128 * (d.size() - std::min(pos, d.size())))) {
    *err = "truncated TGA file";
    return false;
  }
  std::vector<uint8_t> px(npx * 4);
  auto put = [&](size_t k, const uint8_t* p) {
    if (base == 1) {
      const int idx = p[0] - cm_first;
      for (int c = 0; c < 4; ++c) px[4 * k + c] = idx >= 0 && idx < cm_len ? pal[4 * (size_t)idx + c] : 0;
    } else {
      decode(p, bpp, &px[4 * k]);
    }
  };
  for (size_t k = 0; k < npx;) {
    if (!rle) {
      if (pos + pb > d.size()) { *err = "truncated TGA file"; return false; }
      put(k++, d.data() + pos);
      pos += pb;
      continue;
    }
    if (pos >= d.size()) { *err = "truncated TGA file"; return false; }
    const int head = d[pos++], n = (head & 127) + 1;
    if (head & 128) {
      if (pos + pb > d.size()) { *err = "truncated TGA file"; return false; }
      for (int r = 0; r < n && k < npx; ++r) put(k++, d.data() + pos);
      pos += pb;
    } else {
      for (int r = 0; r < n && k < npx; ++r) {
        if (pos + pb > d.size()) { *err = "truncated TGA file"; return false; }
        put(k++, d.data() + pos);
        pos += pb;
      }
    }
  }
  const bool top_down = (desc & 0x20) != 0;
  out->width = w;
  out->height = h;
  out->hdr = false;
  out->rgba.resize(npx * 4);
  for (int y = 0; y < h; ++y) {
    const size_t src = (size_t)(top_down ? y : h - 1 - y) * w;
    for (int x = 0; x < w; ++x)
      for (int c = 0; c < 4; ++c) out->rgba[4 * ((size_t)y * w + x) + c] = px[4 * (src + x) + c];
  }
  return true;
}

// binary PGM (P5, maxval <= 255): grey replicated to R, G, B
bool load_pgm(const std::vector<uint8_t>& d, Image* out, std::string* err) {
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
  if (fields < 4 || tok[0] != "P5") { *err = "not a binary PGM file"; return false; }
  const int w = atoi(tok[1].c_str()), h = atoi(tok[2].c_str()), mx = atoi(tok[3].c_str());
  if (w <= 0 || h <= 0 || mx <= 0 || mx > 255 || d.size() < pos + (size_t)w * h) { *err = "truncated PGM file"; return false; }
  out->width = w; out->height = h; out->hdr = false;
  out->rgba.assign((size_t)w * h * 4, 255.0f);
  for (size_t i = 0; i < (size_t)w * h; ++i)
    for (int c = 0; c < 3; ++c) out->rgba[4 * i + c] = (float)d[pos + i];
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
  if (e == "pgm") return load_pgm(d, out, err);
  if (e == "bmp") return load_bmp(d, out, err);
  if (e == "tga") return load_tga(d, out, err);
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
