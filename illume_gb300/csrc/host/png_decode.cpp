// PNG decoding for 8-bit (LDR) bitmap textures.
//
// The reference loads every non-.hdr bitmap with stb_image as 8-bit RGBA
// (src/imageio.cpp:6-13, src/texture.cu:57-63): grey becomes (g, g, g, 255), grey +
// alpha (g, g, g, a), RGB gets alpha 255, palette images are expanded, 16-bit samples
// keep their high byte, and sub-byte grey samples are scaled to 0..255. This decoder
// produces the same texels for PNG files, written from the specifications: the zlib
// container (RFC 1950), deflate (RFC 1951: stored, fixed-Huffman and dynamic-Huffman
// blocks) and PNG (ISO/IEC 15948: chunks, the five scanline filters, Adam7 interlace,
// bit depths 1-16, colour types 0, 2, 3, 4, 6, tRNS transparency).
#include "png_decode.h"

#include <string.h>

namespace illume {

namespace {

// ---------------------------------------------------------------- inflate
struct Bits {
  const uint8_t* p;
  size_t n, pos = 0;
  uint32_t buf = 0;
  int cnt = 0;
  bool over = false;
  int get(int k) {   // k <= 24 bits, least significant first
    while (cnt < k) {
      if (pos >= n) { over = true; return 0; }
      buf |= (uint32_t)p[pos++] << cnt;
      cnt += 8;
    }
    const int v = (int)(buf & ((1u << k) - 1));
    buf >>= k;
    cnt -= k;
    return v;
  }
  void align() { buf = 0; cnt = 0; }
};

// Canonical Huffman code: symbols sorted by code length, counts per length.
struct Huff {
  uint16_t count[16];
  uint16_t sym[320];
  bool build(const uint8_t* len, int nsym) {
    memset(count, 0, sizeof(count));
    for (int i = 0; i < nsym; ++i) count[len[i]]++;
    count[0] = 0;
    int left = 1;
    for (int l = 1; l < 16; ++l) {
      left = 2 * left - count[l];
      if (left < 0) return false;   // over-subscribed
    }
    uint16_t off[16];
    off[1] = 0;
    for (int l = 1; l < 15; ++l) off[l + 1] = off[l] + count[l];
    for (int i = 0; i < nsym; ++i)
      if (len[i]) sym[off[len[i]]++] = (uint16_t)i;
    return true;
  }
  // Walks the code one bit at a time: codes of length l occupy [first, first + count[l]).
  int decode(Bits& b) const {
    int code = 0, first = 0, index = 0;
    for (int l = 1; l < 16; ++l) {
      code |= b.get(1);
      const int c = count[l];
      if (code - first < c) return sym[index + code - first];
      index += c;
      first = (first + c) << 1;
      code <<= 1;
      if (b.over) return -1;
    }
    return -1;
  }
};

const uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31,
                               35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129, 193,
                                257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

bool inflate_codes(Bits& b, const Huff& lit, const Huff& dist, std::vector<uint8_t>& out, size_t limit, std::string* err) {
  for (;;) {
    const int s = lit.decode(b);
    if (s < 0) { *err = "PNG: bad deflate code"; return false; }
    if (s < 256) {
      if (out.size() >= limit) { *err = "PNG: image data longer than expected"; return false; }
      out.push_back((uint8_t)s);
      continue;
    }
    if (s == 256) return true;
    const int li = s - 257;
    if (li >= 29) { *err = "PNG: bad length code"; return false; }
    const int len = kLenBase[li] + b.get(kLenExtra[li]);
    const int di = dist.decode(b);
    if (di < 0 || di >= 30) { *err = "PNG: bad distance code"; return false; }
    const size_t d = kDistBase[di] + b.get(kDistExtra[di]);
    if (b.over) { *err = "PNG: truncated deflate stream"; return false; }
    if (d > out.size()) { *err = "PNG: distance beyond the start of the data"; return false; }
    if (out.size() + len > limit) { *err = "PNG: image data longer than expected"; return false; }
    const size_t from = out.size() - d;
    for (int k = 0; k < len; ++k) out.push_back(out[from + k]);
  }
}

uint32_t be32_adler(const uint8_t* p) {
  return (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | p[3];
}
uint32_t adler32(const uint8_t* p, size_t n);

// zlib stream -> bytes (at most `limit`).
bool zlib_inflate(const std::vector<uint8_t>& in, size_t limit, std::vector<uint8_t>* out, std::string* err) {
  if (in.size() < 6) { *err = "PNG: truncated zlib stream"; return false; }
  const int cmf = in[0], flg = in[1];
  if ((cmf & 15) != 8 || (cmf >> 4) > 7 || ((cmf << 8) | flg) % 31 != 0 || (flg & 32)) {
    *err = "PNG: bad zlib header";
    return false;
  }
  Bits b{in.data() + 2, in.size() - 2};
  std::vector<uint8_t>& o = *out;
  o.clear();
  o.reserve(limit);
  int final_block = 0;
  while (!final_block) {
    final_block = b.get(1);
    const int type = b.get(2);
    if (b.over) { *err = "PNG: truncated deflate stream"; return false; }
    if (type == 0) {
      b.align();
      if (b.pos + 4 > b.n) { *err = "PNG: truncated stored block"; return false; }
      const int len = b.p[b.pos] | b.p[b.pos + 1] << 8, nlen = b.p[b.pos + 2] | b.p[b.pos + 3] << 8;
      b.pos += 4;
      if ((len ^ 0xffff) != nlen || b.pos + len > b.n) { *err = "PNG: bad stored block"; return false; }
      if (o.size() + len > limit) { *err = "PNG: image data longer than expected"; return false; }
      o.insert(o.end(), b.p + b.pos, b.p + b.pos + len);
      b.pos += len;
      b.align();
    } else if (type == 1) {
      struct Fixed { Huff lit, dist; };
      static const Fixed fixed = [] {   // the fixed codes of RFC 1951 section 3.2.6
        Fixed f;
        uint8_t l[288];
        for (int i = 0; i < 144; ++i) l[i] = 8;
        for (int i = 144; i < 256; ++i) l[i] = 9;
        for (int i = 256; i < 280; ++i) l[i] = 7;
        for (int i = 280; i < 288; ++i) l[i] = 8;
        f.lit.build(l, 288);
        uint8_t d[30];
        for (int i = 0; i < 30; ++i) d[i] = 5;
        f.dist.build(d, 30);
        return f;
      }();
      if (!inflate_codes(b, fixed.lit, fixed.dist, o, limit, err)) return false;
    } else if (type == 2) {
      const int hlit = b.get(5) + 257, hdist = b.get(5) + 1, hclen = b.get(4) + 4;
      static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
      uint8_t cl[19] = {0};
      for (int i = 0; i < hclen; ++i) cl[order[i]] = (uint8_t)b.get(3);
      Huff ch;
      if (b.over || !ch.build(cl, 19)) { *err = "PNG: bad code-length code"; return false; }
      uint8_t lens[320] = {0};
      int k = 0;
      while (k < hlit + hdist) {
        const int s = ch.decode(b);
        if (s < 0) { *err = "PNG: bad code lengths"; return false; }
        if (s < 16) { lens[k++] = (uint8_t)s; continue; }
        int rep = 0;
        uint8_t v = 0;
        if (s == 16) {
          if (k == 0) { *err = "PNG: repeat without a previous length"; return false; }
          v = lens[k - 1];
          rep = 3 + b.get(2);
        } else if (s == 17) {
          rep = 3 + b.get(3);
        } else {
          rep = 11 + b.get(7);
        }
        if (k + rep > hlit + hdist) { *err = "PNG: too many code lengths"; return false; }
        while (rep--) lens[k++] = v;
      }
      Huff lit, dist;
      if (!lit.build(lens, hlit) || !dist.build(lens + hlit, hdist)) { *err = "PNG: bad Huffman table"; return false; }
      if (!inflate_codes(b, lit, dist, o, limit, err)) return false;
    } else {
      *err = "PNG: bad deflate block type";
      return false;
    }
  }
  // Adler-32 of the uncompressed data follows the last block, byte aligned
  const size_t at = b.pos;
  if (at + 4 > b.n || be32_adler(b.p + at) != adler32(o.data(), o.size())) {
    *err = "PNG: zlib checksum mismatch";
    return false;
  }
  return true;
}

// ---------------------------------------------------------------- PNG
uint32_t be32(const uint8_t* p) { return (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | p[3]; }

// CRC-32 of chunk type and data (ISO 3309 polynomial, reflected).
uint32_t chunk_crc(const uint8_t* p, size_t n) {
  struct Table { uint32_t t[256]; };
  static const Table table = [] {
    Table tb;
    for (uint32_t i = 0; i < 256; ++i) {
      uint32_t v = i;
      for (int k = 0; k < 8; ++k) v = (v & 1) ? 0xedb88320u ^ (v >> 1) : v >> 1;
      tb.t[i] = v;
    }
    return tb;
  }();
  uint32_t c = 0xffffffffu;
  for (size_t i = 0; i < n; ++i) c = table.t[(c ^ p[i]) & 0xff] ^ (c >> 8);
  return c ^ 0xffffffffu;
}

uint32_t adler32(const uint8_t* p, size_t n) {
  uint32_t a = 1, b = 0;
  for (size_t i = 0; i < n; ++i) {
    a = (a + p[i]) % 65521u;
    b = (b + a) % 65521u;
  }
  return b << 16 | a;
}

int paeth(int a, int b, int c) {
  const int p = a + b - c, pa = p > a ? p - a : a - p, pb = p > b ? p - b : b - p, pc = p > c ? p - c : c - p;
  if (pa <= pb && pa <= pc) return a;
  return pb <= pc ? b : c;
}

// Reverses the scanline filters of one (sub)image in place: rows of 1 + stride bytes.
bool unfilter(uint8_t* data, int rows, size_t stride, int bpp, std::string* err) {
  uint8_t* prev = nullptr;
  for (int y = 0; y < rows; ++y) {
    uint8_t* row = data + (size_t)y * (stride + 1);
    const int f = row[0];
    uint8_t* x = row + 1;
    for (size_t i = 0; i < stride; ++i) {
      const int a = i >= (size_t)bpp ? x[i - bpp] : 0;
      const int b = prev ? prev[i] : 0;
      const int c = prev && i >= (size_t)bpp ? prev[i - bpp] : 0;
      int v = x[i];
      switch (f) {
        case 0: break;
        case 1: v += a; break;
        case 2: v += b; break;
        case 3: v += (a + b) >> 1; break;
        case 4: v += paeth(a, b, c); break;
        default: *err = "PNG: bad filter type"; return false;
      }
      x[i] = (uint8_t)v;
    }
    prev = x;
  }
  return true;
}

}  // namespace

bool decode_png(const std::vector<uint8_t>& d, Image* out, std::string* err) {
  static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
  if (d.size() < 8 || memcmp(d.data(), sig, 8) != 0) { *err = "not a PNG file"; return false; }
  size_t pos = 8;
  int w = 0, h = 0, depth = 0, ctype = -1, interlace = 0;
  std::vector<uint8_t> idat, plte, trns;
  bool seen_end = false;
  while (pos + 8 <= d.size()) {
    const uint32_t len = be32(&d[pos]);
    const char* type = reinterpret_cast<const char*>(&d[pos + 4]);
    if (pos + 12 + (size_t)len > d.size()) { *err = "PNG: truncated chunk"; return false; }
    const uint8_t* c = &d[pos + 8];
    if (chunk_crc(&d[pos + 4], 4 + (size_t)len) != be32(c + len)) { *err = "PNG: chunk CRC mismatch"; return false; }
    if (!memcmp(type, "IHDR", 4)) {
      if (len < 13) { *err = "PNG: short IHDR"; return false; }
      w = (int)be32(c);
      h = (int)be32(c + 4);
      depth = c[8];
      ctype = c[9];
      if (c[10] != 0 || c[11] != 0) { *err = "PNG: unknown compression or filter method"; return false; }
      interlace = c[12];
    } else if (!memcmp(type, "PLTE", 4)) {
      plte.assign(c, c + len);
    } else if (!memcmp(type, "tRNS", 4)) {
      trns.assign(c, c + len);
    } else if (!memcmp(type, "IDAT", 4)) {
      idat.insert(idat.end(), c, c + len);
    } else if (!memcmp(type, "IEND", 4)) {
      seen_end = true;
      break;
    }
    pos += 12 + (size_t)len;
  }
  if (!seen_end || idat.empty()) { *err = "PNG: missing image data"; return false; }
  if (w <= 0 || h <= 0 || (long long)w * h > (1LL << 28)) { *err = "PNG: bad image size"; return false; }
  const int chans = ctype == 0 ? 1 : ctype == 2 ? 3 : ctype == 3 ? 1 : ctype == 4 ? 2 : ctype == 6 ? 4 : 0;
  const bool depth_ok = (ctype == 0 && (depth == 1 || depth == 2 || depth == 4 || depth == 8 || depth == 16)) ||
                        (ctype == 3 && (depth == 1 || depth == 2 || depth == 4 || depth == 8)) ||
                        ((ctype == 2 || ctype == 4 || ctype == 6) && (depth == 8 || depth == 16));
  if (!chans || !depth_ok || interlace > 1) { *err = "PNG: unsupported colour type / bit depth / interlace"; return false; }
  if (ctype == 3 && (plte.empty() || plte.size() % 3)) { *err = "PNG: missing palette"; return false; }
  const int bits_pp = chans * depth;
  const int bpp = bits_pp >= 8 ? bits_pp / 8 : 1;
  // Adam7 passes: start x, start y, step x, step y (one pass without interlace)
  static const int pass_tab[7][4] = {{0, 0, 8, 8}, {4, 0, 8, 8}, {0, 4, 4, 8}, {2, 0, 4, 4},
                                     {0, 2, 2, 4}, {1, 0, 2, 2}, {0, 1, 1, 2}};
  const int npass = interlace ? 7 : 1;
  size_t total = 0;
  int pw[7], ph[7];
  for (int p = 0; p < npass; ++p) {
    const int* t = interlace ? pass_tab[p] : nullptr;
    pw[p] = t ? (w - t[0] + t[2] - 1) / t[2] : w;
    ph[p] = t ? (h - t[1] + t[3] - 1) / t[3] : h;
    if (pw[p] > 0 && ph[p] > 0) total += (size_t)ph[p] * (1 + ((size_t)pw[p] * bits_pp + 7) / 8);
  }
  std::vector<uint8_t> raw;
  if (!zlib_inflate(idat, total, &raw, err)) return false;
  if (raw.size() != total) { *err = "PNG: image data shorter than expected"; return false; }
  out->width = w;
  out->height = h;
  out->hdr = false;
  out->rgba.assign((size_t)w * h * 4, 0.0f);
  const int maxv = (1 << depth) - 1;
  size_t off = 0;
  for (int p = 0; p < npass; ++p) {
    if (pw[p] <= 0 || ph[p] <= 0) continue;
    const size_t stride = ((size_t)pw[p] * bits_pp + 7) / 8;
    uint8_t* img = raw.data() + off;
    if (!unfilter(img, ph[p], stride, bpp, err)) return false;
    for (int y = 0; y < ph[p]; ++y) {
      const uint8_t* row = img + (size_t)y * (stride + 1) + 1;
      for (int x = 0; x < pw[p]; ++x) {
        int s[4];
        for (int k = 0; k < chans; ++k) {
          if (depth == 16) {
            s[k] = row[(size_t)(x * chans + k) * 2];   // high byte
          } else if (depth == 8) {
            s[k] = row[(size_t)x * chans + k];
          } else {
            const size_t bit = (size_t)x * depth;
            s[k] = (row[bit >> 3] >> (8 - depth - (int)(bit & 7))) & maxv;
          }
        }
        // key transparency compares full-precision samples
        auto sample16 = [&](int k) -> int {
          return depth == 16 ? (row[(size_t)(x * chans + k) * 2] << 8 | row[(size_t)(x * chans + k) * 2 + 1]) : s[k];
        };
        float r, g, b, a = 255.0f;
        if (ctype == 3) {
          const int idx = s[0];
          if ((size_t)idx * 3 + 2 >= plte.size()) { *err = "PNG: palette index out of range"; return false; }
          r = plte[3 * idx]; g = plte[3 * idx + 1]; b = plte[3 * idx + 2];
          if ((size_t)idx < trns.size()) a = trns[idx];
        } else if (ctype == 0 || ctype == 4) {
          const int v = depth < 8 ? s[0] * (255 / maxv) : s[0];
          r = g = b = (float)v;
          if (ctype == 4) a = (float)s[1];
          else if (trns.size() >= 2 && sample16(0) == (trns[0] << 8 | trns[1])) a = 0.0f;
        } else {
          r = (float)s[0]; g = (float)s[1]; b = (float)s[2];
          if (ctype == 6) a = (float)s[3];
          else if (trns.size() >= 6 && sample16(0) == (trns[0] << 8 | trns[1]) &&
                   sample16(1) == (trns[2] << 8 | trns[3]) && sample16(2) == (trns[4] << 8 | trns[5]))
            a = 0.0f;
        }
        const int X = interlace ? pass_tab[p][0] + x * pass_tab[p][2] : x;
        const int Y = interlace ? pass_tab[p][1] + y * pass_tab[p][3] : y;
        float* o = &out->rgba[4 * ((size_t)Y * w + X)];
        o[0] = r; o[1] = g; o[2] = b; o[3] = a;
      }
    }
    off += (size_t)ph[p] * (stride + 1);
  }
  return true;
}

}  // namespace illume
