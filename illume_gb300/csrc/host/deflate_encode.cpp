// zlib / deflate encoder (see deflate_encode.h), written from RFC 1950 and RFC 1951.
#include "deflate_encode.h"

#include <algorithm>
#include <atomic>
#include <queue>
#include <thread>
#include <utility>

namespace illume {

namespace {

constexpr int kWindow = 1 << 15;         // deflate's largest distance
constexpr int kMinMatch = 3, kMaxMatch = 258;
constexpr int kHashBits = 15;
constexpr int kMaxChain = 32;            // candidates tried per position
constexpr int kGoodMatch = 16;           // once a match is this long, at most 4 more candidates
constexpr int kNiceMatch = 128;          // a match this long ends the search
constexpr int kLazyLimit = 32;           // shorter matches wait one position for a longer one
constexpr size_t kBlockSymbols = 1 << 15;

// RFC 1951 3.2.5: length codes 257..285 and distance codes 0..29 (base, extra bits)
constexpr int kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                              31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
constexpr int kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
constexpr int kDistBase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,    65,    97,    129,
                               193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
constexpr int kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
// RFC 1951 3.2.7: the order in which the code-length code's lengths are stored
constexpr int kClOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

int len_code(int len) {   // index into kLenBase
  int k = 28;
  while (kLenBase[k] > len) --k;
  return k;
}
int dist_code(int dist) {
  int lo = 0, hi = 29;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (kDistBase[mid] <= dist) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Bits packed from the least significant end, as deflate stores them.
struct BitWriter {
  std::vector<uint8_t>& out;
  uint64_t acc = 0;
  int nbits = 0;
  void put(uint32_t bits, int n) {
    acc |= (uint64_t)bits << nbits;
    nbits += n;
    while (nbits >= 8) {
      out.push_back((uint8_t)acc);
      acc >>= 8;
      nbits -= 8;
    }
  }
  void flush() {
    if (nbits > 0) out.push_back((uint8_t)acc);
    acc = 0;
    nbits = 0;
  }
};

// A literal (dist 0) or a match of `v` bytes at distance `dist`.
struct Sym { uint16_t v, dist; };

// At least two used symbols, so that every tree is a proper (complete) code.
void at_least_two(std::vector<uint32_t>& f) {
  int used = 0;
  for (uint32_t x : f) used += x > 0;
  for (size_t i = 0; used < 2 && i < f.size(); ++i)
    if (f[i] == 0) {
      f[i] = 1;
      ++used;
    }
}

// Huffman code lengths for the frequencies, at most max_len bits: the tree of a priority
// queue (ties by node index, so the result is deterministic); a tree that is too deep is
// rebuilt from frequencies halved (rounded up: no used symbol drops out) until it fits.
std::vector<uint8_t> code_lengths(std::vector<uint32_t> f, int max_len) {
  const int n = (int)f.size();
  std::vector<uint8_t> len(n, 0);
  for (;;) {
    std::vector<int> left, right;
    std::vector<uint64_t> w;
    using Item = std::pair<uint64_t, int>;
    std::priority_queue<Item, std::vector<Item>, std::greater<Item>> q;
    for (int i = 0; i < n; ++i)
      if (f[i] > 0) {
        w.push_back(f[i]);
        left.push_back(-1 - i);   // leaf: -1 - symbol
        right.push_back(-1);
        q.push({f[i], (int)w.size() - 1});
      }
    while (q.size() > 1) {
      const Item a = q.top();
      q.pop();
      const Item b = q.top();
      q.pop();
      w.push_back(a.first + b.first);
      left.push_back(a.second);
      right.push_back(b.second);
      q.push({a.first + b.first, (int)w.size() - 1});
    }
    std::fill(len.begin(), len.end(), 0);
    int deepest = 0;
    std::vector<std::pair<int, int>> st{{q.top().second, 0}};
    while (!st.empty()) {
      const auto [node, d] = st.back();
      st.pop_back();
      if (left[node] < 0) {
        len[-1 - left[node]] = (uint8_t)d;
        deepest = std::max(deepest, d);
        continue;
      }
      st.push_back({left[node], d + 1});
      st.push_back({right[node], d + 1});
    }
    if (deepest <= max_len) return len;
    for (uint32_t& x : f)
      if (x > 0) x = (x + 1) / 2;
  }
}

// Canonical codes of the lengths (RFC 1951 3.2.2), bit-reversed for LSB-first output.
std::vector<uint16_t> codes_of(const std::vector<uint8_t>& len) {
  int count[16] = {0};
  for (uint8_t l : len)
    if (l) ++count[l];
  int next[16] = {0};
  int code = 0;
  for (int bits = 1; bits <= 15; ++bits) {
    code = (code + count[bits - 1]) << 1;
    next[bits] = code;
  }
  std::vector<uint16_t> out(len.size(), 0);
  for (size_t i = 0; i < len.size(); ++i) {
    if (!len[i]) continue;
    const int c = next[len[i]]++;
    int r = 0;
    for (int b = 0; b < len[i]; ++b) r |= ((c >> b) & 1) << (len[i] - 1 - b);
    out[i] = (uint16_t)r;
  }
  return out;
}

void write_block(BitWriter& bw, const std::vector<Sym>& syms, bool final) {
  std::vector<uint32_t> lf(286, 0), df(30, 0);
  for (const Sym& s : syms) {
    if (s.dist == 0) {
      ++lf[s.v];
    } else {
      ++lf[257 + len_code(s.v)];
      ++df[dist_code(s.dist)];
    }
  }
  lf[256] = 1;
  at_least_two(lf);
  at_least_two(df);
  const std::vector<uint8_t> ll = code_lengths(lf, 15), dl = code_lengths(df, 15);
  int hlit = 286, hdist = 30;
  while (hlit > 257 && ll[hlit - 1] == 0) --hlit;
  while (hdist > 1 && dl[hdist - 1] == 0) --hdist;
  // the two trees' lengths, run-length coded: 16 repeats the previous length 3-6 times,
  // 17 and 18 give 3-10 and 11-138 zeros
  std::vector<uint8_t> all(ll.begin(), ll.begin() + hlit);
  all.insert(all.end(), dl.begin(), dl.begin() + hdist);
  std::vector<std::pair<int, int>> rle;   // (symbol, extra-bit value)
  for (size_t i = 0; i < all.size();) {
    const uint8_t v = all[i];
    size_t r = 1;
    while (i + r < all.size() && all[i + r] == v) ++r;
    i += r;
    if (v == 0) {
      while (r >= 11) {
        const size_t t = std::min<size_t>(r, 138);
        rle.push_back({18, (int)t - 11});
        r -= t;
      }
      if (r >= 3) {
        rle.push_back({17, (int)r - 3});
        r = 0;
      }
      while (r--) rle.push_back({0, 0});
    } else {
      rle.push_back({v, 0});
      --r;
      while (r >= 3) {
        const size_t t = std::min<size_t>(r, 6);
        rle.push_back({16, (int)t - 3});
        r -= t;
      }
      while (r--) rle.push_back({v, 0});
    }
  }
  std::vector<uint32_t> cf(19, 0);
  for (const auto& e : rle) ++cf[e.first];
  at_least_two(cf);
  const std::vector<uint8_t> cl = code_lengths(cf, 7);
  int hclen = 19;
  while (hclen > 4 && cl[kClOrder[hclen - 1]] == 0) --hclen;
  const std::vector<uint16_t> lc = codes_of(ll), dc = codes_of(dl), cc = codes_of(cl);

  bw.put(final ? 1 : 0, 1);
  bw.put(2, 2);   // dynamic Huffman codes
  bw.put(hlit - 257, 5);
  bw.put(hdist - 1, 5);
  bw.put(hclen - 4, 4);
  for (int k = 0; k < hclen; ++k) bw.put(cl[kClOrder[k]], 3);
  for (const auto& e : rle) {
    bw.put(cc[e.first], cl[e.first]);
    if (e.first == 16) bw.put(e.second, 2);
    else if (e.first == 17) bw.put(e.second, 3);
    else if (e.first == 18) bw.put(e.second, 7);
  }
  for (const Sym& s : syms) {
    if (s.dist == 0) {
      bw.put(lc[s.v], ll[s.v]);
      continue;
    }
    const int k = len_code(s.v), d = dist_code(s.dist);
    bw.put(lc[257 + k], ll[257 + k]);
    if (kLenExtra[k]) bw.put(s.v - kLenBase[k], kLenExtra[k]);
    bw.put(dc[d], dl[d]);
    if (kDistExtra[d]) bw.put(s.dist - kDistBase[d], kDistExtra[d]);
  }
  bw.put(lc[256], ll[256]);
}


// The deflate blocks of data[begin, end), matches reaching back at most into the 32 KB
// before `begin` (which the decoder has already produced). A segment that is not the last
// ends with an empty stored block, which brings the stream to a byte boundary so that
// the next segment's bytes can follow it directly.
std::vector<uint8_t> deflate_segment(const uint8_t* data, size_t begin, size_t end, bool last) {
  const size_t n = end;
  std::vector<uint8_t> out;
  out.reserve((end - begin) + (end - begin) / 64 + 64);
  BitWriter bw{out};
  std::vector<int> head(1 << kHashBits, -1), prev(kWindow, -1);
  auto hash3 = [&](size_t i) {
    return (int)(((uint32_t)data[i] << 10 ^ (uint32_t)data[i + 1] << 5 ^ (uint32_t)data[i + 2]) & ((1u << kHashBits) - 1));
  };
  auto insert = [&](size_t i) {
    if (i + 2 >= n) return;
    const int h = hash3(i);
    prev[i & (kWindow - 1)] = head[h];
    head[h] = (int)i;
  };
  // the longest earlier match of the bytes at i within the window (0 when under 3 bytes)
  auto longest = [&](size_t i, int* dist) {
    if (i + kMinMatch > n) return 0;
    const int maxlen = (int)std::min<size_t>(kMaxMatch, n - i);
    int best = 0, cand = head[hash3(i)], chain = kMaxChain;
    if (cand < 0) return 0;
    while (cand >= 0 && chain-- > 0 && i - (size_t)cand <= (size_t)kWindow) {
      if (data[cand + best] == data[i + best]) {
        int l = 0;
        while (l < maxlen && data[cand + l] == data[i + l]) ++l;
        if (l > best) {
          best = l;
          *dist = (int)(i - cand);
          if (l >= std::min(maxlen, kNiceMatch)) break;
          if (l >= kGoodMatch) chain = std::min(chain, 4);
        }
      }
      const int next = prev[cand & (kWindow - 1)];
      if (next >= cand) break;   // a slot reused by a later position
      cand = next;
    }
    return best >= kMinMatch ? best : 0;
  };
  // the window before the segment: its positions are match candidates, not output
  for (size_t k = begin > (size_t)kWindow ? begin - kWindow : 0; k < begin; ++k) insert(k);
  std::vector<Sym> syms;
  syms.reserve(kBlockSymbols + 2);
  auto emit = [&](Sym s) {
    syms.push_back(s);
    if (syms.size() >= kBlockSymbols) {
      write_block(bw, syms, false);
      syms.clear();
    }
  };
  size_t i = begin;
  int known_len = -1, known_dist = 0;   // the match at i when the previous step found it
  while (i < n) {
    int d1 = known_dist;
    const int l1 = known_len >= 0 ? known_len : longest(i, &d1);
    known_len = -1;
    if (l1 == 0) {
      emit(Sym{data[i], 0});
      insert(i);
      ++i;
      continue;
    }
    insert(i);
    if (l1 < kLazyLimit && i + 1 < n) {
      int d2 = 0;
      const int l2 = longest(i + 1, &d2);
      if (l2 > l1) {   // a literal here, and the longer match from the next position on
        emit(Sym{data[i], 0});
        ++i;
        known_len = l2;
        known_dist = d2;
        continue;
      }
    }
    emit(Sym{(uint16_t)l1, (uint16_t)d1});
    for (int k = 1; k < l1; ++k) insert(i + k);
    i += l1;
  }
  write_block(bw, syms, last);
  if (!last) {
    bw.put(0, 3);   // stored block, not final
    bw.flush();
    out.push_back(0x00);
    out.push_back(0x00);
    out.push_back(0xff);
    out.push_back(0xff);
  }
  bw.flush();
  return out;
}

}  // namespace

std::vector<uint8_t> zlib_compress(const uint8_t* data, size_t n) {
  // fixed-size segments, compressed on the host threads and joined in order: the bytes do
  // not depend on the number of threads
  constexpr size_t kSegment = size_t(1) << 19;
  const size_t nseg = std::max<size_t>(1, (n + kSegment - 1) / kSegment);
  std::vector<std::vector<uint8_t>> seg(nseg);
  std::atomic<size_t> next{0};
  auto work = [&]() {
    for (size_t k = next++; k < nseg; k = next++)
      seg[k] = deflate_segment(data, k * kSegment, std::min(n, (k + 1) * kSegment), k + 1 == nseg);
  };
  const int threads = (int)std::min<size_t>(nseg, std::max(1u, std::min(16u, std::thread::hardware_concurrency())));
  std::vector<std::thread> pool;
  for (int t = 1; t < threads; ++t) pool.emplace_back(work);
  work();
  for (auto& th : pool) th.join();
  std::vector<uint8_t> out{0x78, 0x9c};   // deflate, 32 KB window, default level; (0x789c % 31) == 0
  size_t total = 6;
  for (const auto& v : seg) total += v.size();
  out.reserve(total);
  for (const auto& v : seg) out.insert(out.end(), v.begin(), v.end());
  // Adler-32 (RFC 1950 8.2), reduced every 5552 bytes (the most that cannot overflow)
  uint32_t a = 1, b = 0;
  for (size_t k = 0; k < n;) {
    const size_t e = std::min(n, k + 5552);
    for (; k < e; ++k) {
      a += data[k];
      b += a;
    }
    a %= 65521;
    b %= 65521;
  }
  const uint32_t adler = (b << 16) | a;
  out.push_back((uint8_t)(adler >> 24));
  out.push_back((uint8_t)(adler >> 16));
  out.push_back((uint8_t)(adler >> 8));
  out.push_back((uint8_t)adler);
  return out;
}

}  // namespace illume
