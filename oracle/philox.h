// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw, "Parallel random
// numbers: as easy as 1, 2, 3", SC'11), written from the paper for the CPU checkers.
//
// TEST INFRASTRUCTURE: this header belongs to the oracle (CPU restatement) and to the
// host shim that runs the reference integrator on the CPU. The product library has its
// own device/host implementation in illume_gb300/csrc/common/philox.cuh; the tests check
// that both produce the same words.
//
// Stream layout shared by every implementation in this project:
//   counter = (pixel, sample, bounce_slot, block), key = (seed, job)
//   bounce_slot 0 = camera ray generation, slot j+1 = bounce j of the path loop.
//   Uniform floats are taken lane by lane: lane d of block d/4.
//   u = ((word >> 8) + 1) * 2^-24, a float in (0, 1] like curand_uniform's range.
#pragma once
#include <stdint.h>

namespace philox {

static inline void round1(uint32_t c[4], const uint32_t k[2]) {
  const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
  const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
  const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
  const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
  const uint32_t n0 = hi1 ^ c[1] ^ k[0];
  const uint32_t n2 = hi0 ^ c[3] ^ k[1];
  c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
}

static inline void philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
  uint32_t k[2] = {key[0], key[1]};
  for (int r = 0; r < 10; ++r) {
    if (r) { k[0] += 0x9E3779B9u; k[1] += 0xBB67AE85u; }
    round1(c, k);
  }
  out[0] = c[0]; out[1] = c[1]; out[2] = c[2]; out[3] = c[3];
}

static inline float word_to_unit(uint32_t w) {
  return (float)((w >> 8) + 1u) * (1.0f / 16777216.0f);
}

// Sequential view of one (pixel, sample, bounce_slot) stream: next() returns lane 0, 1, ...
struct Stream {
  uint32_t ctr[4];
  uint32_t key[2];
  uint32_t buf[4];
  uint32_t dim;
  void init(uint32_t pixel, uint32_t sample, uint32_t slot, uint32_t seed, uint32_t job) {
    ctr[0] = pixel; ctr[1] = sample; ctr[2] = slot; ctr[3] = 0;
    key[0] = seed; key[1] = job;
    dim = 0;
  }
  float next() {
    if ((dim & 3u) == 0) {
      uint32_t c[4] = {ctr[0], ctr[1], ctr[2], dim >> 2};
      philox4x32_10(c, key, buf);
    }
    return word_to_unit(buf[dim++ & 3u]);
  }
};

}  // namespace philox
