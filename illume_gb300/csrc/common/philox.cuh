// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), stateless and counter based.
//
// Stream layout: counter = (pixel, sample, bounce_slot, block), key = (seed, job).
// bounce_slot 0 = camera ray, slot j + 1 = bounce j. The d-th uniform of a slot is lane
// d % 4 of block d / 4, mapped to (0, 1] as ((word >> 8) + 1) * 2^-24. A path's numbers
// therefore depend only on (pixel, sample, bounce, d): never on scheduling, on which
// other paths or jobs share the GPU, or on the number of GPUs.
#pragma once

#include <stdint.h>

namespace illume {

struct Philox4 { uint32_t x, y, z, w; };

__host__ __device__ __forceinline__ Philox4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                                            uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
#ifdef __CUDA_ARCH__
    const uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
    const uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
#else
    const uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
    const uint32_t lo0 = (uint32_t)p0, hi0 = (uint32_t)(p0 >> 32);
    const uint32_t lo1 = (uint32_t)p1, hi1 = (uint32_t)(p1 >> 32);
#endif
    const uint32_t n0 = hi1 ^ c1 ^ k0;
    const uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
  }
  return Philox4{c0, c1, c2, c3};
}

__host__ __device__ __forceinline__ float philox_unit(uint32_t w) {
  return (float)((w >> 8) + 1u) * (1.0f / 16777216.0f);
}

// Sequential reader over one (pixel, sample, slot) stream.
struct RngStream {
  uint32_t pixel, sample, slot, seed, job, dim;
  Philox4 buf;
  __device__ __forceinline__ void init(uint32_t p, uint32_t s, uint32_t sl, uint32_t sd, uint32_t jb) {
    pixel = p; sample = s; slot = sl; seed = sd; job = jb; dim = 0;
  }
  __device__ __forceinline__ void skip(uint32_t n) {
    // position the stream at dimension `n` (the block is generated on the next call)
    dim = n;
    if (n & 3u) buf = philox4x32_10(pixel, sample, slot, n >> 2, seed, job);
  }
  __device__ __forceinline__ float next() {
    if ((dim & 3u) == 0) buf = philox4x32_10(pixel, sample, slot, dim >> 2, seed, job);
    const uint32_t lane = dim++ & 3u;
    const uint32_t w = lane == 0 ? buf.x : lane == 1 ? buf.y : lane == 2 ? buf.z : buf.w;
    return philox_unit(w);
  }
};

}  // namespace illume
