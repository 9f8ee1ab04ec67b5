// Host stand-ins for the CUDA runtime, texture and cuRAND names that the reference
// renderer's sources use, so that those sources compile unchanged with g++ and run on
// the CPU.
//
// TEST INFRASTRUCTURE ONLY. This shim is used by oracle/build_ref.py to build the
// reference's own integrator for the host (output in oracle/_ref/). Nothing in the
// product links it. Without __CUDACC__ the reference's KERNEL_ARGS2 macro expands to
// nothing (src/renderer.cu:29-37), so its __global__ functions become plain host
// functions; the driver (oracle/ref_driver.cpp) calls them once per thread index with
// the thread-local blockIdx/threadIdx below.
//
// Random numbers: curandState is replaced by a Philox4x32-10 stream keyed by
// (pixel, sample, bounce_slot); see oracle/philox.h. The driver sets the key fields
// before each launch, so curand_init's seed is not used.
// Textures: tex2D reads a host copy of the array with wrap addressing and normalised
// coordinates; float4 arrays are filtered bilinearly with exact FP32 weights, uchar4
// arrays are point sampled (the filter modes src/texture.cu:110-115 selects).
#pragma once

#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#include <math.h>

#include "../philox.h"

#define __device__
#define __host__
#define __global__
#define __forceinline__ inline

struct uint3 { unsigned x, y, z; };
struct dim3 { unsigned x = 1, y = 1, z = 1; };
struct float4 { float x, y, z, w; };
struct uchar4 { unsigned char x, y, z, w; };

extern thread_local uint3 blockIdx;
extern thread_local uint3 threadIdx;
extern thread_local uint3 blockDim;

typedef int cudaError_t;
enum { cudaSuccess = 0, cudaErrorMemoryAllocation = 2 };
static inline const char* cudaGetErrorString(cudaError_t e) { return e ? "host shim error" : "no error"; }

enum cudaMemcpyKind { cudaMemcpyHostToHost, cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost, cudaMemcpyDeviceToDevice };
enum cudaLimit { cudaLimitMallocHeapSize };

template <typename T>
static inline cudaError_t cudaMalloc(T** p, size_t n) {
  *p = (T*)calloc(n ? n : 1, 1);
  return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
static inline cudaError_t cudaFree(void* p) { free(p); return cudaSuccess; }
static inline cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind) {
  if (n) memcpy(d, s, n);
  return cudaSuccess;
}
static inline cudaError_t cudaDeviceSetLimit(cudaLimit, size_t) { return cudaSuccess; }

typedef struct ShimEvent* cudaEvent_t;
struct ShimEvent { double t; };
double illume_shim_now_ms();
static inline cudaError_t cudaEventCreate(cudaEvent_t* e) { *e = new ShimEvent{0}; return cudaSuccess; }
static inline cudaError_t cudaEventRecord(cudaEvent_t e, int) { e->t = illume_shim_now_ms(); return cudaSuccess; }
static inline cudaError_t cudaEventSynchronize(cudaEvent_t) { return cudaSuccess; }
static inline cudaError_t cudaEventElapsedTime(float* ms, cudaEvent_t a, cudaEvent_t b) { *ms = (float)(b->t - a->t); return cudaSuccess; }

// ---- arrays and texture objects ----
struct cudaChannelFormatDesc { int bytes; int is_float; };
template <typename T> cudaChannelFormatDesc cudaCreateChannelDesc();
template <> inline cudaChannelFormatDesc cudaCreateChannelDesc<float4>() { return {16, 1}; }
template <> inline cudaChannelFormatDesc cudaCreateChannelDesc<uchar4>() { return {4, 0}; }

struct cudaArray { int width, height, bytes, is_float; unsigned char* data; };
static inline cudaError_t cudaMallocArray(cudaArray** a, const cudaChannelFormatDesc* d, size_t w, size_t h) {
  cudaArray* r = new cudaArray;
  r->width = (int)w; r->height = (int)h; r->bytes = d->bytes; r->is_float = d->is_float;
  r->data = (unsigned char*)calloc(w * (h ? h : 1), d->bytes);
  *a = r;
  return cudaSuccess;
}
static inline cudaError_t cudaMemcpyToArray(cudaArray* a, size_t, size_t, const void* src, size_t n, cudaMemcpyKind) {
  memcpy(a->data, src, n);
  return cudaSuccess;
}
static inline cudaError_t cudaFreeArray(cudaArray* a) { if (a) { free(a->data); delete a; } return cudaSuccess; }

enum cudaResourceType { cudaResourceTypeArray };
struct cudaResourceDesc { cudaResourceType resType; union { struct { cudaArray* array; } array; } res; };
enum cudaTextureAddressMode { cudaAddressModeWrap, cudaAddressModeClamp };
enum cudaTextureFilterMode { cudaFilterModePoint, cudaFilterModeLinear };
enum cudaTextureReadMode { cudaReadModeElementType };
struct cudaTextureDesc {
  cudaTextureAddressMode addressMode[3];
  cudaTextureFilterMode filterMode;
  cudaTextureReadMode readMode;
  int normalizedCoords;
};
typedef unsigned long long cudaTextureObject_t;
struct ShimTexture { cudaArray* a; int linear; };
static inline cudaError_t cudaCreateTextureObject(cudaTextureObject_t* t, const cudaResourceDesc* r, const cudaTextureDesc* d, const void*) {
  ShimTexture* s = new ShimTexture{r->res.array.array, d->filterMode == cudaFilterModeLinear};
  *t = (cudaTextureObject_t)(uintptr_t)s;
  return cudaSuccess;
}
static inline cudaError_t cudaDestroyTextureObject(cudaTextureObject_t t) { delete (ShimTexture*)(uintptr_t)t; return cudaSuccess; }

static inline int shim_wrap(int i, int n) { int r = i % n; return r < 0 ? r + n : r; }

template <typename T> T tex2D(cudaTextureObject_t t, float x, float y);
template <> inline float4 tex2D<float4>(cudaTextureObject_t t, float x, float y) {
  const ShimTexture* s = (const ShimTexture*)(uintptr_t)t;
  const cudaArray* a = s->a;
  const float* d = (const float*)a->data;
  const int w = a->width, h = a->height;
  if (!s->linear) {
    int ix = shim_wrap((int)floorf(x * (float)w), w), iy = shim_wrap((int)floorf(y * (float)h), h);
    const float* p = d + 4 * ((size_t)iy * w + ix);
    return float4{p[0], p[1], p[2], p[3]};
  }
  const float fx = x * (float)w - 0.5f, fy = y * (float)h - 0.5f;
  const float x0f = floorf(fx), y0f = floorf(fy);
  const float ax = fx - x0f, ay = fy - y0f;
  const int x0 = shim_wrap((int)x0f, w), x1 = shim_wrap((int)x0f + 1, w);
  const int y0 = shim_wrap((int)y0f, h), y1 = shim_wrap((int)y0f + 1, h);
  float out[4];
  for (int c = 0; c < 4; ++c) {
    const float t00 = d[4 * ((size_t)y0 * w + x0) + c], t10 = d[4 * ((size_t)y0 * w + x1) + c];
    const float t01 = d[4 * ((size_t)y1 * w + x0) + c], t11 = d[4 * ((size_t)y1 * w + x1) + c];
    const float top = t00 * (1.0f - ax) + t10 * ax;
    const float bot = t01 * (1.0f - ax) + t11 * ax;
    out[c] = top * (1.0f - ay) + bot * ay;
  }
  return float4{out[0], out[1], out[2], out[3]};
}
template <> inline uchar4 tex2D<uchar4>(cudaTextureObject_t t, float x, float y) {
  const ShimTexture* s = (const ShimTexture*)(uintptr_t)t;
  const cudaArray* a = s->a;
  const int w = a->width, h = a->height;
  int ix = shim_wrap((int)floorf(x * (float)w), w), iy = shim_wrap((int)floorf(y * (float)h), h);
  const unsigned char* p = a->data + 4 * ((size_t)iy * w + ix);
  return uchar4{p[0], p[1], p[2], p[3]};
}

// ---- cuRAND stand-in ----
struct curandState {
  uint32_t pixel, sample, slot, seed, job, dim;
  uint32_t buf[4];
};
static inline void curand_init(unsigned long long, unsigned long long, unsigned long long, curandState* s) {
  // Key fields are assigned by the driver (pixel, sample, bounce slot); see header comment.
  s->dim = 0;
}
static inline float curand_uniform(curandState* s) {
  if ((s->dim & 3u) == 0) {
    uint32_t c[4] = {s->pixel, s->sample, s->slot, s->dim >> 2};
    uint32_t k[2] = {s->seed, s->job};
    philox::philox4x32_10(c, k, s->buf);
  }
  return philox::word_to_unit(s->buf[s->dim++ & 3u]);
}
