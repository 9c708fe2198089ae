// cuda_host.h -- TEST INFRASTRUCTURE: run the reference's CUDA device code on
// the CPU, to pin the oracle to the reference's own update rules.
//
// The reference's headers and kernels are compiled by g++ against these
// definitions: CUDA vector types come from cuda_runtime.h; atomics are plain
// sequential read-modify-writes (one emulated thread runs at a time);
// `__shared__` variables become function statics, shared by the threads of
// the CTA being emulated; `__syncthreads()` switches to the next thread of the
// CTA (cooperative contexts, only for kernels that use it); tex2D point-samples
// a registered host image.
#pragma once
#include <cuda_runtime.h>
#include <ucontext.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#undef __shared__
#define __shared__ static

struct EmuIdx {
  unsigned x, y, z;
};
extern EmuIdx threadIdx, blockIdx;
extern dim3 blockDim, gridDim;

inline float __int_as_float(int i) {
  float f;
  std::memcpy(&f, &i, 4);
  return f;
}
inline int __float_as_int(float f) {
  int i;
  std::memcpy(&i, &f, 4);
  return i;
}

inline int atomicAdd(int *a, int v) { int o = *a; *a = o + v; return o; }
inline unsigned atomicAdd(unsigned *a, unsigned v) { unsigned o = *a; *a = o + v; return o; }
inline float atomicAdd(float *a, float v) { float o = *a; *a = o + v; return o; }
inline int atomicSub(int *a, int v) { int o = *a; *a = o - v; return o; }
inline unsigned atomicSub(unsigned *a, unsigned v) { unsigned o = *a; *a = o - v; return o; }
inline int atomicExch(int *a, int v) { int o = *a; *a = v; return o; }
inline unsigned atomicExch(unsigned *a, unsigned v) { unsigned o = *a; *a = v; return o; }
inline int atomicCAS(int *a, int cmp, int v) { int o = *a; if (o == cmp) *a = v; return o; }
inline unsigned atomicCAS(unsigned *a, unsigned cmp, unsigned v) { unsigned o = *a; if (o == cmp) *a = v; return o; }

// host images bound as texture objects (point sampling, unnormalised coords)
struct EmuTexture {
  const void *data;
  int width, height, elem;
};
extern std::vector<EmuTexture> g_emu_textures;
template <class T> inline T tex2D(cudaTextureObject_t t, float x, float y) {
  const EmuTexture &tx = g_emu_textures[(size_t)t];
  int ix = (int)std::floor(x), iy = (int)std::floor(y);
  ix = ix < 0 ? 0 : (ix >= tx.width ? tx.width - 1 : ix);
  iy = iy < 0 ? 0 : (iy >= tx.height ? tx.height - 1 : iy);
  return static_cast<const T *>(tx.data)[(size_t)iy * tx.width + ix];
}

void __syncthreads();

#ifndef MINF
#define MINF __int_as_float(0xff800000)
#endif
