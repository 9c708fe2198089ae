// mh_batch.cuh -- the scene table of a batch and the loops that batched
// kernels run over it.
//
// A batch holds many independent volumes.  Each per-frame stage runs as ONE
// launch for all scenes: the batched twin of a kernel walks the device scene
// table and runs the same body as the single-scene kernel for every scene
// that takes a frame this step.  Persistent (grid-stride) bodies spread each
// scene's work over the whole grid; pixel-tiled bodies walk a virtual tile
// range that concatenates the scenes' tiles.  The scene descriptor is staged
// in shared memory, so the body's field reads are shared loads that the
// compiler knows do not alias the global stores of the body.
#pragma once
#include "mh_internal.cuh"

struct __align__(16) Scene {
  Dev d;
  const float *src;          // this step's depth frame (device, metres)
  float *tv;                 // TV scratch: 9 planes of W x H floats
  float *ray_depth;          // raycast outputs (device; null: not written)
  float4 *ray_vert, *ray_norm;
  int active;                // the scene takes a frame this step
  int recycle;               // run the periodic recycle pass this step
  int starve;                // simple update: starve + garbage + recycle this step
  int alloc_tile0;           // first virtual tile of the scene in the alloc grid
  int ray_tile0;             // first virtual tile of the scene in the raycast grid
  int pix0;                  // first pixel of the scene in the concatenated pixel range
  int tv_tile0;              // first virtual tile of the scene in the tiled-TV grid
  int pad;
};

__device__ __forceinline__ int flat_tid() { return threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z); }
__device__ __forceinline__ int flat_nthreads() { return blockDim.x * blockDim.y * blockDim.z; }

__device__ __forceinline__ void stage_scene(Scene &cur, const Scene *t, int s) {
  const int4 *src = reinterpret_cast<const int4 *>(t + s);
  int4 *dst = reinterpret_cast<int4 *>(&cur);
  for (int i = flat_tid(); i < (int)(sizeof(Scene) / 16); i += flat_nthreads()) dst[i] = src[i];
}

// Runs f(scene) for every active scene, with all threads of the CTA.
template <class F> __device__ __forceinline__ void each_scene(const Scene *t, int n, F &&f) {
  __shared__ Scene cur;
  for (int s = 0; s < n; ++s) {
    __syncthreads();
    stage_scene(cur, t, s);
    __syncthreads();
    if (cur.active) f(cur);
  }
}

// Virtual tiles: tile vt belongs to the last scene whose first tile is <= vt.
// Runs f(scene, local tile) for every tile of an active scene; tile0 selects
// the prefix field (alloc or raycast tiling).
template <class F>
__device__ __forceinline__ void each_tile(const Scene *t, int n, int total, int Scene::*tile0, F &&f) {
  __shared__ Scene cur;
  __shared__ int cur_s;
  if (flat_tid() == 0) cur_s = -1;
  for (int vt = blockIdx.x; vt < total; vt += gridDim.x) {
    int s = 0;
    while (s + 1 < n && t[s + 1].*tile0 <= vt) ++s;
    __syncthreads();
    if (s != cur_s) {
      stage_scene(cur, t, s);
      __syncthreads();
      if (flat_tid() == 0) cur_s = s;
    }
    __syncthreads();
    if (cur.active) f(cur, vt - cur.*tile0);
  }
}
