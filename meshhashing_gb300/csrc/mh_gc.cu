// mh_gc.cu -- block garbage collection (mapping/recycle.cu:15-274).
//
// Low-surfel collection updates every candidate's life counter in one launch
// and tests the six neighbours in a second one, so the neighbour test always
// sees this pass's counters (the reference relies on __syncthreads, which only
// orders threads of one CTA, recycle.cu:94-113).  Recycling frees the flagged
// blocks' triangles, then their unreferenced vertices, and finally returns a
// block with no live vertex to the pool: its hash entry is erased under the
// bucket lock and its voxel and mesh-unit state is cleared (Block::Clear,
// core/block.h:26-40).
#include "mh_internal.cuh"
#include "mh_hash.cuh"
#include "mh_kernels.h"
#include "mh_batch.cuh"

#include <algorithm>


// CollectLowSurfelBlocksKernel, first half (recycle.cu:91-99)
__device__ __forceinline__ void gc_life_body(const Dev &d) {
  const int n = *reinterpret_cast<volatile int *>(&d.ctr->cand_count);
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    d.flags[c] = 0;
    const int ptr = d.cand[c].w;
    if (ptr < 0) continue;
    if (d.inner[ptr] < 10 && d.boundary[ptr] == 0) d.life[ptr] -= 1;
    else d.life[ptr] = MH_BLOCK_LIFE;
  }
}
__global__ void k_gc_life(Dev d) { gc_life_body(d); }
__global__ void k_gc_life_b(const Scene *t, int n) {
  each_scene(t, n, [&](const Scene &c) { gc_life_body(c.d); });
}

// CollectLowSurfelBlocksKernel, second half (recycle.cu:102-113)
__device__ __forceinline__ void gc_flag_body(const Dev &d) {
  const int n = *reinterpret_cast<volatile int *>(&d.ctr->cand_count);
  const int off[6][3] = {{0, 0, 1}, {0, 0, -1}, {0, 1, 0}, {0, -1, 0}, {1, 0, 0}, {-1, 0, 0}};
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    const int4 cb = d.cand[c];
    if (cb.w < 0 || d.life[cb.w] > 0) continue;
    bool ok = true;
    for (int j = 0; j < 6 && ok; ++j) {
      const int q = hash_find(d, cb.x + off[j][0], cb.y + off[j][1], cb.z + off[j][2]);
      if (q >= 0 && d.life[q] != 0) ok = false;
    }
    if (ok) d.flags[c] = 1;
  }
}
__global__ void k_gc_flag(Dev d) { gc_flag_body(d); }
__global__ void k_gc_flag_b(const Scene *t, int n) {
  each_scene(t, n, [&](const Scene &c) { gc_flag_body(c.d); });
}

// StarveOccupiedBlocksKernel (recycle.cu:15-25)
__device__ __forceinline__ void gc_starve_body(const Dev &d) {
  const int n = *reinterpret_cast<volatile int *>(&d.ctr->cand_count);
  for (int c = blockIdx.x; c < n; c += gridDim.x) {
    const int ptr = d.cand[c].w;
    if (ptr < 0) continue;
    float4 *w4 = reinterpret_cast<float4 *>(d.w + (size_t)ptr * MH_BLOCK_VOXELS) + threadIdx.x;
    float4 w = *w4;
    w.x = fmaxf(0.0f, w.x - 1.0f), w.y = fmaxf(0.0f, w.y - 1.0f);
    w.z = fmaxf(0.0f, w.z - 1.0f), w.w = fmaxf(0.0f, w.w - 1.0f);
    *w4 = w;
  }
}
__global__ void __launch_bounds__(128) k_gc_starve(Dev d) { gc_starve_body(d); }
__global__ void __launch_bounds__(128) k_gc_starve_b(const Scene *t, int n) {
  each_scene(t, n, [&](const Scene &c) { if (c.starve) gc_starve_body(c.d); });
}

// CollectGarbageBlockArrayKernel (recycle.cu:28-75)
__device__ __forceinline__ void gc_garbage_body(const Dev &d) {
  __shared__ float smin[4], smax[4];
  const int n = *reinterpret_cast<volatile int *>(&d.ctr->cand_count);
  const float inf = __int_as_float(0x7f800000);
  for (int c = blockIdx.x; c < n; c += gridDim.x) {
    const int ptr = d.cand[c].w;
    if (ptr < 0) {
      if (threadIdx.x == 0) d.flags[c] = 0;
      continue;
    }
    const size_t base = (size_t)ptr * MH_BLOCK_VOXELS + threadIdx.x * 4;
    const float4 S = *reinterpret_cast<const float4 *>(d.sdf + base);
    const float4 W = *reinterpret_cast<const float4 *>(d.w + base);
    const float sv[4] = {S.x, S.y, S.z, S.w}, wv[4] = {W.x, W.y, W.z, W.w};
    float mn = inf, mx = 0.0f;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float s = (double)wv[k] < 1e-6 ? inf : sv[k];
      mn = fminf(mn, fabsf(s));
      mx = fmaxf(mx, wv[k]);
    }
    for (int o = 16; o > 0; o >>= 1) {
      mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
      mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    if ((threadIdx.x & 31) == 0) smin[threadIdx.x >> 5] = mn, smax[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
      mn = fminf(fminf(smin[0], smin[1]), fminf(smin[2], smin[3]));
      mx = fmaxf(fmaxf(smax[0], smax[1]), fmaxf(smax[2], smax[3]));
      const float t = truncate_dist(d.p, 5.0f);
      d.flags[c] = (mn >= t || (double)mx < 1e-6) ? 1 : 0;
    }
    __syncthreads();
  }
}
__global__ void __launch_bounds__(128) k_gc_garbage(Dev d) { gc_garbage_body(d); }
__global__ void __launch_bounds__(128) k_gc_garbage_b(const Scene *t, int n) {
  each_scene(t, n, [&](const Scene &c) { if (c.starve) gc_garbage_body(c.d); });
}

// RecycleGarbageTrianglesKernel (recycle.cu:117-142)
__device__ __forceinline__ void gc_recycle_tri_body(const Dev &d) {
  const int n = *reinterpret_cast<volatile int *>(&d.ctr->cand_count);
  for (int c = blockIdx.x; c < n; c += gridDim.x) {
    const int ptr = d.cand[c].w;
    if (ptr < 0 || !d.flags[c]) continue;
    const int pg = d.page_of[ptr];
    if (pg < 0) continue;
    for (int v = threadIdx.x; v < MH_BLOCK_VOXELS * 5; v += blockDim.x) {
      int *ts = d.tri_slot + (size_t)pg * MH_BLOCK_VOXELS * 5 + v;
      const int tp = *ts;
      if (tp < 0) continue;
      const int4 ot = d.tri[tp];
      atomicSub(&d.vtx[ot.x].ref_count, 1);
      atomicSub(&d.vtx[ot.y].ref_count, 1);
      atomicSub(&d.vtx[ot.z].ref_count, 1);
      d.tri[tp] = make_int4(-1, -1, -1, 0);
      stack_push(&d.ctr->tri_top, d.tri_heap, tp);
      *ts = MH_FREE_PTR;
    }
  }
}
__global__ void __launch_bounds__(128) k_gc_recycle_tri(Dev d) { gc_recycle_tri_body(d); }
__global__ void __launch_bounds__(128) k_gc_recycle_tri_b(const Scene *t, int n, int which) {
  each_scene(t, n, [&](const Scene &c) { if (which ? c.starve : c.recycle) gc_recycle_tri_body(c.d); });
}

// RecycleGarbageVerticesKernel (recycle.cu:144-181) + FreeEntry + Block::Clear
__device__ __forceinline__ void gc_recycle_vtx_body(const Dev &d) {
  __shared__ int live;
  const int n = *reinterpret_cast<volatile int *>(&d.ctr->cand_count);
  for (int c = blockIdx.x; c < n; c += gridDim.x) {
    const int4 cb = d.cand[c];
    if (cb.w < 0 || !d.flags[c]) continue;
    const int ptr = cb.w;
    const int pg = d.page_of[ptr];
    if (threadIdx.x == 0) live = 0;
    __syncthreads();
    int mine = 0, freed = 0;
    if (pg >= 0) {
      for (int v = threadIdx.x; v < MH_BLOCK_VOXELS * 3; v += blockDim.x) {
        int *sp = d.vtx_slot + (size_t)pg * MH_BLOCK_VOXELS * 3 + v;
        const int vp = *sp;
        if (vp < 0) continue;
        if (d.vtx[vp].ref_count <= 0) {
          float4 *v4 = reinterpret_cast<float4 *>(d.vtx + vp);
          v4[0] = make_float4(0.f, 0.f, 0.f, 0.f);
          v4[1] = make_float4(0.f, 0.f, 0.f, 0.f);
          stack_push(&d.ctr->vtx_top, d.vtx_heap, vp);
          *sp = MH_FREE_PTR;
          ++freed;
        } else {
          ++mine;
        }
      }
    }
    if (freed) atomicSub(d.nvtx + ptr, freed);
    if (mine) atomicAdd(&live, mine);
    __syncthreads();
    const bool drop = live == 0;
    __syncthreads();
    if (!drop) continue;
    if (threadIdx.x == 0) {
      hash_erase(d, cb.x, cb.y, cb.z);
      d.block_pos[ptr] = make_int4(0, 0, 0, 0);
      d.life[ptr] = MH_BLOCK_LIFE;
      d.inner[ptr] = 0;
      d.boundary[ptr] = 0;
      d.nvtx[ptr] = 0;
      d.wmax[ptr] = 0.0f;
      d.nnc[ptr] = MH_BLOCK_VOXELS;  // its voxels are zeroed below (sdf 0 is non-negative)
      d.cand[c].w = -1;
      atomicAdd(&d.ctr->gc_freed, 1);
    }
    const size_t base = (size_t)ptr * MH_BLOCK_VOXELS;
    for (int v = threadIdx.x; v < MH_BLOCK_VOXELS; v += blockDim.x)
      d.sdf[base + v] = 0.f, d.w[base + v] = 0.f, d.a[base + v] = 0.f, d.b[base + v] = 0.f;
    // the page has no triangle (freed above) and no vertex left
    if (pg >= 0) release_page_cta(d, ptr, pg);
    __syncthreads();
    if (threadIdx.x == 0) stack_push(&d.ctr->heap_top, d.heap, ptr);
  }
}
__global__ void __launch_bounds__(128) k_gc_recycle_vtx(Dev d) { gc_recycle_vtx_body(d); }
__global__ void __launch_bounds__(128) k_gc_recycle_vtx_b(const Scene *t, int n, int which) {
  each_scene(t, n, [&](const Scene &c) { if (which ? c.starve : c.recycle) gc_recycle_vtx_body(c.d); });
}

int launch_gc_low_surfel(const Dev &d, cudaStream_t s) {
  const int g = mh_sm_count() * 2;
  k_gc_life<<<g, 256, 0, s>>>(d);
  k_gc_flag<<<g, 256, 0, s>>>(d);
  mh_count_launches(2);
  return cudaGetLastError() == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}
int launch_gc_starve(const Dev &d, cudaStream_t s) {
  k_gc_starve<<<mh_sm_count() * 8, 128, 0, s>>>(d);
  mh_count_launches(1);
  return cudaGetLastError() == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}
int launch_gc_collect_garbage(const Dev &d, cudaStream_t s) {
  k_gc_garbage<<<mh_sm_count() * 8, 128, 0, s>>>(d);
  mh_count_launches(1);
  return cudaGetLastError() == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}
int launch_gc_recycle(const Dev &d, cudaStream_t s) {
  const int g = mh_sm_count() * 8;
  k_gc_recycle_tri<<<g, 128, 0, s>>>(d);
  k_gc_recycle_vtx<<<g, 128, 0, s>>>(d);
  mh_count_launches(2);
  return cudaGetLastError() == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}

// ------------------------------------------------------------------ batched
int launch_batch_gc_low_surfel(const Scene *t, int n, cudaStream_t s) {
  const int g = mh_sm_count() * 2;
  k_gc_life_b<<<g, 256, 0, s>>>(t, n);
  k_gc_flag_b<<<g, 256, 0, s>>>(t, n);
  mh_count_launches(2);
  return cudaGetLastError() == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}
// which = 0: scenes due for the periodic recycle; 1: scenes due for starvation
int launch_batch_gc_recycle(const Scene *t, int n, int which, cudaStream_t s) {
  const int g = mh_sm_count() * 8;
  k_gc_recycle_tri_b<<<g, 128, 0, s>>>(t, n, which);
  k_gc_recycle_vtx_b<<<g, 128, 0, s>>>(t, n, which);
  mh_count_launches(2);
  return cudaGetLastError() == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}
int launch_batch_gc_starve(const Scene *t, int n, cudaStream_t s) {
  k_gc_starve_b<<<mh_sm_count() * 8, 128, 0, s>>>(t, n);
  k_gc_garbage_b<<<mh_sm_count() * 8, 128, 0, s>>>(t, n);
  mh_count_launches(2);
  return cudaGetLastError() == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}
