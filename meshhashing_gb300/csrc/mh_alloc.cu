// mh_alloc.cu -- spatial-hash insertion, block allocation and candidate
// collection.
//
// AllocBlockArrayKernel (mapping/allocate.cu:8-99) walks, for every pixel, the
// blocks crossed by [d - mu(d), d + mu(d)] and calls HashTable::AllocEntry for
// each in-frustum block.  Here a 16x16-pixel CTA first gathers the blocks its
// pixels touch into a shared-memory set (most neighbouring pixels touch the
// same few blocks), then inserts each distinct block once into the global
// table.  Insertion is lock-free (64-bit atomicCAS of the packed key into the
// first empty bucket slot); only the rare overflow append and deletions take
// a per-bucket lock, with a bounded wait.  Unlike the reference, which holds a
// bucket mutex for the whole launch and drops competing inserts
// (core/hash_table.h:133-176), every touched block is inserted.
#include "mh_internal.cuh"
#include "mh_hash.cuh"
#include "mh_kernels.h"
#include "mh_batch.cuh"

#include <algorithm>

// ------------------------------------------------------------------ alloc

#define ALLOC_TILE 16
#define ALLOC_SET 1024

__device__ __forceinline__ void alloc_body(const Dev &d, int tile_x, int tile_y) {
  __shared__ unsigned long long set[ALLOC_SET];
  __shared__ float sm[32];
  const int tid = threadIdx.x + threadIdx.y * ALLOC_TILE;
  for (int i = tid; i < ALLOC_SET; i += ALLOC_TILE * ALLOC_TILE) set[i] = MH_KEY_EMPTY;
  if (tid < 16) sm[tid] = d.fc->wTc[tid];
  else if (tid < 32) sm[tid] = d.fc->cTw[tid - 16];
  __syncthreads();
  const float *wTc = sm, *cTw = sm + 16;
  const DevParams &p = d.p;
  const unsigned x = tile_x * ALLOC_TILE + threadIdx.x;
  const unsigned y = tile_y * ALLOC_TILE + threadIdx.y;
  const float vs = p.voxel_size;

  if (x < p.width && y < p.height) {
    const float depth = d.depth[y * p.width + x];
    if (!depth_invalid(p, depth)) {
      const float tr = truncate_dist(p, depth);
      const float near_d = fminf(p.sdf_upper_bound, depth - tr);
      const float far_d = fminf(p.sdf_upper_bound, depth + tr);
      if (near_d < far_d) {
        const float rx = ((float)x - p.cx) / p.fx, ry = ((float)y - p.cy) / p.fy;
        F3 wn = mul_pt(wTc, f3(near_d * rx, near_d * ry, near_d));
        F3 wf = mul_pt(wTc, f3(far_d * rx, far_d * ry, far_d));
        F3 dir = normalize3(f3(wf.x - wn.x, wf.y - wn.y, wf.z - wn.z));
        const int bnx = vox2blk(w2vi(wn.x, vs)), bny = vox2blk(w2vi(wn.y, vs)), bnz = vox2blk(w2vi(wn.z, vs));
        const int bfx = vox2blk(w2vi(wf.x, vs)), bfy = vox2blk(w2vi(wf.y, vs)), bfz = vox2blk(w2vi(wf.z, vs));
        const float sx = dir.x < 0.0f ? -1.0f : 1.0f, sy = dir.y < 0.0f ? -1.0f : 1.0f,
                    sz = dir.z < 0.0f ? -1.0f : 1.0f;
        const float hv = 0.5f * vs;
        const float cenx = (float)((bnx + (sx > 0.0f)) * MH_BLOCK_SIDE) * vs - hv;
        const float ceny = (float)((bny + (sy > 0.0f)) * MH_BLOCK_SIDE) * vs - hv;
        const float cenz = (float)((bnz + (sz > 0.0f)) * MH_BLOCK_SIDE) * vs - hv;
        float tx = (cenx - wn.x) / dir.x, ty = (ceny - wn.y) / dir.y, tz = (cenz - wn.z) / dir.z;
        float dtx = sx * (float)MH_BLOCK_SIDE * vs / dir.x;
        float dty = sy * (float)MH_BLOCK_SIDE * vs / dir.y;
        float dtz = sz * (float)MH_BLOCK_SIDE * vs / dir.z;
        const int ebx = f2i((float)bfx + sx), eby = f2i((float)bfy + sy), ebz = f2i((float)bfz + sz);
        const float inf = __int_as_float(0x7f800000);
        if (dir.x == 0.0f) tx = dtx = inf;
        if (dir.y == 0.0f) ty = dty = inf;
        if (dir.z == 0.0f) tz = dtz = inf;
        int cx = bnx, cy = bny, cz = bnz;
#pragma unroll 1
        for (int it = 0; it < 1024; ++it) {
          if (block_in_frustum(p, cTw, cx, cy, cz)) {
            // add to the CTA's set; fall back to a direct insert when it is full
            const unsigned long long k = pack_key(cx, cy, cz);
            uint32_t h = hash_bucket(cx, cy, cz, ALLOC_SET - 1);
            bool done = false;
            for (int probe = 0; probe < 64; ++probe) {
              unsigned long long old = atomicCAS(&set[h], MH_KEY_EMPTY, k);
              if (old == MH_KEY_EMPTY || old == k) {
                done = true;
                break;
              }
              h = (h + 1) & (ALLOC_SET - 1);
            }
            if (!done) hash_insert(d, cx, cy, cz);
          }
          if (tx < ty && tx < tz) {
            cx = f2i((float)cx + sx);
            if (cx == ebx) break;
            tx += dtx;
          } else if (ty < tz) {
            cy = f2i((float)cy + sy);
            if (cy == eby) break;
            ty += dty;
          } else {
            cz = f2i((float)cz + sz);
            if (cz == ebz) break;
            tz += dtz;
          }
        }
      }
    }
  }
  __syncthreads();
  for (int i = tid; i < ALLOC_SET; i += ALLOC_TILE * ALLOC_TILE) {
    const unsigned long long k = set[i];
    if (k == MH_KEY_EMPTY) continue;
    const int bx = (int)((long long)(k << 1) >> 43);
    const int by = (int)((long long)(k << 22) >> 43);
    const int bz = (int)((long long)(k << 43) >> 43);
    hash_insert(d, bx, by, bz);
  }
}
__global__ void __launch_bounds__(ALLOC_TILE * ALLOC_TILE) k_alloc(Dev d) { alloc_body(d, blockIdx.x, blockIdx.y); }
__global__ void __launch_bounds__(ALLOC_TILE * ALLOC_TILE) k_alloc_b(const Scene *t, int n, int total) {
  each_tile(t, n, total, &Scene::alloc_tile0, [&](const Scene &c, int lt) {
    const int tw = (c.d.p.width + ALLOC_TILE - 1) / ALLOC_TILE;
    alloc_body(c.d, lt % tw, lt / tw);
  });
}

// ------------------------------------------------------------------ collect
// CollectBlocksInFrustumKernel / CollectAllBlocksKernel
// (core/collect_block_array.cu:25-91), over the block pool's live indices
// [0, high_water) instead of all hash entries; warp-ballot compaction with one
// atomic per warp.
__device__ __forceinline__ void collect_body(const Dev &d, int frustum) {
  __shared__ float cTw[16];
  if (threadIdx.x < 16) cTw[threadIdx.x] = d.fc->cTw[threadIdx.x];
  __syncthreads();
  const int hw = *reinterpret_cast<volatile int *>(&d.ctr->high_water);
  const int stride = gridDim.x * blockDim.x;
  for (int base = blockIdx.x * blockDim.x; base < hw; base += stride) {
    const int i = base + threadIdx.x;
    bool keep = false;
    int4 bp = make_int4(0, 0, 0, 0);
    if (i < hw) {
      bp = d.block_pos[i];
      keep = bp.w != 0 && (!frustum || block_in_frustum(d.p, cTw, bp.x, bp.y, bp.z));
    }
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    int slot = 0;
    if (lane_id() == 0 && m) slot = atomicAdd(&d.ctr->cand_count, __popc(m));
    slot = __shfl_sync(0xffffffffu, slot, 0);
    if (keep) d.cand[slot + __popc(m & lanemask_lt())] = make_int4(bp.x, bp.y, bp.z, i);
  }
}
__global__ void __launch_bounds__(256) k_collect(Dev d, int frustum) { collect_body(d, frustum); }
__global__ void __launch_bounds__(256) k_collect_b(const Scene *t, int n) {
  each_scene(t, n, [&](const Scene &c) { collect_body(c.d, 1); });
}

// Insert host-given blocks (state loading) and report their indices.
__global__ void k_insert_list(Dev d, const int *pos, int n, int *ptr_out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  hash_insert(d, pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
}
__global__ void k_find_list(Dev d, const int *pos, int n, int *ptr_out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  ptr_out[i] = hash_find(d, pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
}
__global__ void k_set_candidates(Dev d, const int *pos, const int *ptr, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) d.ctr->cand_count = n;
  if (i >= n) return;
  d.cand[i] = make_int4(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], ptr[i]);
}

int launch_alloc(const Dev &d, cudaStream_t s) {
  dim3 blk(ALLOC_TILE, ALLOC_TILE);
  dim3 grid((d.p.width + ALLOC_TILE - 1) / ALLOC_TILE, (d.p.height + ALLOC_TILE - 1) / ALLOC_TILE);
  k_alloc<<<grid, blk, 0, s>>>(d);
  mh_count_launches(1);
  return cudaGetLastError() == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}

int launch_collect(const Dev &d, int frustum, cudaStream_t s) {
  MH_CUDA_TRY(cudaMemsetAsync(&d.ctr->cand_count, 0, sizeof(int), s));
  k_collect<<<mh_sm_count() * 4, 256, 0, s>>>(d, frustum);
  mh_count_launches(1);
  return cudaGetLastError() == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}

int launch_insert_list(const Dev &d, const int *pos_dev, int n, cudaStream_t s) {
  if (n <= 0) return MH_OK;
  k_insert_list<<<(n + 127) / 128, 128, 0, s>>>(d, pos_dev, n, nullptr);
  mh_count_launches(1);
  return cudaGetLastError() == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}
int launch_find_list(const Dev &d, const int *pos_dev, int n, int *ptr_dev, cudaStream_t s) {
  if (n <= 0) return MH_OK;
  k_find_list<<<(n + 127) / 128, 128, 0, s>>>(d, pos_dev, n, ptr_dev);
  mh_count_launches(1);
  return cudaGetLastError() == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}
int launch_set_candidates(const Dev &d, const int *pos_dev, const int *ptr_dev, int n, cudaStream_t s) {
  k_set_candidates<<<(max(n, 1) + 127) / 128, 128, 0, s>>>(d, pos_dev, ptr_dev, n);
  mh_count_launches(1);
  return cudaGetLastError() == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}

// ------------------------------------------------------------------ batched
int launch_batch_alloc(const Scene *t, int n, int total_tiles, cudaStream_t s) {
  const int grid = std::max(1, std::min(total_tiles, mh_sm_count() * 8));
  k_alloc_b<<<grid, dim3(ALLOC_TILE, ALLOC_TILE), 0, s>>>(t, n, total_tiles);
  mh_count_launches(1);
  return cudaGetLastError() == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}
int launch_batch_collect(const Scene *t, int n, cudaStream_t s) {
  k_collect_b<<<mh_sm_count() * 4, 256, 0, s>>>(t, n);
  mh_count_launches(1);
  return cudaGetLastError() == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}
