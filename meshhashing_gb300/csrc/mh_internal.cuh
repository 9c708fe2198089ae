// mh_internal.cuh -- device data layout and inline device helpers.
//
// HBM layout (one volume):
//   hash     : bucket_count x 4 slots of 16 B {u64 key, i32 ptr, i32 next};
//              slot 0's `next` heads the bucket's overflow chain, whose
//              entries live in a separate pool.  Occupied slots always form
//              a prefix of the bucket.
//   blocks   : SoA voxel fields, each [value_capacity][512] float, voxel x
//              fastest -- sdf, weight (inv_sigma2), a, b -- so one block of
//              one field is 2 KB contiguous and 16 B aligned.
//   meshunit : per voxel: 3 vertex slots (i32), 5 triangle slots (i32),
//              current cube index (u8) and a vertex-claim word (u32), held in
//              18.5 KB mesh pages that only blocks with surface cubes or owned
//              vertices receive (page_of[block]); blocks in free space carry
//              voxel state only.
//   pools    : vertices (32 B: pos, normal, radius, ref_count), triangles
//              (16 B: three vertex indices), each with a free-index stack.
//   counters : one small struct in device memory, so every count a launch
//              needs stays on the device (graph-capturable chain).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/meshhash.h"

#define MH_BLOCK_SIDE 8
#define MH_BLOCK_VOXELS 512
#define MH_BLOCK_LIFE 3            // core/block.h:13
#define MH_FREE_PTR (-2)           // core/common.h:54-57
#define MH_KEY_EMPTY 0xFFFFFFFFFFFFFFFFull
#define MH_SPIN_LIMIT (1 << 20)    // bounded waits: iterations before MH_ERR_TIMEOUT

struct __align__(16) HSlot {
  unsigned long long key;
  int ptr;
  int next;
};

struct __align__(16) Vertex {
  float px, py, pz;
  float nx, ny, nz;
  float radius;
  int ref_count;
};

struct Counters {
  int heap_top;        // free blocks on the block stack
  int vtx_top;         // free vertices
  int tri_top;         // free triangles
  int ovf_top;         // free overflow entries
  int cand_count;      // candidate list length
  int high_water;      // highest block index handed out + 1
  unsigned error;      // sticky MH_ERR_*
  unsigned epoch;      // mesh epoch (vertex claims)
  int frames;          // frames integrated by the fused chain
  int dropped;         // inserts refused (pool / chain full)
  int gc_freed;        // blocks freed by GC
  int vwork_count;     // vertices to (re)compute this mesh pass
  int gc_count;        // flagged blocks of the current GC pass
  int mesh_passes;     // mesh calls since reset
  int page_top;        // free mesh pages
  int mesh_list_count; // candidates holding a mesh page this pass
  int cube_list_count; // candidates the cube pass must tile this pass
  int vtx_list_count;  // candidates owning vertices (inlier prediction)
  int ray_next;        // next ray handed out by the raycast
  unsigned long long cand_sum;   // sum of candidate counts over mesh calls
  unsigned long long vwork_sum;  // sum of computed vertices over mesh calls
  unsigned long long cube_blocks_sum;     // blocks the cube pass loaded a tile for
  unsigned long long mesh_list_sum;       // blocks the triangle/recycle passes walked
  unsigned long long predict_blocks_sum;  // blocks the inlier prediction read
};

// Per-frame pose constants, kept in device memory so that captured graphs can
// read a new pose each replay.
struct FrameConst {
  float wTc[16];
  float cTw[16];
  float rc_cTw[16];
  float rc_wTc[16];
};

struct DevParams {
  uint32_t bucket_mask;
  uint32_t linked_list_size;
  int value_capacity;
  int max_vertex_count, max_triangle_count, overflow_capacity;
  float voxel_size, truncation_distance_scale, truncation_distance, sdf_upper_bound;
  float weight_sample;
  float fx, fy, cx, cy;
  uint32_t width, height;
  float min_depth_range, max_depth_range;
  float rc_fx, rc_fy, rc_cx, rc_cy;
  uint32_t rc_width, rc_height;
  float min_raycast_depth, max_raycast_depth, raycast_step, sample_sdf_threshold, sdf_threshold;
  int enable_gradients, enable_bayesian;
  int compat;  // evaluate the reference's formulas as written
};

// Everything a kernel needs, passed by value (pointers + params).
struct Dev {
  DevParams p;
  HSlot *slots;
  HSlot *overflow;
  int *overflow_free;
  int *bucket_lock;
  int *heap;
  int4 *block_pos;         // x, y, z, alive
  float *sdf, *w, *a, *b;  // [cap * 512]
  int *life, *inner, *boundary, *nvtx;  // per block
  int *page_of;            // per block: mesh page or -1
  float *wmax;             // per block: upper bound of the largest voxel weight
  int *nnc;                // per block: voxels whose sdf is non-negative (sdf_nonneg), 512 = all
  uint8_t *cellok;         // per block, set before a raycast: it and its 7 upper neighbours count 512 (null: unused)
  uint8_t *touch;          // per block: set by the raycast when a ray looks it up (null: not recorded)
  int *vtx_slot;           // [pages * 512 * 3]
  int *tri_slot;           // [pages * 512 * 5]
  uint8_t *cube;           // [pages * 512]
  uint32_t *claim;         // [pages * 512]
  int *page_heap;          // free pages
  int *page_owner;         // per page: block index or -1
  int *mesh_list;          // candidates holding a page (this mesh pass)
  int4 *cube_list;         // candidates the cube pass tiles (x, y, z, block)
  int *vtx_list;           // candidate indices owning vertices
  int page_capacity;
  Vertex *vtx;
  int *vtx_heap;
  int4 *tri;
  int *tri_heap;
  int4 *cand;              // x, y, z, ptr
  uint8_t *flags;          // per candidate
  int4 *vwork;             // mesh pass: (owner block, voxel, slot, -) to compute
  int vwork_capacity;
  float *depth, *inlier;   // current frame (W x H)
  FrameConst *fc;
  Counters *ctr;
};

// ------------------------------------------------------------------ helpers

__device__ __forceinline__ void set_error(const Dev &d, unsigned code) { atomicCAS(&d.ctr->error, 0u, code); }

__device__ __forceinline__ unsigned long long pack_key(int x, int y, int z) {
  const unsigned long long M = 0x1FFFFFull;
  return (((unsigned long long)x & M) << 42) | (((unsigned long long)y & M) << 21) | ((unsigned long long)z & M);
}
__device__ __forceinline__ bool key_in_range(int x, int y, int z) {
  return x >= -(1 << 20) && x < (1 << 20) && y >= -(1 << 20) && y < (1 << 20) && z >= -(1 << 20) && z < (1 << 20);
}
// Teschner hash (core/hash_table.h:259-269); bucket_count is a power of two,
// so the unsigned modulo is a mask.
__device__ __forceinline__ uint32_t hash_bucket(int x, int y, int z, uint32_t mask) {
  uint32_t h = ((uint32_t)x * 73856093u) ^ ((uint32_t)y * 19349669u) ^ ((uint32_t)z * 83492791u);
  return h & mask;
}

// Lookup for kernels that do not modify the table.  Returns the block index
// or -1 (HashTable::GetEntry, core/hash_table.h:57-93).
__device__ __forceinline__ int hash_find(const Dev &d, int x, int y, int z) {
  if (!key_in_range(x, y, z)) return -1;
  const unsigned long long k = pack_key(x, y, z);
  const uint32_t b = hash_bucket(x, y, z, d.p.bucket_mask);
  const int4 *s = reinterpret_cast<const int4 *>(d.slots + (size_t)b * 4);
  int head = -1;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    int4 e = __ldg(s + j);
    unsigned long long ek = ((unsigned long long)(unsigned)e.y << 32) | (unsigned)e.x;
    if (j == 0) head = e.w;
    if (ek == k) return e.z >= 0 ? e.z : -1;
    if (ek == MH_KEY_EMPTY) return -1;
  }
  int n = head;
  for (uint32_t it = 0; it < d.p.linked_list_size && n >= 0; ++it) {
    int4 e = __ldg(reinterpret_cast<const int4 *>(d.overflow + n));
    unsigned long long ek = ((unsigned long long)(unsigned)e.y << 32) | (unsigned)e.x;
    if (ek == k) return e.z >= 0 ? e.z : -1;
    n = e.w;
  }
  return -1;
}

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31; }

// A voxel counts as non-negative when its sdf lies in [0, 1e30) (NaN does
// not).  A trilinear sample whose eight corners are all non-negative is then
// non-negative itself and finite: its weights lie in [0, 1].  Every kernel
// that writes sdf keeps the per-block count of such voxels (nnc) exact; the
// raycast skips the gathers of samples whose corner blocks all count 512.
__device__ __forceinline__ int sdf_nonneg(float s) { return s >= 0.0f && s < 1e30f ? 1 : 0; }
// add the lanes' changes of one block's non-negative count (all active lanes
// of the warp update the same block)
__device__ __forceinline__ void note_nnc(const Dev &d, int blk, int delta) {
  const unsigned act = __activemask();
  const int sum = __reduce_add_sync(act, delta);
  if ((int)lane_id() == __ffs(act) - 1 && sum) atomicAdd(d.nnc + blk, sum);
}
__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Warp-aggregated pop from a free-index stack.  All active lanes call it;
// lanes with need == true get an index (or -1 when the pool ran dry, which
// also sets MH_ERR_CAPACITY).  Pops and pushes never run in the same launch.
__device__ __forceinline__ int warp_pop(const Dev &d, int *top, const int *stack, bool need) {
  const unsigned act = __activemask();
  const unsigned m = __ballot_sync(act, need);
  if (m == 0) return -1;
  const int leader = __ffs(m) - 1;
  const int cnt = __popc(m);
  int base = 0;
  if ((int)lane_id() == leader) {
    base = atomicSub(top, cnt) - cnt;
    if (base < 0) {
      int failed = min(cnt, -base);
      atomicAdd(top, failed);
      set_error(d, MH_ERR_CAPACITY);
      atomicAdd(&d.ctr->dropped, failed);
    }
  }
  base = __shfl_sync(act, base, leader);
  if (!need) return -1;
  const int idx = base + __popc(m & lanemask_lt());
  return idx >= 0 ? stack[idx] : -1;
}

__device__ __forceinline__ void stack_push(int *top, int *stack, int v) {
  int idx = atomicAdd(top, 1);
  stack[idx] = v;
}

// ------------------------------------------------------------------ geometry
// Every expression below keeps the operation order of the reference's
// GeometryHelper (geometry/geometry_helper.h:36-216); the library is built
// with --fmad=false so single-precision results are reproducible on the CPU.

struct F3 {
  float x, y, z;
};
__device__ __forceinline__ F3 f3(float x, float y, float z) { return F3{x, y, z}; }
__device__ __forceinline__ float dot3(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ F3 normalize3(F3 v) {
  float inv = 1.0f / sqrtf(dot3(v, v));
  return f3(v.x * inv, v.y * inv, v.z * inv);
}
__device__ __forceinline__ F3 mul_pt(const float *m, F3 v) {
  return f3(m[0] * v.x + m[1] * v.y + m[2] * v.z + m[3] * 1.0f, m[4] * v.x + m[5] * v.y + m[6] * v.z + m[7] * 1.0f,
            m[8] * v.x + m[9] * v.y + m[10] * v.z + m[11] * 1.0f);
}
__device__ __forceinline__ F3 mul_dir(const float *m, F3 v) {
  return f3(m[0] * v.x + m[1] * v.y + m[2] * v.z + m[3] * 0.0f, m[4] * v.x + m[5] * v.y + m[6] * v.z + m[7] * 0.0f,
            m[8] * v.x + m[9] * v.y + m[10] * v.z + m[11] * 0.0f);
}
__device__ __forceinline__ int f2i(float v) { return __float2int_rz(v); }
// WorldToVoxeli: round half away from zero with sign(0) = +1
__device__ __forceinline__ int w2vi(float w, float vs) {
  float q = w / vs;
  float s = q < 0.0f ? -1.0f : 1.0f;
  return f2i(q + s * 0.5f);
}
__device__ __forceinline__ int vox2blk(int v) { return (v - (v < 0) * (MH_BLOCK_SIDE - 1)) / MH_BLOCK_SIDE; }
__device__ __forceinline__ float truncate_dist(const DevParams &p, float z) {
  return p.truncation_distance + p.truncation_distance_scale * z;
}
__device__ __forceinline__ float normalize_depth(const DevParams &p, float z) {
  return (z - p.min_depth_range) / (p.max_depth_range - p.min_depth_range);
}
__device__ __forceinline__ bool depth_invalid(const DevParams &p, float d) {
  return d == -__int_as_float(0x7f800000) || d == 0.0f || d >= p.sdf_upper_bound;
}
// IsPointInCameraFrustum (geometry_helper.h:186-206)
__device__ __forceinline__ bool point_in_frustum(const DevParams &p, const float *cTw, F3 w) {
  F3 c = mul_pt(cTw, w);
  float u = c.x * p.fx / c.z + p.cx;
  float v = c.y * p.fy / c.z + p.cy;
  float W1 = (float)p.width - 1.0f, H1 = (float)p.height - 1.0f;
  float nx = (2.0f * u - W1) / W1;
  float ny = (H1 - 2.0f * v) / H1;
  float nz = normalize_depth(p, c.z);
  nx = nx * 0.95f, ny = ny * 0.95f, nz = nz * 0.95f;
  return !(nx < -1.0f || nx > 1.0f || ny < -1.0f || ny > 1.0f || nz < 0.0f || nz > 1.0f);
}
// IsBlockInCameraFrustum (geometry_helper.h:208-216): block corner + 3.5 voxels
__device__ __forceinline__ bool block_in_frustum(const DevParams &p, const float *cTw, int bx, int by, int bz) {
  float vs = p.voxel_size;
  float off = vs * 0.5f * ((float)MH_BLOCK_SIDE - 1.0f);
  F3 w = f3((float)(bx * MH_BLOCK_SIDE) * vs + off, (float)(by * MH_BLOCK_SIDE) * vs + off,
            (float)(bz * MH_BLOCK_SIDE) * vs + off);
  return point_in_frustum(p, cTw, w);
}

// ------------------------------------------------------------------ sampling
// Per-thread cache of the last block lookup (hit or miss).
struct BlockCache {
  int bx, by, bz, ptr;
  __device__ __forceinline__ void init() { bx = by = bz = 0x7fffffff; ptr = -1; }
  __device__ __forceinline__ int get(const Dev &d, int x, int y, int z) {
    if (x != bx || y != by || z != bz) {
      bx = x, by = y, bz = z;
      ptr = hash_find(d, x, y, z);
    }
    return ptr;
  }
};

// Corner voxel indices of one axis for GetSpatialValue: exactly
// WorldToVoxeli(p - v/2) and WorldToVoxeli(p - v/2 + v).
__device__ __forceinline__ void corner_pair(float p, float off, float vs, float fl, float fr, int &c0, int &c1) {
  if (fr > 0.01f && fr < 0.99f) {
    c0 = (int)fl;
    c1 = c0 + 1;
  } else {
    const float pc = p - 0.5f * off;
    c0 = w2vi(pc, vs);
    c1 = w2vi(pc + 1.0f * off, vs);
  }
}

// GetSpatialValue (geometry/spatial_query.h:23-66): trilinear sdf (and the
// interpolated sqrt(1/inv_sigma2) when want_radius); false if any corner
// block is missing.  The block of corner 0 is looked up first, so a sample
// inside a block already known to be missing costs three divisions and one
// cache compare; corners in other blocks go through a second cache entry.
template <bool want_radius>
__device__ __forceinline__ bool spatial_sample(const Dev &d, BlockCache &bc, F3 pos, float &sdf, float &radius,
                                               BlockCache *bc2 = nullptr) {
  const float off = d.p.voxel_size;
  const float vs = d.p.voxel_size;
  const float qx = pos.x / vs, qy = pos.y / vs, qz = pos.z / vs;
  const float fx = floorf(qx), fy = floorf(qy), fz = floorf(qz);
  const float rx = qx - fx, ry = qy - fy, rz = qz - fz;
  // The corner voxels are round-half-away((p - v/2)/v) and ((p + v/2)/v), which
  // equal floor(p/v) and floor(p/v) + 1 unless p/v lies within rounding error
  // of an integer; only there are the two extra divisions evaluated.
  int v0x, v0y, v0z, v1x, v1y, v1z;
  corner_pair(pos.x, off, vs, fx, rx, v0x, v1x);
  corner_pair(pos.y, off, vs, fy, ry, v0y, v1y);
  corner_pair(pos.z, off, vs, fz, rz, v0z, v1z);
  const int b0x = vox2blk(v0x), b0y = vox2blk(v0y), b0z = vox2blk(v0z);
  const int p0 = bc.get(d, b0x, b0y, b0z);
  if (p0 < 0) return false;
  float s = 0.0f, rad = 0.0f;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int mx = (i & 4) > 0, my = (i & 2) > 0, mz = (i & 1) > 0;
    const int vx = mx ? v1x : v0x, vy = my ? v1y : v0y, vz = mz ? v1z : v0z;
    const float wx = mx ? rx : 1.0f - rx, wy = my ? ry : 1.0f - ry, wz = mz ? rz : 1.0f - rz;
    const int bx = vox2blk(vx), by = vox2blk(vy), bz = vox2blk(vz);
    int ptr = p0;
    if (bx != b0x || by != b0y || bz != b0z) {
      ptr = bc2 ? bc2->get(d, bx, by, bz) : hash_find(d, bx, by, bz);
      if (ptr < 0) return false;
    }
    const int li = (vx - bx * MH_BLOCK_SIDE) + (vy - by * MH_BLOCK_SIDE) * MH_BLOCK_SIDE +
                   (vz - bz * MH_BLOCK_SIDE) * MH_BLOCK_SIDE * MH_BLOCK_SIDE;
    const size_t gi = (size_t)ptr * MH_BLOCK_VOXELS + li;
    const float w = wx * wy * wz;
    s += w * __ldg(d.sdf + gi);
    if (want_radius) rad += w * sqrtf(1.0f / __ldg(d.w + gi));
  }
  sdf = s;
  radius = rad;
  return true;
}

// GetSpatialSDFGradient (geometry/spatial_query.h:68-97)
__device__ __forceinline__ bool spatial_gradient(const Dev &d, BlockCache &bc, F3 pos, F3 &g) {
  const float h = 0.5f * d.p.voxel_size;
  float sp[3], sn[3], r;
#pragma unroll 1
  for (int i = 0; i < 3; ++i) {
    F3 dm = f3(pos.x - (i == 0 ? h : 0.0f), pos.y - (i == 1 ? h : 0.0f), pos.z - (i == 2 ? h : 0.0f));
    F3 dp = f3(pos.x + (i == 0 ? h : 0.0f), pos.y + (i == 1 ? h : 0.0f), pos.z + (i == 2 ? h : 0.0f));
    if (!spatial_sample<false>(d, bc, dm, sn[i], r)) return false;
    if (!spatial_sample<false>(d, bc, dp, sp[i], r)) return false;
  }
  const float vs = d.p.voxel_size;
  g = f3((sp[0] - sn[0]) / vs, (sp[1] - sn[1]) / vs, (sp[2] - sn[2]) / vs);
  return true;
}

// Mesh page of a block, allocating one on first use.  Pages are popped only
// by the mesh cube pass and pushed only by the recycle passes.  A racing
// allocator waits (bounded) for the winner's page.
__device__ __forceinline__ int ensure_page(const Dev &d, int blk) {
  int pg = *reinterpret_cast<volatile int *>(d.page_of + blk);
  if (pg >= 0) return pg;
  for (int it = 0; it < MH_SPIN_LIMIT; ++it) {
    const int old = atomicCAS(d.page_of + blk, -1, -2);
    if (old >= 0) return old;
    if (old == -1) {
      const int idx = atomicSub(&d.ctr->page_top, 1) - 1;
      if (idx < 0) {
        atomicAdd(&d.ctr->page_top, 1);
        set_error(d, MH_ERR_CAPACITY);
        atomicExch(d.page_of + blk, -1);
        return -1;
      }
      const int p = d.page_heap[idx];
      d.page_owner[p] = blk;
      __threadfence();
      atomicExch(d.page_of + blk, p);
      return p;
    }
    __nanosleep(32);
  }
  set_error(d, MH_ERR_TIMEOUT);
  return -1;
}

// Return a page whose slots are all free: clear its cube and claim words.
__device__ __forceinline__ void release_page_cta(const Dev &d, int blk, int pg) {
  for (int v = threadIdx.x; v < MH_BLOCK_VOXELS; v += blockDim.x) {
    d.cube[(size_t)pg * MH_BLOCK_VOXELS + v] = 0;
    d.claim[(size_t)pg * MH_BLOCK_VOXELS + v] = 0;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    d.page_of[blk] = -1;
    d.page_owner[pg] = -1;
    stack_push(&d.ctr->page_top, d.page_heap, pg);
  }
}

// launch helpers
#define MH_CUDA_TRY(expr)                     \
  do {                                        \
    cudaError_t _e = (expr);                  \
    if (_e != cudaSuccess) return MH_ERR_CUDA; \
  } while (0)

int mh_sm_count();
// CTAs of a persistent grid: resident CTAs per SM (at most cap_per_sm) x SMs
int mh_resident_grid(const void *fn, int block, int cap_per_sm);
// every launcher adds the kernels it launched (reported by mh_launch_count)
void mh_count_launches(int n);
