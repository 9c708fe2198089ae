// mh_volume.cu -- volume lifecycle, frame input, stage entry points and state
// dumps: the extern "C" boundary declared in include/meshhash.h.
//
// MainEngine (engine/main_engine.cc) owns a HashTable, EntryArray, BlockArray
// and Mesh, each holding raw cudaMalloc buffers, and every stage ends with a
// cudaDeviceSynchronize plus a device-to-host read of a counter.  Here one
// mh_volume owns all device state, stages are asynchronous on the caller's
// stream, and counts stay in device memory; only the introspection calls
// synchronise.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <unordered_map>
#include <vector>

#include "mh_internal.cuh"
#include "mh_kernels.h"
#include "mh_volume.h"


static std::atomic<unsigned long long> g_launches{0};
void mh_count_launches(int n) { g_launches.fetch_add((unsigned long long)n, std::memory_order_relaxed); }

// Records a CUDA event pair around one stage when profiling is on.
struct StageScope {
  mh_volume *v;
  int stage;
  cudaStream_t s;
  cudaEvent_t a = nullptr, b = nullptr;
  StageScope(mh_volume *v_, int st, cudaStream_t s_) : v(v_), stage(st), s(s_) {
    if (!v->prof) return;
    a = v->event();
    b = v->event();
    cudaEventRecord(a, s);
  }
  ~StageScope() {
    if (!a) return;
    cudaEventRecord(b, s);
    v->pend[stage].push_back({a, b});
  }
};

// SM count of the current device, cached per device ordinal (threads may
// race to fill an entry; they all store the same value)
int mh_sm_count() {
  static std::atomic<int> cache[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) dev = 0;
  if (dev >= 64) {
    int n = 0;
    return cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && n > 0 ? n : 132;
  }
  int n = cache[dev].load(std::memory_order_relaxed);
  if (n <= 0) {
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 132;
    cache[dev].store(n, std::memory_order_relaxed);
  }
  return n;
}

// Persistent grids: as many CTAs as can be resident at once (at most
// cap_per_sm per SM), so that a grid-stride loop never leaves a second,
// partly filled wave of CTAs behind the first.
int mh_resident_grid(const void *fn, int block, int cap_per_sm) {
  static std::mutex mu;
  static std::unordered_map<const void *, int> cache;
  std::lock_guard<std::mutex> lk(mu);
  auto it = cache.find(fn);
  int per_sm;
  if (it != cache.end()) {
    per_sm = it->second;
  } else {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, block, 0) != cudaSuccess || n <= 0) n = 1;
    per_sm = n;
    cache[fn] = n;
  }
  return std::min(per_sm, cap_per_sm) * mh_sm_count();
}

// ------------------------------------------------------------------ helpers

// 4x4 inverse by cofactors with the term order of float4x4::getInverse
// (extern/cuda/matrix.h:964-1086); compiled without FMA contraction.
void inverse4(const float *m, float *out) {
  float inv[16];
  for (int r = 0; r < 4; ++r) {
    for (int c = 0; c < 4; ++c) {
      int rows[3], cols[3], nr = 0, nc = 0;
      for (int i = 0; i < 4; ++i)
        if (i != c) rows[nr++] = i;
      for (int j = 0; j < 4; ++j)
        if (j != r) cols[nc++] = j;
      auto E = [&](int i, int j) { return m[i * 4 + j]; };
      const int ra = rows[0], rb = rows[1], rc = rows[2];
      const int c0 = cols[0], c1 = cols[1], c2 = cols[2];
      const float s = ((r + c) & 1) ? -1.0f : 1.0f;
      float t[6];
      t[0] = (s * E(ra, c0)) * E(rb, c1) * E(rc, c2);
      t[1] = -((s * E(ra, c0)) * E(rb, c2) * E(rc, c1));
      t[2] = -((s * E(rb, c0)) * E(ra, c1) * E(rc, c2));
      t[3] = (s * E(rb, c0)) * E(ra, c2) * E(rc, c1);
      t[4] = (s * E(rc, c0)) * E(ra, c1) * E(rb, c2);
      t[5] = -((s * E(rc, c0)) * E(ra, c2) * E(rb, c1));
      float acc = t[0];
      for (int k = 1; k < 6; ++k) acc = acc + t[k];
      inv[r * 4 + c] = acc;
    }
  }
  const float det = m[0] * inv[0] + m[1] * inv[4] + m[2] * inv[8] + m[3] * inv[12];
  const float detr = 1.0f / det;
  for (int i = 0; i < 16; ++i) out[i] = inv[i] * detr;
}

__global__ void k_fill_i32(int *p, size_t n, int v) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) p[i] = v;
}
// stack[i] = hi - 1 - i for i < count (pops hand out lo, lo+1, ... first)
__global__ void k_stack_init(int *p, int count, int hi) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) p[i] = hi - 1 - i;
}
__global__ void k_scatter_fields(Dev d, const int *ptr, int n, const float *sdf, const float *w, const float *a,
                                 const float *b) {
  const int blk = blockIdx.x;
  if (blk >= n) return;
  const int p = ptr[blk];
  if (p < 0) return;
  __shared__ int npos;
  if (threadIdx.x == 0) npos = 0;
  __syncthreads();
  int mine = 0;
  for (int v = threadIdx.x; v < MH_BLOCK_VOXELS; v += blockDim.x) {
    const size_t src = (size_t)blk * MH_BLOCK_VOXELS + v, dst = (size_t)p * MH_BLOCK_VOXELS + v;
    if (v == 0) d.wmax[p] = __int_as_float(0x7f800000);
    if (sdf) {
      d.sdf[dst] = sdf[src];
      mine += sdf_nonneg(sdf[src]);
    }
    if (w) d.w[dst] = w[src];
    if (a) d.a[dst] = a[src];
    if (b) d.b[dst] = b[src];
  }
  if (sdf) {
    atomicAdd(&npos, mine);
    __syncthreads();
    if (threadIdx.x == 0) d.nnc[p] = npos;
  }
}

static int grid_for(size_t n, int tpb = 256) {
  size_t g = (n + tpb - 1) / tpb;
  size_t cap = (size_t)mh_sm_count() * 16;
  return (int)(g < cap ? (g > 0 ? g : 1) : cap);
}

static int ensure_scratch(mh_volume *v, size_t bytes) {
  if (v->scratch_bytes >= bytes) return MH_OK;
  if (v->scratch) cudaFree(v->scratch);
  v->scratch = nullptr;
  v->scratch_bytes = 0;
  if (cudaMalloc(&v->scratch, bytes) != cudaSuccess) return MH_ERR_NOMEM;
  v->scratch_bytes = bytes;
  return MH_OK;
}

template <class T> static int dalloc(mh_volume *v, T **p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  if (cudaMalloc((void **)p, sizeof(T) * count) != cudaSuccess) return MH_ERR_NOMEM;
  v->allocs.push_back(*p);
  return MH_OK;
}

static Counters read_counters(mh_volume *v) {
  Counters c;
  cudaMemcpy(&c, v->d.ctr, sizeof(c), cudaMemcpyDeviceToHost);
  return c;
}

#define CHECK_VOL(v)                  \
  do {                                \
    if (!(v)) return MH_ERR_INVALID;  \
  } while (0)
#define TRY(expr)                 \
  do {                            \
    int _r = (expr);              \
    if (_r != MH_OK) return _r;   \
  } while (0)

extern "C" {

int mh_default_params(mh_params *p) {
  if (!p) return MH_ERR_INVALID;
  memset(p, 0, sizeof(*p));
  p->bucket_count = 1u << 20;
  p->bucket_size = 4;
  p->entry_count = p->bucket_count * 4;
  p->linked_list_size = 7;
  p->value_capacity = 100000;
  p->max_vertex_count = 8000000;
  p->max_triangle_count = 8000000;
  p->voxel_size = 0.008f;
  p->truncation_distance_scale = 0.008f;
  p->truncation_distance = 0.012f;
  p->sdf_upper_bound = 4.0f;
  p->weight_sample = 10;
  p->weight_upper_bound = 255;
  p->fx = 481.2f, p->fy = 480.0f, p->cx = 319.5f, p->cy = 239.5f;
  p->width = 640, p->height = 480;
  p->min_depth_range = 0.5f, p->max_depth_range = 4.0f, p->range_factor = 0.0002f;
  p->rc_fx = p->fx, p->rc_fy = p->fy, p->rc_cx = p->cx, p->rc_cy = p->cy;
  p->rc_width = p->width, p->rc_height = p->height;
  p->min_raycast_depth = 0.5f, p->max_raycast_depth = 5.5f, p->raycast_step = 0.016f;
  p->sample_sdf_threshold = 0.808f, p->sdf_threshold = 0.8f;
  p->enable_gradients = 1;
  p->enable_bayesian_update = 1;
  p->enable_sdf_gradient = 1;
  p->overflow_capacity = 1u << 18;
  p->mesh_page_capacity = 50000;
  return MH_OK;
}

uint32_t mh_hash_bucket(int32_t x, int32_t y, int32_t z, uint32_t bucket_count) {
  uint32_t h = ((uint32_t)x * 73856093u) ^ ((uint32_t)y * 19349669u) ^ ((uint32_t)z * 83492791u);
  return bucket_count ? h % bucket_count : 0;
}

int mh_volume_reset(mh_volume *v, void *stream) {
  CHECK_VOL(v);
  cudaStream_t s = (cudaStream_t)stream;
  const mh_params &P = v->hp;
  Dev &d = v->d;
  const size_t cap = P.value_capacity, nv = cap * MH_BLOCK_VOXELS;
  const size_t npg = (size_t)d.page_capacity, pv = npg * MH_BLOCK_VOXELS;
  MH_CUDA_TRY(cudaMemsetAsync(d.slots, 0xFF, sizeof(HSlot) * (size_t)P.bucket_count * 4, s));
  MH_CUDA_TRY(cudaMemsetAsync(d.overflow, 0xFF, sizeof(HSlot) * (size_t)P.overflow_capacity, s));
  MH_CUDA_TRY(cudaMemsetAsync(d.bucket_lock, 0, sizeof(int) * (size_t)P.bucket_count, s));
  MH_CUDA_TRY(cudaMemsetAsync(d.block_pos, 0, sizeof(int4) * cap, s));
  for (float *f : {d.sdf, d.w, d.a, d.b}) MH_CUDA_TRY(cudaMemsetAsync(f, 0, sizeof(float) * nv, s));
  MH_CUDA_TRY(cudaMemsetAsync(d.inner, 0, sizeof(int) * cap, s));
  MH_CUDA_TRY(cudaMemsetAsync(d.boundary, 0, sizeof(int) * cap, s));
  MH_CUDA_TRY(cudaMemsetAsync(d.nvtx, 0, sizeof(int) * cap, s));
  MH_CUDA_TRY(cudaMemsetAsync(d.wmax, 0, sizeof(float) * cap, s));
  MH_CUDA_TRY(cudaMemsetAsync(d.page_of, 0xFF, sizeof(int) * cap, s));
  MH_CUDA_TRY(cudaMemsetAsync(d.page_owner, 0xFF, sizeof(int) * (size_t)npg, s));
  MH_CUDA_TRY(cudaMemsetAsync(d.cube, 0, pv, s));
  MH_CUDA_TRY(cudaMemsetAsync(d.claim, 0, sizeof(uint32_t) * pv, s));
  MH_CUDA_TRY(cudaMemsetAsync(d.vtx, 0, sizeof(Vertex) * (size_t)P.max_vertex_count, s));
  MH_CUDA_TRY(cudaMemsetAsync(d.flags, 0, cap, s));
  k_fill_i32<<<grid_for(cap), 256, 0, s>>>(d.life, cap, MH_BLOCK_LIFE);
  // every voxel starts at sdf 0, which counts as non-negative
  k_fill_i32<<<grid_for(cap), 256, 0, s>>>(d.nnc, cap, MH_BLOCK_VOXELS);
  k_fill_i32<<<grid_for(pv * 3), 256, 0, s>>>(d.vtx_slot, pv * 3, MH_FREE_PTR);
  k_fill_i32<<<grid_for(pv * 5), 256, 0, s>>>(d.tri_slot, pv * 5, MH_FREE_PTR);
  k_stack_init<<<grid_for(npg), 256, 0, s>>>(d.page_heap, (int)npg, (int)npg);
  k_fill_i32<<<grid_for((size_t)P.max_triangle_count * 4), 256, 0, s>>>(reinterpret_cast<int *>(d.tri),
                                                                       (size_t)P.max_triangle_count * 4, -1);
  k_stack_init<<<grid_for(cap), 256, 0, s>>>(d.heap, (int)cap, (int)cap);
  // vertex index 0 is never handed out, so "vertex_ptrs > 0" means "has a vertex"
  k_stack_init<<<grid_for(P.max_vertex_count), 256, 0, s>>>(d.vtx_heap, (int)P.max_vertex_count - 1,
                                                            (int)P.max_vertex_count);
  k_stack_init<<<grid_for(P.max_triangle_count), 256, 0, s>>>(d.tri_heap, (int)P.max_triangle_count,
                                                              (int)P.max_triangle_count);
  k_stack_init<<<grid_for(P.overflow_capacity), 256, 0, s>>>(d.overflow_free, (int)P.overflow_capacity,
                                                             (int)P.overflow_capacity);
  MH_CUDA_TRY(cudaGetLastError());
  Counters c;
  memset(&c, 0, sizeof(c));
  c.heap_top = (int)cap;
  c.vtx_top = (int)P.max_vertex_count - 1;
  c.tri_top = (int)P.max_triangle_count;
  c.ovf_top = (int)P.overflow_capacity;
  c.page_top = d.page_capacity;
  c.epoch = 0;
  MH_CUDA_TRY(cudaMemcpyAsync(d.ctr, &c, sizeof(c), cudaMemcpyHostToDevice, s));
  MH_CUDA_TRY(cudaStreamSynchronize(s));
  v->frames = 0;
  v->has_frame = false;
  return MH_OK;
}

int mh_volume_create(const mh_params *p, mh_volume **out) {
  if (!p || !out) return MH_ERR_INVALID;
  *out = nullptr;
  const mh_params &P = *p;
  if (P.bucket_count == 0 || (P.bucket_count & (P.bucket_count - 1)) != 0) return MH_ERR_INVALID;
  if (P.bucket_size != 4) return MH_ERR_INVALID;
  if (P.value_capacity == 0 || (size_t)P.value_capacity * MH_BLOCK_VOXELS * 5 > (size_t)INT32_MAX * 16)
    return MH_ERR_INVALID;
  if (P.max_vertex_count < 2 || P.max_triangle_count < 1 || P.max_vertex_count > (uint32_t)INT32_MAX ||
      P.max_triangle_count > (uint32_t)INT32_MAX)
    return MH_ERR_INVALID;
  if (P.width == 0 || P.height == 0 || P.rc_width == 0 || P.rc_height == 0) return MH_ERR_INVALID;
  if (!(P.voxel_size > 0.0f) || P.overflow_capacity == 0) return MH_ERR_INVALID;
  // the raycast march must advance t and stay bounded
  if (!(P.raycast_step >= 1e-5f) || !(P.max_raycast_depth > P.min_raycast_depth) ||
      !(P.min_raycast_depth > 0.0f) || (P.max_raycast_depth - P.min_raycast_depth) / P.raycast_step > 1e6f)
    return MH_ERR_INVALID;
  if (P.linked_list_size > 1024) return MH_ERR_INVALID;
  if (P.mesh_page_capacity == 0 || P.mesh_page_capacity > P.value_capacity) return MH_ERR_INVALID;

  mh_volume *v = new mh_volume();
  v->hp = P;
  Dev &d = v->d;
  DevParams &q = d.p;
  q.bucket_mask = P.bucket_count - 1;
  q.linked_list_size = P.linked_list_size;
  q.value_capacity = (int)P.value_capacity;
  q.max_vertex_count = (int)P.max_vertex_count;
  q.max_triangle_count = (int)P.max_triangle_count;
  q.overflow_capacity = (int)P.overflow_capacity;
  q.voxel_size = P.voxel_size;
  q.truncation_distance_scale = P.truncation_distance_scale;
  q.truncation_distance = P.truncation_distance;
  q.sdf_upper_bound = P.sdf_upper_bound;
  q.weight_sample = (float)P.weight_sample;
  q.fx = P.fx, q.fy = P.fy, q.cx = P.cx, q.cy = P.cy;
  q.width = P.width, q.height = P.height;
  q.min_depth_range = P.min_depth_range, q.max_depth_range = P.max_depth_range;
  q.rc_fx = P.rc_fx, q.rc_fy = P.rc_fy, q.rc_cx = P.rc_cx, q.rc_cy = P.rc_cy;
  q.rc_width = P.rc_width, q.rc_height = P.rc_height;
  q.min_raycast_depth = P.min_raycast_depth, q.max_raycast_depth = P.max_raycast_depth;
  q.raycast_step = P.raycast_step;
  q.sample_sdf_threshold = P.sample_sdf_threshold, q.sdf_threshold = P.sdf_threshold;
  q.enable_gradients = P.enable_gradients, q.enable_bayesian = P.enable_bayesian_update;
  q.compat = P.compat_arithmetic != 0;

  const size_t cap = P.value_capacity, nv = cap * MH_BLOCK_VOXELS, npix = (size_t)P.width * P.height;
  const size_t rpix = (size_t)P.rc_width * P.rc_height;
  int r = MH_OK;
  auto A = [&](int rr) {
    if (r == MH_OK) r = rr;
  };
  A(dalloc(v, &d.slots, (size_t)P.bucket_count * 4));
  A(dalloc(v, &d.overflow, P.overflow_capacity));
  A(dalloc(v, &d.overflow_free, P.overflow_capacity));
  A(dalloc(v, &d.bucket_lock, P.bucket_count));
  A(dalloc(v, &d.heap, cap));
  A(dalloc(v, &d.block_pos, cap));
  A(dalloc(v, &d.sdf, nv));
  A(dalloc(v, &d.w, nv));
  A(dalloc(v, &d.a, nv));
  A(dalloc(v, &d.b, nv));
  A(dalloc(v, &d.life, cap));
  A(dalloc(v, &d.inner, cap));
  A(dalloc(v, &d.boundary, cap));
  A(dalloc(v, &d.nvtx, cap));
  d.page_capacity = (int)P.mesh_page_capacity;
  const size_t pv = (size_t)d.page_capacity * MH_BLOCK_VOXELS;
  A(dalloc(v, &d.page_of, cap));
  A(dalloc(v, &d.wmax, cap));
  A(dalloc(v, &d.nnc, cap));
  A(dalloc(v, &d.cellok, cap));
  A(dalloc(v, &d.mesh_list, cap));
  A(dalloc(v, &d.cube_list, cap));
  A(dalloc(v, &d.vtx_list, cap));
  A(dalloc(v, &d.page_heap, (size_t)d.page_capacity));
  A(dalloc(v, &d.page_owner, (size_t)d.page_capacity));
  A(dalloc(v, &d.vtx_slot, pv * 3));
  A(dalloc(v, &d.tri_slot, pv * 5));
  A(dalloc(v, &d.cube, pv));
  A(dalloc(v, &d.claim, pv));
  A(dalloc(v, &d.vtx, P.max_vertex_count));
  A(dalloc(v, &d.vtx_heap, P.max_vertex_count));
  A(dalloc(v, &d.tri, P.max_triangle_count));
  A(dalloc(v, &d.tri_heap, P.max_triangle_count));
  A(dalloc(v, &d.cand, cap));
  A(dalloc(v, &d.flags, cap));
  d.vwork_capacity = (int)P.max_vertex_count;
  A(dalloc(v, &d.vwork, (size_t)d.vwork_capacity));
  A(dalloc(v, &d.depth, npix));
  A(dalloc(v, &d.inlier, npix));
  A(dalloc(v, &d.fc, 1));
  A(dalloc(v, &d.ctr, 1));
  A(dalloc(v, &v->tv, npix * 9));
  A(dalloc(v, &v->rc_stage, rpix * 9));
  if (r == MH_OK) r = mh_volume_reset(v, nullptr);
  if (r != MH_OK) {
    mh_volume_destroy(v);
    return r;
  }
  *out = v;
  return MH_OK;
}

int mh_volume_destroy(mh_volume *v) {
  CHECK_VOL(v);
  cudaDeviceSynchronize();
  for (auto &pv : v->pend)
    for (auto &pr : pv) v->ev_pool.push_back(pr.first), v->ev_pool.push_back(pr.second);
  for (cudaEvent_t e : v->ev_pool) cudaEventDestroy(e);
  for (void *p : v->allocs) cudaFree(p);
  if (v->scratch) cudaFree(v->scratch);
  if (v->acc) cudaFree(v->acc);
  if (v->touch) cudaFree(v->touch);
  mh_pd_free(v);
  delete v;
  return MH_OK;
}

static int set_pose(mh_volume *v, const float wTc[16], cudaStream_t s) {
  FrameConst &fc = v->fc_host;
  memcpy(fc.wTc, wTc, sizeof(float) * 16);
  inverse4(fc.wTc, fc.cTw);
  memcpy(fc.rc_cTw, fc.cTw, sizeof(float) * 16);
  inverse4(fc.rc_cTw, fc.rc_wTc);
  MH_CUDA_TRY(cudaMemcpyAsync(v->d.fc, &fc, sizeof(FrameConst), cudaMemcpyHostToDevice, s));
  return MH_OK;
}

static int frame_set_impl(mh_volume *v, const float *depth, const uint16_t *depth16, int on_device,
                          const float wTc[16], cudaStream_t s) {
  CHECK_VOL(v);
  if ((!depth && !depth16) || !wTc) return MH_ERR_INVALID;
  const size_t n = (size_t)v->hp.width * v->hp.height;
  const float *src = nullptr;
  const uint16_t *src16 = nullptr;
  if (on_device) {
    src = depth;
    src16 = depth16;
  } else {
    // stage host input in the TV buffer (free outside mh_denoise_tv)
    if (depth) {
      MH_CUDA_TRY(cudaMemcpyAsync(v->tv, depth, n * sizeof(float), cudaMemcpyHostToDevice, s));
      src = v->tv;
    } else {
      MH_CUDA_TRY(cudaMemcpyAsync(v->tv, depth16, n * sizeof(uint16_t), cudaMemcpyHostToDevice, s));
      src16 = reinterpret_cast<const uint16_t *>(v->tv);
    }
  }
  {
    StageScope sc(v, MH_STAGE_PREPROCESS, s);
    TRY(launch_preprocess(v->d, src, src16, v->hp.range_factor, s));
  }
  TRY(set_pose(v, wTc, s));
  v->has_frame = true;
  return MH_OK;
}

int mh_frame_set(mh_volume *v, const float *depth, int depth_on_device, const float wTc[16], void *stream) {
  return frame_set_impl(v, depth, nullptr, depth_on_device, wTc, (cudaStream_t)stream);
}
int mh_frame_set_u16(mh_volume *v, const uint16_t *depth, int depth_on_device, const float wTc[16], void *stream) {
  return frame_set_impl(v, nullptr, depth, depth_on_device, wTc, (cudaStream_t)stream);
}

#define NEED_FRAME(v)                            \
  do {                                           \
    CHECK_VOL(v);                                \
    if (!(v)->has_frame) return MH_ERR_STATE;    \
  } while (0)

int mh_allocate(mh_volume *v, void *stream) {
  NEED_FRAME(v);
  StageScope sc(v, MH_STAGE_ALLOC, (cudaStream_t)stream);
  return launch_alloc(v->d, (cudaStream_t)stream);
}
int mh_collect_frustum(mh_volume *v, void *stream) {
  NEED_FRAME(v);
  StageScope sc(v, MH_STAGE_COLLECT, (cudaStream_t)stream);
  return launch_collect(v->d, 1, (cudaStream_t)stream);
}
int mh_collect_all(mh_volume *v, void *stream) {
  CHECK_VOL(v);
  return launch_collect(v->d, 0, (cudaStream_t)stream);
}
int mh_integrate_simple(mh_volume *v, void *stream) {
  NEED_FRAME(v);
  StageScope sc(v, MH_STAGE_INTEGRATE, (cudaStream_t)stream);
  return launch_integrate_simple(v->d, (cudaStream_t)stream);
}
int mh_predict_inlier(mh_volume *v, void *stream) {
  NEED_FRAME(v);
  StageScope sc(v, MH_STAGE_PREDICT, (cudaStream_t)stream);
  return launch_predict_inlier(v->d, (cudaStream_t)stream);
}
int mh_integrate_psdf(mh_volume *v, void *stream) {
  NEED_FRAME(v);
  StageScope sc(v, MH_STAGE_INTEGRATE, (cudaStream_t)stream);
  return launch_integrate_psdf(v->d, (cudaStream_t)stream);
}
int mh_mesh(mh_volume *v, void *stream) {
  CHECK_VOL(v);
  StageScope sc(v, MH_STAGE_MESH, (cudaStream_t)stream);
  return launch_mesh(v->d, (cudaStream_t)stream);
}
int mh_gc_low_surfel(mh_volume *v, void *stream) {
  CHECK_VOL(v);
  return launch_gc_low_surfel(v->d, (cudaStream_t)stream);
}
int mh_gc_recycle(mh_volume *v, void *stream) {
  CHECK_VOL(v);
  return launch_gc_recycle(v->d, (cudaStream_t)stream);
}
int mh_gc_starve(mh_volume *v, void *stream) {
  CHECK_VOL(v);
  return launch_gc_starve(v->d, (cudaStream_t)stream);
}
int mh_gc_collect_garbage(mh_volume *v, void *stream) {
  CHECK_VOL(v);
  return launch_gc_collect_garbage(v->d, (cudaStream_t)stream);
}

int mh_denoise_tv(mh_volume *v, float lambda, int iterations, void *stream) {
  NEED_FRAME(v);
  if (iterations < 0 || !(lambda > 0.0f)) return MH_ERR_INVALID;
  StageScope sc(v, MH_STAGE_TV, (cudaStream_t)stream);
  return launch_denoise_tv(v->d, v->tv, lambda, iterations, (cudaStream_t)stream);
}

static int raycast_impl(mh_volume *v, float *depth, float *vert4, float *norm4, int on_device, cudaStream_t s) {
  const size_t n = (size_t)v->hp.rc_width * v->hp.rc_height;
  if (on_device) {
    StageScope sc(v, MH_STAGE_RAYCAST, s);
    return launch_raycast(v->d, depth, vert4, norm4, s);
  }
  float *dd = depth ? v->rc_stage : nullptr;
  float *dv = vert4 ? v->rc_stage + n : nullptr;
  float *dn = norm4 ? v->rc_stage + 5 * n : nullptr;
  {
    StageScope sc(v, MH_STAGE_RAYCAST, s);
    TRY(launch_raycast(v->d, dd, dv, dn, s));
  }
  if (depth) MH_CUDA_TRY(cudaMemcpyAsync(depth, dd, n * sizeof(float), cudaMemcpyDeviceToHost, s));
  if (vert4) MH_CUDA_TRY(cudaMemcpyAsync(vert4, dv, n * 4 * sizeof(float), cudaMemcpyDeviceToHost, s));
  if (norm4) MH_CUDA_TRY(cudaMemcpyAsync(norm4, dn, n * 4 * sizeof(float), cudaMemcpyDeviceToHost, s));
  MH_CUDA_TRY(cudaStreamSynchronize(s));
  return MH_OK;
}

int mh_raycast(mh_volume *v, const float cTw[16], float *depth, float *vertex4, float *normal4, int out_on_device,
               void *stream) {
  CHECK_VOL(v);
  if (!cTw) return MH_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  FrameConst &fc = v->fc_host;
  memcpy(fc.rc_cTw, cTw, sizeof(float) * 16);
  inverse4(fc.rc_cTw, fc.rc_wTc);
  if (!v->has_frame) {
    memcpy(fc.cTw, cTw, sizeof(float) * 16);
    memcpy(fc.wTc, fc.rc_wTc, sizeof(float) * 16);
  }
  MH_CUDA_TRY(cudaMemcpyAsync(v->d.fc, &fc, sizeof(FrameConst), cudaMemcpyHostToDevice, s));
  return raycast_impl(v, depth, vertex4, normal4, out_on_device, s);
}

int mh_raycast_footprint(mh_volume *v, const float cTw[16], int *blocks_touched, void *stream) {
  CHECK_VOL(v);
  if (!cTw || !blocks_touched) return MH_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  const int cap = v->d.p.value_capacity;
  if (!v->touch) MH_CUDA_TRY(cudaMalloc(&v->touch, (size_t)cap + 16));
  int *dcount = reinterpret_cast<int *>(v->touch + ((size_t)cap + 3) / 4 * 4);
  MH_CUDA_TRY(cudaMemsetAsync(v->touch, 0, (size_t)cap + 16, s));
  FrameConst &fc = v->fc_host;
  memcpy(fc.rc_cTw, cTw, sizeof(float) * 16);
  inverse4(fc.rc_cTw, fc.rc_wTc);
  if (!v->has_frame) {
    memcpy(fc.cTw, cTw, sizeof(float) * 16);
    memcpy(fc.wTc, fc.rc_wTc, sizeof(float) * 16);
  }
  MH_CUDA_TRY(cudaMemcpyAsync(v->d.fc, &fc, sizeof(FrameConst), cudaMemcpyHostToDevice, s));
  Dev d = v->d;
  d.touch = v->touch;
  TRY(launch_raycast(d, nullptr, nullptr, nullptr, s));
  TRY(launch_count_flags(v->touch, cap, dcount, s));
  MH_CUDA_TRY(cudaMemcpyAsync(blocks_touched, dcount, sizeof(int), cudaMemcpyDeviceToHost, s));
  MH_CUDA_TRY(cudaStreamSynchronize(s));
  return MH_OK;
}

int mh_integrate_frame(mh_volume *v, const float *depth, int depth_on_device, const float wTc[16], int tv_iterations,
                       float tv_lambda, float *ray_depth, float *ray_vertex4, float *ray_normal4,
                       int outputs_on_device, void *stream) {
  CHECK_VOL(v);
  cudaStream_t s = (cudaStream_t)stream;
  const Dev &d = v->d;
  TRY(mh_frame_set(v, depth, depth_on_device, wTc, stream));
  if (tv_iterations > 0) TRY(mh_denoise_tv(v, tv_lambda, tv_iterations, stream));
  // MainEngine::Mapping (main_engine.cc:100-154)
  TRY(mh_allocate(v, stream));
  TRY(mh_collect_frustum(v, stream));
  if (v->hp.enable_bayesian_update) {
    TRY(mh_predict_inlier(v, stream));
    TRY(mh_integrate_psdf(v, stream));
  } else {
    TRY(mh_integrate_simple(v, stream));
  }
  v->frames += 1;
  // MainEngine::Meshing (main_engine.cc:156-174)
  TRY(mh_mesh(v, stream));
  {
    StageScope sc(v, MH_STAGE_GC, s);
    TRY(launch_gc_low_surfel(d, s));
    if (v->frames % 10 == 0) TRY(launch_gc_recycle(d, s));
  }
  // RayCaster::Cast from the frame's pose
  if (ray_depth || ray_vertex4 || ray_normal4)
    TRY(raycast_impl(v, ray_depth, ray_vertex4, ray_normal4, outputs_on_device, s));
  // MainEngine::Recycle (main_engine.cc:176-192), simple mode only
  if (!v->hp.enable_bayesian_update && v->frames % 15 == 14) {
    StageScope sc(v, MH_STAGE_GC, s);
    TRY(launch_gc_starve(d, s));
    TRY(launch_gc_collect_garbage(d, s));
    TRY(launch_gc_recycle(d, s));
  }
  return MH_OK;
}

int mh_stats_get(mh_volume *v, mh_stats *out, void *stream) {
  CHECK_VOL(v);
  if (!out) return MH_ERR_INVALID;
  MH_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
  MH_CUDA_TRY(cudaDeviceSynchronize());
  Counters c = read_counters(v);
  out->error = c.error;
  out->blocks_allocated = (uint32_t)(v->hp.value_capacity - c.heap_top);
  out->block_high_water = (uint32_t)c.high_water;
  out->candidates = (uint32_t)c.cand_count;
  out->vertices_allocated = (uint32_t)(v->hp.max_vertex_count - 1 - c.vtx_top);
  out->triangles_allocated = (uint32_t)(v->hp.max_triangle_count - c.tri_top);
  out->overflow_used = (uint32_t)(v->hp.overflow_capacity - c.ovf_top);
  out->frames = (uint32_t)v->frames;
  out->dropped_inserts = (uint32_t)c.dropped;
  out->gc_freed_blocks = (uint32_t)c.gc_freed;
  out->mesh_passes = (uint32_t)c.mesh_passes;
  out->candidate_sum = c.cand_sum;
  out->vertex_work_sum = c.vwork_sum;
  out->cube_blocks_sum = c.cube_blocks_sum;
  out->mesh_list_sum = c.mesh_list_sum;
  out->predict_blocks_sum = c.predict_blocks_sum;
  out->mesh_pages_used = (uint32_t)(v->d.page_capacity - c.page_top);
  return MH_OK;
}

int mh_clear_error(mh_volume *v, void *stream) {
  CHECK_VOL(v);
  MH_CUDA_TRY(cudaMemsetAsync(&v->d.ctr->error, 0, sizeof(unsigned), (cudaStream_t)stream));
  MH_CUDA_TRY(cudaMemsetAsync(&v->d.ctr->dropped, 0, sizeof(int), (cudaStream_t)stream));
  return MH_OK;
}

// ------------------------------------------------------------------ dumps

int mh_dump_blocks(mh_volume *v, int max_blocks, int32_t *pos, float *sdf, float *weight, float *a, float *b,
                   int *n_out) {
  CHECK_VOL(v);
  MH_CUDA_TRY(cudaDeviceSynchronize());
  Counters c = read_counters(v);
  const int hw = c.high_water;
  std::vector<int4> bp(hw > 0 ? hw : 1);
  if (hw > 0) MH_CUDA_TRY(cudaMemcpy(bp.data(), v->d.block_pos, sizeof(int4) * hw, cudaMemcpyDeviceToHost));
  int n = 0;
  std::vector<float> tmp(MH_BLOCK_VOXELS);
  for (int i = 0; i < hw; ++i) {
    if (!bp[i].w) continue;
    if (n < max_blocks) {
      if (pos) pos[3 * n] = bp[i].x, pos[3 * n + 1] = bp[i].y, pos[3 * n + 2] = bp[i].z;
      const float *src[4] = {v->d.sdf, v->d.w, v->d.a, v->d.b};
      float *dst[4] = {sdf, weight, a, b};
      for (int f = 0; f < 4; ++f) {
        if (!dst[f]) continue;
        MH_CUDA_TRY(cudaMemcpy(dst[f] + (size_t)n * MH_BLOCK_VOXELS, src[f] + (size_t)i * MH_BLOCK_VOXELS,
                               sizeof(float) * MH_BLOCK_VOXELS, cudaMemcpyDeviceToHost));
      }
    }
    ++n;
  }
  if (n_out) *n_out = n;
  return MH_OK;
}

static int find_ptrs(mh_volume *v, int n, const int32_t *pos, std::vector<int> &ptr, bool insert) {
  ptr.assign(n, -1);
  if (n <= 0) return MH_OK;
  TRY(ensure_scratch(v, sizeof(int) * 4 * (size_t)n));
  int *dpos = v->scratch, *dptr = v->scratch + 3 * (size_t)n;
  MH_CUDA_TRY(cudaMemcpy(dpos, pos, sizeof(int) * 3 * n, cudaMemcpyHostToDevice));
  if (insert) TRY(launch_insert_list(v->d, dpos, n, nullptr));
  TRY(launch_find_list(v->d, dpos, n, dptr, nullptr));
  MH_CUDA_TRY(cudaMemcpy(ptr.data(), dptr, sizeof(int) * n, cudaMemcpyDeviceToHost));
  return MH_OK;
}

int mh_load_blocks(mh_volume *v, int n, const int32_t *pos, const float *sdf, const float *weight, const float *a,
                   const float *b) {
  CHECK_VOL(v);
  if (n < 0 || (n > 0 && !pos)) return MH_ERR_INVALID;
  MH_CUDA_TRY(cudaDeviceSynchronize());
  // Every position is inserted before any voxel data moves.  On
  // MH_ERR_CAPACITY the blocks that did fit stay allocated with the voxel
  // values they held before (zero for new blocks): the caller may free them
  // with mh_gc_* or reset the volume.
  std::vector<int> ptr;
  TRY(find_ptrs(v, n, pos, ptr, true));
  for (int i = 0; i < n; ++i)
    if (ptr[i] < 0) return MH_ERR_CAPACITY;
  const size_t nv = (size_t)n * MH_BLOCK_VOXELS;
  float *buf = nullptr;
  MH_CUDA_TRY(cudaMalloc(&buf, sizeof(float) * nv * 4 + sizeof(int) * n));
  int *dptr = reinterpret_cast<int *>(buf + nv * 4);
  const float *srcs[4] = {sdf, weight, a, b};
  float *dsts[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaError_t e = cudaSuccess;
  for (int f = 0; f < 4 && e == cudaSuccess; ++f) {
    if (!srcs[f]) continue;
    dsts[f] = buf + nv * f;
    e = cudaMemcpy(dsts[f], srcs[f], sizeof(float) * nv, cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess) e = cudaMemcpy(dptr, ptr.data(), sizeof(int) * n, cudaMemcpyHostToDevice);
  // a failed upload scatters nothing
  if (e == cudaSuccess && n > 0) {
    k_scatter_fields<<<n, 128>>>(v->d, dptr, n, dsts[0], dsts[1], dsts[2], dsts[3]);
    e = cudaGetLastError();
  }
  const cudaError_t es = cudaDeviceSynchronize();
  cudaFree(buf);
  return e == cudaSuccess && es == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}

int mh_dump_candidates(mh_volume *v, int max_n, int32_t *pos, int *n_out) {
  CHECK_VOL(v);
  MH_CUDA_TRY(cudaDeviceSynchronize());
  Counters c = read_counters(v);
  std::vector<int4> cand(c.cand_count > 0 ? c.cand_count : 1);
  if (c.cand_count > 0)
    MH_CUDA_TRY(cudaMemcpy(cand.data(), v->d.cand, sizeof(int4) * c.cand_count, cudaMemcpyDeviceToHost));
  int n = 0;
  for (int i = 0; i < c.cand_count; ++i) {
    if (cand[i].w < 0) continue;
    if (n < max_n && pos) pos[3 * n] = cand[i].x, pos[3 * n + 1] = cand[i].y, pos[3 * n + 2] = cand[i].z;
    ++n;
  }
  if (n_out) *n_out = n;
  return MH_OK;
}

int mh_set_candidates(mh_volume *v, int n, const int32_t *pos) {
  CHECK_VOL(v);
  if (n < 0 || n > (int)v->hp.value_capacity) return MH_ERR_INVALID;
  MH_CUDA_TRY(cudaDeviceSynchronize());
  std::vector<int> ptr;
  TRY(find_ptrs(v, n, pos, ptr, false));
  for (int i = 0; i < n; ++i)
    if (ptr[i] < 0) return MH_ERR_INVALID;
  TRY(ensure_scratch(v, sizeof(int) * 4 * (size_t)(n > 0 ? n : 1)));
  int *dpos = v->scratch, *dptr = v->scratch + 3 * (size_t)n;
  if (n > 0) {
    MH_CUDA_TRY(cudaMemcpy(dpos, pos, sizeof(int) * 3 * n, cudaMemcpyHostToDevice));
    MH_CUDA_TRY(cudaMemcpy(dptr, ptr.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
  }
  TRY(launch_set_candidates(v->d, dpos, dptr, n, nullptr));
  MH_CUDA_TRY(cudaDeviceSynchronize());
  return MH_OK;
}

int mh_dump_inlier(mh_volume *v, float *out) {
  CHECK_VOL(v);
  if (!out) return MH_ERR_INVALID;
  MH_CUDA_TRY(cudaDeviceSynchronize());
  MH_CUDA_TRY(cudaMemcpy(out, v->d.inlier, sizeof(float) * v->hp.width * v->hp.height, cudaMemcpyDeviceToHost));
  return MH_OK;
}
int mh_dump_depth(mh_volume *v, float *out) {
  CHECK_VOL(v);
  if (!out) return MH_ERR_INVALID;
  MH_CUDA_TRY(cudaDeviceSynchronize());
  MH_CUDA_TRY(cudaMemcpy(out, v->d.depth, sizeof(float) * v->hp.width * v->hp.height, cudaMemcpyDeviceToHost));
  return MH_OK;
}

// Mesh state keyed by owners: vertices (x, y, z, slot) + data; triangles
// (cube x, y, z, slot, i0, i1, i2) with i* indices into the vertex list.
int mh_dump_mesh(mh_volume *v, int max_vertices, int32_t *vkeys, float *vdata, int max_triangles, int32_t *tris,
                 int *n_vertices, int *n_triangles) {
  CHECK_VOL(v);
  MH_CUDA_TRY(cudaDeviceSynchronize());
  const int np = v->d.page_capacity;
  std::vector<int> owner(np);
  MH_CUDA_TRY(cudaMemcpy(owner.data(), v->d.page_owner, sizeof(int) * np, cudaMemcpyDeviceToHost));
  std::vector<int> pages;
  for (int i = 0; i < np; ++i)
    if (owner[i] >= 0) pages.push_back(i);
  std::vector<int4> bp(v->hp.value_capacity);
  MH_CUDA_TRY(cudaMemcpy(bp.data(), v->d.block_pos, sizeof(int4) * bp.size(), cudaMemcpyDeviceToHost));
  std::vector<int> vs(MH_BLOCK_VOXELS * 3), ts(MH_BLOCK_VOXELS * 5);
  std::vector<Vertex> vtx(v->hp.max_vertex_count);
  std::vector<int4> tri(v->hp.max_triangle_count);
  MH_CUDA_TRY(cudaMemcpy(vtx.data(), v->d.vtx, sizeof(Vertex) * vtx.size(), cudaMemcpyDeviceToHost));
  MH_CUDA_TRY(cudaMemcpy(tri.data(), v->d.tri, sizeof(int4) * tri.size(), cudaMemcpyDeviceToHost));
  std::unordered_map<int, int> index;
  struct TriRec {
    int x, y, z, t, tp;
  };
  std::vector<TriRec> trecs;
  int nvx = 0;
  for (int pg : pages) {
    const int4 b = bp[owner[pg]];
    MH_CUDA_TRY(cudaMemcpy(vs.data(), v->d.vtx_slot + (size_t)pg * MH_BLOCK_VOXELS * 3, sizeof(int) * vs.size(),
                           cudaMemcpyDeviceToHost));
    MH_CUDA_TRY(cudaMemcpy(ts.data(), v->d.tri_slot + (size_t)pg * MH_BLOCK_VOXELS * 5, sizeof(int) * ts.size(),
                           cudaMemcpyDeviceToHost));
    for (int li = 0; li < MH_BLOCK_VOXELS; ++li) {
      const int gx = b.x * 8 + (li & 7), gy = b.y * 8 + ((li >> 3) & 7), gz = b.z * 8 + (li >> 6);
      for (int s = 0; s < 3; ++s) {
        const int p = vs[li * 3 + s];
        if (p < 0) continue;
        if (nvx < max_vertices && vkeys && vdata) {
          vkeys[4 * nvx] = gx, vkeys[4 * nvx + 1] = gy, vkeys[4 * nvx + 2] = gz, vkeys[4 * nvx + 3] = s;
          const Vertex &x = vtx[p];
          float *o = vdata + 8 * (size_t)nvx;
          o[0] = x.px, o[1] = x.py, o[2] = x.pz, o[3] = x.nx, o[4] = x.ny, o[5] = x.nz, o[6] = x.radius;
          o[7] = (float)x.ref_count;
        }
        index[p] = nvx++;
      }
      for (int t = 0; t < 5; ++t) {
        const int tp = ts[li * 5 + t];
        if (tp >= 0) trecs.push_back({gx, gy, gz, t, tp});
      }
    }
  }
  int nt = 0;
  for (const TriRec &r : trecs) {
    if (nt < max_triangles && tris) {
      int32_t *o = tris + 7 * (size_t)nt;
      o[0] = r.x, o[1] = r.y, o[2] = r.z, o[3] = r.t;
      const int vv[3] = {tri[r.tp].x, tri[r.tp].y, tri[r.tp].z};
      for (int q = 0; q < 3; ++q) {
        auto it = index.find(vv[q]);
        o[4 + q] = it == index.end() ? -1 : it->second;
      }
    }
    ++nt;
  }
  if (n_vertices) *n_vertices = nvx;
  if (n_triangles) *n_triangles = nt;
  return MH_OK;
}

int mh_dump_cubes(mh_volume *v, int n, const int32_t *pos, uint8_t *cube_idx) {
  CHECK_VOL(v);
  if (n < 0 || !cube_idx) return MH_ERR_INVALID;
  MH_CUDA_TRY(cudaDeviceSynchronize());
  std::vector<int> ptr;
  TRY(find_ptrs(v, n, pos, ptr, false));
  for (int i = 0; i < n; ++i) {
    int pg = -1;
    if (ptr[i] >= 0) MH_CUDA_TRY(cudaMemcpy(&pg, v->d.page_of + ptr[i], sizeof(int), cudaMemcpyDeviceToHost));
    if (pg < 0) {
      memset(cube_idx + (size_t)i * MH_BLOCK_VOXELS, 0, MH_BLOCK_VOXELS);
      continue;
    }
    MH_CUDA_TRY(cudaMemcpy(cube_idx + (size_t)i * MH_BLOCK_VOXELS, v->d.cube + (size_t)pg * MH_BLOCK_VOXELS,
                           MH_BLOCK_VOXELS, cudaMemcpyDeviceToHost));
  }
  return MH_OK;
}

int mh_dump_block_meta(mh_volume *v, int n, const int32_t *pos, int32_t *life, int32_t *inner, int32_t *boundary) {
  CHECK_VOL(v);
  if (n < 0) return MH_ERR_INVALID;
  MH_CUDA_TRY(cudaDeviceSynchronize());
  std::vector<int> ptr;
  TRY(find_ptrs(v, n, pos, ptr, false));
  for (int i = 0; i < n; ++i) {
    const int p = ptr[i];
    int32_t *dst[3] = {life, inner, boundary};
    const int *src[3] = {v->d.life, v->d.inner, v->d.boundary};
    for (int f = 0; f < 3; ++f) {
      if (!dst[f]) continue;
      if (p < 0) dst[f][i] = INT32_MIN;
      else MH_CUDA_TRY(cudaMemcpy(dst[f] + i, src[f] + p, sizeof(int), cudaMemcpyDeviceToHost));
    }
  }
  return MH_OK;
}

int mh_dump_nonneg_counts(mh_volume *v, int n, const int32_t *pos, int32_t *count) {
  CHECK_VOL(v);
  if (n < 0 || (n > 0 && (!pos || !count))) return MH_ERR_INVALID;
  MH_CUDA_TRY(cudaDeviceSynchronize());
  std::vector<int> ptr;
  TRY(find_ptrs(v, n, pos, ptr, false));
  std::vector<int> all((size_t)v->d.p.value_capacity);
  MH_CUDA_TRY(cudaMemcpy(all.data(), v->d.nnc, sizeof(int) * all.size(), cudaMemcpyDeviceToHost));
  for (int i = 0; i < n; ++i) count[i] = ptr[i] < 0 ? INT32_MIN : all[ptr[i]];
  return MH_OK;
}

int mh_dump_flags(mh_volume *v, int max_n, uint8_t *flags, int *n_out) {
  CHECK_VOL(v);
  MH_CUDA_TRY(cudaDeviceSynchronize());
  Counters c = read_counters(v);
  const int n = c.cand_count < max_n ? c.cand_count : max_n;
  if (n > 0 && flags) MH_CUDA_TRY(cudaMemcpy(flags, v->d.flags, n, cudaMemcpyDeviceToHost));
  if (n_out) *n_out = c.cand_count;
  return MH_OK;
}

int mh_profile_enable(mh_volume *v, int enable) {
  CHECK_VOL(v);
  v->prof = enable != 0;
  return MH_OK;
}

int mh_profile_read(mh_volume *v, double ms[MH_STAGE_COUNT], int calls[MH_STAGE_COUNT]) {
  CHECK_VOL(v);
  MH_CUDA_TRY(cudaDeviceSynchronize());
  for (int st = 0; st < MH_STAGE_COUNT; ++st) {
    double acc = 0.0;
    for (auto &pr : v->pend[st]) {
      float t = 0.0f;
      cudaEventElapsedTime(&t, pr.first, pr.second);
      acc += t;
      v->ev_pool.push_back(pr.first);
      v->ev_pool.push_back(pr.second);
    }
    if (ms) ms[st] = acc;
    if (calls) calls[st] = (int)v->pend[st].size();
    v->pend[st].clear();
  }
  return MH_OK;
}

uint64_t mh_launch_count(void) { return (uint64_t)g_launches.load(); }

// Algorithmic bytes of one frame at the current counts:
// [alloc, collect, integrate, predict, mesh, raycast].
int mh_bytes_model(mh_volume *v, double out[6]) {
  CHECK_VOL(v);
  if (!out) return MH_ERR_INVALID;
  MH_CUDA_TRY(cudaDeviceSynchronize());
  Counters c = read_counters(v);
  const double nb = c.cand_count, px = (double)v->hp.width * v->hp.height;
  const double rpx = (double)v->hp.rc_width * v->hp.rc_height;
  const bool psdf = v->hp.enable_bayesian_update != 0;
  out[0] = px * 4.0;
  out[1] = (double)c.high_water * 16.0 + nb * 16.0;
  out[2] = nb * 512.0 * (psdf ? 32.0 : 16.0) + px * (psdf ? 8.0 : 4.0);
  out[3] = psdf ? nb * 512.0 * 12.0 + px * 4.0 : 0.0;
  out[4] = nb * 729.0 * 16.0 + nb * 512.0 * (12.0 + 20.0 + 1.0);
  out[5] = rpx * (4.0 + 16.0 + 16.0);
  return MH_OK;
}

}  // extern "C"
