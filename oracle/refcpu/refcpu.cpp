// refcpu.cpp -- TEST INFRASTRUCTURE: the reference's own device code, run on
// the CPU, to pin the oracle (and produce golden fixtures).
//
// Built only where the reference tree is present (it is not shipped): its
// headers are included from the reference tree and its kernels are included
// from oracle/_ref/ref_kernels.inc, which extract.py copies out of the
// reference's .cu files at build time.  This file provides what the
// reference's host code would: storage for HashTable / EntryArray /
// BlockArray / Mesh (host memory instead of cudaMalloc), the bound depth
// texture, and the stage wrappers with the reference's launch shapes
// (mapping/allocate.cu:101-125, core/collect_block_array.cu:245-276,
// mapping/update_simple.cu:79-108, mapping/update_bayesian.cu:372-433,
// meshing/marching_cubes.cu:326-382, mapping/recycle.cu:183-274,
// visualization/ray_caster.cu:190-209, optimize/primal_dual.cu:146-223,
// localizing/point_to_psdf.cu:86-147).  Every emulated CUDA thread runs
// to completion (or to its next __syncthreads) before the next one starts.
#include "cuda_host.h"
#include "helper_math.h"

// From here on the reference's headers take their device-compiler branches
// (e.g. matrix.h would otherwise turn __int_as_float into a numeric cast).
#define __CUDACC__ 1
#include "matrix.h"
#include "core/common.h"
#include "core/params.h"
#include "core/hash_table.h"
#include "core/entry_array.h"
#include "core/block_array.h"
#include "core/mesh.h"
#include "geometry/geometry_helper.h"
#include "geometry/voxel_query.h"
#include "geometry/spatial_query.h"
#include "geometry/isosurface_intersection.h"
#include "geometry/primal_dual_query.h"
#include "visualization/color_util.h"
#include "meshing/mc_tables.h"
#include "visualization/compact_mesh.h"

#include <functional>
#include <unordered_map>

#include "../../include/meshhash.h"

// The fields of SensorData (sensor/rgbd_sensor.h:16-40) the kernels read, and
// the raycaster's sample/output structs (visualization/ray_caster.h:13-26);
// restated here so the OpenCV/GL headers around them are not needed.
struct SensorData {
  cudaTextureObject_t depth_texture;
  cudaTextureObject_t color_texture;
  float4 *color_data;
  float *inlier_ratio;
};
struct RayCasterSample {
  float entropy;
  float sdf;
  float t;
  uint weight;
};
struct RayCasterData {
  float4 *depth;
  float4 *vertex;
  float4 *normal;
  float4 *color;
  float4 *surface;
};

#include "ref_kernels.inc"

// ------------------------------------------------------------------ emulation
EmuIdx threadIdx, blockIdx;
dim3 blockDim, gridDim;
std::vector<EmuTexture> g_emu_textures;

namespace {
ucontext_t g_sched;
std::vector<ucontext_t> g_ctx;
std::vector<char> g_stacks;
std::vector<int> g_state;  // 0 runnable, 1 at barrier, 2 done
int g_cur = 0;
bool g_coop = false;
const std::function<void()> *g_body = nullptr;
const size_t kStack = 1 << 16;

void set_tid(int t) {
  threadIdx.x = t % blockDim.x;
  threadIdx.y = (t / blockDim.x) % blockDim.y;
  threadIdx.z = t / (blockDim.x * blockDim.y);
}
void thread_entry() {
  (*g_body)();
  g_state[g_cur] = 2;
}
}  // namespace

void __syncthreads() {
  if (!g_coop) return;
  g_state[g_cur] = 1;
  swapcontext(&g_ctx[g_cur], &g_sched);
}

// One emulated launch.  `coop` kernels use __syncthreads and run on contexts.
static void launch(dim3 grid, dim3 block, bool coop, const std::function<void()> &body) {
  gridDim = grid;
  blockDim = block;
  const int n = (int)(block.x * block.y * block.z);
  g_body = &body;
  g_coop = coop;
  if (coop) {
    if ((int)g_ctx.size() < n) {
      g_ctx.resize(n);
      g_stacks.resize((size_t)n * kStack);
    }
    g_state.assign(n, 0);
  }
  for (unsigned bz = 0; bz < grid.z; ++bz)
    for (unsigned by = 0; by < grid.y; ++by)
      for (unsigned bx = 0; bx < grid.x; ++bx) {
        blockIdx.x = bx, blockIdx.y = by, blockIdx.z = bz;
        if (!coop) {
          for (int t = 0; t < n; ++t) {
            set_tid(t);
            body();
          }
          continue;
        }
        for (int t = 0; t < n; ++t) {
          getcontext(&g_ctx[t]);
          g_ctx[t].uc_stack.ss_sp = &g_stacks[(size_t)t * kStack];
          g_ctx[t].uc_stack.ss_size = kStack;
          g_ctx[t].uc_link = &g_sched;
          makecontext(&g_ctx[t], (void (*)())thread_entry, 0);
          g_state[t] = 0;
        }
        bool pending = true;
        while (pending) {
          pending = false;
          for (int t = 0; t < n; ++t) {
            if (g_state[t] == 2) continue;
            g_state[t] = 0;
            g_cur = t;
            set_tid(t);
            swapcontext(&g_sched, &g_ctx[t]);
            if (g_state[t] != 2) pending = true;
          }
        }
      }
  g_coop = false;
}

// ------------------------------------------------------------------ storage
// Host-memory versions of the reference classes' allocation methods
// (core/hash_table.cu:344-439, entry_array.cu:356-422, block_array.cu,
// mesh.cu:38-130).

HashTable::HashTable(const HashParams &params) {
  Alloc(params);
  Reset();
}
void HashTable::Alloc(const HashParams &params) {
  if (is_allocated_on_gpu_) return;
  bucket_count = params.bucket_count;
  bucket_size = params.bucket_size;
  entry_count = params.entry_count;
  value_capacity = params.value_capacity;
  linked_list_size = params.linked_list_size;
  heap_ = new uint[value_capacity];
  heap_counter_ = new uint[1];
  entries_ = new HashEntry[entry_count];
  bucket_mutexes_ = new int[bucket_count];
  is_allocated_on_gpu_ = true;
}
void HashTable::Free() {
  if (!is_allocated_on_gpu_) return;
  delete[] heap_;
  delete[] heap_counter_;
  delete[] entries_;
  delete[] bucket_mutexes_;
  is_allocated_on_gpu_ = false;
}
void HashTable::Resize(const HashParams &params) {
  Alloc(params);
  Reset();
}
void HashTable::Reset() {
  ResetMutexes();
  for (uint i = 0; i < entry_count; ++i) entries_[i].Clear();
  heap_counter_[0] = value_capacity - 1;
  for (uint i = 0; i < value_capacity; ++i) heap_[i] = value_capacity - i - 1;
}
void HashTable::ResetMutexes() {
  for (uint i = 0; i < bucket_count; ++i) bucket_mutexes_[i] = FREE_ENTRY;
}

EntryArray::EntryArray(uint entry_count) { Resize(entry_count); }
void EntryArray::Alloc(uint entry_count) {
  if (is_allocated_on_gpu_) return;
  entry_count_ = entry_count;
  entries_ = new HashEntry[entry_count];
  counter_ = new int[1];
  flags_ = new uchar[entry_count];
  is_allocated_on_gpu_ = true;
}
void EntryArray::Free() {
  if (!is_allocated_on_gpu_) return;
  delete[] entries_;
  delete[] counter_;
  delete[] flags_;
  is_allocated_on_gpu_ = false;
}
void EntryArray::Resize(uint entry_count) {
  if (is_allocated_on_gpu_) Free();
  Alloc(entry_count);
  Reset();
}
void EntryArray::Reset() {
  for (uint i = 0; i < entry_count_; ++i) entries_[i].Clear();
  std::memset(flags_, 0, entry_count_);
  counter_[0] = 0;
}
uint EntryArray::count() { return (uint)counter_[0]; }
void EntryArray::reset_count() { counter_[0] = 0; }

BlockArray::BlockArray(uint block_count) { Resize(block_count); }
void BlockArray::Alloc(uint block_count) {
  if (is_allocated_on_gpu_) return;
  block_count_ = block_count;
  blocks_ = new Block[block_count];
  is_allocated_on_gpu_ = true;
}
void BlockArray::Free() {
  if (!is_allocated_on_gpu_) return;
  delete[] blocks_;
  is_allocated_on_gpu_ = false;
}
void BlockArray::Resize(uint block_count) {
  if (is_allocated_on_gpu_) Free();
  Alloc(block_count);
  Reset();
}
void BlockArray::Reset() {
  for (uint i = 0; i < block_count_; ++i) blocks_[i].Clear();
}

void Mesh::Alloc(const MeshParams &mp) {
  if (is_allocated_on_gpu_) return;
  vertex_heap_ = new uint[mp.max_vertex_count];
  vertex_heap_counter_ = new uint[1];
  vertices = new Vertex[mp.max_vertex_count];
  triangle_heap_ = new uint[mp.max_triangle_count];
  triangle_heap_counter_ = new uint[1];
  triangles = new Triangle[mp.max_triangle_count];
  is_allocated_on_gpu_ = true;
}
void Mesh::Free() {
  if (!is_allocated_on_gpu_) return;
  delete[] vertex_heap_;
  delete[] vertex_heap_counter_;
  delete[] vertices;
  delete[] triangle_heap_;
  delete[] triangle_heap_counter_;
  delete[] triangles;
  is_allocated_on_gpu_ = false;
}
void Mesh::Resize(const MeshParams &mp) {
  mesh_params_ = mp;
  if (is_allocated_on_gpu_) Free();
  Alloc(mp);
  Reset();
}
void Mesh::Reset() {
  vertex_heap_counter_[0] = mesh_params_.max_vertex_count - 1;
  triangle_heap_counter_[0] = mesh_params_.max_triangle_count - 1;
  for (uint i = 0; i < mesh_params_.max_vertex_count; ++i) {
    vertex_heap_[i] = mesh_params_.max_vertex_count - i - 1;
    vertices[i].Clear();
  }
  for (uint i = 0; i < mesh_params_.max_triangle_count; ++i) {
    triangle_heap_[i] = mesh_params_.max_triangle_count - i - 1;
    triangles[i].Clear();
  }
}
uint Mesh::vertex_heap_count() { return vertex_heap_counter_[0]; }

// CompactMesh (visualization/compact_mesh.cu:16-95) in host memory
void CompactMesh::Alloc(const MeshParams &mp) {
  if (is_allocated_on_gpu_) return;
  vertex_remapper_ = new int[mp.max_vertex_count];
  vertex_counter_ = new uint[1];
  vertices_ref_count_ = new int[mp.max_vertex_count];
  vertices_ = new float3[mp.max_vertex_count];
  normals_ = new float3[mp.max_vertex_count];
  colors_ = new float3[mp.max_vertex_count];
  triangle_counter_ = new uint[1];
  triangles_ref_count_ = new int[mp.max_triangle_count];
  triangles_ = new int3[mp.max_triangle_count];
  is_allocated_on_gpu_ = true;
}
void CompactMesh::Free() {
  if (!is_allocated_on_gpu_) return;
  delete[] vertex_remapper_;
  delete[] vertex_counter_;
  delete[] vertices_ref_count_;
  delete[] vertices_;
  delete[] normals_;
  delete[] colors_;
  delete[] triangle_counter_;
  delete[] triangles_ref_count_;
  delete[] triangles_;
  is_allocated_on_gpu_ = false;
}
void CompactMesh::Resize(const MeshParams &mp) {
  mesh_params_ = mp;
  Free();
  Alloc(mp);
  Reset();
}
void CompactMesh::Reset() {
  std::memset(vertex_remapper_, 0xff, sizeof(int) * mesh_params_.max_vertex_count);
  std::memset(vertices_ref_count_, 0, sizeof(int) * mesh_params_.max_vertex_count);
  vertex_counter_[0] = 0;
  std::memset(triangles_ref_count_, 0, sizeof(int) * mesh_params_.max_triangle_count);
  triangle_counter_[0] = 0;
}
uint CompactMesh::vertex_count() { return vertex_counter_[0]; }
uint CompactMesh::triangle_count() { return triangle_counter_[0]; }
uint Mesh::triangle_heap_count() { return triangle_heap_counter_[0]; }

// ------------------------------------------------------------------ driver
struct Ref {
  HashParams hp;
  VolumeParams vp;
  SensorParams sp;
  RayCasterParams rp;
  MeshParams mp;
  HashTable ht;
  EntryArray cand;
  BlockArray blocks;
  Mesh mesh;
  GeometryHelper gh;
  std::vector<float> depth, inlier;
  SensorData sd;
  float4x4 wTc, cTw;
  int frames = 0;
};

static dim3 D3(unsigned x, unsigned y = 1) { return dim3(x, y, 1); }

extern "C" {

void *ref_create(const mh_params *p) {
  Ref *r = new Ref;
  r->hp.bucket_count = p->bucket_count;
  r->hp.bucket_size = p->bucket_size;
  r->hp.entry_count = p->bucket_count * p->bucket_size;
  r->hp.linked_list_size = p->linked_list_size;
  r->hp.value_capacity = p->value_capacity;
  r->vp.voxel_size = p->voxel_size;
  r->vp.truncation_distance_scale = p->truncation_distance_scale;
  r->vp.truncation_distance = p->truncation_distance;
  r->vp.sdf_upper_bound = p->sdf_upper_bound;
  r->vp.weight_sample = p->weight_sample;
  r->vp.weight_upper_bound = p->weight_upper_bound;
  r->sp.fx = p->fx, r->sp.fy = p->fy, r->sp.cx = p->cx, r->sp.cy = p->cy;
  r->sp.width = p->width, r->sp.height = p->height;
  r->sp.min_depth_range = p->min_depth_range, r->sp.max_depth_range = p->max_depth_range;
  r->sp.range_factor = p->range_factor;
  r->rp.fx = p->rc_fx, r->rp.fy = p->rc_fy, r->rp.cx = p->rc_cx, r->rp.cy = p->rc_cy;
  r->rp.width = p->rc_width, r->rp.height = p->rc_height;
  r->rp.min_raycast_depth = p->min_raycast_depth, r->rp.max_raycast_depth = p->max_raycast_depth;
  r->rp.raycast_step = p->raycast_step;
  r->rp.sample_sdf_threshold = p->sample_sdf_threshold, r->rp.sdf_threshold = p->sdf_threshold;
  r->rp.enable_gradients = p->enable_gradients != 0;
  r->mp.max_vertex_count = p->max_vertex_count;
  r->mp.max_triangle_count = p->max_triangle_count;
  // MainEngine ctor (engine/main_engine.cc:315-336)
  r->ht.Resize(r->hp);
  r->cand.Resize(r->hp.entry_count);
  r->blocks.Resize(r->hp.value_capacity);
  r->mesh.Resize(r->mp);
  r->gh.Init(r->vp);
  size_t n = (size_t)p->width * p->height;
  r->depth.assign(n, 0.0f);
  r->inlier.assign(n, 0.1f);
  g_emu_textures.push_back({r->depth.data(), (int)p->width, (int)p->height, 4});
  r->sd.depth_texture = g_emu_textures.size() - 1;
  r->sd.color_texture = 0;
  r->sd.color_data = nullptr;
  r->sd.inlier_ratio = r->inlier.data();
  return r;
}

void ref_destroy(void *h) {
  Ref *r = (Ref *)h;
  r->ht.Free();
  r->cand.Free();
  r->blocks.Free();
  r->mesh.Free();
  delete r;
}

// Sensor::Process with float depth: ConvertDepthFormatKernel's range test
// (sensor/preprocess.cu:25-42), ResetInlierRatioKernel (:10-23) and
// Sensor::set_transform (cTw = wTc.getInverse(), sensor/rgbd_sensor.h:47-50).
void ref_frame_set(void *h, const float *depth, const float *wTc) {
  Ref *r = (Ref *)h;
  for (size_t i = 0; i < r->depth.size(); ++i) {
    float d = depth[i];
    r->depth[i] = (d >= r->sp.min_depth_range && d <= r->sp.max_depth_range) ? d : MINF;
    r->inlier[i] = 0.1f;
  }
  for (int i = 0; i < 16; ++i) r->wTc.entries[i] = wTc[i];
  r->cTw = r->wTc.getInverse();
}

void ref_inverse(const float *m, float *out) {
  float4x4 a;
  for (int i = 0; i < 16; ++i) a.entries[i] = m[i];
  float4x4 b = a.getInverse();
  for (int i = 0; i < 16; ++i) out[i] = b.entries[i];
}

int ref_allocated(void *h) {
  Ref *r = (Ref *)h;
  int n = 0;
  for (uint i = 0; i < r->hp.entry_count; ++i) n += r->ht.entry(i).ptr != FREE_ENTRY;
  return n;
}

// AllocBlockArray (mapping/allocate.cu:101-125).  With `until_stable`, the
// launch is repeated (mutexes reset in between, as at the next frame) until
// no block is added, which gives the set without the per-bucket drops.
int ref_alloc(void *h, int until_stable) {
  Ref *r = (Ref *)h;
  int before = -1, now = ref_allocated(h);
  int passes = 0;
  do {
    before = now;
    r->ht.ResetMutexes();
    const uint t = 8;
    launch(D3((r->sp.width + t - 1) / t, (r->sp.height + t - 1) / t), D3(t, t), false,
           [&] { AllocBlockArrayKernel(r->ht, r->sd, r->sp, r->wTc, r->gh); });
    now = ref_allocated(h);
    ++passes;
  } while (until_stable && now != before && passes < 64);
  return now;
}

int ref_collect(void *h) {
  Ref *r = (Ref *)h;
  r->cand.reset_count();
  launch(D3((r->hp.entry_count + 255) / 256), D3(256), true,
         [&] { CollectBlocksInFrustumKernel(r->ht, r->sp, r->cTw, r->gh, r->cand); });
  return (int)r->cand.count();
}

void ref_integrate_simple(void *h) {
  Ref *r = (Ref *)h;
  uint n = r->cand.count();
  if (n == 0) return;
  launch(D3(n), D3(BLOCK_SIZE), false,
         [&] { UpdateBlocksSimpleKernel(r->cand, r->blocks, r->sd, r->sp, r->cTw, r->ht, r->gh); });
}

void ref_predict(void *h) {
  Ref *r = (Ref *)h;
  uint n = r->cand.count();
  if (n == 0) return;
  launch(D3(n), D3(BLOCK_SIZE), false, [&] {
    PredictOutlierRatioKernel(r->cand, r->blocks, r->mesh, r->sd, r->sp, r->cTw, r->ht, r->gh);
  });
}

void ref_integrate_psdf(void *h) {
  Ref *r = (Ref *)h;
  uint n = r->cand.count();
  if (n == 0) return;
  launch(D3(n), D3(BLOCK_SIZE), false,
         [&] { UpdateBlocksBayesianKernel(r->cand, r->blocks, r->sd, r->sp, r->cTw, r->ht, r->gh); });
}

void ref_mesh(void *h) {
  Ref *r = (Ref *)h;
  uint n = r->cand.count();
  if (n == 0) return;
  launch(D3(n), D3(BLOCK_SIZE), false,
         [&] { SurfelExtractionKernel(r->cand, r->blocks, r->mesh, r->ht, r->gh, true); });
  launch(D3(n), D3(BLOCK_SIZE), true,
         [&] { TriangleExtractionKernel(r->cand, r->blocks, r->mesh, r->ht, r->gh, true); });
  launch(D3(n), D3(BLOCK_SIZE), false, [&] { RecycleTrianglesKernel(r->cand, r->blocks, r->mesh); });
  launch(D3(n), D3(BLOCK_SIZE), false, [&] { RecycleVerticesKernel(r->cand, r->blocks, r->mesh); });
}

void ref_gc_low_surfel(void *h) {
  Ref *r = (Ref *)h;
  uint n = r->cand.count();
  if (n == 0) return;
  launch(D3((n + 63) / 64), D3(64), true,
         [&] { CollectLowSurfelBlocksKernel(r->cand, r->blocks, r->ht, r->gh, (int)n); });
}

void ref_gc_recycle(void *h) {
  Ref *r = (Ref *)h;
  uint n = r->cand.count();
  if (n == 0) return;
  launch(D3(n), D3(BLOCK_SIZE), false,
         [&] { RecycleGarbageTrianglesKernel(r->cand, r->blocks, r->mesh, r->ht); });
  launch(D3(n), D3(BLOCK_SIZE), true,
         [&] { RecycleGarbageVerticesKernel(r->cand, r->blocks, r->mesh, r->ht); });
}

// RayCaster::Cast (visualization/ray_caster.cu:190-209); outputs the metric
// depth (vertex.z) and the camera-frame normal, -inf on a miss.
void ref_raycast(void *h, const float *cTw, float *depth, float *normal4) {
  Ref *r = (Ref *)h;
  float4x4 c;
  for (int i = 0; i < 16; ++i) c.entries[i] = cTw[i];
  const float4x4 w = c.getInverse();
  const size_t n = (size_t)r->rp.width * r->rp.height;
  std::vector<float4> d(n), v(n), nn(n), col(n), surf(n);
  RayCasterData rcd{d.data(), v.data(), nn.data(), col.data(), surf.data()};
  const uint t = 8;
  launch(D3((r->rp.width + t - 1) / t, (r->rp.height + t - 1) / t), D3(t, t), false,
         [&] { CastKernel(r->ht, r->blocks, rcd, r->rp, c, w, r->gh); });
  for (size_t i = 0; i < n; ++i) {
    depth[i] = v[i].z;
    if (normal4) {
      normal4[4 * i] = nn[i].x, normal4[4 * i + 1] = nn[i].y;
      normal4[4 * i + 2] = nn[i].z, normal4[4 * i + 3] = nn[i].w;
    }
  }
}

// Replace the candidate list by the entries of the given block positions
// (absent positions are skipped); returns the new count.
int ref_set_candidates(void *h, int n, const int32_t *pos) {
  Ref *r = (Ref *)h;
  r->cand.reset_count();
  for (int i = 0; i < n; ++i) {
    HashEntry e = r->ht.GetEntry(make_int3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]));
    if (e.ptr == FREE_ENTRY) continue;
    r->cand[r->cand.counter()++] = e;
  }
  return (int)r->cand.count();
}

// PrimalDualInit / PrimalDualIterate (optimize/primal_dual.cu:146-223) with
// the reference's launch shapes; the two error accumulators live in host
// memory instead of cudaMalloc'd floats, and are returned instead of printed.
void ref_pd_init(void *h) {
  Ref *r = (Ref *)h;
  uint n = r->cand.count();
  if (n == 0) return;
  launch(D3(n), D3(BLOCK_SIZE), false, [&] { PrimalDualInitKernel(r->cand, r->blocks, r->ht, r->gh); });
}

void ref_pd_iterate(void *h, float lambda, float sigma, float tau, float *err) {
  Ref *r = (Ref *)h;
  uint n = r->cand.count();
  err[0] = err[1] = 0.0f;
  if (n == 0) return;
  launch(D3(n), D3(BLOCK_SIZE), false, [&] {
    PrimalDualIteratePass1Kernel(r->cand, r->blocks, r->ht, r->gh, lambda, sigma, tau, err, err + 1);
  });
  launch(D3(n), D3(BLOCK_SIZE), false,
         [&] { PrimalDualIteratePass2Kernel(r->cand, r->blocks, r->ht, r->gh, lambda, sigma, tau); });
}

// PointToSurface (localizing/point_to_psdf.cu:86-147): the tracker's normal
// equations at the pose wTc over the current depth frame, 16x16 CTAs, the
// accumulators in host memory.
void ref_point_to_psdf(void *h, const float *wTc, float *A, float *b, float *err, int *count) {
  Ref *r = (Ref *)h;
  float4x4 T;
  for (int i = 0; i < 16; ++i) T.entries[i] = wTc[i];
  mat6x6 mA;
  mat6x1 mb;
  mA.setZero();
  mb.setZero();
  float e = 0.0f;
  int c = 0;
  const unsigned t = 16;
  launch(D3((r->sp.width + t - 1) / t, (r->sp.height + t - 1) / t), D3(t, t), false, [&] {
    PointToSurfaceKernel(r->blocks, r->sd, r->sp, T, r->ht, r->gh, &mA, &mb, &e, &c);
  });
  for (int i = 0; i < 36; ++i) A[i] = mA.entries[i];
  for (int i = 0; i < 6; ++i) b[i] = mb.entries[i];
  *err = e;
  *count = c;
}

// Live blocks: pos[3n] and voxel fields [512n] in hash-entry order.
int ref_get_blocks(void *h, int max, int32_t *pos, float *sdf, float *w, float *a, float *b) {
  Ref *r = (Ref *)h;
  int n = 0;
  for (uint i = 0; i < r->hp.entry_count; ++i) {
    const HashEntry &e = r->ht.entry(i);
    if (e.ptr == FREE_ENTRY) continue;
    if (n < max) {
      if (pos) pos[3 * n] = e.pos.x, pos[3 * n + 1] = e.pos.y, pos[3 * n + 2] = e.pos.z;
      const Block &bl = r->blocks[e.ptr];
      for (int k = 0; k < BLOCK_SIZE; ++k) {
        if (sdf) sdf[(size_t)n * BLOCK_SIZE + k] = bl.voxels[k].sdf;
        if (w) w[(size_t)n * BLOCK_SIZE + k] = bl.voxels[k].inv_sigma2;
        if (a) a[(size_t)n * BLOCK_SIZE + k] = bl.voxels[k].a;
        if (b) b[(size_t)n * BLOCK_SIZE + k] = bl.voxels[k].b;
      }
    }
    ++n;
  }
  return n;
}

int ref_get_candidates(void *h, int max, int32_t *pos) {
  Ref *r = (Ref *)h;
  int n = (int)r->cand.count();
  for (int i = 0; i < n && i < max; ++i) {
    const HashEntry &e = r->cand[i];
    pos[3 * i] = e.pos.x, pos[3 * i + 1] = e.pos.y, pos[3 * i + 2] = e.pos.z;
  }
  return n;
}

void ref_get_inlier(void *h, float *out) {
  Ref *r = (Ref *)h;
  std::memcpy(out, r->inlier.data(), r->inlier.size() * 4);
}

// Mesh as owner keys, like the oracle's dump: vertices (x, y, z, slot) +
// (pos, normal, radius, ref_count); triangles (cube x, y, z, slot, i0, i1, i2).
void ref_dump_mesh(void *h, int maxv, int32_t *vkeys, float *vdata, int maxt, int32_t *tris, int *nv, int *nt) {
  Ref *r = (Ref *)h;
  std::unordered_map<int, int> index;
  int v = 0, t = 0;
  for (int pass = 0; pass < 2; ++pass) {
    for (uint i = 0; i < r->hp.entry_count; ++i) {
      const HashEntry &e = r->ht.entry(i);
      if (e.ptr == FREE_ENTRY) continue;
      Block &bl = r->blocks[e.ptr];
      for (int li = 0; li < BLOCK_SIZE; ++li) {
        const int gx = e.pos.x * 8 + li % 8, gy = e.pos.y * 8 + (li / 8) % 8, gz = e.pos.z * 8 + li / 64;
        const MeshUnit &mu = bl.mesh_units[li];
        if (pass == 0) {
          for (int s = 0; s < 3; ++s) {
            const int p = mu.vertex_ptrs[s];
            if (p < 0) continue;
            if (v < maxv && vkeys) {
              vkeys[4 * v] = gx, vkeys[4 * v + 1] = gy, vkeys[4 * v + 2] = gz, vkeys[4 * v + 3] = s;
              const Vertex &x = r->mesh.vertex(p);
              float *o = vdata + 8 * (size_t)v;
              o[0] = x.pos.x, o[1] = x.pos.y, o[2] = x.pos.z;
              o[3] = x.normal.x, o[4] = x.normal.y, o[5] = x.normal.z;
              o[6] = x.radius, o[7] = (float)x.ref_count;
            }
            index[p] = v++;
          }
        } else {
          for (int k = 0; k < N_TRIANGLE; ++k) {
            const int tp = mu.triangle_ptrs[k];
            if (tp < 0) continue;
            if (t < maxt && tris) {
              int32_t *o = tris + 7 * (size_t)t;
              o[0] = gx, o[1] = gy, o[2] = gz, o[3] = k;
              const int3 vv = r->mesh.triangle(tp).vertex_ptrs;
              const int ids[3] = {vv.x, vv.y, vv.z};
              for (int q = 0; q < 3; ++q) {
                auto it = index.find(ids[q]);
                o[4 + q] = it == index.end() ? -1 : it->second;
              }
            }
            ++t;
          }
        }
      }
    }
  }
  *nv = v;
  *nt = t;
}

// MainEngine's mesh output (main_engine.cc:207-216): CollectAllBlocks
// (core/collect_block_array.cu:97-117), then CompressMesh
// (visualization/compress_mesh.cu:96-172) with the reference's launch
// shapes.  Writes at most max_v compact vertices (pos3, normal3) and max_t
// triangles (3 compact indices); stats = (triangles, vertices, sum of the
// compacted vertices' ref_count).
void ref_compress_mesh(void *h, int max_v, float *pos3, float *nrm3, int max_t, int32_t *tri3, int32_t *stats) {
  Ref *r = (Ref *)h;
  r->cand.reset_count();
  launch(D3((r->hp.entry_count + 255) / 256), D3(256), true, [&] { CollectAllBlocksKernel(r->ht, r->cand); });
  CompactMesh cm;
  cm.Resize(r->mp);
  int3 st = make_int3(0, 0, 0);
  const uint n = r->cand.count();
  if (n > 0) {
    launch(D3(n), D3(BLOCK_SIZE), false, [&] { CollectVerticesAndTrianglesKernel(r->cand, r->blocks, r->mesh, cm); });
    uint vref = 0;
    launch(D3((r->mp.max_vertex_count + 255) / 256), D3(256), true,
           [&] { CompressVerticesKernel(r->mesh, cm, r->mp.max_vertex_count, &vref); });
    launch(D3((r->mp.max_triangle_count + 255) / 256), D3(256), true,
           [&] { CompressTrianglesKernel(r->mesh, cm, r->mp.max_triangle_count); });
    st = make_int3((int)cm.triangle_count(), (int)cm.vertex_count(), (int)vref);
  }
  stats[0] = st.x, stats[1] = st.y, stats[2] = st.z;
  for (int i = 0; i < st.y && i < max_v; ++i) {
    const float3 p = cm.vertices()[i], q = cm.normals()[i];
    pos3[3 * i] = p.x, pos3[3 * i + 1] = p.y, pos3[3 * i + 2] = p.z;
    nrm3[3 * i] = q.x, nrm3[3 * i + 1] = q.y, nrm3[3 * i + 2] = q.z;
  }
  for (int i = 0; i < st.x && i < max_t; ++i) {
    const int3 t = cm.triangles()[i];
    tri3[3 * i] = t.x, tri3[3 * i + 1] = t.y, tri3[3 * i + 2] = t.z;
  }
  cm.Free();
}

void ref_cube_indices(void *h, int n, const int32_t *pos, uint8_t *out) {
  Ref *r = (Ref *)h;
  std::memset(out, 0, (size_t)n * BLOCK_SIZE);
  for (uint i = 0; i < r->hp.entry_count; ++i) {
    const HashEntry &e = r->ht.entry(i);
    if (e.ptr == FREE_ENTRY) continue;
    for (int j = 0; j < n; ++j) {
      if (pos[3 * j] != e.pos.x || pos[3 * j + 1] != e.pos.y || pos[3 * j + 2] != e.pos.z) continue;
      for (int k = 0; k < BLOCK_SIZE; ++k) out[(size_t)j * BLOCK_SIZE + k] = (uint8_t)r->blocks[e.ptr].mesh_units[k].curr_cube_idx;
    }
  }
}

}  // extern "C"
