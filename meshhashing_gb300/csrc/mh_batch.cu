// mh_batch.cu -- many independent scenes advanced with one launch per stage.
//
// The step is the per-frame chain of mh_integrate_frame (MainEngine::Mapping,
// Meshing, RayCaster::Cast, Recycle; engine/main_engine.cc:100-192) for every
// active scene at once: the batched twins of the stage kernels walk a device
// scene table (mh_batch.cuh).  Per-step inputs -- the scene table with the
// active / recycle / starve flags and depth pointers, the scenes' pose
// constants, and (for host depth) the depth frames -- are written into one
// of two pinned host blocks and moved by one copy each, so the whole step can
// be captured once as a CUDA graph and replayed with new inputs.
#include <algorithm>
#include <cstring>
#include <vector>

#include "mh_batch.cuh"
#include "mh_kernels.h"
#include "mh_volume.h"

namespace {

// the per-step counter resets the single-scene launchers do with memsets
__global__ void k_frame_begin_b(const Scene *t, int n) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
    if (!t[s].active) continue;
    Counters *c = t[s].d.ctr;
    c->cand_count = 0;
    c->vtx_list_count = 0;
  }
}

const int kCtaCaps[3] = {4, 8, 16};

}  // namespace

struct mh_batch {
  std::vector<mh_volume *> vols;
  int n = 0;
  bool raycast = false;
  bool has_simple = false, has_psdf = false;
  int alloc_tiles = 0, max_pixels = 0, tv_tiles = 0;
  std::vector<int> alloc_tile0, tv_tile0, pix0, rc_w, rc_h;
  size_t pixels = 0;               // sum of the scenes' W x H
  // device: [Scene n][FrameConst n] and the host-depth staging
  char *d_block = nullptr;
  float *d_depth = nullptr;
  size_t block_bytes = 0;
  // pinned, double-buffered step inputs
  char *h_block[2] = {nullptr, nullptr};
  float *h_depth[2] = {nullptr, nullptr};
  cudaEvent_t block_free[2] = {nullptr, nullptr};
  bool block_used[2] = {false, false};
  int step = 0;
  std::vector<float *> out_depth, out_vert, out_norm;
  std::vector<void *> allocs;
  mh_batch_tuning tune{0, 16};
  // graph per pinned block, with the configuration it was captured for
  cudaGraphExec_t exec[2] = {nullptr, nullptr};
  int g_tv_it[2] = {-1, -1}, g_host[2] = {-1, -1};
  float g_lambda[2] = {0, 0};
  mh_batch_tuning g_tune[2];
  cudaStream_t own = nullptr;
  // online autotuning
  int tune_left = 0, tune_k = 0;
  double ray_ms[3] = {0, 0, 0}, int_ms[3] = {0, 0, 0};
  int ray_cnt[3] = {0, 0, 0}, int_cnt[3] = {0, 0, 0};
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  // per-stage times of the tuning steps (events at every stage boundary)
  cudaEvent_t sev[MH_STAGE_COUNT + 1] = {};
  double stage_ms[MH_STAGE_COUNT] = {};
  int stage_steps = 0;

  Scene *table() const { return reinterpret_cast<Scene *>(d_block); }
  int ray_tiles(int shape, std::vector<int> *first) const {
    int tx, ty, total = 0;
    ray_tile_shape(shape, tx, ty);
    for (int s = 0; s < n; ++s) {
      if (first) (*first)[s] = total;
      total += ((rc_w[s] + tx - 1) / tx) * ((rc_h[s] + ty - 1) / ty);
    }
    return total;
  }
};

static void batch_free(mh_batch *b) {
  cudaDeviceSynchronize();
  for (int p = 0; p < 2; ++p) {
    if (b->exec[p]) cudaGraphExecDestroy(b->exec[p]);
    if (b->h_block[p]) cudaFreeHost(b->h_block[p]);
    if (b->h_depth[p]) cudaFreeHost(b->h_depth[p]);
    if (b->block_free[p]) cudaEventDestroy(b->block_free[p]);
  }
  for (cudaEvent_t e : b->ev)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : b->sev)
    if (e) cudaEventDestroy(e);
  for (void *p : b->allocs) cudaFree(p);
  if (b->own) cudaStreamDestroy(b->own);
  delete b;
}

// Enqueue one step from pinned block p.  Nothing here synchronises, so the
// same sequence is what a graph capture records.
static int enqueue(mh_batch *b, int p, bool host_depth, int tv_it, float lambda, bool timed, cudaStream_t s) {
  const Scene *t = b->table();
  const int n = b->n;
  MH_CUDA_TRY(cudaMemcpyAsync(b->d_block, b->h_block[p], b->block_bytes, cudaMemcpyHostToDevice, s));
  if (host_depth)
    MH_CUDA_TRY(cudaMemcpyAsync(b->d_depth, b->h_depth[p], b->pixels * sizeof(float), cudaMemcpyHostToDevice, s));
  k_frame_begin_b<<<(n + 127) / 128, 128, 0, s>>>(t, n);
  mh_count_launches(1);
  auto mark = [&](int st) {
    if (timed) cudaEventRecord(b->sev[st], s);
  };
  int r;
  mark(MH_STAGE_PREPROCESS);
  if ((r = launch_batch_preprocess(t, n, s)) != MH_OK) return r;
  mark(MH_STAGE_TV);
  if (tv_it > 0 && (r = launch_batch_tv(t, n, b->tv_tiles, lambda, tv_it, s)) != MH_OK) return r;
  mark(MH_STAGE_ALLOC);
  if ((r = launch_batch_alloc(t, n, b->alloc_tiles, s)) != MH_OK) return r;
  mark(MH_STAGE_COLLECT);
  if ((r = launch_batch_collect(t, n, s)) != MH_OK) return r;
  mark(MH_STAGE_PREDICT);
  if (b->has_psdf && (r = launch_batch_predict(t, n, s)) != MH_OK) return r;
  mark(MH_STAGE_INTEGRATE);
  if (timed) cudaEventRecord(b->ev[0], s);
  if ((r = launch_batch_integrate(t, n, b->has_simple, b->has_psdf, kCtaCaps[b->tune.integrate_cta_per_sm], s)) !=
      MH_OK)
    return r;
  if (timed) cudaEventRecord(b->ev[1], s);
  mark(MH_STAGE_MESH);
  if ((r = launch_batch_mesh(t, n, s)) != MH_OK) return r;
  mark(MH_STAGE_GC);
  if ((r = launch_batch_gc_low_surfel(t, n, s)) != MH_OK) return r;
  if ((r = launch_batch_gc_recycle(t, n, 0, s)) != MH_OK) return r;
  mark(MH_STAGE_RAYCAST);
  if (b->raycast) {
    if (timed) cudaEventRecord(b->ev[2], s);
    if ((r = launch_raycast_batch(t, n, b->ray_tiles(b->tune.ray_tile_shape, nullptr), b->tune.ray_tile_shape, s)) !=
        MH_OK)
      return r;
    if (timed) cudaEventRecord(b->ev[3], s);
  }
  mark(MH_STAGE_COUNT);
  if (b->has_simple) {
    if ((r = launch_batch_gc_starve(t, n, s)) != MH_OK) return r;
    if ((r = launch_batch_gc_recycle(t, n, 1, s)) != MH_OK) return r;
  }
  return MH_OK;
}

extern "C" {

int mh_batch_create(mh_volume *const *volumes, int count, int raycast, mh_batch **out) {
  if (!volumes || count <= 0 || !out) return MH_ERR_INVALID;
  *out = nullptr;
  mh_batch *b = new mh_batch();
  b->n = count;
  b->raycast = raycast != 0;
  int r = MH_OK;
  for (int s = 0; s < count; ++s) {
    mh_volume *v = volumes[s];
    if (!v) {
      delete b;
      return MH_ERR_INVALID;
    }
    b->vols.push_back(v);
    const int W = (int)v->hp.width, H = (int)v->hp.height;
    b->alloc_tile0.push_back(b->alloc_tiles);
    b->alloc_tiles += ((W + 15) / 16) * ((H + 15) / 16);
    b->tv_tile0.push_back(b->tv_tiles);
    b->tv_tiles += tv_tile_count(W, H);
    b->pix0.push_back((int)b->pixels);
    b->pixels += (size_t)W * H;
    b->max_pixels = std::max(b->max_pixels, W * H);
    b->rc_w.push_back((int)v->hp.rc_width);
    b->rc_h.push_back((int)v->hp.rc_height);
    if (v->hp.enable_bayesian_update) b->has_psdf = true;
    else b->has_simple = true;
  }
  b->block_bytes = (sizeof(Scene) + sizeof(FrameConst)) * count;
  auto dal = [&](void **p, size_t bytes) {
    if (r != MH_OK) return;
    if (cudaMalloc(p, std::max<size_t>(bytes, 16)) != cudaSuccess) r = MH_ERR_NOMEM;
    else b->allocs.push_back(*p);
  };
  dal((void **)&b->d_block, b->block_bytes);
  dal((void **)&b->d_depth, b->pixels * sizeof(float));
  for (int p = 0; p < 2 && r == MH_OK; ++p) {
    if (cudaMallocHost((void **)&b->h_block[p], b->block_bytes) != cudaSuccess ||
        cudaMallocHost((void **)&b->h_depth[p], std::max<size_t>(b->pixels, 1) * sizeof(float)) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->block_free[p], cudaEventDisableTiming) != cudaSuccess)
      r = MH_ERR_NOMEM;
    else
      memset(b->h_block[p], 0, b->block_bytes);
  }
  for (int s = 0; s < count && r == MH_OK; ++s) {
    float *dd = nullptr, *dv = nullptr, *dn = nullptr;
    if (b->raycast) {
      const size_t np = (size_t)b->rc_w[s] * b->rc_h[s];
      dal((void **)&dd, np * sizeof(float));
      dal((void **)&dv, np * 4 * sizeof(float));
      dal((void **)&dn, np * 4 * sizeof(float));
    }
    b->out_depth.push_back(dd);
    b->out_vert.push_back(dv);
    b->out_norm.push_back(dn);
  }
  for (cudaEvent_t &e : b->ev)
    if (r == MH_OK && cudaEventCreate(&e) != cudaSuccess) r = MH_ERR_CUDA;
  for (cudaEvent_t &e : b->sev)
    if (r == MH_OK && cudaEventCreate(&e) != cudaSuccess) r = MH_ERR_CUDA;
  if (r == MH_OK && cudaStreamCreateWithFlags(&b->own, cudaStreamNonBlocking) != cudaSuccess) r = MH_ERR_CUDA;
  if (r == MH_OK) {
    mh_sm_count();
    batch_warm_occupancy();
    if (cudaGetLastError() != cudaSuccess) r = MH_ERR_CUDA;
  }
  if (r != MH_OK) {
    batch_free(b);
    return r;
  }
  *out = b;
  return MH_OK;
}

int mh_batch_destroy(mh_batch *b) {
  if (!b) return MH_ERR_INVALID;
  batch_free(b);
  return MH_OK;
}

int mh_batch_outputs(mh_batch *b, int scene, float **depth, float **vertex4, float **normal4) {
  if (!b || scene < 0 || scene >= b->n) return MH_ERR_INVALID;
  if (depth) *depth = b->out_depth[scene];
  if (vertex4) *vertex4 = b->out_vert[scene];
  if (normal4) *normal4 = b->out_norm[scene];
  return MH_OK;
}

int mh_batch_dump_raycast(mh_batch *b, int scene, float *depth, float *vertex4, float *normal4) {
  if (!b || scene < 0 || scene >= b->n || !b->raycast) return MH_ERR_INVALID;
  const size_t np = (size_t)b->rc_w[scene] * b->rc_h[scene];
  MH_CUDA_TRY(cudaDeviceSynchronize());
  if (depth) MH_CUDA_TRY(cudaMemcpy(depth, b->out_depth[scene], np * sizeof(float), cudaMemcpyDeviceToHost));
  if (vertex4) MH_CUDA_TRY(cudaMemcpy(vertex4, b->out_vert[scene], np * 16, cudaMemcpyDeviceToHost));
  if (normal4) MH_CUDA_TRY(cudaMemcpy(normal4, b->out_norm[scene], np * 16, cudaMemcpyDeviceToHost));
  return MH_OK;
}

int mh_batch_get_tuning(mh_batch *b, mh_batch_tuning *out) {
  if (!b || !out) return MH_ERR_INVALID;
  *out = b->tune;
  out->integrate_cta_per_sm = kCtaCaps[b->tune.integrate_cta_per_sm];
  return MH_OK;
}

int mh_batch_set_tuning(mh_batch *b, const mh_batch_tuning *t) {
  if (!b || !t || t->ray_tile_shape < 0 || t->ray_tile_shape >= ray_tile_shapes()) return MH_ERR_INVALID;
  int k = -1;
  for (int i = 0; i < 3; ++i)
    if (kCtaCaps[i] == t->integrate_cta_per_sm) k = i;
  if (k < 0) return MH_ERR_INVALID;
  b->tune.ray_tile_shape = t->ray_tile_shape;
  b->tune.integrate_cta_per_sm = k;
  return MH_OK;
}

int mh_batch_autotune(mh_batch *b, int trials) {
  if (!b || trials <= 0) return MH_ERR_INVALID;
  b->tune_left = trials * 9;
  b->tune_k = 0;
  b->stage_steps = 0;
  for (double &x : b->stage_ms) x = 0.0;
  for (int i = 0; i < 3; ++i) b->ray_ms[i] = b->int_ms[i] = 0.0, b->ray_cnt[i] = b->int_cnt[i] = 0;
  return MH_OK;
}

int mh_batch_stage_times(mh_batch *b, double ms[MH_STAGE_COUNT]) {
  if (!b || !ms) return MH_ERR_INVALID;
  for (int st = 0; st < MH_STAGE_COUNT; ++st) ms[st] = b->stage_steps ? b->stage_ms[st] / b->stage_steps : -1.0;
  return MH_OK;
}

int mh_batch_tuning_times(mh_batch *b, double ray_ms[3], double integrate_ms[3]) {
  if (!b || !ray_ms || !integrate_ms) return MH_ERR_INVALID;
  for (int i = 0; i < 3; ++i) {
    ray_ms[i] = b->ray_cnt[i] ? b->ray_ms[i] / b->ray_cnt[i] : -1.0;
    integrate_ms[i] = b->int_cnt[i] ? b->int_ms[i] / b->int_cnt[i] : -1.0;
  }
  return MH_OK;
}

int mh_batch_step(mh_batch *b, const float *const *depth, int depth_on_device, const float *wTc, const int *active,
                  int tv_iterations, float tv_lambda, int use_graph, void *stream) {
  if (!b || !depth || !wTc || tv_iterations < 0 || (tv_iterations > 0 && !(tv_lambda > 0.0f))) return MH_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  const int n = b->n;
  const int p = b->step & 1;
  // the block of two steps ago must have been consumed before it is rewritten
  if (b->block_used[p]) MH_CUDA_TRY(cudaEventSynchronize(b->block_free[p]));
  const bool tuning = b->tune_left > 0;
  if (tuning) {
    b->tune.ray_tile_shape = b->tune_k % 3;
    b->tune.integrate_cta_per_sm = (b->tune_k / 3) % 3;
  }
  Scene *tab = reinterpret_cast<Scene *>(b->h_block[p]);
  FrameConst *fcs = reinterpret_cast<FrameConst *>(b->h_block[p] + sizeof(Scene) * n);
  FrameConst *d_fc = reinterpret_cast<FrameConst *>(b->d_block + sizeof(Scene) * n);
  std::vector<int> ray0(n);
  b->ray_tiles(b->tune.ray_tile_shape, &ray0);
  for (int i = 0; i < n; ++i) {
    mh_volume *v = b->vols[i];
    Scene &sc = tab[i];
    const bool act = !active || active[i];
    sc.d = v->d;
    sc.d.fc = d_fc + i;
    sc.d.cellok = nullptr;  // the batched raycast runs without the per-block cell flags
    sc.tv = v->tv;
    sc.ray_depth = b->out_depth[i];
    sc.ray_vert = reinterpret_cast<float4 *>(b->out_vert[i]);
    sc.ray_norm = reinterpret_cast<float4 *>(b->out_norm[i]);
    sc.alloc_tile0 = b->alloc_tile0[i];
    sc.tv_tile0 = b->tv_tile0[i];
    sc.ray_tile0 = ray0[i];
    sc.pix0 = b->pix0[i];
    sc.active = act ? 1 : 0;
    sc.recycle = sc.starve = 0;
    if (!act) continue;
    const size_t np = (size_t)v->hp.width * v->hp.height;
    if (!depth[i]) return MH_ERR_INVALID;
    if (depth_on_device) {
      sc.src = depth[i];
    } else {
      memcpy(b->h_depth[p] + b->pix0[i], depth[i], np * sizeof(float));
      sc.src = b->d_depth + b->pix0[i];
    }
    // MainEngine's frame counter: recycle every 10 frames, starvation
    // (simple update) at frame 14 of every 15 (main_engine.cc:163-191)
    v->frames += 1;
    sc.recycle = v->frames % 10 == 0;
    sc.starve = !v->hp.enable_bayesian_update && v->frames % 15 == 14;
    FrameConst &fc = fcs[i];
    memcpy(fc.wTc, wTc + 16 * i, sizeof(float) * 16);
    inverse4(fc.wTc, fc.cTw);
    memcpy(fc.rc_cTw, fc.cTw, sizeof(float) * 16);
    inverse4(fc.rc_cTw, fc.rc_wTc);
    v->fc_host = fc;
    v->has_frame = true;
  }
  const bool host_depth = !depth_on_device;
  if (use_graph && !tuning) {
    const bool stale = !b->exec[p] || b->g_tv_it[p] != tv_iterations || b->g_lambda[p] != tv_lambda ||
                       b->g_host[p] != (host_depth ? 1 : 0) || b->g_tune[p].ray_tile_shape != b->tune.ray_tile_shape ||
                       b->g_tune[p].integrate_cta_per_sm != b->tune.integrate_cta_per_sm;
    if (stale) {
      if (b->exec[p]) cudaGraphExecDestroy(b->exec[p]);
      b->exec[p] = nullptr;
      cudaGraph_t g = nullptr;
      MH_CUDA_TRY(cudaStreamBeginCapture(b->own, cudaStreamCaptureModeThreadLocal));
      const int r = enqueue(b, p, host_depth, tv_iterations, tv_lambda, false, b->own);
      const cudaError_t e = cudaStreamEndCapture(b->own, &g);
      if (r != MH_OK) return r;
      if (e != cudaSuccess) return MH_ERR_CUDA;
      const cudaError_t ie = cudaGraphInstantiate(&b->exec[p], g, 0);
      cudaGraphDestroy(g);
      if (ie != cudaSuccess) return MH_ERR_CUDA;
      b->g_tv_it[p] = tv_iterations;
      b->g_lambda[p] = tv_lambda;
      b->g_host[p] = host_depth ? 1 : 0;
      b->g_tune[p] = b->tune;
    }
    MH_CUDA_TRY(cudaGraphLaunch(b->exec[p], s));
  } else {
    const int r = enqueue(b, p, host_depth, tv_iterations, tv_lambda, tuning, s);
    if (r != MH_OK) return r;
  }
  MH_CUDA_TRY(cudaEventRecord(b->block_free[p], s));
  b->block_used[p] = true;
  b->step += 1;
  if (tuning) {
    MH_CUDA_TRY(cudaEventSynchronize(b->block_free[p]));
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]) == cudaSuccess) {
      b->int_ms[b->tune.integrate_cta_per_sm] += ms;
      b->int_cnt[b->tune.integrate_cta_per_sm] += 1;
    }
    if (b->raycast && cudaEventElapsedTime(&ms, b->ev[2], b->ev[3]) == cudaSuccess) {
      b->ray_ms[b->tune.ray_tile_shape] += ms;
      b->ray_cnt[b->tune.ray_tile_shape] += 1;
    }
    for (int st = 0; st < MH_STAGE_COUNT; ++st)
      if (cudaEventElapsedTime(&ms, b->sev[st], b->sev[st + 1]) == cudaSuccess) b->stage_ms[st] += ms;
    b->stage_steps += 1;
    b->tune_k += 1;
    if (--b->tune_left == 0) {
      int best_r = 0, best_i = 0;
      for (int i = 1; i < 3; ++i) {
        if (b->ray_cnt[i] && b->ray_ms[i] / b->ray_cnt[i] < b->ray_ms[best_r] / std::max(b->ray_cnt[best_r], 1))
          best_r = i;
        if (b->int_cnt[i] && b->int_ms[i] / b->int_cnt[i] < b->int_ms[best_i] / std::max(b->int_cnt[best_i], 1))
          best_i = i;
      }
      b->tune.ray_tile_shape = best_r;
      b->tune.integrate_cta_per_sm = best_i;
    }
  }
  return MH_OK;
}

}  // extern "C"
