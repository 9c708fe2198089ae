// mh_huber.cu -- volumetric Huber-TV smoothing of the fused sdf.
//
// The reference's primal-dual regulariser (optimize/primal_dual.cu:10-223 with
// the neighbour queries of geometry/primal_dual_query.h:15-234), which its
// engines never call, as an optional post-fusion stage over the candidate
// blocks:
//   init   for voxels with inv_sigma2 >= 1e-6: weight = exp(|grad sdf| / voxel)
//          from forward differences (0 when a +x/+y/+z neighbour is missing or
//          unobserved), sdf0 = sdf, sdf_bar = 0, p = 0, mask set;
//   pass 1 (dual)   data error (sdf - sdf0)^2 and Huber(|grad sdf|, 0.02);
//          p = (p + sigma grad sdf_bar) / (1 + sigma alpha), then p /= max(1, |p|);
//   pass 2 (primal) div = sum_i (p(v - e_i) - p(v))_i; sdf -= tau div;
//          sdf = (sdf + lambda w tau sdf0) / (1 + lambda w tau); sdf = sdf0
//          where w > 2; sdf_bar = 2 sdf - sdf_prev.
// Differences use face neighbours that exist, are observed and carry the
// mask; otherwise the gradient (or divergence) is 0, as in the reference.
// The per-voxel state (7 words, plus one for the per-call work list) lives in
// arrays laid out like the voxel storage, allocated on first use; the mask is an epoch stamp, so voxels not
// initialised by the latest init read as unmasked.  Every pass runs one
// thread per candidate voxel over a face-neighbour table that is built once
// per call, so no pass waits on a hash probe.
#include <cstring>

#include "mh_kernels.h"
#include "mh_volume.h"

namespace {

constexpr float kEps = 1e-6f;     // EPSILON (core/common.h:62)
constexpr float kAlpha = 0.02f;   // Huber threshold (primal_dual.cu:60)

struct PD {
  float *sdf0, *bar, *w, *px, *py, *pz;
  unsigned *mask;
  unsigned epoch;
};

__device__ __forceinline__ float huber(float x, float a) { return fabsf(x) < a ? 0.5f * (x * x) / a : fabsf(x) - 0.5f * a; }

__device__ __forceinline__ int cand_count(const Dev &d) { return *reinterpret_cast<volatile int *>(&d.ctr->cand_count); }

// Face-neighbour table of the candidate list: nbt[6 c + 2 k + (s < 0)] is
// the pool index of the block next to candidate c along axis k, direction
// s (-1 when absent).  One lookup per thread, so the table costs one pass of
// independent hash probes instead of a serial probe per block and pass.
__global__ void __launch_bounds__(256) k_pd_faces(Dev d, int *nbt) {
  const int n = cand_count(d);
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < 6 * n; t += gridDim.x * blockDim.x) {
    const int c = t / 6, j = t - 6 * c;
    const int4 cb = d.cand[c];
    int q = -1;
    if (cb.w >= 0) {
      const int k = j >> 1, s = (j & 1) ? -1 : 1;
      q = hash_find(d, cb.x + (k == 0) * s, cb.y + (k == 1) * s, cb.z + (k == 2) * s);
    }
    nbt[t] = q;
  }
}

// Global voxel index of the face neighbour (axis k, direction s) of local
// voxel li (= x + 8 y + 64 z) of candidate c in pool block blk; -1 when the
// neighbour's block does not exist.
template <int K, int S>
__device__ __forceinline__ long long face(const int *nbt, int c, int blk, int li) {
  constexpr int sh = 3 * K;
  const int cn = ((li >> sh) & 7) + S;
  if ((unsigned)cn > 7u) {
    const int q = __ldg(nbt + 6 * c + 2 * K + (S < 0));
    return q < 0 ? -1 : (long long)q * MH_BLOCK_VOXELS + ((li & ~(7 << sh)) | ((cn & 7) << sh));
  }
  return (long long)blk * MH_BLOCK_VOXELS + li + S * (1 << sh);
}

template <int S>
__device__ __forceinline__ void faces(const int *nbt, int c, int blk, int li, long long (&q)[3]) {
  q[0] = face<0, S>(nbt, c, blk, li);
  q[1] = face<1, S>(nbt, c, blk, li);
  q[2] = face<2, S>(nbt, c, blk, li);
}

// neighbour usable by the masked queries: block exists, voxel observed, mask set
__device__ __forceinline__ bool usable(const Dev &d, const PD &pd, long long g) {
  return g >= 0 && d.w[g] >= kEps && pd.mask[g] == pd.epoch;
}

// The init loop runs one thread per voxel of the candidate list, grid-stride
// over candidates x 512; a warp covers 32 voxels of one block.
#define PD_FOR_EACH_VOXEL(d, n)                                                                   \
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < (long long)(n) * 512; \
       t += (long long)gridDim.x * blockDim.x)

__global__ void __launch_bounds__(256) k_pd_init(Dev d, PD pd, const int *nbt) {
  const int n = cand_count(d);
  PD_FOR_EACH_VOXEL(d, n) {
    const int c = (int)(t >> 9), li = (int)(t & 511);
    const int blk = d.cand[c].w;
    if (blk < 0) continue;
    const long long g = (long long)blk * MH_BLOCK_VOXELS + li;
    if (d.w[g] < kEps) continue;
    long long q[3];
    faces<1>(nbt, c, blk, li, q);
    bool ok = true;
#pragma unroll
    for (int k = 0; k < 3; ++k) ok &= q[k] >= 0 && d.w[q[k]] >= kEps;
    const float s = d.sdf[g];
    float gr[3] = {0.0f, 0.0f, 0.0f};
    if (ok) {
#pragma unroll
      for (int k = 0; k < 3; ++k) gr[k] = d.sdf[q[k]] - s;
    }
    const float len = sqrtf(gr[0] * gr[0] + gr[1] * gr[1] + gr[2] * gr[2]);
    pd.w[g] = expf(len / d.p.voxel_size);
    pd.sdf0[g] = s;
    pd.bar[g] = 0.0f;
    pd.px[g] = pd.py[g] = pd.pz[g] = 0.0f;
    pd.mask[g] = pd.epoch;
  }
}

// Work list of a call: (candidate << 9 | local voxel) of every observed,
// masked candidate voxel, one CTA per candidate block, one atomic per block.
// Each voxel's update reads only the previous pass's state, so the order of
// the list does not change the result.
__global__ void __launch_bounds__(256) k_pd_list(Dev d, PD pd, unsigned *list, int *count) {
  __shared__ int wsum[8], base;
  const int n = cand_count(d);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int c = blockIdx.x; c < n; c += gridDim.x) {
    const int blk = d.cand[c].w;
    bool f[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const long long g = (long long)blk * MH_BLOCK_VOXELS + threadIdx.x + 256 * h;
      f[h] = blk >= 0 && d.w[g] >= kEps && pd.mask[g] == pd.epoch;
    }
    const unsigned b0 = __ballot_sync(0xffffffffu, f[0]), b1 = __ballot_sync(0xffffffffu, f[1]);
    if (lane == 0) wsum[wid] = __popc(b0) + __popc(b1);
    __syncthreads();
    if (threadIdx.x == 0) {
      int tot = 0;
      for (int w = 0; w < 8; ++w) {
        const int x = wsum[w];
        wsum[w] = tot;
        tot += x;
      }
      base = tot ? atomicAdd(count, tot) : 0;
    }
    __syncthreads();
    const unsigned lt = (1u << lane) - 1u;
    int o = base + wsum[wid];
    if (f[0]) list[o + __popc(b0 & lt)] = ((unsigned)c << 9) | threadIdx.x;
    o += __popc(b0);
    if (f[1]) list[o + __popc(b1 & lt)] = ((unsigned)c << 9) | (threadIdx.x + 256);
    __syncthreads();
  }
}

template <int NV> __device__ __forceinline__ void cta_sum(float (&v)[NV], double *acc) {
  __shared__ float red[NV][8];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int k = 0; k < NV; ++k) {
    float x = v[k];
    for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) red[k][wid] = x;
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[threadIdx.x][w];
    atomicAdd(acc + threadIdx.x, s);
  }
}

// dual step and energies (PrimalDualIteratePass1Kernel)
__global__ void __launch_bounds__(256) k_pd_dual(Dev d, PD pd, const int *nbt, const unsigned *list,
                                                 const int *count, float sigma, double *err) {
  const int n = *count;
  float e[2] = {0.0f, 0.0f};
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const unsigned code = list[t];
    const int c = (int)(code >> 9), li = (int)(code & 511);
    const int blk = d.cand[c].w;
    const long long g = (long long)blk * MH_BLOCK_VOXELS + li;
    long long q[3];
    faces<1>(nbt, c, blk, li, q);
    bool ok = true;
#pragma unroll
    for (int k = 0; k < 3; ++k) ok &= usable(d, pd, q[k]);
    const float s = d.sdf[g], b = pd.bar[g];
    float gs[3] = {0.0f, 0.0f, 0.0f}, gb[3] = {0.0f, 0.0f, 0.0f};
    if (ok) {
#pragma unroll
      for (int k = 0; k < 3; ++k) gs[k] = d.sdf[q[k]] - s, gb[k] = pd.bar[q[k]] - b;
    }
    const float dd = fabsf(s - pd.sdf0[g]);
    e[0] += dd * dd;
    e[1] += huber(sqrtf(gs[0] * gs[0] + gs[1] * gs[1] + gs[2] * gs[2]), kAlpha);
    float px = pd.px[g] + sigma * gb[0], py = pd.py[g] + sigma * gb[1], pz = pd.pz[g] + sigma * gb[2];
    const float h = 1.0f + sigma * kAlpha;
    px /= h, py /= h, pz /= h;
    const float nrm = fmaxf(1.0f, sqrtf(px * px + py * py + pz * pz));
    pd.px[g] = px / nrm, pd.py[g] = py / nrm, pd.pz[g] = pz / nrm;
  }
  cta_sum<2>(e, err);
}

// primal step and extrapolation (PrimalDualIteratePass2Kernel)
__global__ void __launch_bounds__(256) k_pd_primal(Dev d, PD pd, const int *nbt, const unsigned *list,
                                                   const int *count, float lambda, float tau) {
  const int n = *count;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const unsigned code = list[t];
    const int c = (int)(code >> 9), li = (int)(code & 511);
    const int blk = d.cand[c].w;
    const long long g = (long long)blk * MH_BLOCK_VOXELS + li;
    long long q[3];
    faces<-1>(nbt, c, blk, li, q);
    bool ok = true;
#pragma unroll
    for (int k = 0; k < 3; ++k) ok &= usable(d, pd, q[k]);
    float div = 0.0f;
    if (ok) div = (pd.px[q[0]] - pd.px[g]) + (pd.py[q[1]] - pd.py[g]) + (pd.pz[q[2]] - pd.pz[g]);
    const float prev = d.sdf[g], s0 = pd.sdf0[g], w = pd.w[g];
    const float lam = lambda * w;
    float s = prev - tau * div;
    s = (s + lam * tau * s0) / (1.0f + lam * tau);
    if (w > 2.0f) s = s0;
    d.sdf[g] = s;
    const int dpos = sdf_nonneg(s) - sdf_nonneg(prev);
    if (dpos) atomicAdd(d.nnc + blk, dpos);
    pd.bar[g] = 2.0f * s - prev;
  }
}

}  // namespace

struct mh_pd_state {
  PD pd;
  size_t voxels = 0;
  double *err = nullptr;
  int *nbt = nullptr;   // face-neighbour table of the candidate list (6 per candidate)
  unsigned *list = nullptr;  // work list of the call (one entry per observed, masked voxel)
  int *count = nullptr;      // its length
};

static int grid_of(const void *fn) { return mh_resident_grid(fn, 256, 8); }

static int pd_ensure(mh_volume *v) {
  if (v->pd) return MH_OK;
  if (v->hp.value_capacity > (1u << 23)) return MH_ERR_INVALID;  // work-list entries hold candidate << 9
  mh_pd_state *st = new mh_pd_state();
  const size_t nv = (size_t)v->hp.value_capacity * MH_BLOCK_VOXELS;
  float **f[6] = {&st->pd.sdf0, &st->pd.bar, &st->pd.w, &st->pd.px, &st->pd.py, &st->pd.pz};
  bool ok = true;
  for (float **p : f) ok = ok && cudaMalloc((void **)p, sizeof(float) * nv) == cudaSuccess;
  ok = ok && cudaMalloc((void **)&st->pd.mask, sizeof(unsigned) * nv) == cudaSuccess;
  ok = ok && cudaMalloc((void **)&st->err, sizeof(double) * 2) == cudaSuccess;
  ok = ok && cudaMalloc((void **)&st->nbt, sizeof(int) * 6 * (size_t)v->hp.value_capacity) == cudaSuccess;
  ok = ok && cudaMalloc((void **)&st->list, sizeof(unsigned) * nv) == cudaSuccess;
  ok = ok && cudaMalloc((void **)&st->count, sizeof(int)) == cudaSuccess;
  ok = ok && cudaMemset(st->pd.mask, 0, sizeof(unsigned) * nv) == cudaSuccess;
  st->pd.epoch = 0;
  st->voxels = nv;
  v->pd = st;
  if (!ok) {
    cudaGetLastError();  // the failed allocation must not surface at the next launch check
    mh_pd_free(v);
    return MH_ERR_NOMEM;
  }
  return MH_OK;
}

void mh_pd_free(mh_volume *v) {
  mh_pd_state *st = v->pd;
  if (!st) return;
  for (void *p : {(void *)st->pd.sdf0, (void *)st->pd.bar, (void *)st->pd.w, (void *)st->pd.px, (void *)st->pd.py,
                  (void *)st->pd.pz, (void *)st->pd.mask, (void *)st->err, (void *)st->nbt,
                  (void *)st->list, (void *)st->count})
    if (p) cudaFree(p);
  delete st;
  v->pd = nullptr;
}

extern "C" {

int mh_huber_tv_init(mh_volume *v, void *stream) {
  if (!v) return MH_ERR_INVALID;
  int r = pd_ensure(v);
  if (r != MH_OK) return r;
  mh_pd_state *st = v->pd;
  st->pd.epoch += 1;
  cudaStream_t s = (cudaStream_t)stream;
  k_pd_faces<<<grid_of((const void *)k_pd_faces), 256, 0, s>>>(v->d, st->nbt);
  k_pd_init<<<grid_of((const void *)k_pd_init), 256, 0, s>>>(v->d, st->pd, st->nbt);
  mh_count_launches(2);
  return cudaGetLastError() == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}

int mh_huber_tv_iterate(mh_volume *v, float lambda, float sigma, float tau, int iterations, double *energy,
                        void *stream) {
  if (!v || iterations < 0) return MH_ERR_INVALID;
  if (!v->pd || v->pd->pd.epoch == 0) return MH_ERR_STATE;
  cudaStream_t s = (cudaStream_t)stream;
  mh_pd_state *st = v->pd;
  double last[2] = {0.0, 0.0};
  if (iterations > 0) {
    // the candidate list may have changed since init: rebuild the face table
    // and the work list of this call (neither pass changes w or the mask)
    k_pd_faces<<<grid_of((const void *)k_pd_faces), 256, 0, s>>>(v->d, st->nbt);
    MH_CUDA_TRY(cudaMemsetAsync(st->count, 0, sizeof(int), s));
    k_pd_list<<<grid_of((const void *)k_pd_list), 256, 0, s>>>(v->d, st->pd, st->list, st->count);
    mh_count_launches(2);
  }
  const int gd = grid_of((const void *)k_pd_dual), gp = grid_of((const void *)k_pd_primal);
  for (int it = 0; it < iterations; ++it) {
    MH_CUDA_TRY(cudaMemsetAsync(st->err, 0, sizeof(double) * 2, s));
    k_pd_dual<<<gd, 256, 0, s>>>(v->d, st->pd, st->nbt, st->list, st->count, sigma, st->err);
    k_pd_primal<<<gp, 256, 0, s>>>(v->d, st->pd, st->nbt, st->list, st->count, lambda, tau);
    mh_count_launches(2);
  }
  MH_CUDA_TRY(cudaGetLastError());
  if (energy && iterations > 0) {
    MH_CUDA_TRY(cudaMemcpyAsync(last, st->err, sizeof(last), cudaMemcpyDeviceToHost, s));
    MH_CUDA_TRY(cudaStreamSynchronize(s));
    // as the reference prints it: lambda / 2 * data + tv, then data, tv
    energy[0] = last[0] * lambda / 2.0 + last[1];
    energy[1] = last[0];
    energy[2] = last[1];
  }
  return MH_OK;
}

}  // extern "C"
