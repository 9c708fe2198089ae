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
// The per-voxel state (7 words) lives in arrays laid out like the voxel
// storage, allocated on first use; the mask is an epoch stamp, so blocks
// reused since the last init read as unmasked.
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

// the CTA's block and its six face neighbours (index 1 + 2k: +axis k, 2 + 2k: -axis k)
__device__ __forceinline__ void load_neighbours(const Dev &d, int4 cb, int *nb) {
  if (threadIdx.x < 7) {
    int q = cb.w;
    if (threadIdx.x > 0) {
      const int k = (threadIdx.x - 1) >> 1, s = ((threadIdx.x - 1) & 1) ? -1 : 1;
      q = hash_find(d, cb.x + (k == 0) * s, cb.y + (k == 1) * s, cb.z + (k == 2) * s);
    }
    nb[threadIdx.x] = q;
  }
  __syncthreads();
}

// global voxel index of the face neighbour (axis k, direction s) of local voxel li
__device__ __forceinline__ long long neighbour(const int *nb, int li, int k, int s) {
  int c[3] = {li & 7, (li >> 3) & 7, li >> 6};
  c[k] += s;
  int blk = nb[0];
  if (c[k] < 0 || c[k] > 7) {
    blk = nb[1 + 2 * k + (s < 0)];
    c[k] &= 7;
  }
  if (blk < 0) return -1;
  return (long long)blk * MH_BLOCK_VOXELS + c[0] + c[1] * 8 + c[2] * 64;
}

__device__ __forceinline__ bool usable(const Dev &d, const PD &pd, long long g) {
  return g >= 0 && d.w[g] >= kEps && pd.mask[g] == pd.epoch;
}

__global__ void __launch_bounds__(256) k_pd_init(Dev d, PD pd) {
  __shared__ int nb[7];
  const int n = *reinterpret_cast<volatile int *>(&d.ctr->cand_count);
  for (int c = blockIdx.x; c < n; c += gridDim.x) {
    const int4 cb = d.cand[c];
    __syncthreads();
    if (cb.w < 0) continue;
    load_neighbours(d, cb, nb);
    for (int li = threadIdx.x; li < MH_BLOCK_VOXELS; li += blockDim.x) {
      const long long g = (long long)cb.w * MH_BLOCK_VOXELS + li;
      if (d.w[g] < kEps) continue;
      const float s = d.sdf[g];
      float gr[3] = {0.0f, 0.0f, 0.0f};
      bool ok = true;
      for (int k = 0; k < 3 && ok; ++k) {
        const long long q = neighbour(nb, li, k, 1);
        ok = q >= 0 && d.w[q] >= kEps;
        if (ok) gr[k] = d.sdf[q] - s;
      }
      if (!ok) gr[0] = gr[1] = gr[2] = 0.0f;
      const float len = sqrtf(gr[0] * gr[0] + gr[1] * gr[1] + gr[2] * gr[2]);
      pd.w[g] = expf(len / d.p.voxel_size);
      pd.sdf0[g] = s;
      pd.bar[g] = 0.0f;
      pd.px[g] = pd.py[g] = pd.pz[g] = 0.0f;
      pd.mask[g] = pd.epoch;
    }
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
  __syncthreads();
}

// forward differences of field f at g (0 when a neighbour is not usable)
__device__ __forceinline__ void fwd_grad(const Dev &d, const PD &pd, const int *nb, int li, long long g,
                                         const float *f, float (&gr)[3]) {
  gr[0] = gr[1] = gr[2] = 0.0f;
  float v[3];
  for (int k = 0; k < 3; ++k) {
    const long long q = neighbour(nb, li, k, 1);
    if (!usable(d, pd, q)) return;
    v[k] = f[q];
  }
  const float c = f[g];
  gr[0] = v[0] - c, gr[1] = v[1] - c, gr[2] = v[2] - c;
}

__global__ void __launch_bounds__(256) k_pd_dual(Dev d, PD pd, float sigma, double *err) {
  __shared__ int nb[7];
  const int n = *reinterpret_cast<volatile int *>(&d.ctr->cand_count);
  float e[2] = {0.0f, 0.0f};
  for (int c = blockIdx.x; c < n; c += gridDim.x) {
    const int4 cb = d.cand[c];
    __syncthreads();
    if (cb.w < 0) continue;
    load_neighbours(d, cb, nb);
    for (int li = threadIdx.x; li < MH_BLOCK_VOXELS; li += blockDim.x) {
      const long long g = (long long)cb.w * MH_BLOCK_VOXELS + li;
      if (d.w[g] < kEps || pd.mask[g] != pd.epoch) continue;
      const float dd = fabsf(d.sdf[g] - pd.sdf0[g]);
      e[0] += dd * dd;
      float gs[3], gb[3];
      fwd_grad(d, pd, nb, li, g, d.sdf, gs);
      e[1] += huber(sqrtf(gs[0] * gs[0] + gs[1] * gs[1] + gs[2] * gs[2]), kAlpha);
      fwd_grad(d, pd, nb, li, g, pd.bar, gb);
      float px = pd.px[g] + sigma * gb[0], py = pd.py[g] + sigma * gb[1], pz = pd.pz[g] + sigma * gb[2];
      const float h = 1.0f + sigma * kAlpha;
      px /= h, py /= h, pz /= h;
      const float nrm = fmaxf(1.0f, sqrtf(px * px + py * py + pz * pz));
      pd.px[g] = px / nrm, pd.py[g] = py / nrm, pd.pz[g] = pz / nrm;
    }
  }
  cta_sum<2>(e, err);
}

__global__ void __launch_bounds__(256) k_pd_primal(Dev d, PD pd, float lambda, float tau) {
  __shared__ int nb[7];
  const int n = *reinterpret_cast<volatile int *>(&d.ctr->cand_count);
  for (int c = blockIdx.x; c < n; c += gridDim.x) {
    const int4 cb = d.cand[c];
    __syncthreads();
    if (cb.w < 0) continue;
    load_neighbours(d, cb, nb);
    for (int li = threadIdx.x; li < MH_BLOCK_VOXELS; li += blockDim.x) {
      const long long g = (long long)cb.w * MH_BLOCK_VOXELS + li;
      if (d.w[g] < kEps || pd.mask[g] != pd.epoch) continue;
      float div = 0.0f;
      {
        float pn[3];
        bool ok = true;
        const float *comp[3] = {pd.px, pd.py, pd.pz};
        for (int k = 0; k < 3 && ok; ++k) {
          const long long q = neighbour(nb, li, k, -1);
          ok = usable(d, pd, q);
          if (ok) pn[k] = comp[k][q];
        }
        if (ok) div = (pn[0] - pd.px[g]) + (pn[1] - pd.py[g]) + (pn[2] - pd.pz[g]);
      }
      const float prev = d.sdf[g];
      const float lam = lambda * pd.w[g];
      float s = prev - tau * div;
      s = (s + lam * tau * pd.sdf0[g]) / (1.0f + lam * tau);
      if (pd.w[g] > 2.0f) s = pd.sdf0[g];
      d.sdf[g] = s;
      pd.bar[g] = 2.0f * s - prev;
    }
  }
}

}  // namespace

struct mh_pd_state {
  PD pd;
  size_t voxels = 0;
  double *err = nullptr;
};

static int pd_ensure(mh_volume *v) {
  if (v->pd) return MH_OK;
  mh_pd_state *st = new mh_pd_state();
  const size_t nv = (size_t)v->hp.value_capacity * MH_BLOCK_VOXELS;
  float **f[6] = {&st->pd.sdf0, &st->pd.bar, &st->pd.w, &st->pd.px, &st->pd.py, &st->pd.pz};
  bool ok = true;
  for (float **p : f) ok = ok && cudaMalloc((void **)p, sizeof(float) * nv) == cudaSuccess;
  ok = ok && cudaMalloc((void **)&st->pd.mask, sizeof(unsigned) * nv) == cudaSuccess;
  ok = ok && cudaMalloc((void **)&st->err, sizeof(double) * 2) == cudaSuccess;
  ok = ok && cudaMemset(st->pd.mask, 0, sizeof(unsigned) * nv) == cudaSuccess;
  st->pd.epoch = 0;
  st->voxels = nv;
  v->pd = st;
  if (!ok) {
    mh_pd_free(v);
    return MH_ERR_NOMEM;
  }
  return MH_OK;
}

void mh_pd_free(mh_volume *v) {
  mh_pd_state *st = v->pd;
  if (!st) return;
  for (void *p : {(void *)st->pd.sdf0, (void *)st->pd.bar, (void *)st->pd.w, (void *)st->pd.px, (void *)st->pd.py,
                  (void *)st->pd.pz, (void *)st->pd.mask, (void *)st->err})
    if (p) cudaFree(p);
  delete st;
  v->pd = nullptr;
}

extern "C" {

int mh_huber_tv_init(mh_volume *v, void *stream) {
  if (!v) return MH_ERR_INVALID;
  int r = pd_ensure(v);
  if (r != MH_OK) return r;
  v->pd->pd.epoch += 1;
  k_pd_init<<<mh_sm_count() * 8, 256, 0, (cudaStream_t)stream>>>(v->d, v->pd->pd);
  mh_count_launches(1);
  return cudaGetLastError() == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}

int mh_huber_tv_iterate(mh_volume *v, float lambda, float sigma, float tau, int iterations, double *energy,
                        void *stream) {
  if (!v || iterations < 0) return MH_ERR_INVALID;
  if (!v->pd || v->pd->pd.epoch == 0) return MH_ERR_STATE;
  cudaStream_t s = (cudaStream_t)stream;
  const int g = mh_sm_count() * 8;
  double last[2] = {0.0, 0.0};
  for (int it = 0; it < iterations; ++it) {
    MH_CUDA_TRY(cudaMemsetAsync(v->pd->err, 0, sizeof(double) * 2, s));
    k_pd_dual<<<g, 256, 0, s>>>(v->d, v->pd->pd, sigma, v->pd->err);
    k_pd_primal<<<g, 256, 0, s>>>(v->d, v->pd->pd, lambda, tau);
    mh_count_launches(2);
  }
  MH_CUDA_TRY(cudaGetLastError());
  if (energy && iterations > 0) {
    MH_CUDA_TRY(cudaMemcpyAsync(last, v->pd->err, sizeof(last), cudaMemcpyDeviceToHost, s));
    MH_CUDA_TRY(cudaStreamSynchronize(s));
    // as the reference prints it: lambda / 2 * data + tv, then data, tv
    energy[0] = last[0] * lambda / 2.0 + last[1];
    energy[1] = last[0];
    energy[2] = last[1];
  }
  return MH_OK;
}

}  // extern "C"
