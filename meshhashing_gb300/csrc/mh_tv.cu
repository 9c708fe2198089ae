// mh_tv.cu -- primal-dual TV-L2 denoising of the input depth frame.
//
// No reference counterpart: the reference's only primal-dual code is a
// volumetric Huber-TV on voxel SDFs that is never called
// (optimize/primal_dual.cu:10-223).  This is Chambolle & Pock (2011),
// Algorithm 1 with theta = 1, on the ROF model
//     min_u  sum_edges |grad u| + lambda/2 * sum_valid (u - f)^2
// with depth in millimetres (the sensor's native unit), forward differences
// over pairs of valid pixels only (invalid pixels are holes with Neumann
// boundaries and stay invalid), tau = sigma = 1/sqrt(8).
//
// Two forms, bit-identical to each other:
//  * k_tv_iter, one launch per iteration (the allocation-free entry point):
//    each thread recomputes the dual update of its own pixel and of its left
//    and upper neighbours (the ones its divergence needs) from the previous
//    iterate, so the dual and primal steps fuse into a single pass with no
//    grid-wide barrier;
//  * k_tv_tile (a volume's frames) and its batch twin k_tv_tile_b: ten
//    iterations per launch on a 64 x 32 tile held in shared memory with a
//    10-pixel halo, so 20 iterations take 2 launches instead of 22.
#include "mh_internal.cuh"
#include "mh_kernels.h"
#include "mh_batch.cuh"

#include <algorithm>

namespace {

struct TvBuf {
  const float *f;
  const float *u, *ub, *px, *py;
  float *u2, *ub2, *px2, *py2;
  int W, H;
  float lambda;
};

__device__ __forceinline__ bool valid_at(const float *f, int i) { return f[i] > -1e30f; }

// dual update at pixel (x, y) from the previous iterate
__device__ __forceinline__ void dual_at(const TvBuf &b, int x, int y, float sigma, float &ox, float &oy) {
  const int i = y * b.W + x;
  const bool vi = valid_at(b.f, i);
  float gx = 0.0f, gy = 0.0f;
  if (vi && x + 1 < b.W && valid_at(b.f, i + 1)) gx = b.ub[i + 1] - b.ub[i];
  if (vi && y + 1 < b.H && valid_at(b.f, i + b.W)) gy = b.ub[i + b.W] - b.ub[i];
  const float qx = b.px[i] + sigma * gx;
  const float qy = b.py[i] + sigma * gy;
  const float nrm = fmaxf(1.0f, sqrtf(qx * qx + qy * qy));
  ox = qx / nrm;
  oy = qy / nrm;
}

}  // namespace

__device__ __forceinline__ void tv_init_body(const float *depth, float *f, float *u, float *ub, float *px, float *py, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float z = depth[i];
    const bool ok = z > 0.0f && z < 1e30f;
    const float v = ok ? z * 1000.0f : -__int_as_float(0x7f800000);
    f[i] = v;
    u[i] = v;
    ub[i] = v;
    px[i] = 0.0f;
    py[i] = 0.0f;
  }
}
__global__ void k_tv_init(const float *depth, float *f, float *u, float *ub, float *px, float *py, int n) { tv_init_body(depth, f, u, ub, px, py, n); }

__device__ __forceinline__ void tv_iter_body(const TvBuf &b) {
  const float tau = 0.35355339059327373f, sigma = 0.35355339059327373f;
  const int n = b.W * b.H;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int x = i % b.W, y = i / b.W;
    float pxc, pyc;
    dual_at(b, x, y, sigma, pxc, pyc);
    b.px2[i] = pxc;
    b.py2[i] = pyc;
    if (!valid_at(b.f, i)) {
      b.u2[i] = b.f[i];
      b.ub2[i] = b.f[i];
      continue;
    }
    float pxl = 0.0f, pyu = 0.0f, dummy;
    if (x > 0) dual_at(b, x - 1, y, sigma, pxl, dummy);
    if (y > 0) dual_at(b, x, y - 1, sigma, dummy, pyu);
    const float div = (pxc - pxl) + (pyc - pyu);
    const float u0 = b.u[i];
    const float un = (u0 + tau * div + tau * b.lambda * b.f[i]) / (1.0f + tau * b.lambda);
    b.u2[i] = un;
    b.ub2[i] = 2.0f * un - u0;
  }
}
__global__ void __launch_bounds__(256) k_tv_iter(TvBuf b) { tv_iter_body(b); }

__device__ __forceinline__ void tv_out_body(const float *f, const float *u, float *depth, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    depth[i] = valid_at(f, i) ? u[i] * 0.001f : -__int_as_float(0x7f800000);
}
__global__ void k_tv_out(const float *f, const float *u, float *depth, int n) { tv_out_body(f, u, depth, n); }
// a batch's TV result after `launches` tiled launches: planes 1-4 hold the
// iterate after an even number of launches, planes 5-8 after an odd number
__global__ void k_tv_out_b(const Scene *t, int n, int launches) {
  each_scene(t, n, [&](const Scene &c) {
    const size_t np = (size_t)c.d.p.width * c.d.p.height;
    tv_out_body(c.tv, c.tv + np * ((launches & 1) ? 5 : 1), c.d.depth, (int)np);
  });
}

// ------------------------------------------------------------------ tiled
// Up to TV_K iterations per launch for one TV_TW x TV_TH tile of pixels: the
// tile and a TV_K-pixel halo sit in shared memory, every iteration runs the
// dual step over the whole region, then the primal step, and values go stale
// by one pixel per iteration from the region's edge inwards, so the tile's
// own pixels stay exact through TV_K iterations.  Each value is computed by
// the same expressions as tv_iter_body (the dual of a neighbour is the
// neighbour's own new dual), so the result is bit-identical to running
// k_tv_iter once per iteration.  The first launch initialises from the depth
// frame (as k_tv_init), the last writes the frame back (as k_tv_out); between
// launches the iterate goes through the ping-pong planes.
#define TV_TW 64
#define TV_TH 32
#define TV_K 10
#define TV_RW (TV_TW + 2 * TV_K)
#define TV_RH (TV_TH + 2 * TV_K)
#define TV_RN (TV_RW * TV_RH)
constexpr size_t kTvTileSmem = sizeof(float) * 5 * TV_RN;

struct TvTile {
  const float *depth_in;  // first launch: the depth frame (metres); else null
  float *depth_out;       // last launch: the frame to write; else null
  float *f;               // input plane (written by the first launch)
  const float *u, *ub, *px, *py;  // iterate in (unused by the first launch)
  float *u2, *ub2, *px2, *py2;    // iterate out (unused by the last launch)
  int W, H, iters;
  float lambda;
};

__device__ __forceinline__ void tv_tile_body(const TvTile &b, int tile_x, int tile_y) {
  extern __shared__ float sm[];
  float *sf = sm, *su = sm + TV_RN, *sub = sm + 2 * TV_RN, *spx = sm + 3 * TV_RN, *spy = sm + 4 * TV_RN;
  const float tau = 0.35355339059327373f, sigma = 0.35355339059327373f;
  const int x0 = tile_x * TV_TW - TV_K, y0 = tile_y * TV_TH - TV_K;
  const float NI = -__int_as_float(0x7f800000);
  for (int r = threadIdx.x; r < TV_RN; r += blockDim.x) {
    const int gx = x0 + r % TV_RW, gy = y0 + r / TV_RW;
    float f = 0.0f, u = 0.0f, ub = 0.0f, px = 0.0f, py = 0.0f;
    if (gx >= 0 && gx < b.W && gy >= 0 && gy < b.H) {
      const int i = gy * b.W + gx;
      if (b.depth_in) {
        const float z = b.depth_in[i];
        const bool ok = z > 0.0f && z < 1e30f;
        f = u = ub = ok ? z * 1000.0f : NI;
      } else {
        f = b.f[i], u = b.u[i], ub = b.ub[i], px = b.px[i], py = b.py[i];
      }
    }
    sf[r] = f, su[r] = u, sub[r] = ub, spx[r] = px, spy[r] = py;
  }
  __syncthreads();
  for (int it = 0; it < b.iters; ++it) {
    // dual step (dual_at): forward differences of ub over valid pairs
    for (int r = threadIdx.x; r < TV_RN; r += blockDim.x) {
      const int lx = r % TV_RW, ly = r / TV_RW, gx = x0 + lx, gy = y0 + ly;
      const bool vi = sf[r] > -1e30f;
      float gxd = 0.0f, gyd = 0.0f;
      if (vi && gx + 1 < b.W && lx + 1 < TV_RW && sf[r + 1] > -1e30f) gxd = sub[r + 1] - sub[r];
      if (vi && gy + 1 < b.H && ly + 1 < TV_RH && sf[r + TV_RW] > -1e30f) gyd = sub[r + TV_RW] - sub[r];
      const float qx = spx[r] + sigma * gxd;
      const float qy = spy[r] + sigma * gyd;
      const float nrm = fmaxf(1.0f, sqrtf(qx * qx + qy * qy));
      spx[r] = qx / nrm;
      spy[r] = qy / nrm;
    }
    __syncthreads();
    // primal step and extrapolation (tv_iter_body)
    for (int r = threadIdx.x; r < TV_RN; r += blockDim.x) {
      if (!(sf[r] > -1e30f)) {
        su[r] = sf[r];
        sub[r] = sf[r];
        continue;
      }
      const int lx = r % TV_RW, ly = r / TV_RW, gx = x0 + lx, gy = y0 + ly;
      const float pxl = (gx > 0 && lx > 0) ? spx[r - 1] : 0.0f;
      const float pyu = (gy > 0 && ly > 0) ? spy[r - TV_RW] : 0.0f;
      const float div = (spx[r] - pxl) + (spy[r] - pyu);
      const float u0 = su[r];
      const float un = (u0 + tau * div + tau * b.lambda * sf[r]) / (1.0f + tau * b.lambda);
      su[r] = un;
      sub[r] = 2.0f * un - u0;
    }
    __syncthreads();
  }
  for (int k = threadIdx.x; k < TV_TW * TV_TH; k += blockDim.x) {
    const int lx = TV_K + k % TV_TW, ly = TV_K + k / TV_TW, gx = x0 + lx, gy = y0 + ly;
    if (gx >= b.W || gy >= b.H) continue;
    const int r = ly * TV_RW + lx, i = gy * b.W + gx;
    if (b.depth_in) b.f[i] = sf[r];
    if (b.depth_out) {
      b.depth_out[i] = sf[r] > -1e30f ? su[r] * 0.001f : NI;
    } else {
      b.u2[i] = su[r], b.ub2[i] = sub[r], b.px2[i] = spx[r], b.py2[i] = spy[r];
    }
  }
}
__global__ void __launch_bounds__(1024) k_tv_tile(TvTile b) { tv_tile_body(b, blockIdx.x, blockIdx.y); }

int tv_tile_count(int W, int H) { return ((W + TV_TW - 1) / TV_TW) * ((H + TV_TH - 1) / TV_TH); }

// Launch `launch` (of ceil(iterations / TV_K)) of the tiled TV for every
// active scene: the scenes' tiles are concatenated (Scene::tv_tile0); planes
// 1-4 of a scene's TV scratch hold the iterate after an even number of
// launches, planes 5-8 after an odd number.  Bit-identical to the single
// scene's launches, and so to one launch per iteration.
__global__ void __launch_bounds__(1024) k_tv_tile_b(const Scene *t, int n, int total, int launch, int iters, int last,
                                                    float lambda) {
  each_tile(t, n, total, &Scene::tv_tile0, [&](const Scene &c, int lt) {
    const int W = c.d.p.width, H = c.d.p.height;
    const size_t np = (size_t)W * H;
    float *A = c.tv + np * ((launch & 1) ? 5 : 1), *B = c.tv + np * ((launch & 1) ? 1 : 5);
    TvTile b;
    b.depth_in = launch == 0 ? c.d.depth : nullptr;
    b.depth_out = (launch > 0 && last) ? c.d.depth : nullptr;
    b.f = c.tv;
    b.u = A, b.ub = A + np, b.px = A + 2 * np, b.py = A + 3 * np;
    b.u2 = B, b.ub2 = B + np, b.px2 = B + 2 * np, b.py2 = B + 3 * np;
    b.W = W, b.H = H, b.iters = iters, b.lambda = lambda;
    const int tw = (W + TV_TW - 1) / TV_TW;
    tv_tile_body(b, lt % tw, lt / tw);
  });
}

int launch_denoise_tv_iterated(const Dev &d, float *tv, float lambda, int iterations, cudaStream_t s);

// tv holds 9 planes of W*H floats: f, (u, ub, px, py) x 2
int launch_denoise_tv(const Dev &d, float *tv, float lambda, int iterations, cudaStream_t s) {
  const int W = d.p.width, H = d.p.height, n = W * H;
  if (iterations <= 0) return launch_denoise_tv_iterated(d, tv, lambda, iterations, s);
  // 87 KB of dynamic shared memory needs the opt-in; the attribute belongs to
  // the current device, so it is set on every call (it is idempotent)
  if (cudaFuncSetAttribute(k_tv_tile, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTvTileSmem) !=
      cudaSuccess)
    return MH_ERR_CUDA;
  float *A[4] = {tv + (size_t)n, tv + 2 * (size_t)n, tv + 3 * (size_t)n, tv + 4 * (size_t)n};
  float *B[4] = {tv + 5 * (size_t)n, tv + 6 * (size_t)n, tv + 7 * (size_t)n, tv + 8 * (size_t)n};
  const dim3 grid((W + TV_TW - 1) / TV_TW, (H + TV_TH - 1) / TV_TH);
  int launches = 0;
  for (int done = 0; done < iterations; done += TV_K) {
    TvTile b;
    b.depth_in = done == 0 ? d.depth : nullptr;
    b.iters = std::min(TV_K, iterations - done);
    // the first launch reads the frame, so it never writes it back (other
    // tiles may still be reading their halos)
    b.depth_out = (done > 0 && done + b.iters == iterations) ? d.depth : nullptr;
    b.f = tv;
    b.u = A[0], b.ub = A[1], b.px = A[2], b.py = A[3];
    b.u2 = B[0], b.ub2 = B[1], b.px2 = B[2], b.py2 = B[3];
    b.W = W, b.H = H, b.lambda = lambda;
    k_tv_tile<<<grid, 1024, kTvTileSmem, s>>>(b);
    ++launches;
    for (int k = 0; k < 4; ++k) std::swap(A[k], B[k]);
  }
  if (iterations <= TV_K) {
    const int g = min((n + 255) / 256, mh_sm_count() * 8);
    k_tv_out<<<g, 256, 0, s>>>(tv, A[0], d.depth, n);
    ++launches;
  }
  mh_count_launches(launches);
  return cudaGetLastError() == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}

// the one-launch-per-iteration form (zero iterations, and the reference
// timing of the tiled form)
int launch_denoise_tv_iterated(const Dev &d, float *tv, float lambda, int iterations, cudaStream_t s) {
  const int W = d.p.width, H = d.p.height, n = W * H;
  const int g = min((n + 255) / 256, mh_sm_count() * 8);
  float *f = tv;
  float *A[4] = {tv + (size_t)n, tv + 2 * (size_t)n, tv + 3 * (size_t)n, tv + 4 * (size_t)n};
  float *B[4] = {tv + 5 * (size_t)n, tv + 6 * (size_t)n, tv + 7 * (size_t)n, tv + 8 * (size_t)n};
  k_tv_init<<<g, 256, 0, s>>>(d.depth, f, A[0], A[1], A[2], A[3], n);
  for (int it = 0; it < iterations; ++it) {
    TvBuf b;
    b.f = f;
    b.u = A[0], b.ub = A[1], b.px = A[2], b.py = A[3];
    b.u2 = B[0], b.ub2 = B[1], b.px2 = B[2], b.py2 = B[3];
    b.W = W, b.H = H, b.lambda = lambda;
    k_tv_iter<<<g, 256, 0, s>>>(b);
    for (int k = 0; k < 4; ++k) {
      float *t = A[k];
      A[k] = B[k];
      B[k] = t;
    }
  }
  k_tv_out<<<g, 256, 0, s>>>(f, A[0], d.depth, n);
  mh_count_launches(2 + iterations);
  return cudaGetLastError() == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}

// ------------------------------------------------------------------ no-alloc
// TV denoising for callers that cannot allocate device memory: the nine
// scratch planes live in a fixed file-scope device array.  See
// mh_denoise_tv_static in include/meshhash.h.
#include <mutex>

static __device__ __align__(256) float g_tv_static_scratch[(size_t)MH_TV_STATIC_MAX_PIXELS * 9];

namespace {
std::mutex g_tv_static_mu;
float *g_tv_static_ptr[64] = {nullptr};  // per device: address of the array above
}  // namespace

extern "C" int mh_denoise_tv_static(const float *depth_in, float *depth_out, int width, int height, float lambda,
                                    int iterations, void *stream) {
  if (!depth_in || !depth_out || width <= 0 || height <= 0 || iterations < 0 || !(lambda > 0.0f))
    return MH_ERR_INVALID;
  if ((long long)width * height > (long long)MH_TV_STATIC_MAX_PIXELS) return MH_ERR_CAPACITY;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return MH_ERR_CUDA;
  cudaStream_t s = (cudaStream_t)stream;
  float *scratch = nullptr;
  {
    // Host code only sees a host-side stand-in for the array, so its device
    // address is looked up with the device current.  Outside a stream
    // capture the lookup runs on every call: after cudaDeviceReset the
    // module is loaded again and the array may sit at another address.
    // While the stream captures, the address found by the last call outside
    // a capture on this device is used.
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) return MH_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_tv_static_mu);
    if (cap == cudaStreamCaptureStatusNone) {
      void *p = nullptr;
      if (cudaGetSymbolAddress(&p, g_tv_static_scratch) != cudaSuccess || !p) return MH_ERR_CUDA;
      g_tv_static_ptr[dev] = static_cast<float *>(p);
    }
    scratch = g_tv_static_ptr[dev];
    if (!scratch) return MH_ERR_INVALID;
  }
  const int n = width * height;
  const int g = min((n + 255) / 256, mh_sm_count() * 8);
  float *f = scratch;
  float *A[4] = {scratch + (size_t)n, scratch + 2 * (size_t)n, scratch + 3 * (size_t)n, scratch + 4 * (size_t)n};
  float *B[4] = {scratch + 5 * (size_t)n, scratch + 6 * (size_t)n, scratch + 7 * (size_t)n,
                 scratch + 8 * (size_t)n};
  // every plane the iterations read is written here first, so no state from
  // an earlier call leaks into this one
  k_tv_init<<<g, 256, 0, s>>>(depth_in, f, A[0], A[1], A[2], A[3], n);
  for (int it = 0; it < iterations; ++it) {
    TvBuf b;
    b.f = f;
    b.u = A[0], b.ub = A[1], b.px = A[2], b.py = A[3];
    b.u2 = B[0], b.ub2 = B[1], b.px2 = B[2], b.py2 = B[3];
    b.W = width, b.H = height, b.lambda = lambda;
    k_tv_iter<<<g, 256, 0, s>>>(b);
    for (int k = 0; k < 4; ++k) {
      float *t = A[k];
      A[k] = B[k];
      B[k] = t;
    }
  }
  k_tv_out<<<g, 256, 0, s>>>(f, A[0], depth_out, n);
  mh_count_launches(2 + iterations);
  return cudaGetLastError() == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}

// ------------------------------------------------------------------ batched
// The batch's TV: the tiled kernel over all scenes' tiles, TV_K iterations
// per launch (20 iterations: 2 launches instead of 22).
int launch_batch_tv(const Scene *t, int n, int tv_tiles, float lambda, int iterations, cudaStream_t s) {
  if (iterations <= 0 || tv_tiles <= 0) return MH_OK;
  if (cudaFuncSetAttribute(k_tv_tile_b, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTvTileSmem) !=
      cudaSuccess)
    return MH_ERR_CUDA;
  const int launches = (iterations + TV_K - 1) / TV_K;
  const int g = std::max(1, std::min(tv_tiles, mh_sm_count() * 2));
  for (int k = 0; k < launches; ++k) {
    const int iters = std::min(TV_K, iterations - k * TV_K);
    k_tv_tile_b<<<g, 1024, kTvTileSmem, s>>>(t, n, tv_tiles, k, iters, k == launches - 1 ? 1 : 0, lambda);
  }
  int count = launches;
  if (launches == 1) {
    // one launch reads the frame, so the result is written back separately
    const int g2 = std::max(1, mh_sm_count() * 8);
    k_tv_out_b<<<g2, 256, 0, s>>>(t, n, 1);
    ++count;
  }
  mh_count_launches(count);
  return cudaGetLastError() == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}
