// mh_raycast.cu -- trilinear raycast of the zero level set.
//
// CastKernel (visualization/ray_caster.cu:16-150): one thread per pixel
// marches the camera ray with a fixed step from min to max raycast depth,
// samples the SDF trilinearly (GetSpatialValue, geometry/spatial_query.h:23-66),
// and on a + to - sign change refines the hit with three regula-falsi steps
// (BisectionIntersection, geometry/isosurface_intersection.h:21-55).  The
// sample positions, the accumulation of t and every comparison follow the
// reference's single-precision order exactly.
//
// GB300 structure.  The march is bound by instruction issue and by the
// latency of its dependent loads, not by HBM bandwidth, so the work per
// sample is what is cut, never the sample sequence itself:
//  * one gather for every sample: the eight corners' blocks come from a
//    per-ray table of the first corner block's 2x2x2 neighbourhood, filled by
//    hash lookups only when a sample first needs an entry.  Samples whose
//    corners straddle a block face take the same instructions as the others,
//    so the lanes of a warp stay together (a separate slow path for the third
//    of samples that straddle a face cost 1.45x in time).
//  * one out-of-line sampler serves the march, the refinement and the
//    gradient.  Inlined three times the kernel outgrew the instruction cache
//    and its register budget (measured 1.5x slower).
//  * empty-space skip: when the block holding a sample's first corner is
//    missing, every later sample of the ray whose first corner falls in that
//    block fails the same way.  The t interval in which the ray stays inside
//    the block shrunk by a margin (0.1 voxel plus the float error of the
//    position) is computed once, and samples inside it only advance t
//    (t += step, the same accumulation as the full loop).
//  * 16x8-pixel CTAs keep neighbouring rays in one warp; they walk the same
//    blocks at about the same t.
#include "mh_internal.cuh"
#include "mh_kernels.h"
#include "mh_batch.cuh"

#include <algorithm>

#define RC_TX 16
#define RC_TY 8

namespace {

struct RayCache {
  int bx, by, bz;  // block of the first corner of the last sample
  int valid;       // bit n: p[n] holds the lookup of block (bx, by, bz) + (n & 1, n >> 1 & 1, n >> 2 & 1)
  int p[8];
  __device__ __forceinline__ void init() {
    bx = by = bz = 0x7fffffff;
    valid = 0;
  }
};

enum { RS_OK = 0, RS_MISS0 = 1, RS_MISS0_NEW = 2, RS_MISS = 3 };

// GetSpatialValue (geometry/spatial_query.h:23-66) for the raycast: the same
// corners, weights and summation order as spatial_sample.  Every sample runs
// the same gather: corner i lies in block b0 + (mx & ex, my & ey, mz & ez),
// where e is the block step between the two corner voxels of each axis, and
// the up to eight blocks of b0's 2x2x2 neighbourhood are looked up once per
// b0 and only when a sample needs them.  Returns RS_OK, or why the sample
// failed: its first corner's block is missing (RS_MISS0_NEW when that block
// was just looked up) or another corner's block is missing.
__device__ __noinline__ int ray_sample(const Dev &d, RayCache &c, F3 pos, float &sdf) {
  const float off = d.p.voxel_size;
  const float vs = d.p.voxel_size;
  const float qx = pos.x / vs, qy = pos.y / vs, qz = pos.z / vs;
  const float fx = floorf(qx), fy = floorf(qy), fz = floorf(qz);
  const float rx = qx - fx, ry = qy - fy, rz = qz - fz;
  int v0x, v0y, v0z, v1x, v1y, v1z;
  corner_pair(pos.x, off, vs, fx, rx, v0x, v1x);
  corner_pair(pos.y, off, vs, fy, ry, v0y, v1y);
  corner_pair(pos.z, off, vs, fz, rz, v0z, v1z);
  const int b0x = vox2blk(v0x), b0y = vox2blk(v0y), b0z = vox2blk(v0z);
  if (b0x != c.bx || b0y != c.by || b0z != c.bz) {
    c.bx = b0x, c.by = b0y, c.bz = b0z;
    c.valid = 0;
  }
  const int ex = vox2blk(v1x) - b0x, ey = vox2blk(v1y) - b0y, ez = vox2blk(v1z) - b0z;
  // blocks the eight corners use: every subset of the axes that step
  int need = 1;
  if (ex) need |= need << 1;
  if (ey) need |= need << 2;
  if (ez) need |= need << 4;
  const int fresh = need & ~c.valid;
  if (fresh & 1) c.p[0] = hash_find(d, b0x, b0y, b0z);
  c.valid |= fresh & 1;
  if (c.p[0] < 0) return (fresh & 1) ? RS_MISS0_NEW : RS_MISS0;
  for (int todo = fresh & ~1; todo; todo &= todo - 1) {
    const int n = __ffs(todo) - 1;
    c.p[n] = hash_find(d, b0x + (n & 1), b0y + ((n >> 1) & 1), b0z + ((n >> 2) & 1));
  }
  c.valid |= fresh;
  for (int m = need & ~1; m; m &= m - 1)
    if (c.p[__ffs(m) - 1] < 0) return RS_MISS;
  const float w0x = 1.0f - rx, w0y = 1.0f - ry, w0z = 1.0f - rz;
  // local voxel coordinates of the two corners of each axis
  const int l0x = v0x - b0x * MH_BLOCK_SIDE, l1x = v1x - (b0x + ex) * MH_BLOCK_SIDE;
  const int l0y = v0y - b0y * MH_BLOCK_SIDE, l1y = v1y - (b0y + ey) * MH_BLOCK_SIDE;
  const int l0z = v0z - b0z * MH_BLOCK_SIDE, l1z = v1z - (b0z + ez) * MH_BLOCK_SIDE;
  float s = 0.0f;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int mx = (i & 4) > 0, my = (i & 2) > 0, mz = (i & 1) > 0;
    const float w = (mx ? rx : w0x) * (my ? ry : w0y) * (mz ? rz : w0z);
    const int n = (mx & ex) | ((my & ey) << 1) | ((mz & ez) << 2);
    const int li = (mx ? l1x : l0x) + (my ? l1y : l0y) * MH_BLOCK_SIDE +
                   (mz ? l1z : l0z) * MH_BLOCK_SIDE * MH_BLOCK_SIDE;
    s += w * __ldg(d.sdf + (size_t)c.p[n] * MH_BLOCK_VOXELS + li);
  }
  sdf = s;
  return RS_OK;
}

// One axis of the slab test: narrows [lo, hi] to the t for which the ray's
// coordinate lies strictly inside (a, b).
__device__ __forceinline__ void slab(float o, float dir, float a, float b, float &lo, float &hi) {
  if (dir != 0.0f) {
    const float t1 = (a - o) / dir, t2 = (b - o) / dir;
    lo = fmaxf(lo, fminf(t1, t2));
    hi = fminf(hi, fmaxf(t1, t2));
  } else if (!(o > a && o < b)) {
    lo = __int_as_float(0x7f800000);
    hi = -__int_as_float(0x7f800000);
  }
}

// t interval in which every sample of the ray cam + t * wd has its first
// corner in block (bx, by, bz).  A position at least 0.1 voxel inside the
// block's faces has floor(p / v) -- and, where p / v is within 0.01 of an
// integer, round-half-away(p / v - 1/2) -- inside the block.  The margin adds
// 8 units in the last place of the coordinates for the rounding of the
// position and of the interval ends.
__device__ __forceinline__ void miss_interval(const DevParams &p, int bx, int by, int bz, F3 cam, F3 wd, float &lo,
                                              float &hi) {
  const float vs = p.voxel_size;
  const float side = (float)MH_BLOCK_SIDE * vs;
  lo = -__int_as_float(0x7f800000);
  hi = __int_as_float(0x7f800000);
  const float ax = (float)(bx * MH_BLOCK_SIDE) * vs, ay = (float)(by * MH_BLOCK_SIDE) * vs,
              az = (float)(bz * MH_BLOCK_SIDE) * vs;
  const float mx = 0.1f * vs + 5e-7f * (fabsf(ax) + side + fabsf(cam.x));
  const float my = 0.1f * vs + 5e-7f * (fabsf(ay) + side + fabsf(cam.y));
  const float mz = 0.1f * vs + 5e-7f * (fabsf(az) + side + fabsf(cam.z));
  slab(cam.x, wd.x, ax + mx, ax + side - mx, lo, hi);
  slab(cam.y, wd.y, ay + my, ay + side - my, lo, hi);
  slab(cam.z, wd.z, az + mz, az + side - mz, lo, hi);
}

__device__ __forceinline__ bool ray_gradient(const Dev &d, RayCache &c, F3 pos, F3 &g) {
  const float h = 0.5f * d.p.voxel_size;
  const float vs = d.p.voxel_size;
  float gx = 0.0f, gy = 0.0f, gz = 0.0f;
#pragma unroll 1
  for (int i = 0; i < 3; ++i) {
    F3 dm = f3(pos.x - (i == 0 ? h : 0.0f), pos.y - (i == 1 ? h : 0.0f), pos.z - (i == 2 ? h : 0.0f));
    F3 dp = f3(pos.x + (i == 0 ? h : 0.0f), pos.y + (i == 1 ? h : 0.0f), pos.z + (i == 2 ? h : 0.0f));
    float sn, sp;
    if (ray_sample(d, c, dm, sn) != RS_OK) return false;
    if (ray_sample(d, c, dp, sp) != RS_OK) return false;
    const float gi = (sp - sn) / vs;
    gx = i == 0 ? gi : gx;
    gy = i == 1 ? gi : gy;
    gz = i == 2 ? gi : gz;
  }
  g = f3(gx, gy, gz);
  return true;
}

}  // namespace

template <int TX, int TY>
__device__ __forceinline__ void raycast_body(const Dev &d, int tile_x, int tile_y, float *out_depth, float4 *out_vert, float4 *out_norm) {
  __shared__ float sm[32];
  const int tid = threadIdx.x + threadIdx.y * TX;
  if (tid < 16) sm[tid] = d.fc->rc_wTc[tid];
  else if (tid < 32) sm[tid] = d.fc->rc_cTw[tid - 16];
  __syncthreads();
  const float *wTc = sm, *cTw = sm + 16;
  const DevParams &p = d.p;
  const unsigned x = tile_x * TX + threadIdx.x;
  const unsigned y = tile_y * TY + threadIdx.y;
  if (x >= p.rc_width || y >= p.rc_height) return;
  const size_t pix = (size_t)y * p.rc_width + x;
  const float NI = -__int_as_float(0x7f800000);
  float o_depth = NI;
  float4 o_vert = make_float4(NI, NI, NI, NI), o_norm = make_float4(NI, NI, NI, NI);

  const float rx = ((float)x - p.rc_cx) / p.rc_fx, ry = ((float)y - p.rc_cy) / p.rc_fy;
  const F3 cd = normalize3(f3(1.0f * rx, 1.0f * ry, 1.0f));
  const float t_min = p.min_raycast_depth / cd.z;
  const float t_max = p.max_raycast_depth / cd.z;
  const F3 cam = mul_pt(wTc, f3(0.0f, 0.0f, 0.0f));
  const F3 wd = normalize3(mul_dir(wTc, cd));

  RayCache c;
  c.init();
  bool have_prev = false;
  float prev_sdf = 0.0f, prev_t = 0.0f;
  float skip_lo = 1.0f, skip_hi = 0.0f;
  const float step = p.raycast_step;
  float t = t_min;
#pragma unroll 1
  while (true) {
#pragma unroll 1
    while (t > skip_lo && t < skip_hi && t < t_max) t += step;
    if (!(t < t_max)) break;
    float s;
    const int rs = ray_sample(d, c, f3(cam.x + t * wd.x, cam.y + t * wd.y, cam.z + t * wd.z), s);
    if (rs != RS_OK) {
      if (rs == RS_MISS0_NEW) miss_interval(p, c.bx, c.by, c.bz, cam, wd, skip_lo, skip_hi);
      t += step;
      continue;
    }
    if (have_prev && prev_sdf > 0.0f && s < 0.0f) {
      float l = prev_t, r = t, m = (l + r) * 0.5f;
      float ls = prev_sdf, rs_ = s;
      bool found = true;
#pragma unroll 1
      for (int k = 0; k < 3; ++k) {
        m = l + (ls / (ls - rs_)) * (r - l);
        float ms;
        if (ray_sample(d, c, f3(cam.x + m * wd.x, cam.y + m * wd.y, cam.z + m * wd.z), ms) != RS_OK) {
          found = false;
          break;
        }
        if (ls * ms > 0.0f) {
          l = m, ls = ms;
        } else {
          r = m, rs_ = ms;
        }
      }
      if (found && fabsf(prev_sdf - s) < p.sample_sdf_threshold && fabsf(s) < p.sdf_threshold) {
        const float dz = m * cd.z;
        o_depth = dz;
        o_vert = make_float4(dz * rx, dz * ry, dz, 1.0f);
        if (p.enable_gradients && out_norm) {
          const F3 iso = f3(cam.x + m * wd.x, cam.y + m * wd.y, cam.z + m * wd.z);
          F3 g;
          const bool ok = ray_gradient(d, c, iso, g);
          const float len = sqrtf(dot3(g, g));
          F3 nn = f3(0.0f, 0.0f, 0.0f);
          if (ok && len > 0.0f) nn = f3(g.x / len, g.y / len, g.z / len);
          nn = f3(-nn.x, -nn.y, -nn.z);
          const F3 nc = mul_dir(cTw, nn);
          o_norm = make_float4(nc.x, nc.y, nc.z, 1.0f);
        }
        break;
      }
    }
    prev_sdf = s, prev_t = t, have_prev = true;
    t += step;
  }
  if (out_depth) out_depth[pix] = o_depth;
  if (out_vert) out_vert[pix] = o_vert;
  if (out_norm) out_norm[pix] = o_norm;
}
__global__ void __launch_bounds__(RC_TX *RC_TY) k_raycast(Dev d, float *out_depth, float4 *out_vert, float4 *out_norm) { raycast_body<RC_TX, RC_TY>(d, blockIdx.x, blockIdx.y, out_depth, out_vert, out_norm); }
// batched raycast over the scenes' concatenated TX x TY tiles; the tile shape
// is an autotuned choice (the scene table's ray_tile0 follows it)
template <int TX, int TY>
__global__ void __launch_bounds__(TX *TY, 65536 / (TX * TY * 72)) k_raycast_b(const Scene *t, int n, int total) {
  each_tile(t, n, total, &Scene::ray_tile0, [&](const Scene &c, int lt) {
    const int tw = (c.d.p.rc_width + TX - 1) / TX;
    raycast_body<TX, TY>(c.d, lt % tw, lt / tw, c.ray_depth, c.ray_vert, c.ray_norm);
  });
}

// tile shapes the batch autotuner chooses from
static const int kRayTiles[][2] = {{16, 8}, {8, 8}, {32, 4}};
int ray_tile_shapes() { return 3; }
void ray_tile_shape(int i, int &tx, int &ty) {
  tx = kRayTiles[i][0];
  ty = kRayTiles[i][1];
}

int launch_raycast_batch(const Scene *t, int n, int total, int shape, cudaStream_t s) {
  const int grid = std::max(1, std::min(total, mh_sm_count() * 16));
  switch (shape) {
    case 1: k_raycast_b<8, 8><<<grid, dim3(8, 8), 0, s>>>(t, n, total); break;
    case 2: k_raycast_b<32, 4><<<grid, dim3(32, 4), 0, s>>>(t, n, total); break;
    default: k_raycast_b<16, 8><<<grid, dim3(16, 8), 0, s>>>(t, n, total); break;
  }
  mh_count_launches(1);
  return cudaGetLastError() == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}

int launch_raycast(const Dev &d, float *depth, float *vert4, float *norm4, cudaStream_t s) {
  dim3 blk(RC_TX, RC_TY);
  dim3 grid((d.p.rc_width + RC_TX - 1) / RC_TX, (d.p.rc_height + RC_TY - 1) / RC_TY);
  k_raycast<<<grid, blk, 0, s>>>(d, depth, reinterpret_cast<float4 *>(vert4), reinterpret_cast<float4 *>(norm4));
  mh_count_launches(1);
  return cudaGetLastError() == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}
