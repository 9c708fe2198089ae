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

// GetSpatialSDFGradient: central differences h = half a voxel either side
// (spacing = 0.5); a wider spacing gives a smoother normal
__device__ __forceinline__ bool ray_gradient(const Dev &d, RayCache &c, F3 pos, F3 &g, float spacing = 0.5f) {
  const float h = spacing * d.p.voxel_size;
  const float vs = d.p.voxel_size;
  float gx = 0.0f, gy = 0.0f, gz = 0.0f;
#pragma unroll 1
  for (int i = 0; i < 3; ++i) {
    F3 dm = f3(pos.x - (i == 0 ? h : 0.0f), pos.y - (i == 1 ? h : 0.0f), pos.z - (i == 2 ? h : 0.0f));
    F3 dp = f3(pos.x + (i == 0 ? h : 0.0f), pos.y + (i == 1 ? h : 0.0f), pos.z + (i == 2 ? h : 0.0f));
    float sn, sp;
    if (ray_sample(d, c, dm, sn) != RS_OK) return false;
    if (ray_sample(d, c, dp, sp) != RS_OK) return false;
    const float gi = (sp - sn) / (vs * (2.0f * spacing));
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

// ------------------------------------------------------------------ backward
// Reverse-mode derivative of the raycast (no reference counterpart; the
// reference's raycaster is forward only).  For each pixel the march is run
// again with the forward's own code, so every discrete decision -- which
// samples are valid, where the sign changes, which end each regula-falsi step
// replaces -- is the forward's.  With those fixed, the rendered depth
// D = m * cd.z is a smooth function of
//   * the voxel sdf values (each sample is a trilinear sum, linear in them),
//   * the camera pose (every sample sits at cam + t * wd),
// through the two bracketing samples and the three regula-falsi steps
// m = l + ls / (ls - rs) * (r - l); the normal adds six gradient samples
// around the hit and a normalisation.  The kernel propagates adjoints back
// through exactly these steps, so its result is the derivative of what the
// forward computes (what central differences of the forward measure), not
// of an idealised surface.  Pose derivatives are for a left perturbation
// wTc <- exp(xi) wTc, xi = (translation v, rotation w), to first order:
// cam += w x cam + v, wd += w x wd, and the camera-frame normal R^T n
// changes by R^T (n x w).
namespace {

// a sample with what the backward needs: value (bit-identical to
// ray_sample's), spatial gradient, and the eight corners with their weights
struct SampleD {
  float s;
  F3 g;
  int ptr[8], li[8];
  float w[8];
};

__device__ __noinline__ bool ray_sample_d(const Dev &d, RayCache &c, F3 pos, SampleD &o) {
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
  int need = 1;
  if (ex) need |= need << 1;
  if (ey) need |= need << 2;
  if (ez) need |= need << 4;
  for (int todo = need & ~c.valid; todo; todo &= todo - 1) {
    const int n = __ffs(todo) - 1;
    c.p[n] = hash_find(d, b0x + (n & 1), b0y + ((n >> 1) & 1), b0z + ((n >> 2) & 1));
  }
  c.valid |= need;
  for (int m = need; m; m &= m - 1)
    if (c.p[__ffs(m) - 1] < 0) return false;
  const float w0x = 1.0f - rx, w0y = 1.0f - ry, w0z = 1.0f - rz;
  const int l0x = v0x - b0x * MH_BLOCK_SIDE, l1x = v1x - (b0x + ex) * MH_BLOCK_SIDE;
  const int l0y = v0y - b0y * MH_BLOCK_SIDE, l1y = v1y - (b0y + ey) * MH_BLOCK_SIDE;
  const int l0z = v0z - b0z * MH_BLOCK_SIDE, l1z = v1z - (b0z + ez) * MH_BLOCK_SIDE;
  float s = 0.0f, gx = 0.0f, gy = 0.0f, gz = 0.0f;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int mx = (i & 4) > 0, my = (i & 2) > 0, mz = (i & 1) > 0;
    const float wx = mx ? rx : w0x, wy = my ? ry : w0y, wz = mz ? rz : w0z;
    const float w = wx * wy * wz;
    const int n = (mx & ex) | ((my & ey) << 1) | ((mz & ez) << 2);
    const int li = (mx ? l1x : l0x) + (my ? l1y : l0y) * MH_BLOCK_SIDE + (mz ? l1z : l0z) * MH_BLOCK_SIDE * MH_BLOCK_SIDE;
    const float v = __ldg(d.sdf + (size_t)c.p[n] * MH_BLOCK_VOXELS + li);
    s += w * v;
    // d(weight)/d(position): the fractions move at 1/voxel per metre
    gx += (mx ? 1.0f : -1.0f) * wy * wz * v;
    gy += (my ? 1.0f : -1.0f) * wx * wz * v;
    gz += (mz ? 1.0f : -1.0f) * wx * wy * v;
    o.ptr[i] = c.p[n];
    o.li[i] = li;
    o.w[i] = w;
  }
  o.s = s;
  o.g = f3(gx / vs, gy / vs, gz / vs);
  return true;
}

struct RayTrace {
  bool hit;
  float t0, t1;  // the bracketing samples
  int side;      // bit k: regula-falsi step k replaced the left end
};

// the forward's march (k_raycast), recording its decisions instead of outputs
__device__ __noinline__ RayTrace ray_trace(const Dev &d, RayCache &c, F3 cam, F3 wd, float t_min, float t_max) {
  const DevParams &p = d.p;
  RayTrace tr{false, 0.0f, 0.0f, 0};
  bool have_prev = false;
  float prev_sdf = 0.0f, prev_t = 0.0f;
  float skip_lo = 1.0f, skip_hi = 0.0f;
  const float step = p.raycast_step;
  float t = t_min;
  while (true) {
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
      float l = prev_t, r = t, ls = prev_sdf, rs_ = s;
      bool found = true;
      int side = 0;
      for (int k = 0; k < 3; ++k) {
        const float m = l + (ls / (ls - rs_)) * (r - l);
        float ms;
        if (ray_sample(d, c, f3(cam.x + m * wd.x, cam.y + m * wd.y, cam.z + m * wd.z), ms) != RS_OK) {
          found = false;
          break;
        }
        if (ls * ms > 0.0f) {
          l = m, ls = ms, side |= 1 << k;
        } else {
          r = m, rs_ = ms;
        }
      }
      if (found && fabsf(prev_sdf - s) < p.sample_sdf_threshold && fabsf(s) < p.sdf_threshold) {
        tr.hit = true, tr.t0 = prev_t, tr.t1 = t, tr.side = side;
        return tr;
      }
    }
    prev_sdf = s, prev_t = t, have_prev = true;
    t += step;
  }
  return tr;
}

__device__ __forceinline__ F3 cross3(F3 a, F3 b) {
  return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ void scatter(float *grad, const SampleD &o, float a) {
  if (!grad || a == 0.0f) return;
#pragma unroll
  for (int i = 0; i < 8; ++i) atomicAdd(grad + (size_t)o.ptr[i] * MH_BLOCK_VOXELS + o.li[i], a * o.w[i]);
}

// Adjoints of one pixel's depth (aD) and camera-frame normal (aN): voxel
// adjoints go to grad (may be null), pose adjoints to (av, aw).  Returns
// false when the hit cannot be re-evaluated.
__device__ bool pixel_backward(const Dev &d, RayCache &c, const float *cTw, F3 cam, F3 wd, float cdz,
                               const RayTrace &tr, float aD, F3 aN, bool normals, float *grad, F3 &av, F3 &aw) {
  const float vs = d.p.voxel_size;
  F3 a_cam = f3(0.0f, 0.0f, 0.0f), a_wd = f3(0.0f, 0.0f, 0.0f), a_w_extra = f3(0.0f, 0.0f, 0.0f);
  // forward values of the regula falsi, in the forward's operation order
  SampleD S0, S1, Sm[3];
  if (!ray_sample_d(d, c, f3(cam.x + tr.t0 * wd.x, cam.y + tr.t0 * wd.y, cam.z + tr.t0 * wd.z), S0)) return false;
  if (!ray_sample_d(d, c, f3(cam.x + tr.t1 * wd.x, cam.y + tr.t1 * wd.y, cam.z + tr.t1 * wd.z), S1)) return false;
  float L[3], Rr[3], LS[3], RS[3], M[3];
  float l = tr.t0, r = tr.t1, ls = S0.s, rs = S1.s;
  for (int k = 0; k < 3; ++k) {
    L[k] = l, Rr[k] = r, LS[k] = ls, RS[k] = rs;
    const float m = l + (ls / (ls - rs)) * (r - l);
    M[k] = m;
    if (!ray_sample_d(d, c, f3(cam.x + m * wd.x, cam.y + m * wd.y, cam.z + m * wd.z), Sm[k])) return false;
    if ((tr.side >> k) & 1) l = m, ls = Sm[k].s;
    else r = m, rs = Sm[k].s;
  }
  const float m = M[2];
  float am = aD * cdz;
  if (normals && (aN.x != 0.0f || aN.y != 0.0f || aN.z != 0.0f)) {
    const F3 iso = f3(cam.x + m * wd.x, cam.y + m * wd.y, cam.z + m * wd.z);
    const float h = 0.5f * vs;
    SampleD P[3], N[3];
    bool ok = true;
    for (int i = 0; i < 3 && ok; ++i) {
      F3 dm = f3(iso.x - (i == 0 ? h : 0.0f), iso.y - (i == 1 ? h : 0.0f), iso.z - (i == 2 ? h : 0.0f));
      F3 dp = f3(iso.x + (i == 0 ? h : 0.0f), iso.y + (i == 1 ? h : 0.0f), iso.z + (i == 2 ? h : 0.0f));
      ok = ray_sample_d(d, c, dm, N[i]) && ray_sample_d(d, c, dp, P[i]);
    }
    const F3 g = f3((P[0].s - N[0].s) / vs, (P[1].s - N[1].s) / vs, (P[2].s - N[2].s) / vs);
    const float len = sqrtf(dot3(g, g));
    if (ok && len > 0.0f) {
      const F3 u = f3(g.x / len, g.y / len, g.z / len);
      const F3 nn = f3(-u.x, -u.y, -u.z);
      // nc = Rc nn with Rc the rotation of cTw: a_nn = Rc^T aN
      const F3 a_nn = f3(cTw[0] * aN.x + cTw[4] * aN.y + cTw[8] * aN.z, cTw[1] * aN.x + cTw[5] * aN.y + cTw[9] * aN.z,
                         cTw[2] * aN.x + cTw[6] * aN.y + cTw[10] * aN.z);
      a_w_extra = cross3(a_nn, nn);
      const F3 a_u = f3(-a_nn.x, -a_nn.y, -a_nn.z);
      const float ua = dot3(u, a_u);
      const float ag[3] = {(a_u.x - u.x * ua) / len, (a_u.y - u.y * ua) / len, (a_u.z - u.z * ua) / len};
      F3 a_iso = f3(0.0f, 0.0f, 0.0f);
      for (int i = 0; i < 3; ++i) {
        const float ap = ag[i] / vs, an = -ag[i] / vs;
        scatter(grad, P[i], ap);
        scatter(grad, N[i], an);
        a_iso = f3(a_iso.x + ap * P[i].g.x + an * N[i].g.x, a_iso.y + ap * P[i].g.y + an * N[i].g.y,
                   a_iso.z + ap * P[i].g.z + an * N[i].g.z);
      }
      a_cam = f3(a_cam.x + a_iso.x, a_cam.y + a_iso.y, a_cam.z + a_iso.z);
      a_wd = f3(a_wd.x + m * a_iso.x, a_wd.y + m * a_iso.y, a_wd.z + m * a_iso.z);
      am += dot3(a_iso, wd);
    }
  }
  // regula falsi, last step first; (al, ar, als, ars) are the adjoints of
  // the state after step k
  float al = 0.0f, ar = 0.0f, als = 0.0f, ars = 0.0f;
  for (int k = 2; k >= 0; --k) {
    const bool left = (tr.side >> k) & 1;
    float a_mk = (k == 2 ? am : 0.0f) + (left ? al : ar);
    const float a_ms = left ? als : ars;
    if (left) al = 0.0f, als = 0.0f;
    else ar = 0.0f, ars = 0.0f;
    // ms_k = S(cam + m_k wd)
    scatter(grad, Sm[k], a_ms);
    const F3 ap = f3(a_ms * Sm[k].g.x, a_ms * Sm[k].g.y, a_ms * Sm[k].g.z);
    a_cam = f3(a_cam.x + ap.x, a_cam.y + ap.y, a_cam.z + ap.z);
    a_wd = f3(a_wd.x + M[k] * ap.x, a_wd.y + M[k] * ap.y, a_wd.z + M[k] * ap.z);
    a_mk += dot3(ap, wd);
    // m_k = l + q (r - l), q = ls / (ls - rs)
    const float den = LS[k] - RS[k], q = LS[k] / den, span = Rr[k] - L[k];
    al += a_mk * (1.0f - q);
    ar += a_mk * q;
    als += a_mk * span * (-RS[k]) / (den * den);
    ars += a_mk * span * LS[k] / (den * den);
  }
  // the bracketing samples sit at fixed t
  scatter(grad, S0, als);
  scatter(grad, S1, ars);
  const F3 p0 = f3(als * S0.g.x, als * S0.g.y, als * S0.g.z), p1 = f3(ars * S1.g.x, ars * S1.g.y, ars * S1.g.z);
  a_cam = f3(a_cam.x + p0.x + p1.x, a_cam.y + p0.y + p1.y, a_cam.z + p0.z + p1.z);
  a_wd = f3(a_wd.x + tr.t0 * p0.x + tr.t1 * p1.x, a_wd.y + tr.t0 * p0.y + tr.t1 * p1.y,
            a_wd.z + tr.t0 * p0.z + tr.t1 * p1.z);
  av = a_cam;
  const F3 c1 = cross3(cam, a_cam), c2 = cross3(wd, a_wd);
  aw = f3(c1.x + c2.x + a_w_extra.x, c1.y + c2.y + a_w_extra.y, c1.z + c2.z + a_w_extra.z);
  return true;
}

// sum of NV values over the CTA into acc (doubles)
template <int NV> __device__ __forceinline__ void cta_accumulate(float (&v)[NV], double *acc) {
  __shared__ float red[NV][32];
  const int tid = threadIdx.x + threadIdx.y * blockDim.x, lane = tid & 31, wid = tid >> 5;
  const int nw = (blockDim.x * blockDim.y + 31) >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    float x = v[k];
    for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) red[k][wid] = x;
  }
  __syncthreads();
  if (tid < NV) {
    double s = 0.0;
    for (int w = 0; w < nw; ++w) s += red[tid][w];
    atomicAdd(acc + tid, s);
  }
}

}  // namespace

// mode 0: accumulate dL/dsdf into grad (if given) and dL/dxi into acc[0..5]
//         for L = sum dLdD * depth + dLdN . normal;
// mode 1: Gauss-Newton normal equations of frame-to-model alignment over
//         pixels with a hit, a valid observation and |depth - obs| < max_res:
//         the observed point on the pixel's ray against the tangent plane of
//         the model at the raycast hit (normal from the raycast's gradient),
//         r = n . (p_obs - p_hit), J = [n, p_obs x n] for the left increment;
//         acc = [J^T J upper triangle (21), J^T r (6), sum r^2, count].
__global__ void __launch_bounds__(RC_TX *RC_TY) k_raycast_grad(Dev d, int mode, const float *dLdD, const float4 *dLdN,
                                                              float *grad, const float *obs, float max_res,
                                                              double *acc) {
  __shared__ float sm[32];
  const int tid = threadIdx.x + threadIdx.y * RC_TX;
  if (tid < 16) sm[tid] = d.fc->rc_wTc[tid];
  else if (tid < 32) sm[tid] = d.fc->rc_cTw[tid - 16];
  __syncthreads();
  const float *wTc = sm, *cTw = sm + 16;
  const DevParams &p = d.p;
  const unsigned x = blockIdx.x * RC_TX + threadIdx.x;
  const unsigned y = blockIdx.y * RC_TY + threadIdx.y;
  F3 av = f3(0.0f, 0.0f, 0.0f), aw = f3(0.0f, 0.0f, 0.0f);
  float res = 0.0f;
  bool used = false;
  if (x < p.rc_width && y < p.rc_height) {
    const size_t pix = (size_t)y * p.rc_width + x;
    const float rx = ((float)x - p.rc_cx) / p.rc_fx, ry = ((float)y - p.rc_cy) / p.rc_fy;
    const F3 cd = normalize3(f3(1.0f * rx, 1.0f * ry, 1.0f));
    const float t_min = p.min_raycast_depth / cd.z;
    const float t_max = p.max_raycast_depth / cd.z;
    const F3 cam = mul_pt(wTc, f3(0.0f, 0.0f, 0.0f));
    const F3 wd = normalize3(mul_dir(wTc, cd));
    float aD = 0.0f;
    F3 aN = f3(0.0f, 0.0f, 0.0f);
    bool want = false;
    if (mode == 0) {
      aD = dLdD ? dLdD[pix] : 0.0f;
      if (dLdN) {
        const float4 q = dLdN[pix];
        aN = f3(q.x, q.y, q.z);
      }
      want = aD != 0.0f || aN.x != 0.0f || aN.y != 0.0f || aN.z != 0.0f;
    } else {
      const float o = obs[pix];
      want = o > 0.0f && o < 1e30f;
    }
    if (want) {
      RayCache c;
      c.init();
      const RayTrace tr = ray_trace(d, c, cam, wd, t_min, t_max);
      if (tr.hit) {
        if (mode == 1) {
          // the forward's hit and normal
          float l = tr.t0, r = tr.t1, ls, rs_, m = 0.0f;
          ray_sample(d, c, f3(cam.x + l * wd.x, cam.y + l * wd.y, cam.z + l * wd.z), ls);
          ray_sample(d, c, f3(cam.x + r * wd.x, cam.y + r * wd.y, cam.z + r * wd.z), rs_);
          for (int k = 0; k < 3; ++k) {
            m = l + (ls / (ls - rs_)) * (r - l);
            float ms;
            ray_sample(d, c, f3(cam.x + m * wd.x, cam.y + m * wd.y, cam.z + m * wd.z), ms);
            if ((tr.side >> k) & 1) l = m, ls = ms;
            else r = m, rs_ = ms;
          }
          const float o = obs[pix];
          const F3 pm = f3(cam.x + m * wd.x, cam.y + m * wd.y, cam.z + m * wd.z);
          // the normal of the alignment is taken 2.5 voxels either side
          // (inside the truncation band): the half-voxel normal of the
          // rendered image follows the noise of the fused surface, and a
          // noisy normal in J shrinks every Gauss-Newton step (measured: from
          // 2-8 cm / 1-2.5 degree starts, 8 iterations reached 15-90 mm with
          // the half-voxel normal and 1-3 mm on three of four with this one)
          const float spacing = fminf(2.5f, 0.8f * p.truncation_distance / p.voxel_size);
          F3 g;
          if (fabsf(m * cd.z - o) < max_res && ray_gradient(d, c, pm, g, spacing)) {
            const float gl = sqrtf(dot3(g, g));
            if (gl > 0.0f) {
              // projective point-to-plane: the observed point on the same ray
              // against the tangent plane of the model at the hit
              const F3 n = f3(g.x / gl, g.y / gl, g.z / gl);
              const float to = o / cd.z;
              const F3 po = f3(cam.x + to * wd.x, cam.y + to * wd.y, cam.z + to * wd.z);
              res = dot3(n, f3(po.x - pm.x, po.y - pm.y, po.z - pm.z));
              av = n;
              aw = cross3(po, n);
              used = true;
            }
          }
        } else {
          used = pixel_backward(d, c, cTw, cam, wd, cd.z, tr, aD, aN, dLdN != nullptr, grad, av, aw);
        }
      }
    }
  }
  if (!used) av = f3(0.0f, 0.0f, 0.0f), aw = f3(0.0f, 0.0f, 0.0f), res = 0.0f;
  if (mode == 0) {
    float v[6] = {av.x, av.y, av.z, aw.x, aw.y, aw.z};
    cta_accumulate<6>(v, acc);
  } else {
    const float J[6] = {av.x, av.y, av.z, aw.x, aw.y, aw.z};
    float v[29];
    int k = 0;
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
      for (int j = i; j < 6; ++j) v[k++] = J[i] * J[j];
#pragma unroll
    for (int i = 0; i < 6; ++i) v[21 + i] = J[i] * res;
    v[27] = res * res;
    v[28] = used ? 1.0f : 0.0f;
    cta_accumulate<29>(v, acc);
  }
}

int launch_raycast_grad(const Dev &d, int mode, const float *dLdD, const float *dLdN4, float *grad, const float *obs,
                        float max_res, double *acc, cudaStream_t s) {
  dim3 blk(RC_TX, RC_TY);
  dim3 grid((d.p.rc_width + RC_TX - 1) / RC_TX, (d.p.rc_height + RC_TY - 1) / RC_TY);
  k_raycast_grad<<<grid, blk, 0, s>>>(d, mode, dLdD, reinterpret_cast<const float4 *>(dLdN4), grad, obs, max_res,
                                      acc);
  mh_count_launches(1);
  return cudaGetLastError() == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}
