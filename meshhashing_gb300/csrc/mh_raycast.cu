// mh_raycast.cu -- trilinear raycast of the zero level set.
//
// CastKernel (visualization/ray_caster.cu:16-150): one thread per pixel
// marches the camera ray with a fixed step from min to max raycast depth,
// samples the SDF trilinearly (GetSpatialValue, geometry/spatial_query.h:23-66),
// and on a + to - sign change refines the hit with three regula-falsi steps
// (BisectionIntersection, geometry/isosurface_intersection.h:21-55).  The
// sample positions, the accumulation of t and every comparison follow the
// reference's single-precision order exactly, and so does every value the
// output depends on.
//
// GB300 structure.  The march is bound by instruction issue and by the
// latency of its dependent loads, not by HBM bandwidth, so the work per
// sample is what is cut, never the sample sequence itself:
//  * all state in registers: one sampler, inlined once, serves the march, the
//    lazily evaluated previous sample, the regula falsi and the gradient
//    (a phase variable picks the next position); the first corner's 2x2x2
//    block neighbourhood is a register table filled by hash lookups only
//    when a sample first needs an entry, so a sample's eight corners come
//    from one branch-uniform gather;
//  * exact skips (see ray_march): samples whose corner blocks hold only
//    non-negative voxels are never gathered, and the t intervals inside
//    missing blocks and inside non-negative blocks only advance t;
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

}  // namespace

// ------------------------------------------------------------------ forward
// The forward march keeps its whole state in registers: one sampler is
// inlined once, and a phase variable chooses where the next sample goes --
// the march itself, the lazily evaluated previous sample, the three
// regula-falsi steps, the six gradient samples of the normal.  The first
// corner's 2x2x2 block neighbourhood is a register table with three masks
// (looked up, missing, all voxels non-negative), filled by hash lookups only
// when a sample first needs an entry.
//
// Skips, all exact.  A march sample matters only when it is negative right
// after a positive one (the zero crossing), and then the previous sample's
// value matters too.  A sample whose corner blocks hold only non-negative
// voxels (per-block count nnc == 512) is valid and >= 0, so it can never be
// the negative end of a crossing: its gather is skipped and it becomes the
// "previous sample" lazily -- its value is computed only when the next
// evaluated sample is negative, and the crossing is taken if that value is
// > 0.  Three kinds of t interval are skipped with nothing but t += step:
// where the first corner's block is missing (every sample invalid); where it
// lies in a block flagged before the raycast (cellok: the block and its seven
// upper neighbours exist and count 512, so every sample whose first corner
// is there is valid and >= 0); and, otherwise, the interior of a block that
// counts 512, where all eight corners lie in that block.
namespace {

enum { SM_OK = 0, SM_POS = 1, SM_MISS0 = 2, SM_MISS0_NEW = 3, SM_MISS = 4 };

struct Nbhd {
  int bx, by, bz;    // block of the first corner of the last sample
  unsigned looked;   // bit n: block n = (bx, by, bz) + (n & 1, n >> 1 & 1, n >> 2 & 1) looked up
  unsigned miss;     // bit n: block n is missing
  unsigned pos;      // bit n: every voxel of block n is non-negative
  int p[8];          // block indices, indexed with constants only (registers)
  __device__ __forceinline__ void init() {
    bx = by = bz = 0x7fffffff;
    looked = miss = pos = 0u;
#pragma unroll
    for (int j = 0; j < 8; ++j) p[j] = -1;
  }
};

// GetSpatialValue (geometry/spatial_query.h:23-66) with the same corners,
// weights and summation order as spatial_sample.  Returns SM_OK with the
// value in s, SM_POS when allow_pos and every corner block is non-negative
// (value not computed), or why the sample is invalid.  b0_fresh: the first
// corner's block was looked up by this call.
__device__ __forceinline__ int nb_sample(const Dev &d, Nbhd &c, F3 pos, bool allow_pos, float &s, bool &b0_fresh) {
  const float off = d.p.voxel_size;
  const float vs = d.p.voxel_size;
  const float qx = pos.x / vs, qy = pos.y / vs, qz = pos.z / vs;
  const float fx = floorf(qx), fy = floorf(qy), fz = floorf(qz);
  const float rx = qx - fx, ry = qy - fy, rz = qz - fz;
  int v0x, v0y, v0z, v1x, v1y, v1z;
  corner_pair(pos.x, off, vs, fx, rx, v0x, v1x);
  corner_pair(pos.y, off, vs, fy, ry, v0y, v1y);
  corner_pair(pos.z, off, vs, fz, rz, v0z, v1z);
  // VoxelToBlock: floor division by 8 (geometry_helper.h:82-90)
  const int b0x = v0x >> 3, b0y = v0y >> 3, b0z = v0z >> 3;
  if (b0x != c.bx || b0y != c.by || b0z != c.bz) {
    c.bx = b0x, c.by = b0y, c.bz = b0z;
    c.looked = c.miss = c.pos = 0u;
  }
  const int ex = (v1x >> 3) - b0x, ey = (v1y >> 3) - b0y, ez = (v1z >> 3) - b0z;
  unsigned need = 1u;
  if (ex) need |= need << 1;
  if (ey) need |= need << 2;
  if (ez) need |= need << 4;
  unsigned fresh = need & ~c.looked;
  b0_fresh = fresh & 1u;
  if (b0_fresh) {
    const int q = hash_find(d, b0x, b0y, b0z);
    c.p[0] = q;
    if (q >= 0 && d.touch) d.touch[q] = 1;
    if (q < 0) c.miss |= 1u;
    else if (__ldg(d.nnc + q) == MH_BLOCK_VOXELS) c.pos |= 1u;
    c.looked |= 1u;
    fresh &= ~1u;
  }
  if (c.miss & 1u) return b0_fresh ? SM_MISS0_NEW : SM_MISS0;
  while (fresh) {
    const int n = __ffs(fresh) - 1;
    fresh &= fresh - 1;
    const int q = hash_find(d, b0x + (n & 1), b0y + ((n >> 1) & 1), b0z + ((n >> 2) & 1));
#pragma unroll
    for (int j = 1; j < 8; ++j)
      if (j == n) c.p[j] = q;
    if (q >= 0 && d.touch) d.touch[q] = 1;
    if (q < 0) c.miss |= 1u << n;
    else if (__ldg(d.nnc + q) == MH_BLOCK_VOXELS) c.pos |= 1u << n;
  }
  c.looked |= need;
  if (need & c.miss) return SM_MISS;
  if (allow_pos && (need & ~c.pos) == 0u) return SM_POS;
  // block of each corner (mx, my, mz): p[(mx & ex) | (my & ey) << 1 | (mz & ez) << 2]
  const int B0 = c.p[0];
  const int BX = ex ? c.p[1] : B0;
  const int BY = ey ? c.p[2] : B0;
  const int BXY = ey ? (ex ? c.p[3] : c.p[2]) : BX;
  const int BZ = ez ? c.p[4] : B0;
  const int BXZ = ez ? (ex ? c.p[5] : c.p[4]) : BX;
  const int BYZ = ez ? (ey ? c.p[6] : c.p[4]) : BY;
  const int BXYZ = ez ? (ey ? (ex ? c.p[7] : c.p[6]) : (ex ? c.p[5] : c.p[4])) : BXY;
  const int blk[8] = {B0, BZ, BY, BYZ, BX, BXZ, BXY, BXYZ};
  // local voxel coordinates of the two corners of each axis
  const int l0x = v0x & 7, l1x = v1x & 7;
  const int yz[4] = {(v0y & 7) * 8 + (v0z & 7) * 64, (v0y & 7) * 8 + (v1z & 7) * 64,
                     (v1y & 7) * 8 + (v0z & 7) * 64, (v1y & 7) * 8 + (v1z & 7) * 64};
  const float w0x = 1.0f - rx, w0y = 1.0f - ry, w0z = 1.0f - rz;
  const float wxy[4] = {w0x * w0y, w0x * ry, rx * w0y, rx * ry};
  float v[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int mx = (i >> 2) & 1, lyz = i & 3;
    v[i] = __ldg(d.sdf + (size_t)(blk[i] * MH_BLOCK_VOXELS + (mx ? l1x : l0x) + yz[lyz]));
  }
  float acc = 0.0f;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int mz = i & 1;
    acc += wxy[i >> 1] * (mz ? rz : w0z) * v[i];
  }
  s = acc;
  return SM_OK;
}

// One axis of a slab test with the direction's reciprocal: narrows [lo, hi]
// to the t for which the ray's coordinate lies inside (a, b).  The bounds
// carry a few ulp of rounding; the box margins below absorb them.
__device__ __forceinline__ void slab_r(float o, float dir, float idir, float a, float b, float &lo, float &hi) {
  if (dir != 0.0f) {
    const float t1 = (a - o) * idir, t2 = (b - o) * idir;
    lo = fmaxf(lo, fminf(t1, t2));
    hi = fminf(hi, fmaxf(t1, t2));
  } else if (!(o > a && o < b)) {
    lo = __int_as_float(0x7f800000);
    hi = -__int_as_float(0x7f800000);
  }
}

// t interval in which every sample of the ray cam + t * wd has its first
// corner voxel at local coordinates [0, cells) of block (bx, by, bz) on each
// axis: cells = 8 puts the first corner in the block, cells = 7 all eight
// corners.  A coordinate at least 0.1 voxel inside those faces has floor(p / v)
// -- and, where p / v is within 0.01 of an integer, round-half-away(p / v -
// 1/2) -- in range; the margin adds 8 units in the last place of the
// coordinates for the rounding of the position and of the interval ends.
__device__ __forceinline__ void block_interval(const DevParams &p, int bx, int by, int bz, int cells, F3 cam, F3 wd,
                                               F3 iwd, float &lo, float &hi) {
  const float vs = p.voxel_size;
  const float side = (float)MH_BLOCK_SIDE * vs, span = (float)cells * vs;
  lo = -__int_as_float(0x7f800000);
  hi = __int_as_float(0x7f800000);
  const float ax = (float)(bx * MH_BLOCK_SIDE) * vs, ay = (float)(by * MH_BLOCK_SIDE) * vs,
              az = (float)(bz * MH_BLOCK_SIDE) * vs;
  const float mx = 0.1f * vs + 5e-7f * (fabsf(ax) + side + fabsf(cam.x));
  const float my = 0.1f * vs + 5e-7f * (fabsf(ay) + side + fabsf(cam.y));
  const float mz = 0.1f * vs + 5e-7f * (fabsf(az) + side + fabsf(cam.z));
  slab_r(cam.x, wd.x, iwd.x, ax + mx, ax + span - mx, lo, hi);
  slab_r(cam.y, wd.y, iwd.y, ay + my, ay + span - my, lo, hi);
  slab_r(cam.z, wd.z, iwd.z, az + mz, az + span - mz, lo, hi);
}

}  // namespace

// What one ray's march found: whether a hit was accepted, the two march
// samples around the zero crossing, which end each regula-falsi step
// replaced, the last regula-falsi point and, when asked, the spatial
// gradient at that point (g_ok false if a gradient sample was invalid).
struct March {
  bool hit, g_ok;
  float t0, t1, m;
  int side;  // bit k: regula-falsi step k replaced the left end
  F3 g;
};

// RayCaster::CastKernel's march (visualization/ray_caster.cu:62-150) for the
// ray cam + t * wd, t from t_min while t < t_max, with the exact skips
// described above; spacing > 0 also evaluates GetSpatialSDFGradient at the hit
// with central differences `spacing` voxels either side (spatial_query.h:68-97
// uses 0.5).
__device__ __forceinline__ March ray_march(const Dev &d, F3 cam, F3 wd, float t_min, float t_max, float spacing) {
  const DevParams &p = d.p;
  const F3 iwd = f3(wd.x != 0.0f ? 1.0f / wd.x : 0.0f, wd.y != 0.0f ? 1.0f / wd.y : 0.0f,
                    wd.z != 0.0f ? 1.0f / wd.z : 0.0f);
  const float vs = p.voxel_size;
  const float step = p.raycast_step;
  enum { PH_MARCH, PH_PREV, PH_REFINE, PH_GRAD };
  March out;
  out.hit = false, out.g_ok = false, out.t0 = out.t1 = out.m = 0.0f, out.side = 0;
  out.g = f3(0.0f, 0.0f, 0.0f);
  Nbhd c;
  c.init();
  int phase = PH_MARCH, k = 0, side = 0;
  bool have_prev = false, prev_lazy = false, skip_pos = false;
  float prev_sdf = 0.0f, prev_t = 0.0f, skip_lo = 1.0f, skip_hi = 0.0f;
  float t = t_min, cur_s = 0.0f, l = 0.0f, r = 0.0f, ls = 0.0f, rs = 0.0f, m = 0.0f, g_minus = 0.0f;
  F3 iso = f3(0.0f, 0.0f, 0.0f);
#pragma unroll 1
  while (true) {
    F3 pos;
    if (phase == PH_MARCH) {
      if (t > skip_lo && t < skip_hi && t < t_max) {
        float last;
#pragma unroll 1
        do {
          last = t;
          t += step;
        } while (t < skip_hi && t < t_max);
        if (skip_pos) have_prev = true, prev_lazy = true, prev_t = last;
      }
      if (!(t < t_max)) break;
      pos = f3(cam.x + t * wd.x, cam.y + t * wd.y, cam.z + t * wd.z);
    } else if (phase == PH_PREV) {
      pos = f3(cam.x + prev_t * wd.x, cam.y + prev_t * wd.y, cam.z + prev_t * wd.z);
    } else if (phase == PH_REFINE) {
      m = l + (ls / (ls - rs)) * (r - l);
      pos = f3(cam.x + m * wd.x, cam.y + m * wd.y, cam.z + m * wd.z);
    } else {
      // axis k / 2, minus side first
      const float h = spacing * vs;
      const int ax = k >> 1;
      if (k & 1) pos = f3(iso.x + (ax == 0 ? h : 0.0f), iso.y + (ax == 1 ? h : 0.0f), iso.z + (ax == 2 ? h : 0.0f));
      else pos = f3(iso.x - (ax == 0 ? h : 0.0f), iso.y - (ax == 1 ? h : 0.0f), iso.z - (ax == 2 ? h : 0.0f));
    }
    float s = 0.0f;
    bool b0_fresh = false;
    const int res = nb_sample(d, c, pos, phase == PH_MARCH, s, b0_fresh);
    if (phase == PH_MARCH) {
      if (b0_fresh) {
        if (res == SM_MISS0_NEW) {
          block_interval(p, c.bx, c.by, c.bz, MH_BLOCK_SIDE, cam, wd, iwd, skip_lo, skip_hi);
          skip_pos = false;
        } else if (res != SM_MISS0 && d.cellok && __ldg(d.cellok + c.p[0])) {
          block_interval(p, c.bx, c.by, c.bz, MH_BLOCK_SIDE, cam, wd, iwd, skip_lo, skip_hi);
          skip_pos = true;
        } else if (c.pos & 1u) {
          block_interval(p, c.bx, c.by, c.bz, MH_BLOCK_SIDE - 1, cam, wd, iwd, skip_lo, skip_hi);
          skip_pos = true;
        }
      }
      if (res == SM_POS) {
        have_prev = true, prev_lazy = true, prev_t = t;
      } else if (res == SM_OK) {
        if (have_prev && s < 0.0f && (prev_lazy || prev_sdf > 0.0f)) {
          // zero crossing: the previous sample's value is needed first
          cur_s = s;
          if (prev_lazy) {
            phase = PH_PREV;
          } else {
            l = prev_t, r = t, ls = prev_sdf, rs = s, k = 0, side = 0;
            phase = PH_REFINE;
          }
          continue;
        }
        prev_sdf = s, prev_t = t, have_prev = true, prev_lazy = false;
      }
      t += step;
      continue;
    }
    if (phase == PH_PREV) {
      prev_lazy = false;
      // the previous sample was valid; an invalid one here cannot happen
      // while every sdf writer keeps nnc exact
      if (res != SM_OK) set_error(d, MH_ERR_STATE);
      if (res != SM_OK || !(s > 0.0f)) {
        // no crossing (ray_caster.cu:87-88 needs prev > 0): the march goes on
        // from the negative sample
        prev_sdf = cur_s, prev_t = t, have_prev = true;
        t += step;
        phase = PH_MARCH;
        continue;
      }
      prev_sdf = s;
      l = prev_t, r = t, ls = prev_sdf, rs = cur_s, k = 0, side = 0;
      phase = PH_REFINE;
      continue;
    }
    if (phase == PH_REFINE) {
      bool hit = false;
      if (res == SM_OK) {
        if (ls * s > 0.0f) l = m, ls = s, side |= 1 << k;
        else r = m, rs = s;
        if (++k < 3) continue;
        hit = fabsf(prev_sdf - cur_s) < p.sample_sdf_threshold && fabsf(cur_s) < p.sdf_threshold;
      }
      if (!hit) {
        // BisectionIntersection failed or the sample is not good enough:
        // the march goes on from this sample (ray_caster.cu:119-122)
        prev_sdf = cur_s, prev_t = t, have_prev = true, prev_lazy = false;
        t += step;
        phase = PH_MARCH;
        continue;
      }
      out.hit = true, out.t0 = prev_t, out.t1 = t, out.m = m, out.side = side;
      if (!(spacing > 0.0f)) break;
      iso = f3(cam.x + m * wd.x, cam.y + m * wd.y, cam.z + m * wd.z);
      k = 0;
      out.g_ok = true;
      phase = PH_GRAD;
      continue;
    }
    // PH_GRAD
    if (res != SM_OK) {
      out.g_ok = false;
      break;
    }
    if (!(k & 1)) {
      g_minus = s;
    } else {
      const float gi = (s - g_minus) / (vs * (2.0f * spacing));
      const int ax = k >> 1;
      out.g = f3(ax == 0 ? gi : out.g.x, ax == 1 ? gi : out.g.y, ax == 2 ? gi : out.g.z);
    }
    if (++k == 6) break;
  }
  return out;
}

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
  const bool want_normal = p.enable_gradients && out_norm;
  const March mr = ray_march(d, cam, wd, t_min, t_max, want_normal ? 0.5f : 0.0f);
  if (mr.hit) {
    const float dz = mr.m * cd.z;
    o_depth = dz;
    o_vert = make_float4(dz * rx, dz * ry, dz, 1.0f);
    if (want_normal) {
      const F3 g = mr.g;
      const float len = sqrtf(dot3(g, g));
      F3 nn = f3(0.0f, 0.0f, 0.0f);
      if (mr.g_ok && len > 0.0f) nn = f3(g.x / len, g.y / len, g.z / len);
      nn = f3(-nn.x, -nn.y, -nn.z);
      const F3 nc = mul_dir(cTw, nn);
      o_norm = make_float4(nc.x, nc.y, nc.z, 1.0f);
    }
  }
  if (out_depth) out_depth[pix] = o_depth;
  if (out_vert) out_vert[pix] = o_vert;
  if (out_norm) out_norm[pix] = o_norm;
}
// six resident CTAs per SM (at most 80 registers; a few bytes spill) ran
// 1.5 % faster than the five that 86 registers allow, with the same output
__global__ void __launch_bounds__(RC_TX *RC_TY, 6) k_raycast(Dev d, float *out_depth, float4 *out_vert, float4 *out_norm) { raycast_body<RC_TX, RC_TY>(d, blockIdx.x, blockIdx.y, out_depth, out_vert, out_norm); }
// batched raycast over the scenes' concatenated TX x TY tiles; the tile shape
// is an autotuned choice (the scene table's ray_tile0 follows it)
template <int TX, int TY>
__global__ void __launch_bounds__(TX *TY, 4) k_raycast_b(const Scene *t, int n, int total) {
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

// Before a raycast: flag the candidate blocks whose own voxels and those of
// their seven upper neighbours (the blocks at +1 in x, y, z and their
// combinations, which a sample whose first corner lies in the block may
// reach) all exist and count 512 non-negative voxels.  Blocks outside the
// candidate list stay unflagged, which only turns their skip off.
__global__ void __launch_bounds__(256) k_ray_cells(Dev d) {
  const int n = *reinterpret_cast<volatile int *>(&d.ctr->cand_count);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int4 cb = d.cand[i];
    if (cb.w < 0) continue;
    bool ok = __ldg(d.nnc + cb.w) == MH_BLOCK_VOXELS;
#pragma unroll 1
    for (int j = 1; j < 8 && ok; ++j) {
      const int q = hash_find(d, cb.x + (j & 1), cb.y + ((j >> 1) & 1), cb.z + ((j >> 2) & 1));
      ok = q >= 0 && __ldg(d.nnc + q) == MH_BLOCK_VOXELS;
    }
    d.cellok[cb.w] = ok ? 1 : 0;
  }
}
static int prepare_cells(const Dev &d, cudaStream_t s) {
  if (!d.cellok) return MH_OK;
  MH_CUDA_TRY(cudaMemsetAsync(d.cellok, 0, (size_t)d.p.value_capacity, s));
  k_ray_cells<<<mh_sm_count() * 8, 256, 0, s>>>(d);
  mh_count_launches(1);
  return cudaGetLastError() == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}

// number of nonzero bytes of flags[0, n) added to *out
__global__ void k_count_flags(const uint8_t *flags, int n, int *out) {
  int c = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) c += flags[i] != 0;
  c = __reduce_add_sync(0xffffffffu, c);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}
int launch_count_flags(const uint8_t *flags, int n, int *out, cudaStream_t s) {
  k_count_flags<<<std::max(1, std::min((n + 255) / 256, mh_sm_count() * 8)), 256, 0, s>>>(flags, n, out);
  mh_count_launches(1);
  return cudaGetLastError() == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}

int launch_raycast(const Dev &d, float *depth, float *vert4, float *norm4, cudaStream_t s) {
  const int r = prepare_cells(d, s);
  if (r != MH_OK) return r;
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
      // the forward's march: mode 1 takes its hit point and the alignment
      // normal, taken 2.5 voxels either side (inside the truncation band):
      // the half-voxel normal of the rendered image follows the noise of the
      // fused surface, and a noisy normal in J shrinks every Gauss-Newton
      // step (measured: from 2-8 cm / 1-2.5 degree starts, 8 iterations
      // reached 15-90 mm with the half-voxel normal and 1-3 mm on three of
      // four with this one)
      const float spacing = mode == 1 ? fminf(2.5f, 0.8f * p.truncation_distance / p.voxel_size) : 0.0f;
      const March mr = ray_march(d, cam, wd, t_min, t_max, spacing);
      if (mr.hit) {
        if (mode == 1) {
          const float m = mr.m;
          const float o = obs[pix];
          const F3 pm = f3(cam.x + m * wd.x, cam.y + m * wd.y, cam.z + m * wd.z);
          const F3 g = mr.g;
          if (fabsf(m * cd.z - o) < max_res && mr.g_ok) {
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
          // the adjoints re-evaluate the bracketing samples and the three
          // regula-falsi steps along the march's decisions
          RayCache c;
          c.init();
          const RayTrace tr{true, mr.t0, mr.t1, mr.side};
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
  const int r = prepare_cells(d, s);
  if (r != MH_OK) return r;
  dim3 blk(RC_TX, RC_TY);
  dim3 grid((d.p.rc_width + RC_TX - 1) / RC_TX, (d.p.rc_height + RC_TY - 1) / RC_TY);
  k_raycast_grad<<<grid, blk, 0, s>>>(d, mode, dLdD, reinterpret_cast<const float4 *>(dLdN4), grad, obs, max_res,
                                      acc);
  mh_count_launches(1);
  return cudaGetLastError() == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}
