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
// GB300 structure: each thread keeps a one-entry cache of the last block
// lookup (hit or miss), so a sample whose eight corners lie in the block of the
// previous sample costs no hash probe, and samples inside a block already known
// to be missing cost only arithmetic (empty-space skip).  Outputs are written
// once per pixel.
#include "mh_internal.cuh"
#include "mh_kernels.h"

// Rays are handed out in 8x4-pixel tiles by one global counter; a lane whose
// ray terminates takes the next ray at once (warp-aggregated atomic), so a
// warp keeps all lanes marching until the pool is empty instead of waiting
// for its longest ray.  Each loop iteration advances every lane's ray by one
// sample; the per-ray sequence of samples and decisions is exactly the
// reference's.
#define RC_THREADS 128
#define RC_TILE_W 8
#define RC_TILE_H 4

struct RayState {
  int pix;
  unsigned x, y;
  float rx, ry, t, t_max, prev_sdf, prev_t;
  F3 cd, wd;
  bool have_prev;
};

__global__ void __launch_bounds__(RC_THREADS) k_raycast(Dev d, float *out_depth, float4 *out_vert, float4 *out_norm) {
  __shared__ float sm[32];
  const int tid = threadIdx.x;
  if (tid < 16) sm[tid] = d.fc->rc_wTc[tid];
  else if (tid < 32) sm[tid] = d.fc->rc_cTw[tid - 16];
  __syncthreads();
  const float *wTc = sm, *cTw = sm + 16;
  const DevParams &p = d.p;
  const unsigned W = p.rc_width, H = p.rc_height;
  const unsigned tiles_x = (W + RC_TILE_W - 1) / RC_TILE_W, tiles_y = (H + RC_TILE_H - 1) / RC_TILE_H;
  const int n_rays = (int)(tiles_x * tiles_y * RC_TILE_W * RC_TILE_H);
  const F3 cam = mul_pt(wTc, f3(0.0f, 0.0f, 0.0f));
  const float step = p.raycast_step;
  const float NI = -__int_as_float(0x7f800000);
  int *counter = &d.ctr->ray_next;

  RayState r;
  r.pix = -1;
  BlockCache bc, bc2;
  float r_unused;
  while (true) {
    const bool need = r.pix < 0;
    const unsigned act = __activemask();
    const unsigned m = __ballot_sync(act, need);
    if (m) {
      const int leader = __ffs(m) - 1;
      int base = 0;
      if ((int)lane_id() == leader) base = atomicAdd(counter, __popc(m));
      base = __shfl_sync(act, base, leader);
      if (need) {
        const int id = base + __popc(m & lanemask_lt());
        if (id >= n_rays) break;
        const unsigned tile = (unsigned)id / (RC_TILE_W * RC_TILE_H), k = (unsigned)id % (RC_TILE_W * RC_TILE_H);
        r.x = (tile % tiles_x) * RC_TILE_W + k % RC_TILE_W;
        r.y = (tile / tiles_x) * RC_TILE_H + k / RC_TILE_W;
        if (r.x >= W || r.y >= H) continue;
        r.pix = (int)(r.y * W + r.x);
        r.rx = ((float)r.x - p.rc_cx) / p.rc_fx;
        r.ry = ((float)r.y - p.rc_cy) / p.rc_fy;
        r.cd = normalize3(f3(1.0f * r.rx, 1.0f * r.ry, 1.0f));
        r.t = p.min_raycast_depth / r.cd.z;
        r.t_max = p.max_raycast_depth / r.cd.z;
        r.wd = normalize3(mul_dir(wTc, r.cd));
        r.have_prev = false;
        r.prev_sdf = 0.0f, r.prev_t = 0.0f;
        bc.init();
        bc2.init();
        if (!(r.t < r.t_max)) {
          if (out_depth) out_depth[r.pix] = NI;
          if (out_vert) out_vert[r.pix] = make_float4(NI, NI, NI, NI);
          if (out_norm) out_norm[r.pix] = make_float4(NI, NI, NI, NI);
          r.pix = -1;
          continue;
        }
      }
    }
    // one sample of this lane's ray (visualization/ray_caster.cu:64-148)
    const float t = r.t;
    const F3 sp = f3(cam.x + t * r.wd.x, cam.y + t * r.wd.y, cam.z + t * r.wd.z);
    float s;
    bool hit = false;
    if (spatial_sample<false>(d, bc, sp, s, r_unused, &bc2)) {
      if (r.have_prev && r.prev_sdf > 0.0f && s < 0.0f) {
        float l = r.prev_t, rr = t, mm = (l + rr) * 0.5f;
        float ls = r.prev_sdf, rs = s;
        bool found = true;
#pragma unroll 1
        for (int k = 0; k < 3; ++k) {
          mm = l + (ls / (ls - rs)) * (rr - l);
          float ms;
          if (!spatial_sample<false>(d, bc, f3(cam.x + mm * r.wd.x, cam.y + mm * r.wd.y, cam.z + mm * r.wd.z), ms,
                                     r_unused, &bc2)) {
            found = false;
            break;
          }
          if (ls * ms > 0.0f) {
            l = mm, ls = ms;
          } else {
            rr = mm, rs = ms;
          }
        }
        if (found && fabsf(r.prev_sdf - s) < p.sample_sdf_threshold && fabsf(s) < p.sdf_threshold) {
          const float dz = mm * r.cd.z;
          if (out_depth) out_depth[r.pix] = dz;
          if (out_vert) out_vert[r.pix] = make_float4(dz * r.rx, dz * r.ry, dz, 1.0f);
          if (out_norm) {
            float4 o_norm = make_float4(NI, NI, NI, NI);
            if (p.enable_gradients) {
              const F3 iso = f3(cam.x + mm * r.wd.x, cam.y + mm * r.wd.y, cam.z + mm * r.wd.z);
              F3 g;
              const bool ok = spatial_gradient(d, bc, iso, g);
              const float len = sqrtf(dot3(g, g));
              F3 nn = f3(0.0f, 0.0f, 0.0f);
              if (ok && len > 0.0f) nn = f3(g.x / len, g.y / len, g.z / len);
              nn = f3(-nn.x, -nn.y, -nn.z);
              const F3 nc = mul_dir(cTw, nn);
              o_norm = make_float4(nc.x, nc.y, nc.z, 1.0f);
            }
            out_norm[r.pix] = o_norm;
          }
          hit = true;
        }
      }
      if (!hit) r.prev_sdf = s, r.prev_t = t, r.have_prev = true;
    }
    if (!hit) {
      r.t = t + step;
      if (!(r.t < r.t_max)) {
        if (out_depth) out_depth[r.pix] = NI;
        if (out_vert) out_vert[r.pix] = make_float4(NI, NI, NI, NI);
        if (out_norm) out_norm[r.pix] = make_float4(NI, NI, NI, NI);
        hit = true;
      }
    }
    if (hit) r.pix = -1;
  }
}

int launch_raycast(const Dev &d, float *depth, float *vert4, float *norm4, cudaStream_t s) {
  MH_CUDA_TRY(cudaMemsetAsync(&d.ctr->ray_next, 0, sizeof(int), s));
  k_raycast<<<mh_sm_count() * 8, RC_THREADS, 0, s>>>(d, depth, reinterpret_cast<float4 *>(vert4),
                                                      reinterpret_cast<float4 *>(norm4));
  mh_count_launches(1);
  return cudaGetLastError() == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}
