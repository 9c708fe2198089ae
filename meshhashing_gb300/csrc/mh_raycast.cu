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
// GB300 structure: 16x8-pixel CTAs keep neighbouring rays in one warp (they
// walk the same blocks); each thread caches its last two block lookups (hit
// or miss), so a sample whose corners lie in the blocks of the previous
// sample costs no hash probe, and a sample inside a block already known to be
// missing costs three divisions and a compare (empty-space skip).  Outputs are
// written once per pixel.
#include "mh_internal.cuh"
#include "mh_kernels.h"

#define RC_TX 16
#define RC_TY 8

__global__ void __launch_bounds__(RC_TX *RC_TY) k_raycast(Dev d, float *out_depth, float4 *out_vert, float4 *out_norm) {
  __shared__ float sm[32];
  const int tid = threadIdx.x + threadIdx.y * RC_TX;
  if (tid < 16) sm[tid] = d.fc->rc_wTc[tid];
  else if (tid < 32) sm[tid] = d.fc->rc_cTw[tid - 16];
  __syncthreads();
  const float *wTc = sm, *cTw = sm + 16;
  const DevParams &p = d.p;
  const unsigned x = blockIdx.x * RC_TX + threadIdx.x;
  const unsigned y = blockIdx.y * RC_TY + threadIdx.y;
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

  BlockCache bc, bc2;
  bc.init();
  bc2.init();
  bool have_prev = false;
  float prev_sdf = 0.0f, prev_t = 0.0f;
  const float step = p.raycast_step;
  float r_unused;
#pragma unroll 1
  for (float t = t_min; t < t_max; t += step) {
    const F3 sp = f3(cam.x + t * wd.x, cam.y + t * wd.y, cam.z + t * wd.z);
    float s;
    if (!spatial_sample<false>(d, bc, sp, s, r_unused, &bc2)) continue;
    if (have_prev && prev_sdf > 0.0f && s < 0.0f) {
      float l = prev_t, r = t, m = (l + r) * 0.5f;
      float ls = prev_sdf, rs = s;
      bool found = true;
#pragma unroll 1
      for (int k = 0; k < 3; ++k) {
        m = l + (ls / (ls - rs)) * (r - l);
        float ms;
        if (!spatial_sample<false>(d, bc, f3(cam.x + m * wd.x, cam.y + m * wd.y, cam.z + m * wd.z), ms, r_unused,
                                   &bc2)) {
          found = false;
          break;
        }
        if (ls * ms > 0.0f) {
          l = m, ls = ms;
        } else {
          r = m, rs = ms;
        }
      }
      if (found && fabsf(prev_sdf - s) < p.sample_sdf_threshold && fabsf(s) < p.sdf_threshold) {
        const float dz = m * cd.z;
        o_depth = dz;
        o_vert = make_float4(dz * rx, dz * ry, dz, 1.0f);
        if (p.enable_gradients && out_norm) {
          const F3 iso = f3(cam.x + m * wd.x, cam.y + m * wd.y, cam.z + m * wd.z);
          F3 g;
          const bool ok = spatial_gradient(d, bc, iso, g);
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
  }
  if (out_depth) out_depth[pix] = o_depth;
  if (out_vert) out_vert[pix] = o_vert;
  if (out_norm) out_norm[pix] = o_norm;
}

int launch_raycast(const Dev &d, float *depth, float *vert4, float *norm4, cudaStream_t s) {
  dim3 blk(RC_TX, RC_TY);
  dim3 grid((d.p.rc_width + RC_TX - 1) / RC_TX, (d.p.rc_height + RC_TY - 1) / RC_TY);
  k_raycast<<<grid, blk, 0, s>>>(d, depth, reinterpret_cast<float4 *>(vert4), reinterpret_cast<float4 *>(norm4));
  mh_count_launches(1);
  return cudaGetLastError() == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}
