// mh_pose.cu -- host side of the differentiable raycast: gradients of the
// rendered depth and normals, Gauss-Newton normal equations of depth
// alignment, and frame-to-model pose refinement driven by them.
//
// No reference counterpart for the gradients.  Two trackers: the reference's
// point-to-PSDF Gauss-Newton over the frame's points (localizing/
// point_to_psdf.cu, MainEngine::Localizing), and a projective point-to-plane
// refinement against the raycast of the model, differentiated through the
// raycast itself (kernels in mh_raycast.cu).  Pose perturbations are left
// se(3) increments wTc <- exp(xi) wTc with xi = (v, w): translation first,
// then rotation (Sophus's tangent order).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "mh_kernels.h"
#include "mh_volume.h"

int launch_raycast_grad(const Dev &d, int mode, const float *dLdD, const float *dLdN4, float *grad, const float *obs,
                        float max_res, double *acc, cudaStream_t s);

namespace {

// the raycast pose for a launch (as mh_raycast sets it)
int set_raycast_pose(mh_volume *v, const float cTw[16], cudaStream_t s) {
  FrameConst &fc = v->fc_host;
  memcpy(fc.rc_cTw, cTw, sizeof(float) * 16);
  inverse4(fc.rc_cTw, fc.rc_wTc);
  if (!v->has_frame) {
    memcpy(fc.cTw, cTw, sizeof(float) * 16);
    memcpy(fc.wTc, fc.rc_wTc, sizeof(float) * 16);
  }
  return cudaMemcpyAsync(v->d.fc, &fc, sizeof(FrameConst), cudaMemcpyHostToDevice, s) == cudaSuccess ? MH_OK
                                                                                                        : MH_ERR_CUDA;
}

int ensure_acc(mh_volume *v) {
  if (v->acc) return MH_OK;
  return cudaMalloc((void **)&v->acc, sizeof(double) * 32) == cudaSuccess ? MH_OK : MH_ERR_NOMEM;
}

// exp of a left se(3) increment applied to a row-major 4x4 pose (double)
void se3_left_update(const double xi[6], double T[16]) {
  const double w[3] = {xi[3], xi[4], xi[5]}, u[3] = {xi[0], xi[1], xi[2]};
  const double th2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2], th = std::sqrt(th2);
  double A, B, C;  // sin(t)/t, (1 - cos t)/t^2, (t - sin t)/t^3
  if (th < 1e-5) {
    A = 1.0 - th2 / 6.0, B = 0.5 - th2 / 24.0, C = 1.0 / 6.0 - th2 / 120.0;
  } else {
    A = std::sin(th) / th, B = (1.0 - std::cos(th)) / th2, C = (th - std::sin(th)) / (th2 * th);
  }
  const double W[9] = {0, -w[2], w[1], w[2], 0, -w[0], -w[1], w[0], 0};
  double W2[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0;
      for (int k = 0; k < 3; ++k) s += W[3 * i + k] * W[3 * k + j];
      W2[3 * i + j] = s;
    }
  double Rd[9], V[9];
  for (int i = 0; i < 9; ++i) {
    const double I = (i % 4 == 0) ? 1.0 : 0.0;
    Rd[i] = I + A * W[i] + B * W2[i];
    V[i] = I + B * W[i] + C * W2[i];
  }
  double td[3];
  for (int i = 0; i < 3; ++i) td[i] = V[3 * i] * u[0] + V[3 * i + 1] * u[1] + V[3 * i + 2] * u[2];
  double out[16] = {0};
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 4; ++j) {
      double s = 0;
      for (int k = 0; k < 3; ++k) s += Rd[3 * i + k] * T[4 * k + j];
      out[4 * i + j] = s + (j == 3 ? td[i] : 0.0);
    }
  }
  out[15] = 1.0;
  memcpy(T, out, sizeof(out));
}

// solve the symmetric positive definite 6x6 system A x = b (Cholesky)
bool solve6(const double A_in[36], const double b[6], double x[6]) {
  double L[36] = {0};
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j <= i; ++j) {
      double s = A_in[6 * i + j];
      for (int k = 0; k < j; ++k) s -= L[6 * i + k] * L[6 * j + k];
      if (i == j) {
        if (!(s > 0.0)) return false;
        L[6 * i + i] = std::sqrt(s);
      } else {
        L[6 * i + j] = s / L[6 * j + j];
      }
    }
  double y[6];
  for (int i = 0; i < 6; ++i) {
    double s = b[i];
    for (int k = 0; k < i; ++k) s -= L[6 * i + k] * y[k];
    y[i] = s / L[6 * i + i];
  }
  for (int i = 5; i >= 0; --i) {
    double s = y[i];
    for (int k = i + 1; k < 6; ++k) s -= L[6 * k + i] * x[k];
    x[i] = s / L[6 * i + i];
  }
  return true;
}

// the pose becomes the frame's pose for the mapping stages and the raycast
int adopt_frame_pose(mh_volume *v, const float wTc[16], cudaStream_t s) {
  if (!v->has_frame) return MH_OK;
  FrameConst &fc = v->fc_host;
  memcpy(fc.wTc, wTc, sizeof(float) * 16);
  inverse4(fc.wTc, fc.cTw);
  memcpy(fc.rc_cTw, fc.cTw, sizeof(float) * 16);
  inverse4(fc.rc_cTw, fc.rc_wTc);
  return cudaMemcpyAsync(v->d.fc, &fc, sizeof(FrameConst), cudaMemcpyHostToDevice, s) == cudaSuccess ? MH_OK
                                                                                                      : MH_ERR_CUDA;
}

struct Pose16 {
  float m[16];
};

// PointToSurfaceKernel (localizing/point_to_psdf.cu:19-84): one thread per
// pixel with odd x and odd y.  A valid depth is reprojected
// (ImageReprojectToCamera, geometry_helper.h:164-170), moved to the world by
// wTc, and contributes when its trilinear sdf D and gradient g both exist:
// J = [g, p x g] (the reference writes J[2] = g.x, point_to_psdf.cu:70,
// kept when ref_j is set), A += J J^T, b += D J, err += D^2, count += 1.
// acc = [A upper triangle (21), b (6), err, count], CTA sums added as doubles.
__global__ void __launch_bounds__(256) k_point_to_psdf(Dev d, Pose16 T, int ref_j, double *acc) {
  const DevParams &p = d.p;
  const unsigned x = 2 * (blockIdx.x * 16 + threadIdx.x) + 1, y = 2 * (blockIdx.y * 16 + threadIdx.y) + 1;
  float v[29];
#pragma unroll
  for (int k = 0; k < 29; ++k) v[k] = 0.0f;
  if (x < p.width && y < p.height) {
    const float dep = d.depth[(size_t)y * p.width + x];
    if (!depth_invalid(p, dep)) {
      const float rx = ((float)x - p.cx) / p.fx, ry = ((float)y - p.cy) / p.fy;
      const F3 pw = mul_pt(T.m, f3(dep * rx, dep * ry, dep));
      BlockCache bc, bc2;
      bc.init();
      bc2.init();
      float s, r;
      F3 g;
      if (spatial_sample<false>(d, bc, pw, s, r, &bc2) && spatial_gradient(d, bc, pw, g)) {
        const float J[6] = {g.x, g.y, ref_j ? g.x : g.z, -g.y * pw.z + g.z * pw.y, -g.z * pw.x + g.x * pw.z,
                            -g.x * pw.y + g.y * pw.x};
        int k = 0;
#pragma unroll
        for (int i = 0; i < 6; ++i)
#pragma unroll
          for (int j = i; j < 6; ++j) v[k++] = J[i] * J[j];
#pragma unroll
        for (int i = 0; i < 6; ++i) v[21 + i] = s * J[i];
        v[27] = s * s;
        v[28] = 1.0f;
      }
    }
  }
  __shared__ float red[29][8];
  const int tid = threadIdx.x + 16 * threadIdx.y, lane = tid & 31, wid = tid >> 5;
#pragma unroll
  for (int k = 0; k < 29; ++k) {
    float z = v[k];
    for (int o = 16; o; o >>= 1) z += __shfl_xor_sync(0xffffffffu, z, o);
    if (lane == 0) red[k][wid] = z;
  }
  __syncthreads();
  if (tid < 29) {
    double sum = 0.0;
    for (int w = 0; w < 8; ++w) sum += red[tid][w];
    if (sum != 0.0) atomicAdd(acc + tid, sum);
  }
}

}  // namespace

extern "C" {

int mh_point_to_psdf_normal_equations(mh_volume *v, const float wTc[16], int reference_jacobian, double A[36],
                                      double b[6], double *err, int *count, void *stream) {
  if (!v || !wTc) return MH_ERR_INVALID;
  if (!v->has_frame) return MH_ERR_STATE;
  cudaStream_t s = (cudaStream_t)stream;
  int r;
  if ((r = ensure_acc(v)) != MH_OK) return r;
  if (cudaMemsetAsync(v->acc, 0, sizeof(double) * 32, s) != cudaSuccess) return MH_ERR_CUDA;
  Pose16 T;
  memcpy(T.m, wTc, sizeof(T.m));
  const unsigned hw = (v->hp.width / 2 + 15) / 16, hh = (v->hp.height / 2 + 15) / 16;
  k_point_to_psdf<<<dim3(hw ? hw : 1, hh ? hh : 1), dim3(16, 16), 0, s>>>(v->d, T, reference_jacobian ? 1 : 0,
                                                                          v->acc);
  mh_count_launches(1);
  if (cudaGetLastError() != cudaSuccess) return MH_ERR_CUDA;
  double h[29];
  if (cudaMemcpyAsync(h, v->acc, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return MH_ERR_CUDA;
  if (A) {
    int k = 0;
    for (int i = 0; i < 6; ++i)
      for (int j = i; j < 6; ++j, ++k) A[6 * i + j] = A[6 * j + i] = h[k];
  }
  if (b) memcpy(b, h + 21, sizeof(double) * 6);
  if (err) *err = h[27];
  if (count) *count = (int)h[28];
  return MH_OK;
}

// MainEngine::Localizing (engine/main_engine.cc:70-98): per iteration the
// normal equations at the current pose; none -> stop; otherwise
// dxi = -(A + lambda I)^-1 b and wTc <- exp(dxi) wTc (SolveAndConvertDeltaXi,
// main_engine.cc:28-54, with Eigen's LDLT and Sophus's exp restated: a
// Cholesky solve and the closed-form SE(3) exponential, in double).
int mh_track_point_to_psdf(mh_volume *v, float wTc[16], int iterations, float lambda, int reference_jacobian,
                           double *final_err, int *final_count, void *stream) {
  if (!v || !wTc || iterations < 0 || !(lambda >= 0.0f)) return MH_ERR_INVALID;
  if (!v->has_frame) return MH_ERR_STATE;
  double T[16];
  for (int i = 0; i < 16; ++i) T[i] = wTc[i];
  double err = 0.0;
  int count = 0;
  for (int it = 0; it < iterations; ++it) {
    float Tf[16];
    for (int i = 0; i < 16; ++i) Tf[i] = (float)T[i];
    double A[36], b[6];
    int r = mh_point_to_psdf_normal_equations(v, Tf, reference_jacobian, A, b, &err, &count, stream);
    if (r != MH_OK) return r;
    if (count == 0) break;
    for (int i = 0; i < 6; ++i) A[7 * i] += lambda;
    double nb[6], x[6];
    for (int i = 0; i < 6; ++i) nb[i] = -b[i];
    if (!solve6(A, nb, x)) break;
    se3_left_update(x, T);
  }
  for (int i = 0; i < 16; ++i) wTc[i] = (float)T[i];
  if (final_err) *final_err = err;
  if (final_count) *final_count = count;
  return adopt_frame_pose(v, wTc, (cudaStream_t)stream);
}

int mh_raycast_backward(mh_volume *v, const float cTw[16], const float *dL_ddepth, const float *dL_dnormal4,
                        float *grad_sdf, double dL_dxi[6], void *stream) {
  if (!v || !cTw || (!dL_ddepth && !dL_dnormal4)) return MH_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  int r;
  if ((r = ensure_acc(v)) != MH_OK) return r;
  if ((r = set_raycast_pose(v, cTw, s)) != MH_OK) return r;
  if (cudaMemsetAsync(v->acc, 0, sizeof(double) * 32, s) != cudaSuccess) return MH_ERR_CUDA;
  if ((r = launch_raycast_grad(v->d, 0, dL_ddepth, dL_dnormal4, grad_sdf, nullptr, 0.0f, v->acc, s)) != MH_OK)
    return r;
  double h[6];
  if (cudaMemcpyAsync(h, v->acc, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return MH_ERR_CUDA;
  if (dL_dxi) memcpy(dL_dxi, h, sizeof(h));
  return MH_OK;
}

int mh_raycast_normal_equations(mh_volume *v, const float cTw[16], const float *obs_depth, float max_residual,
                                double JtJ[36], double Jtr[6], double *cost, int *count, void *stream) {
  if (!v || !cTw || !(max_residual > 0.0f)) return MH_ERR_INVALID;
  const float *obs = obs_depth;
  if (!obs) {
    if (!v->has_frame || v->hp.width != v->hp.rc_width || v->hp.height != v->hp.rc_height) return MH_ERR_STATE;
    obs = v->d.depth;
  }
  cudaStream_t s = (cudaStream_t)stream;
  int r;
  if ((r = ensure_acc(v)) != MH_OK) return r;
  if ((r = set_raycast_pose(v, cTw, s)) != MH_OK) return r;
  if (cudaMemsetAsync(v->acc, 0, sizeof(double) * 32, s) != cudaSuccess) return MH_ERR_CUDA;
  if ((r = launch_raycast_grad(v->d, 1, nullptr, nullptr, nullptr, obs, max_residual, v->acc, s)) != MH_OK) return r;
  double h[29];
  if (cudaMemcpyAsync(h, v->acc, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return MH_ERR_CUDA;
  if (JtJ) {
    int k = 0;
    for (int i = 0; i < 6; ++i)
      for (int j = i; j < 6; ++j, ++k) JtJ[6 * i + j] = JtJ[6 * j + i] = h[k];
  }
  if (Jtr) memcpy(Jtr, h + 21, sizeof(double) * 6);
  if (cost) *cost = h[27];
  if (count) *count = (int)h[28];
  return MH_OK;
}

int mh_refine_pose(mh_volume *v, const float *obs_depth, float wTc[16], int iterations, float max_residual,
                   double *final_cost, int *final_count, void *stream) {
  if (!v || !wTc || iterations < 0 || !(max_residual > 0.0f)) return MH_ERR_INVALID;
  double T[16];
  for (int i = 0; i < 16; ++i) T[i] = wTc[i];
  double cost = 0.0;
  int count = 0;
  for (int it = 0; it <= iterations; ++it) {
    float Tf[16], cTw[16];
    for (int i = 0; i < 16; ++i) Tf[i] = (float)T[i];
    inverse4(Tf, cTw);
    double A[36], b[6];
    // the residual gate opens at 4x max_residual and halves per iteration
    // down to it: a start centimetres off keeps enough pixels, the last
    // steps keep only close ones
    const float gate = std::max(max_residual, 4.0f * max_residual * std::ldexp(1.0f, -it));
    int r = mh_raycast_normal_equations(v, cTw, obs_depth, it == iterations ? max_residual : gate, A, b, &cost,
                                        &count, stream);
    if (r != MH_OK) return r;
    if (it == iterations || count < 6) break;
    // Gauss-Newton step with a tiny Levenberg term for rank-deficient views
    double tr = 0.0;
    for (int i = 0; i < 6; ++i) tr += A[7 * i];
    for (int i = 0; i < 6; ++i) A[7 * i] += 1e-9 * tr + 1e-12;
    double nb[6], x[6];
    for (int i = 0; i < 6; ++i) nb[i] = -b[i];
    if (!solve6(A, nb, x)) break;
    se3_left_update(x, T);
  }
  for (int i = 0; i < 16; ++i) wTc[i] = (float)T[i];
  if (final_cost) *final_cost = cost;
  if (final_count) *final_count = count;
  // the refined pose becomes the frame's pose for the mapping stages
  return adopt_frame_pose(v, wTc, (cudaStream_t)stream);
}

int mh_dump_block_field(mh_volume *v, const float *field, int max_blocks, int32_t *pos, float *out, int *n_out) {
  if (!v || !field) return MH_ERR_INVALID;
  if (cudaDeviceSynchronize() != cudaSuccess) return MH_ERR_CUDA;
  Counters c;
  if (cudaMemcpy(&c, v->d.ctr, sizeof(c), cudaMemcpyDeviceToHost) != cudaSuccess) return MH_ERR_CUDA;
  const int hw = c.high_water;
  std::vector<int4> bp(hw > 0 ? hw : 1);
  std::vector<float> all((size_t)(hw > 0 ? hw : 1) * MH_BLOCK_VOXELS);
  if (hw > 0) {
    if (cudaMemcpy(bp.data(), v->d.block_pos, sizeof(int4) * hw, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(all.data(), field, sizeof(float) * MH_BLOCK_VOXELS * hw, cudaMemcpyDeviceToHost) != cudaSuccess)
      return MH_ERR_CUDA;
  }
  int n = 0;
  for (int i = 0; i < hw; ++i) {
    if (!bp[i].w) continue;
    if (n < max_blocks) {
      if (pos) pos[3 * n] = bp[i].x, pos[3 * n + 1] = bp[i].y, pos[3 * n + 2] = bp[i].z;
      if (out) memcpy(out + (size_t)n * MH_BLOCK_VOXELS, all.data() + (size_t)i * MH_BLOCK_VOXELS,
                      sizeof(float) * MH_BLOCK_VOXELS);
    }
    ++n;
  }
  if (n_out) *n_out = n;
  return MH_OK;
}

}  // extern "C"
