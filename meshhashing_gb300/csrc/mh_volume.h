// mh_volume.h -- host-side state of one volume (shared by the volume and the
// batch entry points).
#pragma once
#include <cuda_runtime.h>

#include <utility>
#include <vector>

#include "mh_internal.cuh"

struct mh_pd_state;

struct mh_volume {
  mh_params hp;
  Dev d;
  float *tv = nullptr;
  float *rc_stage = nullptr;  // device staging for host raycast outputs
  double *acc = nullptr;      // reduction target of the raycast gradients (allocated on first use)
  uint8_t *touch = nullptr;   // raycast footprint flags, one per block (allocated on first use)
  mh_pd_state *pd = nullptr;  // Huber-TV state (allocated on first use)
  int *scratch = nullptr;     // device scratch for list operations
  size_t scratch_bytes = 0;
  FrameConst fc_host;
  bool has_frame = false;
  int frames = 0;
  std::vector<void *> allocs;
  // per-stage CUDA-event timing (events are pooled and reused)
  bool prof = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pend[MH_STAGE_COUNT];
  std::vector<cudaEvent_t> ev_pool;
  cudaEvent_t event() {
    cudaEvent_t e = nullptr;
    if (!ev_pool.empty()) {
      e = ev_pool.back();
      ev_pool.pop_back();
    } else {
      cudaEventCreate(&e);
    }
    return e;
  }
};

// 4x4 inverse by cofactors with the term order of float4x4::getInverse
// (extern/cuda/matrix.h:964-1086)
void inverse4(const float *m, float *out);
// releases the Huber-TV state of a volume (mh_huber.cu)
void mh_pd_free(mh_volume *v);
