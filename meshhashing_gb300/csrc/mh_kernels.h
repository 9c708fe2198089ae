// mh_kernels.h -- host-side launchers of the device stages (one per .cu file).
#pragma once
#include <cuda_runtime.h>

#include "mh_internal.cuh"

int launch_alloc(const Dev &d, cudaStream_t s);
int launch_collect(const Dev &d, int frustum, cudaStream_t s);
int launch_insert_list(const Dev &d, const int *pos_dev, int n, cudaStream_t s);
int launch_find_list(const Dev &d, const int *pos_dev, int n, int *ptr_dev, cudaStream_t s);
int launch_set_candidates(const Dev &d, const int *pos_dev, const int *ptr_dev, int n, cudaStream_t s);

int launch_preprocess(const Dev &d, const float *src, const uint16_t *src16, float range_factor, cudaStream_t s);
int launch_integrate_simple(const Dev &d, cudaStream_t s);
int launch_integrate_psdf(const Dev &d, cudaStream_t s);
int launch_predict_inlier(const Dev &d, cudaStream_t s);

int launch_mesh(const Dev &d, cudaStream_t s);

int launch_raycast(const Dev &d, float *depth, float *vert4, float *norm4, cudaStream_t s);

int launch_gc_low_surfel(const Dev &d, cudaStream_t s);
int launch_gc_starve(const Dev &d, cudaStream_t s);
int launch_gc_collect_garbage(const Dev &d, cudaStream_t s);
int launch_gc_recycle(const Dev &d, cudaStream_t s);

int launch_denoise_tv(const Dev &d, float *tv, float lambda, int iterations, cudaStream_t s);
