// mh_kernels.h -- host-side launchers of the device stages (one per .cu file).
#pragma once
#include <cuda_runtime.h>

#include "mh_internal.cuh"

struct Scene;

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
int launch_count_flags(const uint8_t *flags, int n, int *out, cudaStream_t s);

int launch_gc_low_surfel(const Dev &d, cudaStream_t s);
int launch_gc_starve(const Dev &d, cudaStream_t s);
int launch_gc_collect_garbage(const Dev &d, cudaStream_t s);
int launch_gc_recycle(const Dev &d, cudaStream_t s);

int launch_denoise_tv(const Dev &d, float *tv, float lambda, int iterations, cudaStream_t s);

// batched twins: one launch per stage for every active scene of a scene table
int launch_batch_preprocess(const Scene *t, int n, cudaStream_t s);
int launch_batch_tv(const Scene *t, int n, int tv_tiles, float lambda, int iterations, cudaStream_t s);
// tiles of the tiled TV kernel for a W x H frame
int tv_tile_count(int W, int H);
int launch_batch_alloc(const Scene *t, int n, int total_tiles, cudaStream_t s);
int launch_batch_collect(const Scene *t, int n, cudaStream_t s);
int launch_batch_predict(const Scene *t, int n, cudaStream_t s);
int launch_batch_integrate(const Scene *t, int n, int has_simple, int has_psdf, int cta_per_sm, cudaStream_t s);
int launch_batch_mesh(const Scene *t, int n, cudaStream_t s);
int launch_batch_gc_low_surfel(const Scene *t, int n, cudaStream_t s);
int launch_batch_gc_recycle(const Scene *t, int n, int which, cudaStream_t s);
int launch_batch_gc_starve(const Scene *t, int n, cudaStream_t s);
int launch_raycast_batch(const Scene *t, int n, int total_tiles, int shape, cudaStream_t s);
int ray_tile_shapes();
void ray_tile_shape(int i, int &tx, int &ty);
void batch_warm_occupancy();
