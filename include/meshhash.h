/*
 * meshhash.h -- C ABI of the GB300 volumetric-fusion hot path.
 *
 * Drop-in boundary for MeshHashing's engine entry points: the spatial hash and
 * block pool (src/core), block allocation and the simple / Bayesian (PSDF)
 * voxel update (src/mapping), per-block marching cubes with shared vertices
 * (src/meshing) and the trilinear raycaster (src/visualization).
 *
 * Conventions
 *  - Every entry point returns an int status (MH_OK == 0).  Device-side
 *    failures (pool exhaustion, bounded-wait overruns) set a sticky error word
 *    in the volume that mh_stats() reads back; no call exits the process.
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 *    Stage calls are asynchronous on that stream; counts stay on the device.
 *  - Poses are row-major float 4x4: wTc maps camera to world, cTw world to
 *    camera, as Sensor::wTc()/cTw() in sensor/rgbd_sensor.h:47-58.
 *  - Depth is float32 metres, row-major width x height, z-depth (not range).
 *  - Pointers marked "device" must be device memory; "host" pointers may be
 *    pageable or pinned.  The library never frees caller memory.
 */
#ifndef MESHHASH_H
#define MESHHASH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MH_OK            0
#define MH_ERR_INVALID   1   /* bad argument or parameter */
#define MH_ERR_CUDA      2   /* a CUDA runtime call failed */
#define MH_ERR_CAPACITY  3   /* block / vertex / triangle / overflow pool exhausted */
#define MH_ERR_TIMEOUT   4   /* a bounded device-side wait ran out */
#define MH_ERR_NOMEM     5   /* device allocation failed at create time */
#define MH_ERR_STATE     6   /* call out of order (e.g. no frame set) */

/* Parameters: restates HashParams, MeshParams, VolumeParams, SensorParams,
 * RayCasterParams and the RuntimeParams flags of core/params.h:16-99. */
typedef struct mh_params {
  /* HashParams (core/params.h:16-24) */
  uint32_t bucket_count;          /* power of two */
  uint32_t bucket_size;           /* slots per bucket; this build supports 4 */
  uint32_t entry_count;           /* informational: bucket_count * bucket_size */
  uint32_t linked_list_size;      /* longest overflow chain per bucket */
  uint32_t value_capacity;        /* blocks in the pool */
  /* MeshParams (core/params.h:26-29) */
  uint32_t max_vertex_count;
  uint32_t max_triangle_count;
  /* VolumeParams (core/params.h:31-40) */
  float    voxel_size;
  float    truncation_distance_scale;
  float    truncation_distance;
  float    sdf_upper_bound;
  uint32_t weight_sample;
  uint32_t weight_upper_bound;    /* parsed but unused, as in the reference */
  /* SensorParams (core/params.h:62-74) */
  float    fx, fy, cx, cy;
  uint32_t width, height;
  float    min_depth_range;
  float    max_depth_range;
  float    range_factor;          /* used by mh_frame_set_u16 only */
  /* RayCasterParams (core/params.h:42-58) */
  float    rc_fx, rc_fy, rc_cx, rc_cy;
  uint32_t rc_width, rc_height;
  float    min_raycast_depth;
  float    max_raycast_depth;
  float    raycast_step;
  float    sample_sdf_threshold;
  float    sdf_threshold;
  int32_t  enable_gradients;      /* raycast normals */
  /* RuntimeParams subset (core/params.h:77-99) */
  int32_t  enable_bayesian_update;
  int32_t  enable_sdf_gradient;   /* vertex normals from the SDF gradient */
  /* this build */
  uint32_t overflow_capacity;     /* entries in the hash overflow pool */
  uint32_t mesh_page_capacity;    /* mesh pages (per-voxel mesh units of one
                                     block, 18.5 KB); only blocks with surface
                                     cubes or owned vertices take one */
  int32_t  compat_arithmetic;     /* 1: evaluate the reference's single-precision
                                     formulas as written (results bit-compatible
                                     with the reference's own kernels);
                                     0 (default): algebraically equal forms
                                     without the reference's cancellations --
                                     the PSDF update with 4 divisions (variance
                                     and Beta moments restated), the simple
                                     update's weight as (dmax - d) / (dmax - dmin) */
} mh_params;

typedef struct mh_stats {
  uint32_t error;                 /* sticky MH_ERR_* set by device code, 0 if none */
  uint32_t blocks_allocated;      /* live blocks in the pool */
  uint32_t block_high_water;      /* highest block index handed out + 1 */
  uint32_t candidates;            /* entries of the current candidate list */
  uint32_t vertices_allocated;
  uint32_t triangles_allocated;
  uint32_t overflow_used;         /* hash overflow entries in use */
  uint32_t frames;                /* frames integrated by mh_integrate_frame */
  uint32_t dropped_inserts;       /* inserts refused because a pool was full */
  uint32_t gc_freed_blocks;       /* blocks returned by garbage collection */
  uint32_t mesh_passes;           /* mh_mesh calls since reset */
  uint64_t candidate_sum;         /* candidate-list lengths summed over mesh passes */
  uint64_t vertex_work_sum;       /* vertices (re)computed, summed over mesh passes */
  uint64_t cube_blocks_sum;       /* blocks whose corner tile the cube pass loaded */
  uint64_t mesh_list_sum;         /* blocks walked by the triangle and recycle passes */
  uint64_t predict_blocks_sum;    /* blocks the inlier prediction read */
  uint32_t mesh_pages_used;       /* mesh pages held by blocks */
} mh_stats;

typedef struct mh_volume mh_volume;

/* ICL-like defaults (config/ICL.yml) with a 4-slot bucket layout. */
int mh_default_params(mh_params *p);

/* HashTable / BlockArray / EntryArray / Mesh ::Resize + GeometryHelper::Init,
 * as done by the MainEngine constructor (engine/main_engine.cc:315-336). */
int mh_volume_create(const mh_params *p, mh_volume **out);
/* MainEngine::~MainEngine (engine/main_engine.cc:338-344). */
int mh_volume_destroy(mh_volume *v);
/* MainEngine::Reset (engine/main_engine.cc:347-355). */
int mh_volume_reset(mh_volume *v, void *stream);

/* Sensor::Process + Sensor::set_transform (sensor/rgbd_sensor.cu:118-137,
 * sensor/rgbd_sensor.h:47-50): takes float depth, marks depth outside
 * [min_depth_range, max_depth_range] invalid as ConvertDepthFormatKernel does
 * (sensor/preprocess.cu:25-42), resets the inlier-ratio image to 0.1
 * (preprocess.cu:10-23) and stores wTc and cTw = inverse(wTc). */
int mh_frame_set(mh_volume *v, const float *depth, int depth_on_device,
                 const float wTc[16], void *stream);
/* Same, from raw 16-bit depth scaled by range_factor (preprocess.cu:25-42,
 * whose source image is a short*): raw values are read as signed, so 32768
 * and above are negative depths and come out invalid, as in the reference. */
int mh_frame_set_u16(mh_volume *v, const uint16_t *depth, int depth_on_device,
                     const float wTc[16], void *stream);

/* AllocBlockArray (mapping/allocate.h:16-20, allocate.cu:101-125). */
int mh_allocate(mh_volume *v, void *stream);
/* CollectBlocksInFrustum (core/collect_block_array.h:26-31). */
int mh_collect_frustum(mh_volume *v, void *stream);
/* CollectAllBlocks (core/collect_block_array.h:16-19). */
int mh_collect_all(mh_volume *v, void *stream);
/* UpdateBlocksSimple (mapping/update_simple.h:21-27). */
int mh_integrate_simple(mh_volume *v, void *stream);
/* PredictOutlierRatio (mapping/update_bayesian.h:41-47). */
int mh_predict_inlier(mh_volume *v, void *stream);
/* UpdateBlocksBayesian (mapping/update_bayesian.h:33-39). */
int mh_integrate_psdf(mh_volume *v, void *stream);
/* MarchingCubes (meshing/marching_cubes.h:18-24): surfel pass, triangle pass
 * and the two recycle passes over the current candidate list. */
int mh_mesh(mh_volume *v, void *stream);
/* CollectLowSurfelBlocks (mapping/recycle.h:40-44). */
int mh_gc_low_surfel(mh_volume *v, void *stream);
/* RecycleGarbageBlockArray (mapping/recycle.h:46-50). */
int mh_gc_recycle(mh_volume *v, void *stream);
/* StarveOccupiedBlockArray (mapping/recycle.h:18-21). */
int mh_gc_starve(mh_volume *v, void *stream);
/* CollectGarbageBlockArray (mapping/recycle.h:23-27). */
int mh_gc_collect_garbage(mh_volume *v, void *stream);

/* RayCaster::Cast (visualization/ray_caster.h:37-41).  Outputs (any may be
 * NULL): depth = metric z of the hit (-inf on a miss), vertex = camera-frame
 * point (x, y, z, 1), normal = camera-frame -grad(sdf) / |grad| (x, y, z, 1);
 * misses are -inf.  Width x height = rc_width x rc_height. */
int mh_raycast(mh_volume *v, const float cTw[16], float *depth, float *vertex4,
               float *normal4, int out_on_device, void *stream);

/* Primal-dual (Chambolle-Pock) TV-L2 denoising of the current depth frame, in
 * place; invalid pixels stay invalid.  No reference counterpart: the
 * reference's only primal-dual code is volumetric (optimize/primal_dual.h). */
int mh_denoise_tv(mh_volume *v, float lambda, int iterations, void *stream);

/* Allocation-free variant of mh_denoise_tv for callers that cannot call
 * cudaMalloc: code whose device memory is owned by another allocator with a
 * fixed budget (a framework's caching allocator), or latency-critical frame
 * loops in which cudaMalloc/cudaFree would synchronise the device.  No
 * counterpart in the reference (which has no 2-D depth denoiser).
 *
 * depth_in / depth_out: device pointers, width x height float32 metres
 * (they may be the same buffer); pixels <= 0 or non-finite are invalid and
 * come out as -inf.  The nine scratch planes live in one fixed device array of
 * MH_TV_STATIC_MAX_PIXELS * 9 floats (about 11 MB), held by every GPU that
 * loads the library until the process exits; images with more than
 * MH_TV_STATIC_MAX_PIXELS pixels are rejected with MH_ERR_CAPACITY.  Each
 * call made while `stream` is not capturing looks up the array's device
 * address with the current device (a lookup, not an allocation), so a
 * cudaDeviceReset, after which the array may move, is followed; a call made
 * while the stream captures reuses the address the last such lookup found on
 * that device, so make one call on each device before any stream capture.
 * All calls share the array: each call initialises every plane it
 * reads, and calls that overlap on the GPU (other streams, other threads) race
 * on it.  Nothing is allocated or freed, on the device or the host. */
#define MH_TV_STATIC_MAX_PIXELS (640 * 480)
int mh_denoise_tv_static(const float *depth_in, float *depth_out, int width, int height, float lambda,
                         int iterations, void *stream);

/* Introspection, no reference counterpart: raycasts from cTw (outputs
 * discarded, the same march as mh_raycast) and counts the distinct blocks the
 * rays looked up and found -- the raycast's block footprint, used by the
 * byte model.  Allocates one byte per block of the pool on first use;
 * synchronises `stream`. */
int mh_raycast_footprint(mh_volume *v, const float cTw[16], int *blocks_touched, void *stream);

/* One MainEngine frame (app/reconstruction.cc:82-100): frame set, optional TV
 * denoise (tv_iterations > 0), Mapping (main_engine.cc:100-154), Meshing
 * (:156-174), raycast into the caller's buffers (may be NULL) and the
 * simple-mode Recycle (:176-192).  `outputs_on_device` applies to the raycast
 * outputs. */
int mh_integrate_frame(mh_volume *v, const float *depth, int depth_on_device,
                       const float wTc[16], int tv_iterations, float tv_lambda,
                       float *ray_depth, float *ray_vertex4, float *ray_normal4,
                       int outputs_on_device, void *stream);

/* Synchronises `stream`, then reads the counters and the sticky error word:
 * the counts the reference reads back or logs (EntryArray::count(),
 * core/entry_array.h:20; heap and mesh counters, core/hash_table.h,
 * core/mesh.h; engine/logging_engine.cc:61-93). */
int mh_stats_get(mh_volume *v, mh_stats *out, void *stream);
/* Clears the sticky error word (no counterpart: the reference exits through
 * checkCudaErrors or printf()s device-side failures). */
int mh_clear_error(mh_volume *v, void *stream);

/* Host copies of state (synchronising).  Blocks are returned in pool order:
 * pos[3n] block coordinates; sdf/weight/a/b [512n], voxel x fastest
 * (geometry/geometry_helper.h:115-131).  Any array may be NULL.  *n_out gets
 * the number of live blocks; at most max_blocks are written. */
int mh_dump_blocks(mh_volume *v, int max_blocks, int32_t *pos, float *sdf,
                   float *weight, float *a, float *b, int *n_out);
/* Overwrite the voxel state of existing blocks (same layout as the dump);
 * blocks not present are inserted.  Used to hand a state to the stages (no
 * counterpart; the reference's block replay is LoggingEngine's,
 * engine/logging_engine.cc:101-233). */
int mh_load_blocks(mh_volume *v, int n, const int32_t *pos, const float *sdf,
                   const float *weight, const float *a, const float *b);
/* Current candidate list as block coordinates pos[3n] (EntryArray,
 * core/entry_array.h:10-50, as CollectBlocksInFrustum leaves it). */
int mh_dump_candidates(mh_volume *v, int max_n, int32_t *pos, int *n_out);
/* Replace the candidate list by the given existing blocks (the reference's
 * stages read whatever EntryArray holds, core/entry_array.h:10-50). */
int mh_set_candidates(mh_volume *v, int n, const int32_t *pos);
/* Inlier-ratio image (width x height floats; SensorData::inlier_ratio,
 * sensor/rgbd_sensor.h:16-40, after PredictOutlierRatio). */
int mh_dump_inlier(mh_volume *v, float *out);
/* Current (preprocessed) depth frame (width x height floats; the depth
 * texture of SensorData after ConvertDepthFormatKernel,
 * sensor/preprocess.cu:25-42). */
int mh_dump_depth(mh_volume *v, float *out);

/* Mesh state in pool-independent form.  For every live vertex slot:
 * vkeys[4i] = (voxel x, y, z, slot) of its owner, vdata[8i] = pos xyz,
 * normal xyz, radius, ref_count (as float).  For every live triangle:
 * tkeys[13 t] = owner cube voxel (x, y, z), triangle slot index, then its
 * three vertices as (slot-owner voxel index into vkeys) ... see mesh.cu.
 * Pass NULL arrays to query counts only. */
int mh_dump_mesh(mh_volume *v, int max_vertices, int32_t *vkeys, float *vdata,
                 int max_triangles, int32_t *tris, int *n_vertices, int *n_triangles);
/* Per-voxel cube index of a block list (MeshUnit::curr_cube_idx,
 * core/voxel.h:27-60), 512 per block. */
int mh_dump_cubes(mh_volume *v, int n, const int32_t *pos, uint8_t *cube_idx);
/* Block bookkeeping for garbage collection (Block, core/block.h:15-40):
 * life_count_down, inner and boundary surfel counts; and the GC flag of each
 * candidate (EntryArray::flag, core/entry_array.h:29-31). */
int mh_dump_block_meta(mh_volume *v, int n, const int32_t *pos, int32_t *life,
                       int32_t *inner, int32_t *boundary);
int mh_dump_flags(mh_volume *v, int max_n, uint8_t *flags, int *n_out);
/* Introspection, no reference counterpart: per block (INT32_MIN if absent)
 * the count the library keeps of voxels whose sdf lies in [0, 1e30); every
 * sdf writer maintains it, and the raycast skips the trilinear gathers of
 * samples whose corner blocks all count 512. */
int mh_dump_nonneg_counts(mh_volume *v, int n, const int32_t *pos, int32_t *count);

/* Per-stage GPU time, measured with CUDA events recorded on each stage's
 * stream around its launches (the reference's per-stage Timer and logging,
 * util/timer.h, engine/logging_engine.cc:61-93).  Stage order: */
#define MH_STAGE_PREPROCESS 0
#define MH_STAGE_TV         1
#define MH_STAGE_ALLOC      2
#define MH_STAGE_COLLECT    3
#define MH_STAGE_PREDICT    4
#define MH_STAGE_INTEGRATE  5
#define MH_STAGE_MESH       6
#define MH_STAGE_GC         7
#define MH_STAGE_RAYCAST    8
#define MH_STAGE_COUNT      9
int mh_profile_enable(mh_volume *v, int enable);
/* Synchronises, returns the accumulated ms and call counts per stage since
 * the last read, and resets them. */
int mh_profile_read(mh_volume *v, double ms[MH_STAGE_COUNT], int calls[MH_STAGE_COUNT]);
/* Number of kernels this library has launched in the process (no
 * counterpart; a measurement aid). */
uint64_t mh_launch_count(void);

/* Dense copy of the mesh (CompressMesh, visualization/compress_mesh.cu:10-172):
 * the vertices referenced by live triangles (position and normal, 3 floats
 * each) and the triangles with their indices remapped, in pool order, so the
 * result does not vary between calls.  At most max_* entries are written
 * (host or device buffers per out_on_device); n_* receive the totals.
 * Allocates and frees its device staging; synchronising. */
int mh_mesh_compact(mh_volume *v, int max_vertices, float *positions3, float *normals3, int max_triangles,
                    int32_t *triangles3, int *n_vertices, int *n_triangles, int out_on_device, void *stream);
/* The dense mesh as a binary little-endian PLY file (io/mesh_writer.cc:14-150
 * writes the reference's): float x y z nx ny nz per vertex, uchar-int lists. */
int mh_write_ply(mh_volume *v, const char *path);
/* The same mesh as Wavefront OBJ text (SaveObj, io/mesh_writer.cc:14-73):
 * v, vn and 1-based "f a//a b//b c//c" lines. */
int mh_write_obj(mh_volume *v, const char *path);

/* Block checkpoint (the reference's block recording,
 * engine/logging_engine.cc:101-233): every allocated block's position and
 * voxel fields (sdf and weight; with the Bayesian update also a and b) in one
 * binary file, streamed in chunks.  Synchronising. */
int mh_save_volume(mh_volume *v, const char *path);
/* Resume: insert the file's blocks (the voxel size must match; existing blocks
 * at the same positions are overwritten).  The mesh is re-extracted by the
 * next mesh pass (e.g. mh_collect_all + mh_mesh).  n_blocks may be NULL. */
int mh_load_volume(mh_volume *v, const char *path, int *n_blocks);

/* Volumetric Huber-TV smoothing of the sdf over the current candidate blocks
 * (PrimalDualInit / PrimalDualIterate, optimize/primal_dual.cu:10-223; the
 * reference never calls them).  init records sdf0 and the per-voxel data
 * weight exp(|grad sdf| / voxel) and allocates the state on first use (32 B
 * per voxel of the block pool; pools up to 2^23 blocks, else MH_ERR_INVALID);
 * iterate runs dual + primal steps and writes
 * the smoothed sdf in place.  energy (may be NULL): [lambda/2 data + tv, data,
 * tv] before the last iteration's primal step, as the reference reports it. */
int mh_huber_tv_init(mh_volume *v, void *stream);
int mh_huber_tv_iterate(mh_volume *v, float lambda, float sigma, float tau, int iterations, double energy[3],
                        void *stream);

/* ------------------------------------------------------------------ gradients
 * Differentiable raycast.  No reference counterpart (the reference's
 * RayCaster::Cast, visualization/ray_caster.cu:16-224, is forward only).  The
 * march is re-run with the forward's code, so its discrete decisions are the
 * forward's; the derivative is taken through the two bracketing samples, the
 * three regula-falsi steps and the gradient-based normal, i.e. it is the
 * derivative of what mh_raycast computes.  Pose derivatives are for a left
 * se(3) increment wTc <- exp(xi) wTc, xi = (tx, ty, tz, wx, wy, wz).
 */
/* For L = sum_pixels dL_ddepth * depth + dL_dnormal4.xyz . normal (device
 * W x H float and W x H float4, either may be NULL): adds dL/dsdf into
 * grad_sdf (device, value_capacity x 512 floats indexed like the volume's
 * own voxel storage, NULL to skip; read it with mh_dump_block_field) and
 * writes dL/dxi (host).  Synchronising. */
int mh_raycast_backward(mh_volume *v, const float cTw[16], const float *dL_ddepth, const float *dL_dnormal4,
                        float *grad_sdf, double dL_dxi[6], void *stream);
/* No reference counterpart (the reference tracks with the point-to-PSDF
 * residual below, engine/main_engine.cc:70-98).
 * Gauss-Newton normal equations of frame-to-model alignment, driven by the
 * raycast: for every pixel with a hit, an observation (> 0, finite) and
 * |rendered - observed depth| < max_residual, the observed point on the
 * pixel's ray is compared with the tangent plane of the model at the hit
 * (normal from central sdf differences 2.5 voxels either side, at most
 * 0.8 truncation distances): r = n . (p_obs - p_hit),
 * J = dr/dxi = [n, p_obs x n] (projective point-to-plane).  The exact
 * derivative of the rendered depth (mh_raycast_backward) follows the
 * millimetre-scale bumps of a fused surface and makes a poor Gauss-Newton
 * model; the tangent plane does not.  Outputs J^T J (6 x 6 row-major),
 * J^T r, sum r^2 and the pixel count. */
int mh_raycast_normal_equations(mh_volume *v, const float cTw[16], const float *obs_depth, float max_residual,
                                double JtJ[36], double Jtr[6], double *cost, int *count, void *stream);
/* Frame-to-model pose refinement: `iterations` Gauss-Newton steps on the
 * alignment above, starting from wTc (updated in place); the residual gate
 * starts at 4 x max_residual and halves per step down to max_residual.  When a frame
 * is set, its pose becomes the refined one.  final_cost / final_count (may be
 * NULL): the residual at the returned pose. */
int mh_refine_pose(mh_volume *v, const float *obs_depth, float wTc[16], int iterations, float max_residual,
                   double *final_cost, int *final_count, void *stream);

/* The reference's tracker, MainEngine::Localizing (engine/main_engine.cc:70-98)
 * over PointToSurface (localizing/point_to_psdf.cu:19-147).  Normal
 * equations of the point-to-PSDF residual at pose wTc over the current
 * frame's pixels with odd x and y: A = sum J J^T (6 x 6 row-major),
 * b = sum D J, err = sum D^2, count; D is the trilinear sdf at the
 * frame point moved to the world, J = [grad D, p x grad D].  The reference
 * writes J[2] = dD/dx (point_to_psdf.cu:70); reference_jacobian = 1 keeps
 * that, 0 uses dD/dz.  Needs a frame (mh_frame_set). */
int mh_point_to_psdf_normal_equations(mh_volume *v, const float wTc[16], int reference_jacobian, double A[36],
                                      double b[6], double *err, int *count, void *stream);
/* `iterations` steps dxi = -(A + lambda I)^-1 b, wTc <- exp(dxi) wTc (the
 * reference uses lambda = 1e5), stopping when no pixel contributes; wTc is
 * updated in place and becomes the frame's pose.  final_err / final_count
 * (may be NULL): the sums of the last evaluated pose. */
int mh_track_point_to_psdf(mh_volume *v, float wTc[16], int iterations, float lambda, int reference_jacobian,
                           double *final_err, int *final_count, void *stream);
/* Like mh_dump_blocks for a caller's device field laid out like the voxel
 * storage (value_capacity x 512 floats), e.g. the grad_sdf above (no
 * counterpart). */
int mh_dump_block_field(mh_volume *v, const float *field, int max_blocks, int32_t *pos, float *out, int *n_out);

/* ------------------------------------------------------------------ batches
 * Many independent volumes (scenes) advanced together.  No reference
 * counterpart: the reference runs one MainEngine per process.  A step runs
 * one MainEngine frame (the mh_integrate_frame chain) for every active scene,
 * with ONE launch per stage for all scenes: the batched kernels walk a device
 * scene table and share the single-scene kernels' code, so each scene's
 * results are those of mh_integrate_frame on the same inputs.  Scenes may
 * differ in resolution, voxel size and update mode.  With use_graph the whole
 * step (table upload, depth upload, every stage) is captured once as a CUDA
 * graph and replayed; the per-step inputs travel in a double-buffered pinned
 * block, so a replay needs no re-capture.  While a volume belongs to a batch,
 * its standalone stage calls need mh_frame_set first (the batch keeps the
 * scenes' poses in its own device table).
 */
typedef struct mh_batch mh_batch;

typedef struct mh_batch_tuning {
  int ray_tile_shape;        /* raycast CTA tile: 0 = 16x8, 1 = 8x8, 2 = 32x4 */
  int integrate_cta_per_sm;  /* cap on resident CTAs per SM of the integrate grid */
} mh_batch_tuning;

/* Build a batch over `count` volumes (the caller keeps ownership and must
 * destroy the batch first).  raycast != 0 allocates per-scene raycast outputs
 * (depth W x H float, vertex and normal W x H float4) written every step. */
int mh_batch_create(mh_volume *const *volumes, int count, int raycast, mh_batch **out);
int mh_batch_destroy(mh_batch *b);
/* One frame for every scene s with active[s] != 0 (active == NULL: all):
 * depth[s] is W_s x H_s metres (device pointers if depth_on_device, else host),
 * wTc is count x 16 row-major camera-to-world poses (host). */
int mh_batch_step(mh_batch *b, const float *const *depth, int depth_on_device, const float *wTc,
                  const int *active, int tv_iterations, float tv_lambda, int use_graph, void *stream);
/* device pointers of scene s's raycast outputs (NULL where not allocated) */
int mh_batch_outputs(mh_batch *b, int scene, float **depth, float **vertex4, float **normal4);
/* copy scene s's last raycast outputs to host buffers (NULL: skipped; synchronising) */
int mh_batch_dump_raycast(mh_batch *b, int scene, float *depth, float *vertex4, float *normal4);
int mh_batch_get_tuning(mh_batch *b, mh_batch_tuning *out);
int mh_batch_set_tuning(mh_batch *b, const mh_batch_tuning *t);
/* Online autotuning: the next (raycast tile shapes x integrate CTA caps x
 * trials) steps each run one combination, timed with CUDA events around the
 * two stages it affects; then the fastest choice per stage is kept.  The
 * steps do their normal work (launch shapes do not change results). */
int mh_batch_autotune(mh_batch *b, int trials);
/* ms per step of the integrate and raycast stages measured by the autotuner
 * for each choice (3 shapes, 3 caps), -1 where not measured */
int mh_batch_tuning_times(mh_batch *b, double ray_ms[3], double integrate_ms[3]);
/* ms per step of each stage (MH_STAGE_*) averaged over the autotuning steps,
 * -1 before any; the raycast entry covers the raycast only */
int mh_batch_stage_times(mh_batch *b, double ms[MH_STAGE_COUNT]);

/* Teschner hash of a block position (HashBucketForBlockPos,
 * core/hash_table.h:259-269). */
uint32_t mh_hash_bucket(int32_t x, int32_t y, int32_t z, uint32_t bucket_count);
/* Bytes the last frame's stages needed by the algorithmic model (no
 * counterpart; a measurement aid): the voxel fields and image pixels each
 * stage must read and write for the blocks and pixels it visited, per stage
 * [alloc, collect, integrate, predict, mesh, raycast]. */
int mh_bytes_model(mh_volume *v, double out[6]);

#ifdef __cplusplus
}
#endif
#endif /* MESHHASH_H */
