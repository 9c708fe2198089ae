"""ctypes mirror of include/meshhash.h (structs and status codes)."""
import ctypes as C

MH_OK, MH_ERR_INVALID, MH_ERR_CUDA, MH_ERR_CAPACITY, MH_ERR_TIMEOUT, MH_ERR_NOMEM, MH_ERR_STATE = range(7)
STATUS_NAMES = {0: "MH_OK", 1: "MH_ERR_INVALID", 2: "MH_ERR_CUDA", 3: "MH_ERR_CAPACITY",
                4: "MH_ERR_TIMEOUT", 5: "MH_ERR_NOMEM", 6: "MH_ERR_STATE"}

_u32, _f32, _i32 = C.c_uint32, C.c_float, C.c_int32


class MhParams(C.Structure):
    _fields_ = [
        ("bucket_count", _u32), ("bucket_size", _u32), ("entry_count", _u32),
        ("linked_list_size", _u32), ("value_capacity", _u32),
        ("max_vertex_count", _u32), ("max_triangle_count", _u32),
        ("voxel_size", _f32), ("truncation_distance_scale", _f32), ("truncation_distance", _f32),
        ("sdf_upper_bound", _f32), ("weight_sample", _u32), ("weight_upper_bound", _u32),
        ("fx", _f32), ("fy", _f32), ("cx", _f32), ("cy", _f32),
        ("width", _u32), ("height", _u32),
        ("min_depth_range", _f32), ("max_depth_range", _f32), ("range_factor", _f32),
        ("rc_fx", _f32), ("rc_fy", _f32), ("rc_cx", _f32), ("rc_cy", _f32),
        ("rc_width", _u32), ("rc_height", _u32),
        ("min_raycast_depth", _f32), ("max_raycast_depth", _f32), ("raycast_step", _f32),
        ("sample_sdf_threshold", _f32), ("sdf_threshold", _f32), ("enable_gradients", _i32),
        ("enable_bayesian_update", _i32), ("enable_sdf_gradient", _i32),
        ("overflow_capacity", _u32), ("mesh_page_capacity", _u32), ("compat_arithmetic", _i32),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class MhStats(C.Structure):
    _fields_ = [(n, _u32) for n in (
        "error", "blocks_allocated", "block_high_water", "candidates", "vertices_allocated",
        "triangles_allocated", "overflow_used", "frames", "dropped_inserts", "gc_freed_blocks",
        "mesh_passes")] + [(n, C.c_uint64) for n in (
        "candidate_sum", "vertex_work_sum", "cube_blocks_sum", "mesh_list_sum", "predict_blocks_sum")] + [
        ("mesh_pages_used", _u32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class MhBatchTuning(C.Structure):
    """mh_batch_tuning (include/meshhash.h)."""
    _fields_ = [("ray_tile_shape", C.c_int32), ("integrate_cta_per_sm", C.c_int32)]
