"""Volume parameters of the fusion workloads (restating core/params.h fields).

Values the reference leaves to per-dataset YAML (config/ICL.yml) are taken
from there: depth range [0.5, 4.0] m, sdf_upper_bound 4 m, raycast depth range
[0.5, 5.5] m, sample/sdf thresholds 0.808/0.800.  The raycast step follows the
reference's own rule of 0.8 x truncation (core/params.h:50).
"""
from ._abi import MhParams


def make_params(width, height, fx, fy, cx, cy, voxel_size, truncation, bayesian,
                bucket_count, value_capacity, weight_sample=10, max_vertex_count=1 << 22,
                max_triangle_count=1 << 22, overflow_capacity=None, raycast_step=None,
                linked_list_size=7, mesh_page_capacity=None, compat_arithmetic=0) -> MhParams:
    p = MhParams()
    p.bucket_count = bucket_count
    p.bucket_size = 4
    p.entry_count = bucket_count * 4
    p.linked_list_size = linked_list_size
    p.value_capacity = value_capacity
    p.max_vertex_count = max_vertex_count
    p.max_triangle_count = max_triangle_count
    p.voxel_size = voxel_size
    p.truncation_distance_scale = 0.0
    p.truncation_distance = truncation
    p.sdf_upper_bound = 4.0
    p.weight_sample = weight_sample
    p.weight_upper_bound = 255
    p.fx, p.fy, p.cx, p.cy = fx, fy, cx, cy
    p.width, p.height = width, height
    p.min_depth_range, p.max_depth_range = 0.5, 4.0
    p.range_factor = 0.0002
    p.rc_fx, p.rc_fy, p.rc_cx, p.rc_cy = fx, fy, cx, cy
    p.rc_width, p.rc_height = width, height
    p.min_raycast_depth, p.max_raycast_depth = 0.5, 5.5
    p.raycast_step = raycast_step if raycast_step is not None else 0.8 * truncation
    p.sample_sdf_threshold, p.sdf_threshold = 0.808, 0.800
    p.enable_gradients = 1
    p.enable_bayesian_update = 1 if bayesian else 0
    p.enable_sdf_gradient = 1
    p.overflow_capacity = overflow_capacity if overflow_capacity is not None else max(bucket_count // 4, 1024)
    p.compat_arithmetic = compat_arithmetic
    p.mesh_page_capacity = (mesh_page_capacity if mesh_page_capacity is not None
                            else max(min(value_capacity, 1 << 20) // 2, min(value_capacity, 1024)))
    return p


def params_for(workload, **over) -> MhParams:
    """Parameters of a scene.Workload by name."""
    cam = workload.camera
    if workload.name.endswith("_circle"):
        # plain TSDF: 8 mm voxels, truncation 3 voxels, 2^18 x 4 hash, simple update;
        # weight_sample raised so the MC weight gate (1/voxel^2) is reachable
        kw = dict(voxel_size=0.008, truncation=0.024, bayesian=False, bucket_count=1 << 18,
                  value_capacity=1 << 17, weight_sample=200)
    else:
        # PSDF: 4 mm voxels, truncation 12 mm, 2^21 buckets
        kw = dict(voxel_size=0.004, truncation=0.012, bayesian=True, bucket_count=1 << 21,
                  value_capacity=1 << 20)
    kw.update(over)
    return make_params(cam.width, cam.height, cam.fx, cam.fy, cam.cx, cam.cy, **kw)
