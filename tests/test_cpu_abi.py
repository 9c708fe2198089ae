"""C-ABI host logic that runs without a GPU: mh_volume_create refuses every
invalid parameter before touching the device (MH_ERR_INVALID, no handle),
argument checks of the other entry points, and mh_hash_bucket against the
Teschner hash (core/hash_table.h:259-269) restated in numpy."""
import ctypes as C

import numpy as np
import pytest

from meshhashing_gb300 import _lib
from meshhashing_gb300._abi import MhParams

MH_ERR_INVALID = 1


def _params(**over):
    L = _lib.load()
    p = MhParams()
    L.mh_default_params(C.byref(p))
    for k, v in over.items():
        setattr(p, k, v)
    return p


@pytest.mark.parametrize("over", [
    dict(bucket_count=0), dict(bucket_count=1000), dict(bucket_size=5), dict(value_capacity=0),
    dict(value_capacity=20_000_000), dict(max_vertex_count=1), dict(max_triangle_count=0),
    dict(width=0), dict(rc_height=0), dict(voxel_size=0.0), dict(voxel_size=-0.004), dict(voxel_size=float("nan")),
    dict(overflow_capacity=0), dict(raycast_step=0.0), dict(raycast_step=1e-7),
    dict(min_raycast_depth=0.0), dict(min_raycast_depth=6.0), dict(linked_list_size=4096),
    dict(mesh_page_capacity=0), dict(value_capacity=1000, mesh_page_capacity=2000),
])
def test_volume_create_refuses_invalid_parameters(built, over):
    L = _lib.load()
    v = C.c_void_p(12345)
    assert L.mh_volume_create(C.byref(_params(**over)), C.byref(v)) == MH_ERR_INVALID
    assert not v.value


def test_null_arguments_are_refused(built):
    L = _lib.load()
    v = C.c_void_p()
    assert L.mh_volume_create(None, C.byref(v)) == MH_ERR_INVALID
    assert L.mh_volume_create(C.byref(_params()), None) == MH_ERR_INVALID
    for name, args in (("mh_huber_tv_init", (None, None)),
                       ("mh_write_ply", (None, b"x.ply")), ("mh_write_obj", (None, b"x.obj")),
                       ("mh_track_point_to_psdf", (None, None, 1, C.c_float(1.0), 0, None, None, None))):
        assert getattr(L, name)(*args) == MH_ERR_INVALID, name


def test_hash_bucket_matches_teschner():
    L = _lib.load()
    rng = np.random.default_rng(9)
    xyz = rng.integers(-(1 << 20), 1 << 20, size=(2000, 3)).astype(np.int64)
    for bits in (10, 18, 21):
        n = 1 << bits
        u = lambda a: (a & 0xFFFFFFFF).astype(np.uint64)  # noqa: E731  (int32 wrap-around)
        h = ((u(xyz[:, 0]) * 73856093) & 0xFFFFFFFF) ^ ((u(xyz[:, 1]) * 19349669) & 0xFFFFFFFF) ^ \
            ((u(xyz[:, 2]) * 83492791) & 0xFFFFFFFF)
        want = h % n
        got = np.array([L.mh_hash_bucket(int(x), int(y), int(z), n) for x, y, z in xyz], np.uint64)
        np.testing.assert_array_equal(got, want)
