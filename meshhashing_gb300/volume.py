"""Host-side mirror of MeshHashing's engine API over the C ABI.

``Volume`` plays the role of ``MainEngine`` (engine/main_engine.h:21-100):
it owns the hash table, block pool, candidate list and mesh pools, and
exposes the reference's stage functions under their reference names
(``alloc_block_array`` = AllocBlockArray, ``update_blocks_bayesian`` =
UpdateBlocksBayesian, ...).  Every call goes through libmeshhash.so; the
stages are asynchronous on the volume's CUDA stream (``stream`` is a
``cudaStream_t`` as an int, 0 = legacy default stream) and device-side
failures surface through ``stats()['error']``.

Arrays: host inputs are numpy arrays; device inputs/outputs are given as
integer device pointers or objects with ``data_ptr()`` (e.g. torch CUDA
tensors), which is how PyTorch serves as plumbing for device memory.  The C
side trusts the pointers it gets, so the frame, raycast and gradient buffers
given as arrays or tensors are checked here for size, float32 type, layout
and device (ValueError); raw integer pointers are taken as given.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _lib
from ._abi import MhParams, MhStats


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _ptr(a, ct=C.c_float):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(ct))


def _hptr(x):
    """Host buffer pointer: numpy arrays or CPU tensors (e.g. pinned torch tensors)."""
    if x is None:
        return None
    if hasattr(x, "data_ptr"):
        return C.c_void_p(x.data_ptr())
    return x.ctypes.data_as(C.c_void_p)


def _dev(x):
    if x is None:
        return None
    if hasattr(x, "data_ptr"):
        return C.c_void_p(x.data_ptr())
    return C.c_void_p(int(x))


def _check_tensor(x, n, what, cuda):
    """A torch tensor handed to the library as a buffer of n float32 values:
    the C side trusts the pointer, so size, type, layout and device are
    checked here (raw integer pointers cannot be)."""
    if str(x.dtype) != "torch.float32":
        raise ValueError(f"{what}: expected a float32 tensor, got {x.dtype}")
    if x.numel() != n:
        raise ValueError(f"{what}: expected {n} values, got {x.numel()}")
    if not x.is_contiguous():
        raise ValueError(f"{what}: tensor must be contiguous")
    if bool(x.is_cuda) != cuda:
        raise ValueError(f"{what}: expected a {'CUDA' if cuda else 'host'} tensor")


def _dev_buf(x, n, what):
    """Device buffer of n float32 values: a CUDA tensor (checked) or an
    integer device pointer (taken as given)."""
    if x is not None and hasattr(x, "data_ptr"):
        _check_tensor(x, n, what, cuda=True)
    return _dev(x)


def _host_out(x, n, what):
    """Host output buffer of n float32 values: a numpy array or a CPU tensor."""
    if x is None:
        return None
    if hasattr(x, "data_ptr"):
        _check_tensor(x, n, what, cuda=False)
        return C.c_void_p(x.data_ptr())
    if not isinstance(x, np.ndarray) or x.dtype != np.float32 or x.size != n or not x.flags.c_contiguous \
            or not x.flags.writeable:
        raise ValueError(f"{what}: expected a writable C-contiguous float32 array of {n} values")
    return x.ctypes.data_as(C.c_void_p)


def default_params() -> MhParams:
    p = MhParams()
    _lib.check("mh_default_params", _lib.load().mh_default_params(C.byref(p)))
    return p


def launch_count() -> int:
    """Kernels launched by libmeshhash.so in this process."""
    return int(_lib.load().mh_launch_count())


def hash_bucket(x, y, z, bucket_count) -> int:
    """HashTable::HashBucketForBlockPos (core/hash_table.h:259-269)."""
    return int(_lib.load().mh_hash_bucket(int(x), int(y), int(z), int(bucket_count)))


class Volume:
    def __init__(self, params: MhParams, stream: int = 0):
        self.L = _lib.load()
        self.params = params
        self.stream = C.c_void_p(int(stream))
        self.h = C.c_void_p()
        _lib.check("mh_volume_create", self.L.mh_volume_create(C.byref(params), C.byref(self.h)))
        self.W, self.H = params.width, params.height
        self.RW, self.RH = params.rc_width, params.rc_height

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.L.mh_volume_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _c(self, name, *args):
        _lib.check(name, getattr(self.L, name)(self.h, *args))

    # ---------------------------------------------------------- lifecycle / input
    def reset(self):
        self._c("mh_volume_reset", self.stream)

    def set_frame(self, depth, wTc, on_device: bool = False):
        """Sensor::Process + Sensor::set_transform."""
        m = _f32(wTc).reshape(16)
        if on_device:
            self._c("mh_frame_set", _dev_buf(depth, self.W * self.H, "depth"), 1, _ptr(m), self.stream)
        else:
            d = _f32(depth).reshape(-1)
            if d.size != self.W * self.H:
                raise ValueError(f"depth: expected {self.W * self.H} values, got {d.size}")
            self._c("mh_frame_set", d.ctypes.data_as(C.c_void_p), 0, _ptr(m), self.stream)

    def set_frame_u16(self, depth, wTc):
        d = np.ascontiguousarray(depth, np.uint16).reshape(-1)
        if d.size != self.W * self.H:
            raise ValueError(f"depth: expected {self.W * self.H} values, got {d.size}")
        m = _f32(wTc).reshape(16)
        self._c("mh_frame_set_u16", d.ctypes.data_as(C.c_void_p), 0, _ptr(m), self.stream)

    # ---------------------------------------------------------- reference stages
    def alloc_block_array(self):
        self._c("mh_allocate", self.stream)

    def collect_blocks_in_frustum(self):
        self._c("mh_collect_frustum", self.stream)

    def collect_all_blocks(self):
        self._c("mh_collect_all", self.stream)

    def update_blocks_simple(self):
        self._c("mh_integrate_simple", self.stream)

    def predict_outlier_ratio(self):
        self._c("mh_predict_inlier", self.stream)

    def update_blocks_bayesian(self):
        self._c("mh_integrate_psdf", self.stream)

    def marching_cubes(self):
        self._c("mh_mesh", self.stream)

    def collect_low_surfel_blocks(self):
        self._c("mh_gc_low_surfel", self.stream)

    def recycle_garbage_block_array(self):
        self._c("mh_gc_recycle", self.stream)

    def starve_occupied_block_array(self):
        self._c("mh_gc_starve", self.stream)

    def collect_garbage_block_array(self):
        self._c("mh_gc_collect_garbage", self.stream)

    def denoise_tv(self, lam: float = 0.1, iterations: int = 20):
        self._c("mh_denoise_tv", C.c_float(lam), int(iterations), self.stream)

    def raycast(self, cTw, depth_out=None, vertex_out=None, normal_out=None):
        """RayCaster::Cast.  Without outputs given, returns host arrays
        (depth (H, W), vertex (H, W, 4), normal (H, W, 4)); with device
        outputs (pointers / tensors) writes them on the device."""
        m = _f32(cTw).reshape(16)
        if depth_out is None and vertex_out is None and normal_out is None:
            d = np.empty(self.RW * self.RH, np.float32)
            v = np.empty(self.RW * self.RH * 4, np.float32)
            n = np.empty(self.RW * self.RH * 4, np.float32)
            self._c("mh_raycast", _ptr(m), d.ctypes.data_as(C.c_void_p), v.ctypes.data_as(C.c_void_p),
                    n.ctypes.data_as(C.c_void_p), 0, self.stream)
            return d.reshape(self.RH, self.RW), v.reshape(self.RH, self.RW, 4), n.reshape(self.RH, self.RW, 4)
        n = self.RW * self.RH
        self._c("mh_raycast", _ptr(m), _dev_buf(depth_out, n, "depth_out"), _dev_buf(vertex_out, 4 * n, "vertex_out"),
                _dev_buf(normal_out, 4 * n, "normal_out"), 1, self.stream)
        return None

    def raycast_footprint(self, cTw) -> int:
        """Distinct blocks the raycast from cTw looks up and finds (its block
        footprint); the outputs are discarded."""
        m = _f32(cTw).reshape(16)
        n = C.c_int32(0)
        self._c("mh_raycast_footprint", _ptr(m), C.byref(n), self.stream)
        return n.value

    # ---------------------------------------------------------- mesh export
    def compact_mesh(self):
        """(positions (V, 3), normals (V, 3), triangles (T, 3) int32): the
        dense mesh in pool order."""
        nv, nt = C.c_int32(), C.c_int32()
        self._c("mh_mesh_compact", 0, None, None, 0, None, C.byref(nv), C.byref(nt), 0, self.stream)
        V, T = nv.value, nt.value
        pos = np.zeros((max(V, 1), 3), np.float32)
        nrm = np.zeros((max(V, 1), 3), np.float32)
        tri = np.zeros((max(T, 1), 3), np.int32)
        self._c("mh_mesh_compact", V, pos.ctypes.data_as(C.c_void_p), nrm.ctypes.data_as(C.c_void_p), T,
                tri.ctypes.data_as(C.c_void_p), C.byref(nv), C.byref(nt), 0, self.stream)
        return pos[:V], nrm[:V], tri[:T]

    def write_ply(self, path: str):
        self._c("mh_write_ply", str(path).encode())

    def write_obj(self, path: str):
        self._c("mh_write_obj", str(path).encode())

    def save(self, path: str):
        """Block checkpoint (positions and voxel fields) to a file."""
        self._c("mh_save_volume", str(path).encode())

    def load(self, path: str) -> int:
        """Insert a checkpoint's blocks; returns their count."""
        n = C.c_int32()
        self._c("mh_load_volume", str(path).encode(), C.byref(n))
        return n.value

    # ---------------------------------------------------------- Huber-TV
    def huber_tv_init(self):
        """Record sdf0 and the data weights over the current candidate blocks
        (PrimalDualInit, optimize/primal_dual.cu:15-40)."""
        self._c("mh_huber_tv_init", self.stream)

    def huber_tv_iterate(self, lam: float, sigma: float, tau: float, iterations: int = 1) -> np.ndarray:
        """Primal-dual Huber-TV steps on the sdf in place (PrimalDualIterate,
        optimize/primal_dual.cu:176-223).  Returns [lam/2 data + tv, data, tv]
        of the last iteration's dual pass."""
        e = (C.c_double * 3)()
        self._c("mh_huber_tv_iterate", float(lam), float(sigma), float(tau), int(iterations), e, self.stream)
        return np.array(list(e))

    # ---------------------------------------------------------- gradients
    def raycast_backward(self, cTw, dL_ddepth, dL_dnormal=None, grad_sdf=None):
        """dL/dxi (left se(3) increment of wTc, translation first) for
        L = sum dL_ddepth * depth + dL_dnormal[..., :3] . normal of the raycast
        from cTw; dL_ddepth (H, W) and dL_dnormal (H, W, 4) are CUDA tensors or
        device pointers.  grad_sdf (a CUDA tensor of value_capacity * 512
        floats, laid out like the voxel storage) receives dL/dsdf added in."""
        m = _f32(cTw).reshape(16)
        xi = (C.c_double * 6)()
        n = self.RW * self.RH
        self._c("mh_raycast_backward", _ptr(m), _dev_buf(dL_ddepth, n, "dL_ddepth"),
                _dev_buf(dL_dnormal, 4 * n, "dL_dnormal"),
                _dev_buf(grad_sdf, self.params.value_capacity * 512, "grad_sdf"), xi, self.stream)
        return np.array(list(xi))

    def normal_equations(self, cTw, obs_depth=None, max_residual: float = 0.1):
        """(J^T J (6, 6), J^T r (6,), sum r^2, count) of r = rendered - observed
        depth; obs_depth a CUDA tensor / device pointer, or None for the frame's."""
        m = _f32(cTw).reshape(16)
        A = (C.c_double * 36)()
        b = (C.c_double * 6)()
        cost = C.c_double()
        cnt = C.c_int32()
        self._c("mh_raycast_normal_equations", _ptr(m), _dev_buf(obs_depth, self.RW * self.RH, "obs_depth"),
                C.c_float(max_residual), A, b, C.byref(cost), C.byref(cnt), self.stream)
        return np.array(list(A)).reshape(6, 6), np.array(list(b)), cost.value, cnt.value

    def refine_pose(self, wTc, iterations: int = 10, obs_depth=None, max_residual: float = 0.1):
        """Gauss-Newton frame-to-model refinement; returns (wTc, cost, count)."""
        m = np.ascontiguousarray(np.asarray(wTc, np.float32).reshape(16))
        cost = C.c_double()
        cnt = C.c_int32()
        self._c("mh_refine_pose", _dev_buf(obs_depth, self.RW * self.RH, "obs_depth"), _ptr(m), int(iterations),
                C.c_float(max_residual), C.byref(cost), C.byref(cnt), self.stream)
        return m.reshape(4, 4), cost.value, cnt.value

    def point_to_psdf(self, wTc, reference_jacobian: bool = False):
        """Normal equations of the reference's point-to-PSDF tracker at wTc
        over the current frame: (A[6, 6], b[6], err, count)."""
        m = _f32(wTc).reshape(16)
        A, b, e, n = (C.c_double * 36)(), (C.c_double * 6)(), C.c_double(), C.c_int32()
        self._c("mh_point_to_psdf_normal_equations", _ptr(m), 1 if reference_jacobian else 0, A, b, C.byref(e),
                C.byref(n), self.stream)
        return np.array(list(A)).reshape(6, 6), np.array(list(b)), e.value, n.value

    def track_point_to_psdf(self, wTc, iterations: int = 10, lam: float = 1e5, reference_jacobian: bool = False):
        """The reference's tracker (MainEngine::Localizing): returns the
        tracked pose, the last sum of squared sdf and its point count; the
        pose becomes the frame's."""
        m = _f32(wTc).reshape(16).copy()
        e, n = C.c_double(), C.c_int32()
        self._c("mh_track_point_to_psdf", _ptr(m), int(iterations), C.c_float(lam), 1 if reference_jacobian else 0,
                C.byref(e), C.byref(n), self.stream)
        return m.reshape(4, 4).astype(np.float64), e.value, n.value

    def dump_block_field(self, field):
        """(positions, rows) of a device per-voxel field laid out like the
        voxel storage (e.g. the grad_sdf of raycast_backward)."""
        n = C.c_int32()
        fp = _dev_buf(field, self.params.value_capacity * 512, "field")
        self._c("mh_dump_block_field", fp, 0, None, None, C.byref(n))
        cnt = n.value
        pos = np.zeros((max(cnt, 1), 3), np.int32)
        out = np.zeros((max(cnt, 1), 512), np.float32)
        self._c("mh_dump_block_field", fp, cnt, _ptr(pos, C.c_int32), _ptr(out), C.byref(n))
        return pos[:cnt], out[:cnt]

    def integrate_frame(self, depth, wTc, on_device: bool = False, tv_iterations: int = 0, tv_lambda: float = 0.1,
                        ray_depth=None, ray_vertex=None, ray_normal=None, outputs_on_device: bool = False):
        """One MainEngine frame: Mapping, Meshing, raycast, Recycle."""
        m = _f32(wTc).reshape(16)
        npx, nray = self.W * self.H, self.RW * self.RH
        if on_device:
            dp = _dev_buf(depth, npx, "depth")
        elif hasattr(depth, "data_ptr"):
            _check_tensor(depth, npx, "depth", cuda=False)
            dp = _hptr(depth)
        else:
            d = _f32(depth).reshape(-1)
            if d.size != npx:
                raise ValueError(f"depth: expected {npx} values, got {d.size}")
            dp = d.ctypes.data_as(C.c_void_p)
        conv = _dev_buf if outputs_on_device else _host_out
        self._c("mh_integrate_frame", dp, 1 if on_device else 0, _ptr(m), int(tv_iterations), C.c_float(tv_lambda),
                conv(ray_depth, nray, "ray_depth"), conv(ray_vertex, 4 * nray, "ray_vertex"),
                conv(ray_normal, 4 * nray, "ray_normal"), 1 if outputs_on_device else 0, self.stream)

    # ---------------------------------------------------------- introspection
    def stats(self) -> dict:
        s = MhStats()
        self._c("mh_stats_get", C.byref(s), self.stream)
        return s.as_dict()

    def clear_error(self):
        self._c("mh_clear_error", self.stream)

    def dump_blocks(self, fields=("sdf", "w", "a", "b")):
        """All live blocks: (pos[n, 3], {field: [n, 512]}) in pool order."""
        n = C.c_int32(0)
        self._c("mh_dump_blocks", 0, None, None, None, None, None, C.byref(n))
        cnt = n.value
        pos = np.zeros((max(cnt, 1), 3), np.int32)
        arrs = {f: np.zeros((max(cnt, 1), 512), np.float32) for f in fields}
        self._c("mh_dump_blocks", cnt, _ptr(pos, C.c_int32), *[_ptr(arrs.get(f)) for f in ("sdf", "w", "a", "b")],
                C.byref(n))
        return pos[:cnt], {f: a[:cnt] for f, a in arrs.items()}

    def load_blocks(self, pos, sdf=None, w=None, a=None, b=None):
        pos = _i32(pos).reshape(-1, 3)
        n = len(pos)
        conv = [None if x is None else _f32(x).reshape(n, 512) for x in (sdf, w, a, b)]
        self._c("mh_load_blocks", n, _ptr(pos, C.c_int32), *[_ptr(x) for x in conv])

    def candidates(self):
        n = C.c_int32(0)
        self._c("mh_dump_candidates", 0, None, C.byref(n))
        pos = np.zeros((max(n.value, 1), 3), np.int32)
        cnt = n.value
        self._c("mh_dump_candidates", cnt, _ptr(pos, C.c_int32), C.byref(n))
        return pos[:cnt]

    def set_candidates(self, pos):
        pos = _i32(pos).reshape(-1, 3)
        self._c("mh_set_candidates", len(pos), _ptr(pos, C.c_int32))

    def inlier(self):
        out = np.empty(self.W * self.H, np.float32)
        self._c("mh_dump_inlier", _ptr(out))
        return out.reshape(self.H, self.W)

    def depth(self):
        out = np.empty(self.W * self.H, np.float32)
        self._c("mh_dump_depth", _ptr(out))
        return out.reshape(self.H, self.W)

    def dump_mesh(self):
        """(vkeys[n, 4] = owner voxel xyz + slot, vdata[n, 8] = pos, normal,
        radius, ref_count, tris[t, 7] = cube voxel xyz, slot, 3 vertex indices)."""
        nv, nt = C.c_int32(0), C.c_int32(0)
        self._c("mh_dump_mesh", 0, None, None, 0, None, C.byref(nv), C.byref(nt))
        vk = np.zeros((max(nv.value, 1), 4), np.int32)
        vd = np.zeros((max(nv.value, 1), 8), np.float32)
        tr = np.zeros((max(nt.value, 1), 7), np.int32)
        a, b = nv.value, nt.value
        self._c("mh_dump_mesh", a, _ptr(vk, C.c_int32), _ptr(vd), b, _ptr(tr, C.c_int32), C.byref(nv), C.byref(nt))
        return vk[:a], vd[:a], tr[:b]

    def cubes(self, pos):
        pos = _i32(pos).reshape(-1, 3)
        out = np.zeros((len(pos), 512), np.uint8)
        self._c("mh_dump_cubes", len(pos), _ptr(pos, C.c_int32), _ptr(out, C.c_uint8))
        return out

    def block_meta(self, pos):
        pos = _i32(pos).reshape(-1, 3)
        n = len(pos)
        life, inner, bnd = (np.zeros(n, np.int32) for _ in range(3))
        self._c("mh_dump_block_meta", n, _ptr(pos, C.c_int32), _ptr(life, C.c_int32), _ptr(inner, C.c_int32),
                _ptr(bnd, C.c_int32))
        return life, inner, bnd

    def nonneg_counts(self, pos):
        """Per block: the library's count of voxels with sdf in [0, 1e30)."""
        pos = _i32(pos).reshape(-1, 3)
        out = np.zeros(len(pos), np.int32)
        self._c("mh_dump_nonneg_counts", len(pos), _ptr(pos, C.c_int32), _ptr(out, C.c_int32))
        return out

    def flags(self):
        n = C.c_int32(0)
        self._c("mh_dump_flags", 0, None, C.byref(n))
        out = np.zeros(max(n.value, 1), np.uint8)
        cnt = n.value
        self._c("mh_dump_flags", cnt, _ptr(out, C.c_uint8), C.byref(n))
        return out[:cnt]

    STAGES = ("preprocess", "tv", "alloc", "collect", "predict", "integrate", "mesh", "gc", "raycast")

    def profile(self, enable: bool = True):
        self._c("mh_profile_enable", 1 if enable else 0)

    def profile_read(self):
        """{stage: (ms, calls)} since the last read (synchronising)."""
        ms = (C.c_double * 9)()
        calls = (C.c_int32 * 9)()
        self._c("mh_profile_read", ms, calls)
        return {k: (ms[i], calls[i]) for i, k in enumerate(self.STAGES)}

    def bytes_model(self):
        out = (C.c_double * 6)()
        self._c("mh_bytes_model", out)
        return dict(zip(("alloc", "collect", "integrate", "predict", "mesh", "raycast"), list(out)))
