"""TEST INFRASTRUCTURE ONLY: ctypes wrapper of the CPU oracle (liboracle.so).

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
checker; the product never imports it.  ``Oracle(params, fp64=True)`` is the
FP64 restatement of the reference's update rules, ``fp64=False`` the
FP32-faithful one (same operation order, IEEE single, no FMA contraction).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
SRC = os.path.join(HERE, "mh_oracle.cpp")


def build(force: bool = False) -> str:
    """Compile liboracle.so with g++ (OpenMP, no FMA contraction)."""
    deps = [SRC, os.path.join(HERE, "..", "meshhashing_gb300", "csrc", "mc_cases.inc"),
            os.path.join(HERE, "..", "meshhashing_gb300", "csrc", "mh_exp.h"),
            os.path.join(HERE, "..", "include", "meshhash.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
           "-fPIC", "-shared", "-o", LIB + ".tmp", SRC]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        vp, i32p, f32p, u8p = C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_float), C.POINTER(C.c_uint8)
        L.orc_create.restype = vp
        L.orc_create.argtypes = [vp, C.c_int]
        L.orc_destroy.argtypes = [vp]
        L.orc_hash_bucket.restype = C.c_uint32
        L.orc_hash_bucket.argtypes = [C.c_int, C.c_int, C.c_int, C.c_uint32]
        for name in ("orc_frame_set",):
            getattr(L, name).argtypes = [vp, f32p, f32p]
        L.orc_inverse.argtypes = [f32p, f32p]
        L.orc_allocate.restype = C.c_int
        L.orc_allocate.argtypes = [vp]
        L.orc_get_touched.restype = C.c_int
        L.orc_get_touched.argtypes = [vp, i32p, C.c_int]
        for name in ("orc_collect_frustum", "orc_collect_all", "orc_block_count"):
            getattr(L, name).restype = C.c_int
            getattr(L, name).argtypes = [vp]
        L.orc_get_candidates.restype = C.c_int
        L.orc_get_candidates.argtypes = [vp, i32p, C.c_int]
        L.orc_set_candidates.restype = C.c_int
        L.orc_set_candidates.argtypes = [vp, C.c_int, i32p]
        L.orc_get_blocks.restype = C.c_int
        L.orc_get_blocks.argtypes = [vp, C.c_int, i32p, f32p, f32p, f32p, f32p]
        L.orc_set_blocks.argtypes = [vp, C.c_int, i32p, f32p, f32p, f32p, f32p]
        for name in ("orc_integrate_simple", "orc_predict_inlier", "orc_integrate_psdf", "orc_mesh",
                     "orc_gc_low_surfel", "orc_gc_starve", "orc_gc_collect_garbage"):
            getattr(L, name).argtypes = [vp]
        L.orc_gc_recycle.restype = C.c_int
        L.orc_gc_recycle.argtypes = [vp]
        L.orc_get_inlier.argtypes = [vp, f32p]
        L.orc_set_inlier.argtypes = [vp, f32p]
        L.orc_dump_mesh.argtypes = [vp, C.c_int, i32p, f32p, C.c_int, i32p, i32p, i32p]
        L.orc_load_mesh.argtypes = [vp, C.c_int, i32p, f32p, C.c_int, i32p]
        L.orc_get_cubes.argtypes = [vp, C.c_int, i32p, u8p]
        L.orc_set_cubes.argtypes = [vp, C.c_int, i32p, u8p]
        L.orc_get_block_meta.argtypes = [vp, C.c_int, i32p, i32p, i32p, i32p, u8p]
        L.orc_set_block_meta.argtypes = [vp, C.c_int, i32p, i32p, i32p, i32p]
        L.orc_raycast.argtypes = [vp, f32p, f32p, f32p, f32p]
        L.orc_frame.argtypes = [vp, f32p, f32p, C.c_int, C.c_float, f32p, f32p, f32p]
        L.orc_denoise_tv.argtypes = [vp, C.c_float, C.c_int]
        L.orc_get_depth.argtypes = [vp, f32p]
        L.orc_set_depth.argtypes = [vp, f32p]
        L.orc_expf.argtypes = [C.c_int, f32p, f32p]
        L.orc_huber_init.argtypes = [vp]
        L.orc_point_to_psdf.argtypes = [vp, f32p, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                        C.POINTER(C.c_double), i32p]
        L.orc_huber_iterate.argtypes = [vp, C.c_float, C.c_float, C.c_float, C.c_int, C.POINTER(C.c_double)]
        L.orc_debug_ray.argtypes = [vp, f32p, C.c_int, C.c_int, C.POINTER(C.c_double)]
        L.orc_raycast_backward.argtypes = [vp, f32p, f32p, f32p, C.POINTER(C.c_double)]
        L.orc_grad_blocks.restype = C.c_int
        L.orc_grad_blocks.argtypes = [vp, C.c_int, i32p, C.POINTER(C.c_double)]
        L.orc_trace.argtypes = [vp, f32p, i32p]
        L.orc_num_threads.restype = C.c_int
        L.orc_set_threads.argtypes = [C.c_int]
        _lib = L
    return _lib


def _p(a, ct):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(ct))


def f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def hash_bucket(x, y, z, bucket_count):
    return lib().orc_hash_bucket(int(x), int(y), int(z), int(bucket_count))


def inverse(m):
    m = f32(m).reshape(16)
    out = np.zeros(16, np.float32)
    lib().orc_inverse(_p(m, C.c_float), _p(out, C.c_float))
    return out.reshape(4, 4)


def expf(x):
    """The library's single-precision exp (mh_exp.h) evaluated on the CPU."""
    x = f32(x).reshape(-1)
    out = np.empty_like(x)
    lib().orc_expf(x.size, _p(x, C.c_float), _p(out, C.c_float))
    return out


def convert_depth_u16(raw, range_factor, min_depth, max_depth):
    """ConvertDepthFormatKernel (sensor/preprocess.cu:25-42) in numpy: the raw
    image is a short*, depth = range_factor * src in single precision, valid
    inside [min, max], else -inf."""
    src = np.asarray(raw).astype(np.uint16).view(np.int16).astype(np.float32)
    z = np.float32(range_factor) * src
    ok = (z >= np.float32(min_depth)) & (z <= np.float32(max_depth))
    return np.where(ok, z, np.float32(-np.inf)).astype(np.float32)


def set_threads(n):
    lib().orc_set_threads(int(n))


def num_threads():
    return lib().orc_num_threads()


class Oracle:
    def __init__(self, params, fp64: bool = True):
        self.params = params
        self.fp64 = fp64
        self.L = lib()
        self.h = self.L.orc_create(C.byref(params), 1 if fp64 else 0)
        self.W, self.H = params.width, params.height

    def __del__(self):
        try:
            if self.h:
                self.L.orc_destroy(self.h)
                self.h = None
        except Exception:
            pass

    # ---- frame and stages
    def frame_set(self, depth, wTc):
        d, m = f32(depth).reshape(-1), f32(wTc).reshape(16)
        self.L.orc_frame_set(self.h, _p(d, C.c_float), _p(m, C.c_float))

    def allocate(self):
        """Run the allocation; returns the blocks it touched (sorted by key)."""
        n = self.L.orc_allocate(self.h)
        out = np.zeros((max(n, 1), 3), np.int32)
        self.L.orc_get_touched(self.h, _p(out, C.c_int32), n)
        return out[:n]

    def collect_frustum(self):
        return self.L.orc_collect_frustum(self.h)

    def collect_all(self):
        return self.L.orc_collect_all(self.h)

    def candidates(self):
        n = self.L.orc_get_candidates(self.h, None, 0)
        out = np.zeros((max(n, 1), 3), np.int32)
        self.L.orc_get_candidates(self.h, _p(out, C.c_int32), n)
        return out[:n]

    def set_candidates(self, pos):
        pos = i32(pos).reshape(-1, 3)
        bad = self.L.orc_set_candidates(self.h, len(pos), _p(pos, C.c_int32))
        assert bad == 0, f"{bad} candidate blocks missing in the oracle"

    def integrate_simple(self):
        self.L.orc_integrate_simple(self.h)

    def predict_inlier(self):
        self.L.orc_predict_inlier(self.h)

    def integrate_psdf(self):
        self.L.orc_integrate_psdf(self.h)

    def inlier(self):
        out = np.zeros(self.W * self.H, np.float32)
        self.L.orc_get_inlier(self.h, _p(out, C.c_float))
        return out.reshape(self.H, self.W)

    def set_inlier(self, img):
        a = f32(img).reshape(-1)
        self.L.orc_set_inlier(self.h, _p(a, C.c_float))

    def mesh(self):
        self.L.orc_mesh(self.h)

    def gc_low_surfel(self):
        self.L.orc_gc_low_surfel(self.h)

    def gc_starve(self):
        self.L.orc_gc_starve(self.h)

    def gc_collect_garbage(self):
        self.L.orc_gc_collect_garbage(self.h)

    def gc_recycle(self):
        return self.L.orc_gc_recycle(self.h)

    def raycast(self, cTw):
        W, H = self.params.rc_width, self.params.rc_height
        d = np.zeros(W * H, np.float32)
        v = np.zeros(W * H * 4, np.float32)
        n = np.zeros(W * H * 4, np.float32)
        m = f32(cTw).reshape(16)
        self.L.orc_raycast(self.h, _p(m, C.c_float), _p(d, C.c_float), _p(v, C.c_float), _p(n, C.c_float))
        return d.reshape(H, W), v.reshape(H, W, 4), n.reshape(H, W, 4)

    def raycast_backward(self, cTw, dL_ddepth, dL_dnormal=None):
        """dL/dxi (6, left se(3) increment of wTc, translation first) for
        L = sum dL_ddepth * depth + dL_dnormal . normal; the voxel gradient is
        kept for grad_blocks()."""
        a = f32(dL_ddepth).reshape(-1)
        nrm = None if dL_dnormal is None else f32(dL_dnormal).reshape(-1)
        xi = (C.c_double * 6)()
        m = f32(cTw).reshape(16)
        self.L.orc_raycast_backward(self.h, _p(m, C.c_float), _p(a, C.c_float), _p(nrm, C.c_float), xi)
        return np.array(list(xi))

    def grad_blocks(self):
        """(positions (n, 3), dL/dsdf (n, 512)) of the last raycast_backward."""
        n = self.L.orc_grad_blocks(self.h, 0, None, None)
        pos = np.zeros((max(n, 1), 3), np.int32)
        g = np.zeros((max(n, 1), 512), np.float64)
        self.L.orc_grad_blocks(self.h, n, _p(pos, C.c_int32), g.ctypes.data_as(C.POINTER(C.c_double)))
        return pos[:n], g[:n]

    def trace(self, cTw):
        """Per pixel (H, W, 4) int32: hit, regula-falsi sides, bits of t0 and t1
        of the single-precision march (the raycast's discrete decisions)."""
        W, H = self.params.rc_width, self.params.rc_height
        out = np.zeros(W * H * 4, np.int32)
        m = f32(cTw).reshape(16)
        self.L.orc_trace(self.h, _p(m, C.c_float), _p(out, C.c_int32))
        return out.reshape(H, W, 4)

    def debug_ray(self, cTw, x, y):
        out = (C.c_double * 16)()
        m = f32(cTw).reshape(16)
        self.L.orc_debug_ray(self.h, _p(m, C.c_float), int(x), int(y), out)
        return list(out)

    def frame(self, depth, wTc, raycast=False, tv_iterations=0, tv_lambda=0.1):
        """One MainEngine frame (optional TV pre-filter, Mapping, Meshing,
        raycast, Recycle); returns the raycast depth when asked."""
        d, m = f32(depth).reshape(-1), f32(wTc).reshape(16)
        if raycast:
            W, H = self.params.rc_width, self.params.rc_height
            rd = np.zeros(W * H, np.float32)
            self.L.orc_frame(self.h, _p(d, C.c_float), _p(m, C.c_float), int(tv_iterations), float(tv_lambda),
                             _p(rd, C.c_float), None, None)
            return rd.reshape(H, W)
        self.L.orc_frame(self.h, _p(d, C.c_float), _p(m, C.c_float), int(tv_iterations), float(tv_lambda),
                         None, None, None)
        return None

    def denoise_tv(self, lam=0.1, iterations=20):
        self.L.orc_denoise_tv(self.h, float(lam), int(iterations))

    def point_to_psdf(self, wTc, fix_jacobian=False):
        """PointToSurface normal equations at wTc over the current frame:
        (A[6, 6], b[6], err, count), sums in double."""
        m = f32(wTc).reshape(16)
        A, b, e = (C.c_double * 36)(), (C.c_double * 6)(), C.c_double(0)
        n = C.c_int32(0)
        self.L.orc_point_to_psdf(self.h, _p(m, C.c_float), 1 if fix_jacobian else 0, A, b, C.byref(e), C.byref(n))
        return np.array(list(A)).reshape(6, 6), np.array(list(b)), e.value, n.value

    def huber_tv_init(self):
        """PrimalDualInit over the current candidate blocks."""
        self.L.orc_huber_init(self.h)

    def huber_tv_iterate(self, lam, sigma, tau, iterations=1):
        """Dual + primal steps; returns [lam/2 data + tv, data, tv] of the
        last iteration's dual pass."""
        e = (C.c_double * 2)()
        self.L.orc_huber_iterate(self.h, float(lam), float(sigma), float(tau), int(iterations), e)
        return np.array([e[0] * np.float32(lam) / 2 + e[1], e[0], e[1]])

    def depth(self):
        out = np.zeros(self.W * self.H, np.float32)
        self.L.orc_get_depth(self.h, _p(out, C.c_float))
        return out.reshape(self.H, self.W)

    def set_depth(self, img):
        """Replace the current frame's preprocessed depth (after frame_set)."""
        a = f32(img).reshape(-1)
        assert a.size == self.W * self.H
        self.L.orc_set_depth(self.h, _p(a, C.c_float))

    # ---- state exchange
    def block_count(self):
        return self.L.orc_block_count(self.h)

    def blocks(self):
        """(pos[n,3], sdf[n,512], w, a, b) sorted by packed key."""
        n = self.block_count()
        pos = np.zeros((max(n, 1), 3), np.int32)
        arrs = [np.zeros((max(n, 1), 512), np.float32) for _ in range(4)]
        self.L.orc_get_blocks(self.h, n, _p(pos, C.c_int32), *[_p(a, C.c_float) for a in arrs])
        return (pos[:n],) + tuple(a[:n] for a in arrs)

    def set_blocks(self, pos, sdf=None, w=None, a=None, b=None):
        pos = i32(pos).reshape(-1, 3)
        conv = [None if x is None else f32(x).reshape(len(pos), 512) for x in (sdf, w, a, b)]
        self.L.orc_set_blocks(self.h, len(pos), _p(pos, C.c_int32), *[_p(x, C.c_float) for x in conv])

    def dump_mesh(self):
        nv, nt = C.c_int32(0), C.c_int32(0)
        self.L.orc_dump_mesh(self.h, 0, None, None, 0, None, C.byref(nv), C.byref(nt))
        vk = np.zeros((max(nv.value, 1), 4), np.int32)
        vd = np.zeros((max(nv.value, 1), 8), np.float32)
        tr = np.zeros((max(nt.value, 1), 7), np.int32)
        self.L.orc_dump_mesh(self.h, nv.value, _p(vk, C.c_int32), _p(vd, C.c_float), nt.value,
                             _p(tr, C.c_int32), C.byref(nv), C.byref(nt))
        return vk[:nv.value], vd[:nv.value], tr[:nt.value]

    def load_mesh(self, vkeys, vdata, tris):
        vk, vd, tr = i32(vkeys).reshape(-1, 4), f32(vdata).reshape(-1, 8), i32(tris).reshape(-1, 7)
        self.L.orc_load_mesh(self.h, len(vk), _p(vk, C.c_int32), _p(vd, C.c_float), len(tr), _p(tr, C.c_int32))

    def cubes(self, pos):
        pos = i32(pos).reshape(-1, 3)
        out = np.zeros((len(pos), 512), np.uint8)
        self.L.orc_get_cubes(self.h, len(pos), _p(pos, C.c_int32), _p(out, C.c_uint8))
        return out

    def set_cubes(self, pos, cubes):
        pos = i32(pos).reshape(-1, 3)
        c = np.ascontiguousarray(cubes, np.uint8)
        self.L.orc_set_cubes(self.h, len(pos), _p(pos, C.c_int32), _p(c, C.c_uint8))

    def block_meta(self, pos):
        pos = i32(pos).reshape(-1, 3)
        n = len(pos)
        life, inner, bnd = (np.zeros(n, np.int32) for _ in range(3))
        flag = np.zeros(n, np.uint8)
        self.L.orc_get_block_meta(self.h, n, _p(pos, C.c_int32), _p(life, C.c_int32), _p(inner, C.c_int32),
                                  _p(bnd, C.c_int32), _p(flag, C.c_uint8))
        return life, inner, bnd, flag

    def set_block_meta(self, pos, life=None, inner=None, boundary=None):
        pos = i32(pos).reshape(-1, 3)
        conv = [None if x is None else i32(x) for x in (life, inner, boundary)]
        self.L.orc_set_block_meta(self.h, len(pos), _p(pos, C.c_int32), *[_p(x, C.c_int32) for x in conv])
