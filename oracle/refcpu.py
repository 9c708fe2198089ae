"""TEST INFRASTRUCTURE: the reference's own device code built for the CPU.

``build(ref_root)`` extracts the reference's kernels (refcpu/extract.py) and
compiles them with refcpu/refcpu.cpp into oracle/_ref/librefcpu.so; it needs
the reference tree, so it runs only where that tree is present (this is how
tests/golden/ fixtures are produced; see tests/golden/make_golden.py).
``RefCPU`` drives the reference's stages (AllocBlockArray,
CollectBlocksInFrustum, UpdateBlocksSimple / Bayesian, MarchingCubes, GC,
RayCaster::Cast, PrimalDualInit / Iterate, PointToSurface) with the reference's launch shapes, one emulated CUDA
thread at a time.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT_DIR, "librefcpu.so")
# where the reference tree is read from: MESHHASHING_REFERENCE, else the
# read-only mount this recipe was written for
DEFAULT_REF = "/root/reference"


def reference_dir() -> str:
    """The reference source tree (``$MESHHASHING_REFERENCE`` overrides)."""
    return os.environ.get("MESHHASHING_REFERENCE", DEFAULT_REF)


def have_reference() -> bool:
    return os.path.isdir(os.path.join(reference_dir(), "src"))


def build(ref_root: str = None, force: bool = False) -> str:
    ref_root = ref_root or reference_dir()
    src = os.path.join(HERE, "refcpu", "refcpu.cpp")
    deps = [src, os.path.join(HERE, "refcpu", "cuda_host.h"), os.path.join(HERE, "refcpu", "extract.py")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    gen = os.path.join(OUT_DIR, "ref_kernels.inc")
    subprocess.check_call([sys.executable, os.path.join(HERE, "refcpu", "extract.py"), ref_root, gen],
                          stdout=subprocess.DEVNULL)
    cuda_inc = "/usr/local/cuda/include"
    cmd = ["g++", "-O2", "-std=c++14", "-ffp-contract=off", "-fPIC", "-shared", "-w",
           "-I", os.path.join(HERE, "refcpu", "stubs"), "-I", os.path.join(ref_root, "src"),
           "-I", os.path.join(ref_root, "src", "extern", "cuda"), "-I", cuda_inc,
           "-I", OUT_DIR, "-I", os.path.join(HERE, "refcpu"), "-o", LIB + ".tmp", src]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(LIB)
        vp, i32p, f32p = C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_float)
        L.ref_create.restype = vp
        L.ref_create.argtypes = [vp]
        L.ref_destroy.argtypes = [vp]
        L.ref_frame_set.argtypes = [vp, f32p, f32p]
        L.ref_alloc.restype = C.c_int
        L.ref_alloc.argtypes = [vp, C.c_int]
        for n in ("ref_collect", "ref_allocated"):
            getattr(L, n).restype = C.c_int
            getattr(L, n).argtypes = [vp]
        for n in ("ref_integrate_simple", "ref_predict", "ref_integrate_psdf", "ref_mesh", "ref_gc_low_surfel",
                  "ref_gc_recycle"):
            getattr(L, n).argtypes = [vp]
        L.ref_raycast.argtypes = [vp, f32p, f32p, f32p]
        L.ref_get_blocks.restype = C.c_int
        L.ref_get_blocks.argtypes = [vp, C.c_int, i32p, f32p, f32p, f32p, f32p]
        L.ref_get_candidates.restype = C.c_int
        L.ref_get_candidates.argtypes = [vp, C.c_int, i32p]
        L.ref_get_inlier.argtypes = [vp, f32p]
        L.ref_dump_mesh.argtypes = [vp, C.c_int, i32p, f32p, C.c_int, i32p, i32p, i32p]
        L.ref_inverse.argtypes = [f32p, f32p]
        L.ref_cube_indices.argtypes = [vp, C.c_int, i32p, C.POINTER(C.c_uint8)]
        L.ref_compress_mesh.argtypes = [vp, C.c_int, f32p, f32p, C.c_int, i32p, i32p]
        L.ref_pd_init.argtypes = [vp]
        L.ref_point_to_psdf.argtypes = [vp, f32p, f32p, f32p, f32p, i32p]
        L.ref_set_candidates.restype = C.c_int
        L.ref_set_candidates.argtypes = [vp, C.c_int, i32p]
        L.ref_pd_iterate.argtypes = [vp, C.c_float, C.c_float, C.c_float, f32p]
        _lib = L
    return _lib


def _p(a, ct):
    return None if a is None else a.ctypes.data_as(C.POINTER(ct))


def inverse(m):
    a = np.ascontiguousarray(m, np.float32).reshape(16)
    out = np.zeros(16, np.float32)
    lib().ref_inverse(_p(a, C.c_float), _p(out, C.c_float))
    return out.reshape(4, 4)


class RefCPU:
    def __init__(self, params):
        self.p = params
        self.L = lib()
        self.h = self.L.ref_create(C.byref(params))

    def __del__(self):
        try:
            self.L.ref_destroy(self.h)
        except Exception:
            pass

    def frame_set(self, depth, wTc):
        d = np.ascontiguousarray(depth, np.float32).reshape(-1)
        m = np.ascontiguousarray(wTc, np.float32).reshape(16)
        self.L.ref_frame_set(self.h, _p(d, C.c_float), _p(m, C.c_float))

    def alloc(self, until_stable=True):
        return self.L.ref_alloc(self.h, 1 if until_stable else 0)

    def collect(self):
        return self.L.ref_collect(self.h)

    def integrate_simple(self):
        self.L.ref_integrate_simple(self.h)

    def predict(self):
        self.L.ref_predict(self.h)

    def integrate_psdf(self):
        self.L.ref_integrate_psdf(self.h)

    def mesh(self):
        self.L.ref_mesh(self.h)

    def gc_low_surfel(self):
        self.L.ref_gc_low_surfel(self.h)

    def gc_recycle(self):
        self.L.ref_gc_recycle(self.h)

    def set_candidates(self, pos):
        pos = np.ascontiguousarray(pos, np.int32).reshape(-1, 3)
        return self.L.ref_set_candidates(self.h, len(pos), _p(pos, C.c_int32))

    def point_to_psdf(self, wTc):
        """PointToSurface at pose wTc: (A[6, 6], b[6], err, count), float sums."""
        m = np.ascontiguousarray(wTc, np.float32).reshape(16)
        A, b, e = np.zeros(36, np.float32), np.zeros(6, np.float32), np.zeros(1, np.float32)
        n = C.c_int32(0)
        self.L.ref_point_to_psdf(self.h, _p(m, C.c_float), _p(A, C.c_float), _p(b, C.c_float), _p(e, C.c_float),
                                 C.byref(n))
        return A.reshape(6, 6), b, float(e[0]), n.value

    def pd_init(self):
        self.L.ref_pd_init(self.h)

    def pd_iterate(self, lam, sigma, tau):
        """One PrimalDualIterate; returns (err_data, err_tv) of its pass 1."""
        e = np.zeros(2, np.float32)
        self.L.ref_pd_iterate(self.h, float(lam), float(sigma), float(tau), _p(e, C.c_float))
        return e

    def raycast(self, cTw):
        W, H = self.p.rc_width, self.p.rc_height
        d = np.zeros(W * H, np.float32)
        n = np.zeros(W * H * 4, np.float32)
        m = np.ascontiguousarray(cTw, np.float32).reshape(16)
        self.L.ref_raycast(self.h, _p(m, C.c_float), _p(d, C.c_float), _p(n, C.c_float))
        return d.reshape(H, W), n.reshape(H, W, 4)

    def blocks(self):
        n = self.L.ref_get_blocks(self.h, 0, None, None, None, None, None)
        pos = np.zeros((max(n, 1), 3), np.int32)
        arrs = [np.zeros((max(n, 1), 512), np.float32) for _ in range(4)]
        self.L.ref_get_blocks(self.h, n, _p(pos, C.c_int32), *[_p(a, C.c_float) for a in arrs])
        return (pos[:n],) + tuple(a[:n] for a in arrs)

    def candidates(self):
        n = self.L.ref_get_candidates(self.h, 0, None)
        out = np.zeros((max(n, 1), 3), np.int32)
        self.L.ref_get_candidates(self.h, n, _p(out, C.c_int32))
        return out[:n]

    def inlier(self):
        out = np.zeros(self.p.width * self.p.height, np.float32)
        self.L.ref_get_inlier(self.h, _p(out, C.c_float))
        return out.reshape(self.p.height, self.p.width)

    def dump_mesh(self):
        nv, nt = C.c_int32(0), C.c_int32(0)
        self.L.ref_dump_mesh(self.h, 0, None, None, 0, None, C.byref(nv), C.byref(nt))
        vk = np.zeros((max(nv.value, 1), 4), np.int32)
        vd = np.zeros((max(nv.value, 1), 8), np.float32)
        tr = np.zeros((max(nt.value, 1), 7), np.int32)
        a, b = nv.value, nt.value
        self.L.ref_dump_mesh(self.h, a, _p(vk, C.c_int32), _p(vd, C.c_float), b, _p(tr, C.c_int32),
                             C.byref(nv), C.byref(nt))
        return vk[:a], vd[:a], tr[:b]

    def compress_mesh(self):
        """MainEngine's compact mesh (CollectAllBlocks + CompressMesh):
        (positions[nv, 3], normals[nv, 3], triangles[nt, 3], stats (nt, nv,
        sum of the compacted vertices' ref_count))."""
        st = np.zeros(3, np.int32)
        self.L.ref_compress_mesh(self.h, 0, None, None, 0, None, _p(st, C.c_int32))
        nt, nv = int(st[0]), int(st[1])
        pos, nrm = np.zeros((max(nv, 1), 3), np.float32), np.zeros((max(nv, 1), 3), np.float32)
        tri = np.zeros((max(nt, 1), 3), np.int32)
        self.L.ref_compress_mesh(self.h, nv, _p(pos, C.c_float), _p(nrm, C.c_float), nt, _p(tri, C.c_int32),
                                 _p(st, C.c_int32))
        return pos[:nv], nrm[:nv], tri[:nt], st.copy()

    def cubes(self, pos):
        pos = np.ascontiguousarray(pos, np.int32).reshape(-1, 3)
        out = np.zeros((len(pos), 512), np.uint8)
        self.L.ref_cube_indices(self.h, len(pos), _p(pos, C.c_int32), out.ctypes.data_as(C.POINTER(C.c_uint8)))
        return out
