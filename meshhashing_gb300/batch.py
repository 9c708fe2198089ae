"""Host-side mirror of the batch entry points (mh_batch_* in include/meshhash.h).

A Batch advances many independent Volumes by one MainEngine frame per step,
with one launch per stage for all scenes (optionally replayed from a captured
CUDA graph).  Each scene's results are those of Volume.integrate_frame on the
same inputs.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._abi import MhBatchTuning
from .volume import _check_tensor

RAY_TILE_SHAPES = ((16, 8), (8, 8), (32, 4))
INTEGRATE_CTA_CAPS = (4, 8, 16)


class Batch:
    def __init__(self, volumes, raycast: bool = True):
        self.L = _lib.load()
        self.volumes = list(volumes)            # keeps the volumes alive while the batch lives
        arr = (C.c_void_p * len(self.volumes))(*[v.h.value for v in self.volumes])
        self.h = C.c_void_p()
        _lib.check("mh_batch_create", self.L.mh_batch_create(arr, len(self.volumes), 1 if raycast else 0,
                                                             C.byref(self.h)))
        self.raycast_enabled = raycast

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.L.mh_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _c(self, name, *args):
        _lib.check(name, getattr(self.L, name)(self.h, *args))

    def step(self, depths, poses, active=None, on_device: bool = False, tv_iterations: int = 0,
             tv_lambda: float = 0.1, use_graph: bool = False, stream: int = 0):
        """One frame for every active scene.  depths: per scene an (H, W) float32
        array (host) or a CUDA tensor / device pointer (on_device); inactive
        scenes may pass None.  poses: per scene a 4x4 camera-to-world matrix.
        Arrays and tensors are checked against each scene's frame size
        (ValueError); raw device pointers are taken as given."""
        n = len(self.volumes)
        if len(depths) != n or len(poses) != n:
            raise ValueError(f"depths and poses need one entry per scene ({n})")
        if active is not None and len(active) != n:
            raise ValueError(f"active needs one entry per scene ({n})")
        keep = []
        ptrs = (C.c_void_p * n)()
        for i, d in enumerate(depths):
            npx = self.volumes[i].W * self.volumes[i].H
            if d is None:
                ptrs[i] = None
            elif on_device:
                if hasattr(d, "data_ptr"):
                    _check_tensor(d, npx, f"depths[{i}]", cuda=True)
                ptrs[i] = d.data_ptr() if hasattr(d, "data_ptr") else int(d)
            else:
                a = np.ascontiguousarray(d, np.float32)
                if a.size != npx:
                    raise ValueError(f"depths[{i}]: expected {npx} values, got {a.size}")
                keep.append(a)
                ptrs[i] = a.ctypes.data
        P = np.zeros((n, 16), np.float32)
        for i, T in enumerate(poses):
            if T is not None:
                P[i] = np.asarray(T, np.float32).reshape(16)
        act = None
        if active is not None:
            act = np.ascontiguousarray(np.asarray(active, np.int32))
        self._c("mh_batch_step", ptrs, 1 if on_device else 0, P.ctypes.data_as(C.POINTER(C.c_float)),
                act.ctypes.data_as(C.POINTER(C.c_int32)) if act is not None else None, int(tv_iterations),
                C.c_float(tv_lambda), 1 if use_graph else 0, C.c_void_p(int(stream)))

    def outputs(self, scene: int):
        """Device pointers (depth, vertex4, normal4) of a scene's raycast outputs."""
        d, v, n = C.c_void_p(), C.c_void_p(), C.c_void_p()
        self._c("mh_batch_outputs", int(scene), C.byref(d), C.byref(v), C.byref(n))
        return d.value, v.value, n.value

    def raycast(self, scene: int):
        """Host copies (depth (H, W), vertex (H, W, 4), normal (H, W, 4)) of a
        scene's last raycast."""
        vol = self.volumes[scene]
        W, H = vol.RW, vol.RH
        d = np.empty(W * H, np.float32)
        v = np.empty(W * H * 4, np.float32)
        n = np.empty(W * H * 4, np.float32)
        f = C.POINTER(C.c_float)
        self._c("mh_batch_dump_raycast", int(scene), d.ctypes.data_as(f), v.ctypes.data_as(f), n.ctypes.data_as(f))
        return d.reshape(H, W), v.reshape(H, W, 4), n.reshape(H, W, 4)

    def tuning(self):
        t = MhBatchTuning()
        self._c("mh_batch_get_tuning", C.byref(t))
        return {"ray_tile": RAY_TILE_SHAPES[t.ray_tile_shape], "integrate_cta_per_sm": t.integrate_cta_per_sm}

    def set_tuning(self, ray_tile_shape: int, integrate_cta_per_sm: int):
        t = MhBatchTuning(int(ray_tile_shape), int(integrate_cta_per_sm))
        self._c("mh_batch_set_tuning", C.byref(t))

    def autotune(self, trials: int = 1):
        """The next 9 * trials steps try every (tile shape, CTA cap) pair."""
        self._c("mh_batch_autotune", int(trials))

    def tuning_times(self):
        r = (C.c_double * 3)()
        i = (C.c_double * 3)()
        self._c("mh_batch_tuning_times", r, i)
        return {"raycast_ms": dict(zip(RAY_TILE_SHAPES, list(r))),
                "integrate_ms": dict(zip(INTEGRATE_CTA_CAPS, list(i)))}

    STAGES = ("preprocess", "tv", "alloc", "collect", "predict", "integrate", "mesh", "gc", "raycast")

    def stage_times(self):
        """ms per step of each stage, averaged over the autotuning steps."""
        ms = (C.c_double * 9)()
        self._c("mh_batch_stage_times", ms)
        return dict(zip(self.STAGES, list(ms)))
