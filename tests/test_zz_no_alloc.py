"""The allocation-free TV entry point against the allocating one.

mh_denoise_tv_static serves callers that cannot allocate device memory (their
memory belongs to another allocator with a fixed budget, or cudaMalloc's
implicit synchronisation would stall their frame loop): its scratch planes
live in a fixed device array inside the library.  This test calls it through
the C ABI twice in a row on the same frame and checks both results against
mh_denoise_tv on a volume, bit for bit (the per-iteration kernels it runs
and the tiled kernel of the volume path compute the same values).  It runs last in collection order and must pass both alone
and after the other tests (the shared scratch keeps the previous call's data).
"""
import ctypes as C

import numpy as np
import pytest

from meshhashing_gb300 import MeshHashError, Volume, _lib, config, scene

pytestmark = pytest.mark.gpu


def test_denoise_tv_static_matches_volume_path(built):
    import torch
    wl = scene.full_spline(4)
    p = config.params_for(wl, value_capacity=1 << 12, bucket_count=1 << 12, max_vertex_count=1 << 12,
                          max_triangle_count=1 << 12, mesh_page_capacity=1 << 10)
    v = Volume(p)
    L = _lib.load()
    H, W = p.height, p.width
    assert W * H <= 640 * 480
    for frame in (0, 3):
        v.set_frame(wl.frame(frame), wl.pose(frame))
        prep = v.depth()                       # preprocessed input (-inf = invalid)
        v.denoise_tv(0.1, 20)
        want = v.depth()
        dev_in = torch.from_numpy(prep.copy()).cuda()
        for call in range(2):
            dev_out = torch.full((H, W), float("nan"), dtype=torch.float32, device="cuda")
            rc = L.mh_denoise_tv_static(C.c_void_p(dev_in.data_ptr()), C.c_void_p(dev_out.data_ptr()), W, H,
                                        C.c_float(0.1), 20, None)
            assert rc == 0, rc
            torch.cuda.synchronize()
            got = dev_out.cpu().numpy()
            ok = np.isfinite(want)
            np.testing.assert_array_equal(np.isfinite(got), ok)
            assert np.all(got[~ok] == -np.inf)
            # the per-iteration kernels of the static path and the tiled
            # kernel of the volume path compute the same bits
            np.testing.assert_array_equal(got[ok].view(np.uint32), want[ok].view(np.uint32),
                                          err_msg=f"frame {frame}, call {call}")
    # sizes beyond the fixed scratch are refused, before any launch
    big = torch.zeros((481, 640), dtype=torch.float32, device="cuda")
    rc = L.mh_denoise_tv_static(C.c_void_p(big.data_ptr()), C.c_void_p(big.data_ptr()), 640, 481,
                                C.c_float(0.1), 20, None)
    assert rc == 3  # MH_ERR_CAPACITY
    assert v.stats()["error"] == 0
