"""The depth TV denoiser on the GPU.

* The tiled form a volume runs (k_tv_tile: ten iterations per launch in
  shared memory) against the one-launch-per-iteration form
  (mh_denoise_tv_static, k_tv_iter) on the same preprocessed frame: bit for
  bit, for iteration counts that need one launch, exactly two, and a
  remainder, on an image whose size is not a multiple of the tile.
* Against the oracle's restatement of the same published method (Chambolle
  & Pock 2011, evaluated in double) on a 640x480 frame with outliers and
  holes: the same valid pixels, depths within 1e-5 m after 20 iterations.
"""
import ctypes as C

import numpy as np
import pytest

from meshhashing_gb300 import Volume, _lib, config, scene
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def test_tiled_tv_bit_identical_to_per_iteration(built):
    import torch
    wl = scene.full_spline(4, width=200, height=150)
    p = config.params_for(wl, value_capacity=1 << 12, bucket_count=1 << 12, max_vertex_count=1 << 12,
                          max_triangle_count=1 << 12, mesh_page_capacity=1 << 10)
    v = Volume(p)
    L = _lib.load()
    H, W = p.height, p.width
    for iters in (1, 3, 10, 11, 20, 23):
        v.set_frame(wl.frame(2), wl.pose(2))
        prep = v.depth()
        v.denoise_tv(0.1, iters)
        want = v.depth()
        dev_in = torch.from_numpy(prep.copy()).cuda()
        dev_out = torch.full((H, W), float("nan"), dtype=torch.float32, device="cuda")
        rc = L.mh_denoise_tv_static(C.c_void_p(dev_in.data_ptr()), C.c_void_p(dev_out.data_ptr()), W, H,
                                    C.c_float(0.1), iters, None)
        assert rc == 0, rc
        torch.cuda.synchronize()
        got = dev_out.cpu().numpy()
        np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32), err_msg=f"{iters} iterations")
        assert np.isfinite(want).mean() > 0.9
    assert v.stats()["error"] == 0


def test_tv_matches_fp64_oracle(built):
    wl = scene.full_spline(4)
    p = config.params_for(wl, value_capacity=1 << 12, bucket_count=1 << 12, max_vertex_count=1 << 12,
                          max_triangle_count=1 << 12, mesh_page_capacity=1 << 10)
    v = Volume(p)
    o = Oracle(p, fp64=True)
    d, T = wl.frame(1), wl.pose(1)
    v.set_frame(d, T)
    o.frame_set(d, T)
    before = v.depth()
    v.denoise_tv(0.1, 20)
    o.denoise_tv(0.1, 20)
    got, want = v.depth(), o.depth()
    ok = np.isfinite(want)
    np.testing.assert_array_equal(np.isfinite(got), ok)
    err = np.abs(got[ok] - want[ok]).max()
    moved = np.abs(got[ok] - before[ok]).max()
    print(f"TV vs FP64: max |ddepth| = {err:.3e} m; the denoiser moved depths by up to {moved:.3e} m")
    assert moved > 1e-3 and err <= 1e-5, (err, moved)
