"""The FP64 oracle's depth TV denoiser against a second, independent
restatement of the same published method, written here with numpy arrays:
Chambolle & Pock (2011), Algorithm 1 (theta = 1) for the ROF model
min_u |grad u|_1 + lambda/2 |u - f|^2, with tau = sigma = 1/sqrt(8), depth in
millimetres, forward differences only between two valid pixels (the
divergence is their negative adjoint) and invalid pixels left invalid.  The
reference has no 2-D depth denoiser, so this pins the oracle to the method,
not to reference code."""
import numpy as np

from meshhashing_gb300 import config, scene
from oracle import oracle as O


def chambolle_pock_tv(depth, lam, iters):
    ok = (depth > 0) & (depth < 1e30)
    f = np.where(ok, depth.astype(np.float64) * 1000.0, 0.0)
    ex = ok[:, :-1] & ok[:, 1:]                 # valid horizontal edges
    ey = ok[:-1, :] & ok[1:, :]                 # valid vertical edges
    tau = sigma = 1.0 / np.sqrt(8.0)
    u, ub = f.copy(), f.copy()
    px, py = np.zeros_like(f), np.zeros_like(f)
    for _ in range(iters):
        gx, gy = np.zeros_like(f), np.zeros_like(f)
        gx[:, :-1] = np.where(ex, ub[:, 1:] - ub[:, :-1], 0.0)
        gy[:-1, :] = np.where(ey, ub[1:, :] - ub[:-1, :], 0.0)
        qx, qy = px + sigma * gx, py + sigma * gy
        nr = np.maximum(1.0, np.sqrt(qx * qx + qy * qy))
        px, py = qx / nr, qy / nr
        pxl, pyu = np.zeros_like(f), np.zeros_like(f)
        pxl[:, 1:], pyu[1:, :] = px[:, :-1], py[:-1, :]
        div = (px - pxl) + (py - pyu)
        un = np.where(ok, (u + tau * div + tau * lam * f) / (1.0 + tau * lam), f)
        ub = np.where(ok, 2.0 * un - u, f)
        u = un
    return np.where(ok, u * 0.001, -np.inf), ok


def test_oracle_tv_matches_published_method(built):
    wl = scene.full_spline(8, width=160, height=120)
    p = config.params_for(wl, value_capacity=1 << 12)
    o = O.Oracle(p, fp64=True)
    for i, (lam, iters) in enumerate(((0.1, 20), (0.5, 7), (0.02, 40))):
        o.frame_set(wl.frame(i), wl.pose(i))
        pre = o.depth()                             # preprocessed input, -inf = invalid
        o.denoise_tv(lam, iters)
        got = o.depth()
        want, ok = chambolle_pock_tv(pre, lam, iters)
        assert ok.sum() > 0.9 * ok.size and (~ok).sum() > 0     # missing pixels are exercised
        np.testing.assert_array_equal(np.isfinite(got), ok)
        assert np.all(got[~ok] == -np.inf)
        # both in double; the oracle rounds its output to float32 metres
        err = np.abs(got[ok].astype(np.float64) - want[ok])
        assert err.max() <= 2.0 * np.spacing(np.float32(5.0)), err.max()
        assert np.abs(got[ok] - pre[ok]).max() > 1e-4         # the filter did something
