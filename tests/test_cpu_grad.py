"""Raycast derivative of the FP64 oracle against central finite differences
of its own raycast (h = 1e-4), on the CPU.

Pixels whose single-precision trace (hit and bracketing samples) changes
under a perturbation are left out of both sides: there the raycast jumps and
no derivative exists.  So are pixels where the output has a kink inside the
stencil (second difference above the float32 resolution of the output): the
trilinear field is only continuous across cell faces, so the hit's
derivative jumps where the root crosses one -- at grazing rays within a
fraction of a millimetre -- and a central difference there averages two
slopes.  A regula-falsi step whose value is within rounding of
zero may take either side; both give the same depth and, on a segment where
the sdf is linear, the same derivative, so those pixels are kept.
"""
import numpy as np

from meshhashing_gb300 import config, scene
from meshhashing_gb300.pose import left_update
from oracle import oracle as O

H_FD = 1e-4


def _volume(fp64=True, width=64, height=48):
    wl = scene.small_circle(60)
    f = 262.5 * width / 320
    wl.camera = scene.Camera(width, height, f, f, (width - 1) / 2, (height - 1) / 2)
    p = config.params_for(wl, value_capacity=1 << 15, bucket_count=1 << 14)
    o = O.Oracle(p, fp64=fp64)
    for i in range(0, 24, 4):
        o.frame(wl.frame(i), wl.pose(i))
    T = wl.pose(26).astype(np.float64)
    return wl, p, o, T


def _render(o, T):
    cTw = np.linalg.inv(T).astype(np.float32)
    d, _, n = o.raycast(cTw)
    tr = o.trace(cTw)
    tr[..., 1] = 0
    return d.astype(np.float64), n[..., :3].astype(np.float64), tr


def _smooth(p, m, c):
    """Second difference at most 2 % of the first (or at the float32
    resolution of the output): the slope hardly changes across the stencil."""
    return np.abs(p + m - 2.0 * c) <= 0.02 * np.abs(p - m) + 1e-6


def _pose_check(with_normals):
    wl, p, o, T = _volume()
    cTw = np.linalg.inv(T).astype(np.float32)
    d0, n0, tr0 = _render(o, T)
    hit = tr0[..., 0] == 1
    assert hit.sum() > 500
    rng = np.random.default_rng(1)
    a = rng.standard_normal(d0.shape) * (0.0 if with_normals else 1.0)
    b = rng.standard_normal(n0.shape) * (1.0 if with_normals else 0.0)
    for k in range(6):
        e = np.zeros(6)
        e[k] = H_FD
        dp, np_, trp = _render(o, left_update(T, e))
        dm, nm, trm = _render(o, left_update(T, -e))
        keep = hit & np.all(trp == tr0, axis=-1) & np.all(trm == tr0, axis=-1)
        if with_normals:
            keep &= np.all(_smooth(np_, nm, n0), axis=-1)
        else:
            keep &= _smooth(dp, dm, d0)
        assert keep.sum() > (0.3 if with_normals else 0.7) * hit.sum(), (k, keep.sum(), hit.sum())
        with np.errstate(invalid="ignore"):
            fd = (np.sum((a * (dp - dm))[keep]) + np.sum((b * (np_ - nm))[keep])) / (2 * H_FD)
        am = np.where(keep, a, 0.0).astype(np.float32)
        bm = np.where(keep[..., None], b, 0.0).astype(np.float32)
        bw = o.raycast_backward(cTw, am, bm if with_normals else None)[k]
        assert abs(bw - fd) <= 2e-2 * abs(bw) + 1e-2, (k, bw, fd)


def test_fp64_depth_pose_gradient_matches_central_differences(built):
    _pose_check(with_normals=False)


def test_fp64_normal_pose_gradient_matches_central_differences(built):
    _pose_check(with_normals=True)


def test_fp64_voxel_gradient_matches_central_differences(built):
    """Voxels drawn from the bulk of the gradient (the largest entries belong
    to rays that barely cross zero, where the depth has a kink in reach of
    any stencil)."""
    wl, p, o, T = _volume()
    cTw = np.linalg.inv(T).astype(np.float32)
    d0, n0, tr0 = _render(o, T)
    hit = tr0[..., 0] == 1
    rng = np.random.default_rng(2)
    a = np.where(hit, rng.standard_normal(d0.shape), 0.0)
    o.raycast_backward(cTw, a.astype(np.float32))
    gpos, g = o.grad_blocks()
    assert len(gpos) > 0
    pos, s, w, A, B = o.blocks()
    idx = {tuple(int(c) for c in q): i for i, q in enumerate(pos)}
    mag = np.abs(g).reshape(-1)
    lo, hi = np.percentile(mag[mag > 0], [50, 90])
    cand = np.flatnonzero((mag >= lo) & (mag <= hi))
    checked = 0
    for f in rng.choice(cand, 8, replace=False):
        bi, li = divmod(int(f), 512)
        row = idx[tuple(int(c) for c in gpos[bi])]
        vals = []
        for sgn in (1, -1):
            s2 = s.copy()
            s2[row, li] += sgn * H_FD
            o.set_blocks(pos[row:row + 1], s2[row:row + 1], w[row:row + 1], A[row:row + 1], B[row:row + 1])
            vals.append(_render(o, T))
        o.set_blocks(pos[row:row + 1], s[row:row + 1], w[row:row + 1], A[row:row + 1], B[row:row + 1])
        (dp, _, trp), (dm, _, trm) = vals
        keep = hit & np.all(trp == tr0, axis=-1) & np.all(trm == tr0, axis=-1) & _smooth(dp, dm, d0)
        with np.errstate(invalid="ignore"):
            fd = np.sum((a * (dp - dm))[keep]) / (2 * H_FD)
        o.raycast_backward(cTw, np.where(keep, a, 0.0).astype(np.float32))
        gp, gk = o.grad_blocks()
        gi = {tuple(int(c) for c in q): i for i, q in enumerate(gp)}
        bw = gk[gi[tuple(int(c) for c in gpos[bi])], li] if tuple(int(c) for c in gpos[bi]) in gi else 0.0
        # the rendered depth is a float32: each difference carries up to one
        # unit in the last place of either side
        quant = np.sum((np.abs(a) * np.spacing(d0.astype(np.float32)))[keep]) / (2 * H_FD)
        assert abs(fd - bw) <= 2e-2 * abs(bw) + quant, (fd, bw, quant)
        checked += 1
    assert checked == 8
