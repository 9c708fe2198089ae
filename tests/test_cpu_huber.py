"""Volumetric Huber-TV (PrimalDualInit / PrimalDualIterate,
optimize/primal_dual.cu:10-223) in the oracle against a second, independent
restatement: dense numpy arrays over a small block grid, in the same
precision.  The grid has a missing block, unobserved voxels and a
non-candidate block, and gradients on both sides of the weight-2 pin
(|grad| = ln 2 voxel).  The two sides may differ by the last place of exp().
"""
import numpy as np

from meshhashing_gb300 import config, scene
from oracle import oracle as O

EPS = np.float32(1e-6)
ALPHA = 0.02


def _grid(seed=0):
    """3 x 2 x 2 blocks minus one; voxel (x, y, z) dense, indexed [x, y, z]."""
    rng = np.random.default_rng(seed)
    nb = (3, 2, 2)
    present = np.ones(nb, bool)
    present[2, 1, 1] = False
    cand = present.copy()
    cand[0, 1, 0] = False
    shape = tuple(8 * n for n in nb)
    x = np.arange(shape[0])[:, None, None]
    vs = 0.008
    sdf = (vs * (0.45 * x + 0.35 * rng.standard_normal(shape)) - 0.05).astype(np.float32)
    w = rng.uniform(0.5, 3.0, shape).astype(np.float32)
    w[rng.random(shape) < 0.1] = 0.0
    up = lambda a: np.repeat(np.repeat(np.repeat(a, 8, 0), 8, 1), 8, 2)  # noqa: E731
    return sdf, w, up(present), up(cand), nb


def _to_blocks(nb, dense_fields, present_blocks):
    pos, rows = [], [[] for _ in dense_fields]
    for bx in range(nb[0]):
        for by in range(nb[1]):
            for bz in range(nb[2]):
                if not present_blocks[bx, by, bz]:
                    continue
                pos.append((bx, by, bz))
                for r, f in zip(rows, dense_fields):
                    blk = f[8 * bx:8 * bx + 8, 8 * by:8 * by + 8, 8 * bz:8 * bz + 8]
                    r.append(blk.transpose(2, 1, 0).reshape(512))   # local index x + 8 y + 64 z
    return np.array(pos, np.int32), [np.array(r) for r in rows]


def _from_blocks(nb, pos, rows):
    out = np.zeros(tuple(8 * n for n in nb), rows.dtype)
    for (bx, by, bz), r in zip(pos, rows):
        out[8 * bx:8 * bx + 8, 8 * by:8 * by + 8, 8 * bz:8 * bz + 8] = r.reshape(8, 8, 8).transpose(2, 1, 0)
    return out


def _shift(a, k, s, fill):
    """a at voxel + s e_k, fill outside the grid."""
    out = np.full_like(a, fill)
    src = [slice(None)] * 3
    dst = [slice(None)] * 3
    if s > 0:
        src[k], dst[k] = slice(1, None), slice(None, -1)
    else:
        src[k], dst[k] = slice(None, -1), slice(1, None)
    out[tuple(dst)] = a[tuple(src)]
    return out


def huber_dense(sdf, w, present, cand, vs, lam, sigma, tau, iters, dt):
    """The reference's init + iterate on dense arrays, in precision dt."""
    f = lambda v: dt(v)  # noqa: E731
    sdf = sdf.astype(dt)
    obs = present & (w >= EPS)
    ok = np.all([_shift(obs, k, 1, False) for k in range(3)], axis=0)
    g = [np.where(ok, _shift(sdf, k, 1, 0) - sdf, f(0)) for k in range(3)]
    W = np.exp(np.sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]) / f(vs)).astype(dt)
    mask = cand & obs
    sdf0, bar = sdf.copy(), np.zeros_like(sdf)
    p = [np.zeros_like(sdf) for _ in range(3)]
    lam, sigma, tau, alpha = f(lam), f(sigma), f(tau), f(np.float32(ALPHA))
    err = (0.0, 0.0)
    for _ in range(iters):
        fok = np.all([_shift(mask, k, 1, False) for k in range(3)], axis=0)
        gs = [np.where(fok, _shift(sdf, k, 1, 0) - sdf, f(0)) for k in range(3)]
        ln = np.sqrt(gs[0] * gs[0] + gs[1] * gs[1] + gs[2] * gs[2])
        hub = np.where(np.abs(ln) < alpha, f(0.5) * (ln * ln) / alpha, np.abs(ln) - f(0.5) * alpha)
        dd = np.abs(sdf - sdf0)
        err = (float(np.sum((dd * dd)[mask], dtype=np.float64)), float(np.sum(hub[mask], dtype=np.float64)))
        gb = [np.where(fok, _shift(bar, k, 1, 0) - bar, f(0)) for k in range(3)]
        q = [(p[k] + sigma * gb[k]) / (f(1) + sigma * alpha) for k in range(3)]
        nrm = np.maximum(f(1), np.sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]))
        p = [np.where(mask, q[k] / nrm, p[k]) for k in range(3)]
        bok = np.all([_shift(mask, k, -1, False) for k in range(3)], axis=0)
        pn = [_shift(p[k], k, -1, 0) for k in range(3)]
        div = np.where(bok, (pn[0] - p[0]) + (pn[1] - p[1]) + (pn[2] - p[2]), f(0))
        lw = lam * W
        x = sdf - tau * div
        x = (x + lw * tau * sdf0) / (f(1) + lw * tau)
        x = np.where(W > f(2), sdf0, x)
        bar = np.where(mask, f(2) * x - sdf, bar)
        sdf = np.where(mask, x, sdf)
    return sdf, err


def _check(fp64):
    wl = scene.small_circle(60)
    p = config.params_for(wl, value_capacity=1 << 10, bucket_count=1 << 10)
    sdf, w, present, cand, nb = _grid()
    present_b, cand_b = present[::8, ::8, ::8], cand[::8, ::8, ::8]
    pos, (rs, rw) = _to_blocks(nb, (sdf, w), present_b)
    o = O.Oracle(p, fp64=fp64)
    o.set_blocks(pos, rs, rw, np.zeros_like(rs), np.zeros_like(rs))
    cpos = np.array([q for q in pos if cand_b[tuple(q)]], np.int32)
    o.set_candidates(cpos)
    lam, sigma, tau, iters = 2.0, 8.0, 0.01, 12
    o.huber_tv_init()
    e = o.huber_tv_iterate(lam, sigma, tau, iters)
    opos, osdf = o.blocks()[:2]
    got = _from_blocks(nb, opos, osdf)
    dt = np.float64 if fp64 else np.float32
    want, err = huber_dense(sdf, w, present, cand, p.voxel_size, np.float32(lam), np.float32(sigma),
                            np.float32(tau), iters, dt)
    want = want.astype(np.float32)
    obs = present & (w >= EPS)
    moved = obs & cand & (sdf != want)
    assert moved.sum() > 500                                   # the smoother did something
    still = present & ~(cand & obs)
    assert np.array_equal(got[still], sdf[still])              # unobserved / non-candidate untouched
    np.testing.assert_allclose(got[present], want[present], rtol=0, atol=2e-6 * np.abs(sdf).max())
    assert np.mean(got[present] == want[present]) > 0.95
    np.testing.assert_allclose(e[1:], err, rtol=1e-4)
    return got


def test_huber_fp32_matches_dense_restatement(built):
    _check(fp64=False)


def test_huber_fp64_matches_dense_restatement(built):
    _check(fp64=True)
