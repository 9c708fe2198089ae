"""Differentiable raycast on the GPU: mh_raycast_backward against the oracle's
backward (FP32 and FP64) on the same state, against central differences of
the GPU's own raycast (h = 1e-4), through the torch.autograd wrapper, and
Gauss-Newton pose refinement (mh_refine_pose) from a perturbed pose.

Finite differences use only pixels whose raycast trace (hit, bracketing
samples; from the FP32 oracle, which takes the same decisions) is unchanged
under the perturbation and whose output is smooth across the stencil.
"""
import numpy as np
import pytest

from meshhashing_gb300 import Volume, config, scene
from meshhashing_gb300.pose import left_update, pose_error
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu
H_FD = 1e-4


def _setup(width=160, height=120, frames=range(0, 32, 4), psdf=False):
    if psdf:
        wl = scene.full_spline(60, width=width, height=height)
        p = config.params_for(wl, value_capacity=1 << 18, bucket_count=1 << 17)
    else:
        wl = scene.small_circle(60)
        f = 262.5 * width / 320
        wl.camera = scene.Camera(width, height, f, f, (width - 1) / 2, (height - 1) / 2)
        p = config.params_for(wl, value_capacity=1 << 17, bucket_count=1 << 16)
    v = Volume(p)
    for i in frames:
        v.integrate_frame(wl.frame(i), wl.pose(i))
    return wl, p, v


def _oracles(p, v):
    pos, f = v.dump_blocks()
    out = []
    for fp64 in (False, True):
        o = Oracle(p, fp64=fp64)
        o.set_blocks(pos, f["sdf"], f["w"], f["a"], f["b"])
        out.append(o)
    return out


def _gpu_backward(v, cTw, a, b=None):
    import torch
    H, W = a.shape
    da = torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()
    db = None
    if b is not None:
        bb = np.zeros((H, W, 4), np.float32)
        bb[..., :3] = b
        db = torch.from_numpy(bb).cuda()
    g = torch.zeros(v.params.value_capacity * 512, dtype=torch.float32, device="cuda")
    xi = v.raycast_backward(cTw, da, db, g)
    torch.cuda.synchronize()
    pos, rows = v.dump_block_field(g)
    keep = np.abs(rows).sum(axis=1) > 0
    return xi, pos[keep], rows[keep]


def _dense(pos, rows):
    return {tuple(int(c) for c in q): r for q, r in zip(pos, rows)}


def test_backward_matches_oracle(built):
    torch = pytest.importorskip("torch")  # noqa: F841
    wl, p, v = _setup()
    T = wl.pose(34).astype(np.float64)
    cTw = np.linalg.inv(T).astype(np.float32)
    o32, o64 = _oracles(p, v)
    d, _, n = v.raycast(cTw)
    hit = np.isfinite(d)
    assert hit.sum() > 5000
    rng = np.random.default_rng(3)
    a = np.where(hit, rng.standard_normal(d.shape), 0.0).astype(np.float32)
    b = np.where(hit[..., None], rng.standard_normal(d.shape + (3,)), 0.0).astype(np.float32)
    xi_g, gp, gr = _gpu_backward(v, cTw, a, b)
    xi_32 = o32.raycast_backward(cTw, a, b)
    xi_64 = o64.raycast_backward(cTw, a, b)
    # same single-precision arithmetic per pixel; sums in another order
    assert np.all(np.abs(xi_g - xi_32) <= 1e-3 * np.abs(xi_32) + 1e-4 * np.abs(xi_32).max()), (xi_g, xi_32)
    # against double precision along the same decisions: the normal terms
    # difference single-precision samples half a voxel apart, so they carry
    # the larger part of this gap (1.2 % of the largest component measured)
    rel64 = np.abs(xi_g - xi_64) / np.abs(xi_64).max()
    assert rel64.max() < 3e-2, (xi_g, xi_64)
    op, og = o32.grad_blocks()
    G, O = _dense(gp, gr), _dense(op, og)
    z = np.zeros(512)
    gmax = max(np.abs(r).max() for r in O.values())
    diff = max(np.abs(G.get(k, z) - O.get(k, z)).max() for k in set(G) | set(O))
    assert diff <= 1e-4 * gmax, (diff, gmax)


def test_backward_matches_central_differences(built):
    torch = pytest.importorskip("torch")  # noqa: F841
    wl, p, v = _setup()
    T = wl.pose(34).astype(np.float64)
    cTw = np.linalg.inv(T).astype(np.float32)
    o32, _ = _oracles(p, v)

    def render(T_):
        c = np.linalg.inv(T_).astype(np.float32)
        d, _, n = v.raycast(c)
        tr = o32.trace(c)
        tr[..., 1] = 0
        return d.astype(np.float64), n[..., :3].astype(np.float64), tr

    d0, n0, tr0 = render(T)
    hit = tr0[..., 0] == 1
    rng = np.random.default_rng(4)
    a = rng.standard_normal(d0.shape)
    for k in range(6):
        e = np.zeros(6)
        e[k] = H_FD
        dp, _, trp = render(left_update(T, e))
        dm, _, trm = render(left_update(T, -e))
        keep = hit & np.all(trp == tr0, axis=-1) & np.all(trm == tr0, axis=-1)
        keep &= np.abs(dp + dm - 2 * d0) <= 0.02 * np.abs(dp - dm) + 1e-6
        assert keep.sum() > 0.7 * hit.sum()
        with np.errstate(invalid="ignore"):
            fd = np.sum((a * (dp - dm))[keep]) / (2 * H_FD)
        xi, _, _ = _gpu_backward(v, cTw, np.where(keep, a, 0.0))
        quant = np.sum((np.abs(a) * np.spacing(d0.astype(np.float32)))[keep]) / (2 * H_FD)
        assert abs(xi[k] - fd) <= 2e-2 * abs(xi[k]) + quant, (k, xi[k], fd, quant)


def test_autograd_wrapper_pose_gradient(built):
    torch = pytest.importorskip("torch")
    from meshhashing_gb300.autograd import RaycastPose
    wl, p, v = _setup(width=128, height=96)
    T0 = wl.pose(34).astype(np.float64)
    xi = torch.zeros(6, dtype=torch.float64, requires_grad=True)
    depth, normal = RaycastPose.apply(xi, v, T0)
    w = torch.randn(depth.shape, generator=torch.Generator().manual_seed(5)).cuda()
    loss = (w * depth).sum()
    loss.backward()
    g = xi.grad.numpy()
    # the same quantity straight through the C ABI
    d = depth.detach().cpu().numpy()
    hit = d > 0
    xi_c, _, _ = _gpu_backward(v, np.linalg.inv(T0).astype(np.float32), np.where(hit, w.cpu().numpy(), 0.0))
    np.testing.assert_allclose(g, xi_c, rtol=1e-6, atol=1e-9)
    # the normal output back-propagates too (its central-difference check is
    # the oracle test; here: same numbers as the C ABI)
    xi2 = torch.zeros(6, dtype=torch.float64, requires_grad=True)
    _, normal2 = RaycastPose.apply(xi2, v, T0)
    wn = torch.randn(normal2.shape, generator=torch.Generator().manual_seed(6)).cuda()
    (wn * normal2).sum().backward()
    xi_n, _, _ = _gpu_backward(v, np.linalg.inv(T0).astype(np.float32), np.zeros(d.shape),
                               np.where(hit[..., None], wn.cpu().numpy(), 0.0))
    np.testing.assert_allclose(xi2.grad.numpy(), xi_n, rtol=1e-5, atol=1e-6)


def test_refine_pose_from_perturbed_start(built):
    """Frame-to-model Gauss-Newton (mh_refine_pose): perturbations of sigma
    1 degree / 2 cm per axis around the true pose, 10 iterations, against the
    plain-TSDF model (8 mm voxels, 24 mm truncation) of the preceding frames.
    Starts up to 8 cm / 2.6 degree off must end within 6 mm / 0.15 degree
    (the depth noise is sigma 1 cm at 3 m; the fused surface carries part of
    it, so the optimum is not exactly the true pose)."""
    torch = pytest.importorskip("torch")  # noqa: F841
    wl = scene.small_circle(60)
    p = config.params_for(wl, value_capacity=1 << 17, bucket_count=1 << 16)
    v = Volume(p)
    for i in range(0, 36, 2):
        v.integrate_frame(wl.frame(i), wl.pose(i))
    rng = np.random.default_rng(6)
    for fi in (38, 42, 46):
        T_true = wl.pose(fi).astype(np.float64)
        xi = np.concatenate([rng.standard_normal(3) * 0.02, rng.standard_normal(3) * np.radians(1.0)])
        T_start = left_update(T_true, xi)
        v.set_frame(wl.frame(fi), T_start)
        T_ref, cost, count = v.refine_pose(T_start, iterations=10, max_residual=0.05)
        assert count > 10000
        tb, rb = pose_error(T_start, T_true)
        ta, ra = pose_error(T_ref, T_true)
        assert ta < 0.006 and ra < 0.15, (fi, (tb, rb), (ta, ra))


def test_autograd_gradcheck_pose_and_voxel_sdf(built):
    """torch.autograd.gradcheck of rendered depth with respect to the pose
    increment and up to eight voxel sdf values together (RaycastPoseSdf),
    against central differences (h = 1e-4) of the GPU's own forward; the
    procedure is tests/_gradcheck.py's."""
    pytest.importorskip("torch")
    from tests._gradcheck import check_pose_sdf
    wl, p, v = _setup(width=128, height=96)

    def block_grad(v, cTw, a):
        _, gp, gr = _gpu_backward(v, cTw, a)
        return gp, gr

    check_pose_sdf(v, wl.pose(34), block_grad, "cuda")
