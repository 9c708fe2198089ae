"""The torch.autograd wrappers of the differentiable raycast on the CPU, with
the single-precision oracle behind the Volume methods they call
(tests/_gradcheck.py's OracleVolume): gradcheck over the pose and voxel sdf
values, and the pose-only wrapper against the oracle's backward.  This covers
the wrappers' own logic (voxel writes, the pool-index map of SdfVoxels,
gradient routing) without a GPU; the GPU test runs the same procedure
through the C ABI."""
import numpy as np
import pytest

from meshhashing_gb300 import config, scene
from oracle import oracle as O
from tests._gradcheck import OracleVolume, check_pose_sdf


def _map(width=128, height=96):
    wl = scene.small_circle(60)
    f = 262.5 * width / 320
    wl.camera = scene.Camera(width, height, f, f, (width - 1) / 2, (height - 1) / 2)
    p = config.params_for(wl, value_capacity=1 << 17, bucket_count=1 << 16)
    o = O.Oracle(p, fp64=False)
    for i in range(0, 32, 4):
        o.frame(wl.frame(i), wl.pose(i))
    return wl, p, o


def _block_grad(v, cTw, a):
    import torch
    g = torch.zeros(v.params.value_capacity * 512, dtype=torch.float32)
    v.raycast_backward(cTw, torch.from_numpy(np.ascontiguousarray(a, np.float32)), None, g)
    pos, rows = v.dump_block_field(g)
    keep = np.abs(rows).sum(axis=1) > 0
    return pos[keep], rows[keep]


def test_gradcheck_pose_and_voxel_sdf_on_oracle(built):
    pytest.importorskip("torch")
    wl, p, o = _map()
    check_pose_sdf(OracleVolume(p, o), wl.pose(34), _block_grad, "cpu")


def test_pose_wrapper_matches_oracle_backward(built):
    torch = pytest.importorskip("torch")
    from meshhashing_gb300.autograd import RaycastPose
    wl, p, o = _map(96, 72)
    v = OracleVolume(p, o)
    T0 = wl.pose(34).astype(np.float64)
    xi = torch.zeros(6, dtype=torch.float64, requires_grad=True)
    depth, normal = RaycastPose.apply(xi, v, T0)
    w = torch.randn(depth.shape, generator=torch.Generator().manual_seed(5))
    (w * depth).sum().backward()
    d = depth.detach().numpy()
    want = o.raycast_backward(np.linalg.inv(T0).astype(np.float32), np.where(d > 0, w.numpy(), 0.0))
    np.testing.assert_allclose(xi.grad.numpy(), want, rtol=1e-6, atol=1e-9)
