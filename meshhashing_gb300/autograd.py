"""torch.autograd wrapper of the differentiable raycast, for gradient checks.

RaycastPose renders depth and camera-frame normals of a Volume from the pose
exp(xi) @ wTc0 (xi: a 6-vector, translation first) and back-propagates
through mh_raycast_backward.  The returned gradient is with respect to a left
increment at the rendered pose, i.e. exact at xi = 0, where Gauss-Newton
steps and finite-difference checks evaluate it.  The voxel sdf values are
not a torch input (they live in the library's storage); their gradient is
available from Volume.raycast_backward(grad_sdf=...).
"""
from __future__ import annotations

import numpy as np

from .pose import left_update


def _torch():
    import torch
    return torch


class RaycastPose:
    """RaycastPose.apply(xi, volume, wTc0) -> (depth (H, W), normal (H, W, 3))."""

    @staticmethod
    def apply(xi, volume, wTc0):
        return _function().apply(xi, volume, wTc0)


_FN = None


def _function():
    global _FN
    if _FN is not None:
        return _FN
    torch = _torch()

    class _RaycastPose(torch.autograd.Function):
        @staticmethod
        def forward(ctx, xi, volume, wTc0):
            T = left_update(np.asarray(wTc0, np.float64), xi.detach().cpu().numpy().astype(np.float64))
            cTw = np.linalg.inv(T).astype(np.float32)
            H, W = volume.RH, volume.RW
            depth = torch.empty((H, W), dtype=torch.float32, device="cuda")
            normal = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
            volume.raycast(cTw, depth_out=depth, normal_out=normal)
            ctx.volume, ctx.cTw = volume, cTw
            ctx.xi_dtype, ctx.xi_device = xi.dtype, xi.device
            hit = torch.isfinite(depth)
            return torch.where(hit, depth, torch.zeros_like(depth)), torch.where(
                hit[..., None], normal[..., :3], torch.zeros_like(normal[..., :3]))

        @staticmethod
        def backward(ctx, g_depth, g_normal):
            gd = g_depth.contiguous().float() if g_depth is not None else None
            gn = None
            if g_normal is not None:
                gn = torch.zeros(g_normal.shape[:-1] + (4,), dtype=torch.float32, device="cuda")
                gn[..., :3] = g_normal
            if gd is None:
                gd = torch.zeros(gn.shape[:-1], dtype=torch.float32, device="cuda")
            dxi = ctx.volume.raycast_backward(ctx.cTw, gd, gn)
            return torch.tensor(dxi, dtype=ctx.xi_dtype, device=ctx.xi_device), None, None

    _FN = _RaycastPose
    return _FN
