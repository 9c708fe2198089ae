"""torch.autograd wrappers of the differentiable raycast, for gradient checks.

RaycastPose renders depth and camera-frame normals of a Volume from the pose
exp(xi) @ wTc0 (xi: a 6-vector, translation first) and back-propagates
through mh_raycast_backward.  RaycastPoseSdf adds a set of voxel sdf values
as a second torch input (SdfVoxels names the voxels): its forward writes the
values into the volume before rendering, its backward returns dL/dxi and
dL/dsdf of those voxels from the same backward kernel.  The pose gradient is
with respect to a left increment at the rendered pose, i.e. exact at xi = 0,
where Gauss-Newton steps and finite-difference checks evaluate it.
"""
from __future__ import annotations

import numpy as np

from .pose import left_update


def _torch():
    import torch
    return torch


def _device(volume):
    return getattr(volume, "torch_device", "cuda")


class SdfVoxels:
    """Voxels of a Volume whose sdf values form one torch input.

    voxels: (K, 4) integers, the block coordinates (x, y, z) and the voxel's
    index inside its block (x fastest, 0..511).  The blocks must be
    allocated.  The blocks' current sdf rows are kept on the host, so write()
    changes only the named voxels; gather() picks their entries out of a
    per-voxel field laid out like the voxel storage (the grad_sdf of
    mh_raycast_backward)."""

    def __init__(self, volume, voxels):
        torch = _torch()
        self.volume = volume
        vox = np.asarray(voxels, np.int64).reshape(-1, 4)
        if np.any(vox[:, 3] < 0) or np.any(vox[:, 3] >= 512):
            raise ValueError("voxel index outside 0..511")
        self.blocks, inv = np.unique(vox[:, :3], axis=0, return_inverse=True)
        self.row_of = inv.reshape(-1)
        self.vidx = vox[:, 3]
        pos, f = volume.dump_blocks(fields=("sdf",))
        lut = {tuple(q): i for i, q in enumerate(pos.tolist())}
        missing = [b for b in self.blocks.tolist() if tuple(b) not in lut]
        if missing:
            raise ValueError(f"blocks not allocated: {missing[:4]}")
        self.rows = np.stack([f["sdf"][lut[tuple(b)]] for b in self.blocks.tolist()]).astype(np.float32)
        # pool index of each block: a field whose first voxel of pool entry i holds i
        cap = volume.params.value_capacity
        dev = _device(volume)
        probe = torch.zeros((cap, 512), dtype=torch.float32, device=dev)
        probe[:, 0] = torch.arange(cap, dtype=torch.float32, device=dev)
        ppos, prows = volume.dump_block_field(probe)
        pool = {tuple(q): int(r[0]) for q, r in zip(ppos.tolist(), prows)}
        block_pool = np.array([pool[tuple(b)] for b in self.blocks.tolist()], np.int64)
        self.flat = torch.from_numpy(block_pool[self.row_of] * 512 + self.vidx).to(dev)

    def values(self) -> np.ndarray:
        """The voxels' current sdf values (float32)."""
        return self.rows[self.row_of, self.vidx].copy()

    def write(self, values):
        rows = self.rows.copy()
        rows[self.row_of, self.vidx] = np.asarray(values, np.float32).reshape(-1)
        self.volume.load_blocks(self.blocks, sdf=rows)

    def gather(self, field):
        return field.reshape(-1)[self.flat]


def _render(volume, xi, wTc0):
    torch = _torch()
    T = left_update(np.asarray(wTc0, np.float64), xi.detach().cpu().numpy().astype(np.float64))
    cTw = np.linalg.inv(T).astype(np.float32)
    H, W, dev = volume.RH, volume.RW, _device(volume)
    depth = torch.empty((H, W), dtype=torch.float32, device=dev)
    normal = torch.empty((H, W, 4), dtype=torch.float32, device=dev)
    volume.raycast(cTw, depth_out=depth, normal_out=normal)
    hit = torch.isfinite(depth)
    return cTw, torch.where(hit, depth, torch.zeros_like(depth)), torch.where(
        hit[..., None], normal[..., :3], torch.zeros_like(normal[..., :3]))


def _backward(volume, cTw, g_depth, g_normal, grad_sdf=None):
    torch = _torch()
    H, W, dev = volume.RH, volume.RW, _device(volume)
    gd = g_depth.contiguous().float() if g_depth is not None else torch.zeros((H, W), dtype=torch.float32,
                                                                               device=dev)
    gn = None
    if g_normal is not None:
        gn = torch.zeros((H, W, 4), dtype=torch.float32, device=dev)
        gn[..., :3] = g_normal
    return volume.raycast_backward(cTw, gd, gn, grad_sdf)


class RaycastPose:
    """RaycastPose.apply(xi, volume, wTc0) -> (depth (H, W), normal (H, W, 3))."""

    @staticmethod
    def apply(xi, volume, wTc0):
        return _functions()[0].apply(xi, volume, wTc0)


class RaycastPoseSdf:
    """RaycastPoseSdf.apply(xi, sdf, voxels: SdfVoxels, wTc0) -> (depth, normal)
    rendered at exp(xi) wTc0 after the voxels' sdf is set to `sdf` (K,)."""

    @staticmethod
    def apply(xi, sdf, voxels, wTc0):
        return _functions()[1].apply(xi, sdf, voxels, wTc0)


_FN = None


def _functions():
    global _FN
    if _FN is not None:
        return _FN
    torch = _torch()

    class _RaycastPose(torch.autograd.Function):
        @staticmethod
        def forward(ctx, xi, volume, wTc0):
            ctx.cTw, depth, normal = _render(volume, xi, wTc0)
            ctx.volume = volume
            ctx.xi_dtype, ctx.xi_device = xi.dtype, xi.device
            return depth, normal

        @staticmethod
        def backward(ctx, g_depth, g_normal):
            dxi = _backward(ctx.volume, ctx.cTw, g_depth, g_normal)
            return torch.tensor(dxi, dtype=ctx.xi_dtype, device=ctx.xi_device), None, None

    class _RaycastPoseSdf(torch.autograd.Function):
        @staticmethod
        def forward(ctx, xi, sdf, voxels, wTc0):
            voxels.write(sdf.detach().cpu().numpy())
            ctx.cTw, depth, normal = _render(voxels.volume, xi, wTc0)
            ctx.voxels = voxels
            ctx.xi_dtype, ctx.xi_device = xi.dtype, xi.device
            ctx.sdf_dtype, ctx.sdf_device = sdf.dtype, sdf.device
            return depth, normal

        @staticmethod
        def backward(ctx, g_depth, g_normal):
            v = ctx.voxels.volume
            g = torch.zeros(v.params.value_capacity * 512, dtype=torch.float32, device=_device(v))
            dxi = _backward(v, ctx.cTw, g_depth, g_normal, g)
            gs = ctx.voxels.gather(g).to(dtype=ctx.sdf_dtype, device=ctx.sdf_device)
            return torch.tensor(dxi, dtype=ctx.xi_dtype, device=ctx.xi_device), gs, None, None

    _FN = (_RaycastPose, _RaycastPoseSdf)
    return _FN
