"""torch.autograd.gradcheck of the raycast over the pose and voxel sdf values
(RaycastPoseSdf), shared by the GPU test (a Volume) and the CPU test (the
FP32 oracle behind the same methods, OracleVolume below).

Procedure (check_pose_sdf):

* The sdf input enters as s0 + 0.3 z, so gradcheck's step (h = 1e-4) moves a
  voxel by 3e-5 m: the regula falsi divides sdf differences of a few
  millimetres, and a 1e-4 m step would bend the difference quotient by a few
  percent.
* Pixels closer than 3 m whose depth is smooth in the pose across the
  stencil (second difference within 1 % of the first: a kink inside the
  stencil, where the hit crosses a cell face, shows as a larger one) are drawn
  at random; each contributes the voxel with the largest sdf gradient of its
  depth among voxels with |sdf| >= 1e-4 m (no sign change under the step).
* The outputs are up to 12 pixels that those voxels move and 12 that they do
  not (zero sdf gradient), all smooth in every input (3 % for the sdf steps,
  which bend the regula falsi more).  The tolerance covers a few float32 ulps
  of those depths over the 2h stencil.
"""
import numpy as np

from meshhashing_gb300.pose import left_update

H_FD = 1e-4
SCALE = 0.3


def check_pose_sdf(v, T0, block_grad, device):
    """v: a Volume or a stand-in; block_grad(v, cTw, a) -> (positions, rows)
    of dL/dsdf for L = sum a * depth; device: where v's tensors live."""
    import torch
    from meshhashing_gb300.autograd import RaycastPoseSdf, SdfVoxels
    T0 = np.asarray(T0, np.float64)
    cTw = np.linalg.inv(T0).astype(np.float32)
    d0, _, _ = v.raycast(cTw)
    bpos, bf = v.dump_blocks(fields=("sdf",))
    rows = {tuple(q): r for q, r in zip(bpos.tolist(), bf["sdf"])}

    def smooth(dp, dm, c, rel):
        with np.errstate(invalid="ignore"):
            return np.isfinite(dp) & np.isfinite(dm) & (np.abs(dp + dm - 2 * c) <= 3e-6 + rel * np.abs(dp - dm))

    def render(xi):
        d, _, _ = v.raycast(np.linalg.inv(left_update(T0, xi)).astype(np.float32))
        return d.astype(np.float64)

    base = d0.astype(np.float64)
    keep = np.isfinite(base) & (base < 3.0)
    for k in range(6):
        e = np.zeros(6)
        e[k] = H_FD
        keep &= smooth(render(e), render(-e), base, 0.01)
    rng = np.random.default_rng(7)
    vox = []
    for px in rng.choice(np.flatnonzero(keep.reshape(-1)), 16, replace=False):
        a = np.zeros(base.size)
        a[px] = 1.0
        gp, gr = block_grad(v, cTw, a.reshape(base.shape))
        sdf_of = np.stack([rows[tuple(q)] for q in gp.tolist()]).reshape(-1)
        score = np.where(np.abs(sdf_of) >= 1e-4, np.abs(gr).reshape(-1), 0.0)
        j = int(np.argmax(score))
        cand = [*gp[j // 512], j % 512]
        if score[j] > 0 and cand not in vox:
            vox.append(cand)
        if len(vox) == 8:
            break
    assert len(vox) >= 4
    sv = SdfVoxels(v, np.array(vox))
    s0 = sv.values().astype(np.float64)

    def depth_at(s):
        sv.write(s)
        return render(np.zeros(6))

    np.testing.assert_array_equal(depth_at(s0), base)
    sens = np.zeros_like(base)
    for k in range(len(s0)):
        dd = []
        for sign in (1.0, -1.0):
            s = s0.copy()
            s[k] += sign * SCALE * H_FD
            dd.append(depth_at(s))
        dp, dm = dd
        keep &= smooth(dp, dm, base, 0.03)
        with np.errstate(invalid="ignore"):
            sens = np.maximum(sens, np.where(keep, np.abs(dp - dm), 0.0))
    sv.write(s0)
    moved = np.flatnonzero(keep.reshape(-1) & (sens.reshape(-1) > 2e-6))
    still = np.flatnonzero(keep.reshape(-1) & (sens.reshape(-1) == 0))
    assert len(moved) >= 4 and len(still) >= 12, (len(moved), len(still))
    pix = torch.from_numpy(np.concatenate([rng.choice(moved, min(12, len(moved)), replace=False),
                                           rng.choice(still, 12, replace=False)])).to(device)
    s0_t = torch.tensor(s0, dtype=torch.float64)

    def f(xi, z):
        d, _ = RaycastPoseSdf.apply(xi, s0_t + SCALE * z, sv, T0)
        return d.reshape(-1)[pix].double().cpu()

    xi = torch.zeros(6, dtype=torch.float64, requires_grad=True)
    z = torch.zeros(len(s0), dtype=torch.float64, requires_grad=True)
    try:
        ok = torch.autograd.gradcheck(f, (xi, z), eps=H_FD, atol=1e-2, rtol=3e-2, nondet_tol=1e-6)
    finally:
        sv.write(s0)
    assert ok
    # the sdf gradient reaches the moved pixels
    d, _ = RaycastPoseSdf.apply(xi, s0_t + SCALE * z, sv, T0)
    d.reshape(-1)[pix[:4]].sum().backward()
    sv.write(s0)
    assert np.abs(z.grad.numpy()).max() > 1e-3


class OracleVolume:
    """The methods of meshhashing_gb300.Volume that the autograd wrappers
    call, served by an oracle on the CPU (torch tensors on the CPU).  Its
    "pool" order is the oracle's block order at construction; blocks added
    later are not supported."""

    torch_device = "cpu"

    def __init__(self, params, oracle):
        self.params, self.o = params, oracle
        self.RW, self.RH = params.rc_width, params.rc_height
        self.order = [tuple(q) for q in oracle.blocks()[0].tolist()]
        self.index = {q: i for i, q in enumerate(self.order)}

    def raycast(self, cTw, depth_out=None, vertex_out=None, normal_out=None):
        import torch
        d, v, n = self.o.raycast(cTw)
        if depth_out is None and vertex_out is None and normal_out is None:
            return d, v, n
        for out, x in ((depth_out, d), (vertex_out, v), (normal_out, n)):
            if out is not None:
                out.copy_(torch.from_numpy(x))
        return None

    def dump_blocks(self, fields=("sdf", "w", "a", "b")):
        pos, s, w, a, b = self.o.blocks()
        m = {"sdf": s, "w": w, "a": a, "b": b}
        return pos, {f: m[f] for f in fields}

    def load_blocks(self, pos, sdf=None, w=None, a=None, b=None):
        P, s0, w0, a0, b0 = self.o.blocks()
        idx = {tuple(q): i for i, q in enumerate(P.tolist())}
        r = [idx[tuple(q)] for q in np.asarray(pos).tolist()]
        self.o.set_blocks(np.asarray(pos, np.int32), *[x0[r] if x is None else np.asarray(x, np.float32)
                                                        for x, x0 in ((sdf, s0), (w, w0), (a, a0), (b, b0))])

    def dump_block_field(self, field):
        f = field.reshape(-1, 512).cpu().numpy()
        return np.array(self.order, np.int32), f[:len(self.order)].copy()

    def raycast_backward(self, cTw, dL_ddepth, dL_dnormal=None, grad_sdf=None):
        import torch
        a = dL_ddepth.cpu().numpy()
        b = None if dL_dnormal is None else dL_dnormal[..., :3].cpu().numpy()
        xi = self.o.raycast_backward(cTw, a, b)
        if grad_sdf is not None:
            gp, gk = self.o.grad_blocks()
            G = grad_sdf.view(-1, 512)
            for q, row in zip(gp.tolist(), gk):
                G[self.index[tuple(q)]] += torch.from_numpy(row.astype(np.float32))
        return xi
