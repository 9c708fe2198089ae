"""Run the golden-fixture chains (tests/golden/make_golden.py) on an
implementation and compare with the reference's recorded outputs."""
import os

import numpy as np

from meshhashing_gb300 import config, scene
from tests._util import mesh_canon, pos_set

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    with np.load(os.path.join(GOLDEN, name)) as z:
        return {k: z[k] for k in z.files}


def simple_params():
    wl = scene.small_circle(60)
    f = 262.5 * 96 / 320
    wl.camera = scene.Camera(96, 72, f, f, 47.5, 35.5)
    return config.params_for(wl, value_capacity=1 << 14, bucket_count=1 << 14, max_vertex_count=1 << 16,
                             max_triangle_count=1 << 16, weight_sample=1000, compat_arithmetic=1)


def psdf_params():
    wl = scene.full_spline(40, width=96, height=72)
    return config.params_for(wl, value_capacity=1 << 15, bucket_count=1 << 17, max_vertex_count=1 << 16,
                             max_triangle_count=1 << 16, compat_arithmetic=1)


class OracleRunner:
    def __init__(self, params):
        from oracle.oracle import Oracle
        self.o = Oracle(params, fp64=False)

    def frame(self, d, T, psdf=False):
        o = self.o
        o.frame_set(d, T)
        o.allocate()
        n = o.block_count()
        o.collect_frustum()
        if psdf:
            o.predict_inlier()
            o.integrate_psdf()
        else:
            o.integrate_simple()
        o.mesh()
        o.gc_low_surfel()
        return n

    def blocks(self):
        pos, s, w, a, b = self.o.blocks()
        return pos, dict(sdf=s, w=w, a=a, b=b)

    def candidates(self):
        return self.o.candidates()

    def mesh(self):
        return self.o.dump_mesh()

    def cubes(self, pos):
        return self.o.cubes(pos)

    def raycast(self, cTw):
        d, _, n = self.o.raycast(cTw)
        return d, n

    def inlier(self):
        return self.o.inlier()

    def track_equations(self, depth, T):
        self.o.frame_set(depth, T)
        return self.o.point_to_psdf(T, fix_jacobian=False)

    def compact(self):
        """The oracle's mesh as compact arrays: the vertices its triangles
        use, the triangles as indices into them, the vertices' summed
        reference counts."""
        vk, vd, tr = self.o.dump_mesh()
        used = np.unique(tr[:, 4:7].reshape(-1))
        remap = -np.ones(len(vd) + 1, np.int64)
        remap[used] = np.arange(len(used))
        return vd[used, :3], remap[tr[:, 4:7]], int(vd[used, 7].sum())


class GpuRunner:
    def __init__(self, params):
        from meshhashing_gb300 import Volume
        self.v = Volume(params)

    def frame(self, d, T, psdf=False):
        v = self.v
        v.set_frame(d, T)
        v.alloc_block_array()
        n = v.stats()["blocks_allocated"]
        v.collect_blocks_in_frustum()
        if psdf:
            v.predict_outlier_ratio()
            v.update_blocks_bayesian()
        else:
            v.update_blocks_simple()
        v.marching_cubes()
        v.collect_low_surfel_blocks()
        return n

    def blocks(self):
        return self.v.dump_blocks()

    def candidates(self):
        return self.v.candidates()

    def mesh(self):
        return self.v.dump_mesh()

    def cubes(self, pos):
        return self.v.cubes(pos)

    def raycast(self, cTw):
        d, _, n = self.v.raycast(cTw)
        return d, n

    def inlier(self):
        return self.v.inlier()

    def track_equations(self, depth, T):
        self.v.set_frame(depth, T)
        return self.v.point_to_psdf(T, reference_jacobian=True)

    def compact(self):
        """mh_mesh_compact's arrays and the summed reference counts of the
        vertices it kept (read from the pools)."""
        pos, _, tri = self.v.compact_mesh()
        vk, vd, tr = self.v.dump_mesh()
        vref = int(vd[np.unique(tr[:, 4:7].reshape(-1)), 7].sum())
        return pos, tri, vref


def _canonical(pos, tri):
    """Triangles as 9-vectors of vertex positions, rotated so the
    lexicographically smallest corner comes first (orientation kept)."""
    t = pos[np.asarray(tri, np.int64)]                      # (n, 3, 3)
    keys = [tuple(map(tuple, x)) for x in t.tolist()]
    out = np.empty((len(t), 9), np.float64)
    for i, k in enumerate(keys):
        j = k.index(min(k))
        out[i] = np.array(k[j:] + k[:j], np.float64).reshape(9)
    return out


def check_compress(runner_cls):
    """CompressMesh (visualization/compress_mesh.cu) on the simple chain's
    map: the same triangle and vertex counts and summed reference counts as
    the reference; the triangles as a multiset of vertex-position triples are
    identical except where a corner is a vertex the reference's last writer
    snapped to the other end of its edge, exactly one voxel away."""
    from scipy.spatial import cKDTree
    fx = load("compress_room96.npz")
    r = runner_cls(simple_params())
    for d, T in zip(fx["depth"], fx["poses"]):
        r.frame(d, T)
    pos, tri, vref = r.compact()
    nt, nv, nref = (int(x) for x in fx["stats"])
    assert nref == 3 * nt
    assert (len(tri), len(pos), vref) == (nt, nv, nref)
    vs = float(simple_params().voxel_size)
    a, b = _canonical(fx["pos"], fx["tris"]), _canonical(pos, tri)
    # triangles as a multiset (degenerate ones, all corners snapped onto one
    # point, repeat): those equal to 1e-5 voxel pair off directly
    from collections import Counter
    ka = [tuple(x) for x in np.round(a / (1e-5 * vs)).astype(np.int64)]
    kb = [tuple(x) for x in np.round(b / (1e-5 * vs)).astype(np.int64)]
    ca, cb = Counter(ka), Counter(kb)
    same = sum((ca & cb).values())
    rest_a = np.array(list((ca - cb).elements()), np.float64).reshape(-1, 9) * (1e-5 * vs)
    rest_b = np.array(list((cb - ca).elements()), np.float64).reshape(-1, 9) * (1e-5 * vs)
    assert len(rest_a) == len(rest_b)
    if len(rest_a):
        d, j = cKDTree(rest_b).query(rest_a, p=np.inf)
        assert np.all(d <= 1.0001 * vs), d.max()
        # per corner: within 1e-4 voxel, or exactly one voxel away (the other
        # end of the edge, where the reference's last writer snapped it)
        corner = np.abs(rest_a - rest_b[j]).reshape(-1, 3, 3).max(axis=2)
        off = corner > 1e-4 * vs
        assert np.all(np.abs(corner[off] - vs) <= 1e-4 * vs)
    # the share of snapped vertices itself is bounded by check_simple, which
    # pairs vertices by owner key on the same chain; here at least 85 % of
    # the triangles are identical as position triples (90.6 % measured)
    assert same >= 0.85 * nt, same / nt
    return nt, same / nt


def rows(pos, field, want):
    idx = {tuple(int(c) for c in p): i for i, p in enumerate(pos)}
    return np.stack([field[idx[tuple(int(c) for c in p)]] for p in want])


def check_simple(runner_cls):
    fx = load("simple_room96.npz")
    r = runner_cls(simple_params())
    counts = [r.frame(d, T) for d, T in zip(fx["depth"], fx["poses"])]
    np.testing.assert_array_equal(counts, fx["counts"])
    pos, f = r.blocks()
    assert pos_set(pos) == pos_set(fx["blocks"])
    assert pos_set(r.candidates()) == pos_set(fx["candidates"])
    # voxel values of the sampled blocks: bit-identical to the reference
    np.testing.assert_array_equal(rows(pos, f["sdf"], fx["sample_pos"]), fx["sample_sdf"])
    np.testing.assert_array_equal(rows(pos, f["w"], fx["sample_pos"]), fx["sample_w"])
    # cube indices (a cube without surface, 0 or 255, may be stored as 0)
    got = r.cubes(fx["sample_pos"])
    want = fx["cubes"]
    np.testing.assert_array_equal(np.where(got == 255, 0, got), np.where(want == 255, 0, want))
    # mesh topology identical; positions identical except where the reference's
    # last writer snapped a shared vertex to the other end of its edge
    vk, vd, tr = r.mesh()
    gv, gt = mesh_canon(vk, vd, tr)
    rvd = np.concatenate([fx["vpos"], np.zeros((len(fx["vpos"]), 4), np.float32),
                          fx["vref"][:, None].astype(np.float32)], axis=1)
    rv, rt = mesh_canon(fx["vkeys"], rvd, fx["tris"])
    assert len(rt) > 0
    assert set(gv) == set(rv), "vertex sets differ"
    assert gt == rt, "triangle topology differs"
    # (the edge endpoints enter VertexIntersection in the writing cube's order,
    # so unsnapped positions may also differ in the last bits)
    vs = float(simple_params().voxel_size)
    other_end = 0
    for k in rv:
        d = np.abs(gv[k][:3] - rv[k][:3])
        if d.max() < 1e-4 * vs:
            continue
        off = np.zeros(3, np.float32)
        off[k[3]] = vs
        assert np.allclose(d, off, atol=1e-4 * vs), (k, d)
        other_end += 1
    assert other_end <= 0.05 * len(rv), other_end
    assert all(gv[k][7] == rv[k][7] for k in rv), "reference counts differ"
    # raycast: same hits, same depth bits
    d, n = r.raycast(fx["ray_cTw"])
    hit = np.isfinite(fx["ray_depth"])
    np.testing.assert_array_equal(np.isfinite(d), hit)
    np.testing.assert_array_equal(d[hit], fx["ray_depth"][hit])
    assert np.abs(n[..., :3][hit] - fx["ray_normal"][hit]).max() < 1e-6
    return len(rt), other_end


def check_psdf(runner_cls):
    fx = load("psdf_room96.npz")
    r = runner_cls(psdf_params())
    counts = [r.frame(d, T, psdf=True) for d, T in zip(fx["depth"], fx["poses"])]
    np.testing.assert_array_equal(counts, fx["counts"])
    pos, f = r.blocks()
    assert pos_set(pos) == pos_set(fx["blocks"])
    worst = 0.0
    for k in ("sdf", "w", "a", "b"):
        got, want = rows(pos, f[k], fx["sample_pos"]), fx["sample_" + k]
        scale = np.maximum(np.abs(want), 1e-3 if k == "sdf" else 1.0)
        rel = float((np.abs(got - want) / scale).max())
        worst = max(worst, rel)
        # expf is not correctly rounded on either side: a few ulp apart
        assert rel < 1e-5, (k, rel)
    got = r.inlier()
    assert np.abs(got - fx["inlier"]).max() < 1e-5
    return worst


def check_huber(impl):
    """PrimalDualInit + iterations on the fixture's cluster.  impl(params,
    pos, sdf, w, cand) returns an object with iterate(lam, sigma, tau) ->
    [total, data, tv] and sdf(cand) -> rows.  Energies are checked here
    against the reference's float sums; returns (final sdf, the reference's
    final sdf, the cluster's sdf before) for the caller's precision checks."""
    fx = load("huber_room96.npz")
    lam, sigma, tau, iters = (float(x) for x in fx["hparams"])
    h = impl(simple_params(), fx["pre_pos"], fx["pre_sdf"], fx["pre_w"], fx["cand"])
    for k in range(int(iters)):
        e = h.iterate(lam, sigma, tau)
        # the reference adds single-precision values one by one
        np.testing.assert_allclose(e[1:], fx["errs"][k], rtol=1e-4, atol=1e-12)
    before = rows(fx["pre_pos"], fx["pre_sdf"], fx["cand"])
    assert np.count_nonzero(fx["post_sdf"] != before) > 5000
    return h.sdf(fx["cand"]), fx["post_sdf"], before


def check_track(runner_cls):
    """The reference's tracker equations (PointToSurface, with its J[2] =
    dD/dx) at the fixture's poses over the simple chain's map: the same
    pixels contribute; A, b and err agree to float summation (the reference
    adds floats one by one)."""
    fx, sc = load("track_room96.npz"), load("simple_room96.npz")
    r = runner_cls(simple_params())
    for d, T in zip(sc["depth"], sc["poses"]):
        r.frame(d, T)
    for k, T in enumerate(fx["poses"]):
        A, b, e, n = r.track_equations(fx["depth"], T)
        assert n == fx["count"][k] and n > 1000
        assert np.abs(A - fx["A"][k]).max() <= 1e-5 * np.abs(fx["A"][k]).max()
        assert np.abs(b - fx["b"][k]).max() <= 1e-5 * np.abs(fx["b"][k]).max()
        assert abs(e - fx["err"][k]) <= 1e-5 * fx["err"][k]
        # the reference's Jacobian repeats dD/dx in place of dD/dz
        np.testing.assert_array_equal(A[:, 2], A[:, 0])
