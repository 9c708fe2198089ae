"""CPU tests: the oracle, the case tables, the scene generator and the ABI.

Nothing here needs a GPU; the C library is only loaded and its exports
checked, no compute entry point is called.
"""
import os
import re

import numpy as np
import pytest

from meshhashing_gb300 import config, scene
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
from oracle.refcpu import reference_dir

REF = reference_dir()


def teschner(x, y, z, n):
    h = ((x * 73856093) & 0xFFFFFFFF) ^ ((y * 19349669) & 0xFFFFFFFF) ^ ((z * 83492791) & 0xFFFFFFFF)
    return h % n


def test_hash_bucket_int32_wrap(built):
    rng = np.random.default_rng(0)
    for _ in range(2000):
        x, y, z = (int(v) for v in rng.integers(-(1 << 20), 1 << 20, 3))
        for n in (1 << 18, 1 << 21, 40000):
            assert O.hash_bucket(x, y, z, n) == teschner(x, y, z, n)
    # values that overflow int32 in the products
    assert O.hash_bucket(100000, -100000, 77777, 1 << 21) == teschner(100000, -100000, 77777, 1 << 21)


def test_capi_exports_every_declared_symbol(built):
    import ctypes
    from meshhashing_gb300 import _lib
    hdr = open(os.path.join(ROOT, "include", "meshhash.h")).read()
    declared = sorted(set(re.findall(r"^(?:int|uint32_t|uint64_t)\s+(mh_[a-z0-9_]+)\s*\(", hdr, re.M)))
    lib = ctypes.CDLL(_lib.LIB_PATH)
    missing = [s for s in declared if not hasattr(lib, s)]
    assert not missing, missing
    assert set(declared) == set(_lib.SYMBOLS)


def test_inverse_matches_numpy(built):
    w = scene.full_spline(5)
    for i in range(5):
        T = w.pose(i)
        inv = O.inverse(T)
        np.testing.assert_allclose(inv, np.linalg.inv(T.astype(np.float64)), atol=2e-6)


def _ref_table(name, shape):
    src = open(os.path.join(REF, "src/meshing/mc_tables.h")).read()
    i = src.index(name)
    body = src[src.index("=", i):src.index("};", i)]
    nums = [int(x, 0) for x in re.findall(r"-?0x[0-9a-fA-F]+|-?\d+", body)]
    return np.array(nums).reshape(shape)


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference sources not present")
def test_mc_case_table_matches_reference():
    from meshhashing_gb300.csrc import gen_mc_cases  # noqa: F401  (module has no side effects)
    tri = _ref_table("kTriangleVertexEdge", (256, 16))
    inc = open(os.path.join(ROOT, "meshhashing_gb300/csrc/mc_cases.inc")).read()
    words = [int(w, 16) for w in re.findall(r"0x([0-9a-f]{16})ull", inc)]
    assert len(words) == 256
    for c in range(256):
        n = words[c] & 0xF
        edges = [(words[c] >> (4 + 4 * k)) & 0xF for k in range(3 * n)]
        ref = [int(e) for e in tri[c] if e >= 0]
        assert edges == ref, c


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference sources not present")
def test_edge_and_owner_tables_match_reference():
    corner = [(0, 1, 1), (1, 1, 1), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 0, 0), (0, 0, 0)]
    ends = [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4), (4, 0), (5, 1), (6, 2), (7, 3)]
    edges_ref = _ref_table("kCubeEdges", (256,))
    for c in range(256):
        m = sum(1 << e for e, (a, b) in enumerate(ends) if ((c >> a) & 1) != ((c >> b) & 1))
        assert m == edges_ref[c]
    assert _ref_table("kVtxOffset", (8, 3)).tolist() == [list(v) for v in corner]
    assert _ref_table("kEdgeEndpointVertices", (12, 2)).tolist() == [list(e) for e in ends]
    owner_ref = _ref_table("kEdgeOwnerCubeOffset", (12, 4))
    for e, (a, b) in enumerate(ends):
        p, q = corner[a], corner[b]
        axis = [i for i in range(3) if p[i] != q[i]][0]
        lo = [min(p[i], q[i]) for i in range(3)]
        assert owner_ref[e].tolist() == lo + [axis]


def test_scene_is_deterministic():
    w = scene.full_spline(4, width=160, height=120)
    a, b = w.frame(2), w.frame(2)
    assert np.array_equal(a, b)
    valid = a > 0
    assert 0.9 < valid.mean() < 0.995        # ~2 % zeros
    speeds = [np.linalg.norm(w.poses[i + 1][:3, 3] - w.poses[i][:3, 3]) * 30 for i in range(3)]
    assert max(speeds) <= 0.5


def _run_oracle(fp64, n_frames=4, width=160, height=120, stride=5):
    wl = scene.small_circle(60)
    cam = scene.Camera(width, height, 262.5 * width / 320, 262.5 * width / 320, (width - 1) / 2, (height - 1) / 2)
    wl.camera = cam
    p = config.params_for(wl, value_capacity=1 << 15)
    o = O.Oracle(p, fp64=fp64)
    for i in range(n_frames):
        o.frame(wl.frame(i * stride), wl.pose(i * stride))
    return wl, p, o


def test_oracle_fp32_close_to_fp64(built):
    """Same start state, one update in each precision: only arithmetic differs."""
    wl, p, o32 = _run_oracle(False)
    o64 = O.Oracle(p, fp64=True)
    pos, s, w, a, b = o32.blocks()
    o64.set_blocks(pos, s, w, a, b)
    d, T = wl.frame(21), wl.pose(21)
    for o in (o32, o64):
        o.frame_set(d, T)
        o.set_candidates(pos)
        o.integrate_simple()
    p32, s32, w32, _, _ = o32.blocks()
    p64, s64, w64, _, _ = o64.blocks()
    from tests._util import align
    g, o, _ = align(p32, s32, p64, s64)
    gw, ow, _ = align(p32, w32, p64, w64)
    both = ow > 0
    assert both.sum() > 1000
    err = np.abs(g - o)[both]
    # FP32 rounding of camera-space depth (|z| < 4 m): a few ulp of 4 m
    assert err.max() < 2e-6, err.max()
    rel_w = np.abs(gw - ow)[both] / ow[both]
    assert rel_w.max() < 1e-5


def test_oracle_psdf_fp32_close_to_fp64(built):
    """One PSDF update from the same state and inlier image in each precision:
    the single-precision form (4 divisions, restated) against the
    reference's expressions evaluated in double.  Weights within 1e-5 and
    the inlier Beta parameters within 5e-6 relative (1.4e-6 measured: the
    restated a', b' avoid the cancellation of f^2 - e); sdf within 2e-6 m absolute, the
    rounding of a single-precision camera depth of a few metres, which both
    forms share (a relative bound is meaningless at the zero crossing)."""
    wl = scene.full_spline(40, width=160, height=120)
    p = config.params_for(wl, value_capacity=1 << 16)
    o32 = O.Oracle(p, fp64=False)
    for i in range(6):
        o32.frame_set(wl.frame(i), wl.pose(i))
        o32.allocate()
        o32.collect_frustum()
        o32.predict_inlier()
        o32.integrate_psdf()
        o32.mesh()
    d, T = wl.frame(6), wl.pose(6)
    o32.frame_set(d, T)
    o32.allocate()
    o32.collect_frustum()
    o32.predict_inlier()
    pos, s, w, a, b = o32.blocks()
    o64 = O.Oracle(p, fp64=True)
    o64.set_blocks(pos, s, w, a, b)
    o64.frame_set(d, T)
    o64.set_inlier(o32.inlier())
    o64.set_candidates(o32.candidates())
    o32.integrate_psdf()
    o64.integrate_psdf()
    p32, s32, w32, a32, b32 = o32.blocks()
    p64, s64, w64, a64, b64 = o64.blocks()
    from tests._util import align
    g, o = [x.reshape(-1) for x in align(p32, s32, p64, s64)[:2]]
    gw, ow = [x.reshape(-1) for x in align(p32, w32, p64, w64)[:2]]
    ga, oa = [x.reshape(-1) for x in align(p32, a32, p64, a64)[:2]]
    gb, ob = [x.reshape(-1) for x in align(p32, b32, p64, b64)[:2]]
    _, w_before = [x.reshape(-1) for x in align(p32, w32, pos, w)[:2]]
    upd = ow > 0
    later = upd & (w_before > 0)          # voxels that went through the Bayesian update
    assert later.sum() > 100000
    assert np.abs(g - o)[upd].max() < 2e-6
    assert (np.abs(gw - ow)[upd] / ow[upd]).max() < 1e-5
    assert (np.abs(ga - oa)[later] / np.abs(oa[later])).max() < 5e-6
    assert (np.abs(gb - ob)[later] / np.abs(ob[later])).max() < 5e-6


def test_oracle_raycast_hits_the_scene(built):
    wl, p, o = _run_oracle(True, n_frames=6)
    i = 25
    cTw = np.linalg.inv(wl.poses[i]).astype(np.float32)
    d, v, n = o.raycast(cTw)
    gt = scene.render_depth(wl.scene, wl.camera, wl.poses[i]).astype(np.float32)
    ok = np.isfinite(d) & (gt > 0)
    assert ok.mean() > 0.5
    assert np.median(np.abs(d - gt)[ok]) < 0.01
    nn = np.linalg.norm(n[..., :3][ok], axis=1)
    assert np.all((np.abs(nn - 1) < 1e-3) | (nn == 0))


def test_oracle_mesh_lies_on_surfaces(built):
    wl, p, o = _run_oracle(True, n_frames=20, stride=1)
    vk, vd, tr = o.dump_mesh()
    assert len(tr) > 0
    pts = vd[:, :3].astype(np.float64)
    # distance to the nearest scene surface along a short probe is small
    ref = wl.scene
    d_room = np.min(np.concatenate([pts - ref.room_lo, ref.room_hi - pts], axis=1), axis=1)
    d_sph = np.min([np.abs(np.linalg.norm(pts - s[:3], axis=1) - s[3]) for s in ref.spheres], axis=0)
    def box_d(b):
        lo, hi = b[:3], b[3:]
        q = np.maximum(lo - pts, pts - hi)
        outside = np.linalg.norm(np.maximum(q, 0), axis=1)
        inside = np.minimum(np.max(q, axis=1), 0)
        return np.abs(outside + inside)
    d_box = np.min([box_d(b) for b in ref.boxes], axis=0)
    dist = np.minimum(np.minimum(d_room, d_sph), d_box)
    assert np.median(dist) < 0.01
    # every triangle references existing vertices
    assert (tr[:, 4:7] >= 0).all()
    # reference counts equal the number of triangle uses
    uses = np.bincount(tr[:, 4:7].ravel(), minlength=len(vk))
    np.testing.assert_array_equal(uses, vd[:, 7].astype(np.int64))


def test_library_exp_within_one_ulp(built):
    """mh_exp.h (the single-precision exp of the PSDF path, shared by the
    kernels and the FP32 oracle) against double-precision exp rounded to
    single: at most 1 ulp on 2 M log-spaced and random arguments, exact at
    0, and the overflow / underflow ends."""
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.uniform(-103.9, 88.7, 1 << 20),
                        -np.logspace(-8, np.log10(103.9), 1 << 19), np.logspace(-8, np.log10(88.7), 1 << 19),
                        [0.0, -0.0, 88.72, -87.33, -103.0, -103.97]]).astype(np.float32)
    got = O.expf(x)
    want = np.exp(x.astype(np.float64)).astype(np.float32)
    gi, wi = got.view(np.int32).astype(np.int64), want.view(np.int32).astype(np.int64)
    assert np.abs(gi - wi).max() <= 1
    assert O.expf(np.array([0.0], np.float32))[0] == 1.0
    assert np.isinf(O.expf(np.array([89.0], np.float32))[0])
    assert O.expf(np.array([-104.0], np.float32))[0] == 0.0
    assert np.isnan(O.expf(np.array([np.nan], np.float32))[0])
