"""The per-block non-negative-voxel counts the raycast's skips rely on.

Every kernel that writes sdf keeps, per block, the number of voxels whose
sdf lies in [0, 1e30) (mh_dump_nonneg_counts); the raycast skips the gathers
of samples whose corner blocks all count 512, the interiors of such blocks,
and whole blocks whose seven upper neighbours count 512 too.  A stale count would change the raycast's output, so the counts
are checked against a recount from the voxels after every kind of writer:
the simple and the PSDF update, the GC that frees blocks (recycle every 10
frames, starvation in simple mode), the volumetric Huber-TV, and
mh_load_blocks.  The raycast of the same state is then compared with the FP32
oracle bit for bit.
"""
import numpy as np
import pytest

from meshhashing_gb300 import Volume, config, scene
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def recount(sdf):
    return ((sdf >= np.float32(0.0)) & (sdf < np.float32(1e30))).sum(axis=1).astype(np.int32)


def check_counts(v, what):
    pos, f = v.dump_blocks(("sdf",))
    got = v.nonneg_counts(pos)
    want = recount(f["sdf"])
    bad = np.nonzero(got != want)[0]
    assert bad.size == 0, f"{what}: {bad.size} of {len(pos)} blocks have stale counts"
    return len(pos), int((want == 512).sum())


def check_raycast(v, p, T, what):
    o = Oracle(p, fp64=False)
    pos, f = v.dump_blocks()
    o.set_blocks(pos, f["sdf"], f["w"], f["a"], f["b"])
    cTw = np.linalg.inv(np.asarray(T, np.float64)).astype(np.float32)
    gd, _, gn = v.raycast(cTw)
    od, _, on = o.raycast(cTw)
    hit = np.isfinite(od)
    assert np.array_equal(np.isfinite(gd), hit), f"{what}: hit masks differ"
    np.testing.assert_array_equal(gd[hit].view(np.uint32), od[hit].view(np.uint32))
    nh = hit & np.isfinite(on[..., 0])
    np.testing.assert_array_equal(gn[nh].view(np.uint32), on[nh].view(np.uint32))
    assert v.stats()["error"] == 0
    return int(hit.sum())


def test_counts_psdf_chain_gc_huber_and_load(built):
    wl = scene.full_spline(32, width=160, height=120)
    p = config.params_for(wl, value_capacity=1 << 17, bucket_count=1 << 16, max_vertex_count=1 << 18,
                          max_triangle_count=1 << 18)
    v = Volume(p)
    for i in range(21):                       # crosses the recycle passes at frames 10 and 20
        v.integrate_frame(wl.frame(i), wl.pose(i), tv_iterations=20, tv_lambda=0.1)
    n, full = check_counts(v, "PSDF chain with GC")
    assert full > 0 and v.stats()["gc_freed_blocks"] > 0
    hits = check_raycast(v, p, wl.pose(21), "PSDF map")
    # the volumetric Huber-TV rewrites the sdf of the candidates' voxels
    v.huber_tv_init()
    v.huber_tv_iterate(2.0, 8.0, 0.01, 5)
    check_counts(v, "after Huber-TV")
    check_raycast(v, p, wl.pose(21), "after Huber-TV")
    # a copy loaded through mh_load_blocks recounts every block it writes
    pos, f = v.dump_blocks()
    u = Volume(p)
    u.load_blocks(pos, f["sdf"], f["w"], f["a"], f["b"])
    check_counts(u, "loaded copy")
    assert hits > 0


def test_counts_simple_chain_with_starvation(built):
    wl = scene.small_circle(32)
    f = 262.5 * 160 / 320
    wl.camera = scene.Camera(160, 120, f, f, 79.5, 59.5)
    p = config.params_for(wl, value_capacity=1 << 16, bucket_count=1 << 15)
    v = Volume(p)
    for i in range(31):                       # starvation passes at frames 15 and 30
        v.integrate_frame(wl.frame(i), wl.pose(i))
    check_counts(v, "simple chain with starvation")
    check_raycast(v, p, wl.pose(31), "simple map")


def test_footprint(built):
    wl = scene.full_spline(12, width=160, height=120)
    p = config.params_for(wl, value_capacity=1 << 16, bucket_count=1 << 16)
    v = Volume(p)
    for i in range(10):
        v.integrate_frame(wl.frame(i), wl.pose(i))
    cTw = np.linalg.inv(np.asarray(wl.pose(10), np.float64)).astype(np.float32)
    n = v.raycast_footprint(cTw)
    assert 0 < n <= v.stats()["blocks_allocated"]
    assert v.raycast_footprint(cTw) == n      # deterministic
