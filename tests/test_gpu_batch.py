"""Batched scenes (mh_batch_*) against the single-scene chain.

Each scene of a batch must end in exactly the state that mh_integrate_frame
gives on the same inputs: same block set and voxel bits, same mesh (as
pool-independent sets), same raycast bits.  The scenes differ in update mode,
resolution and voxel size, some skip steps, and the steps mix plain launches,
autotuning trials and graph replays.
"""
import numpy as np
import pytest

from meshhashing_gb300 import Batch, Volume, config, scene
from tests._util import mesh_canon, pos_set

pytestmark = pytest.mark.gpu


def _scenes():
    a = scene.small_circle(60)
    f = 262.5 * 160 / 320
    a.camera = scene.Camera(160, 120, f, f, 79.5, 59.5)
    pa = config.params_for(a, value_capacity=1 << 16, bucket_count=1 << 15, max_vertex_count=1 << 18,
                           max_triangle_count=1 << 18)
    b = scene.full_spline(40, width=128, height=96)
    pb = config.params_for(b, value_capacity=1 << 17, bucket_count=1 << 16, max_vertex_count=1 << 18,
                           max_triangle_count=1 << 18)
    c = scene.full_spline(40, width=96, height=72, seed=3)
    pc = config.params_for(c, voxel_size=0.006, truncation=0.018, value_capacity=1 << 16, bucket_count=1 << 15,
                           max_vertex_count=1 << 18, max_triangle_count=1 << 18)
    return [(a, pa, 3), (b, pb, 1), (c, pc, 1)]


def _state(v):
    pos, f = v.dump_blocks()
    order = np.lexsort((pos[:, 2], pos[:, 1], pos[:, 0]))
    vk, vd, tr = v.dump_mesh()
    return pos[order], {k: f[k][order] for k in ("sdf", "w", "a", "b")}, mesh_canon(vk, vd, tr)


def test_batch_matches_single_scene_chain(built):
    specs = _scenes()
    steps = 16
    singles = [Volume(p) for _, p, _ in specs]
    batched = [Volume(p) for _, p, _ in specs]
    batch = Batch(batched, raycast=True)
    last = [None] * len(specs)
    for k in range(steps):
        active = [1, 1, 0 if k in (3, 4, 9) else 1]
        depths, poses = [], []
        for i, (wl, p, stride) in enumerate(specs):
            if not active[i]:
                depths.append(None)
                poses.append(None)
                continue
            d, T = wl.frame(k * stride), wl.pose(k * stride)
            depths.append(d)
            poses.append(T)
            out = np.empty((p.rc_height, p.rc_width), np.float32)
            singles[i].integrate_frame(d, T, tv_iterations=3, tv_lambda=0.1, ray_depth=out)
            last[i] = out
        if k == 2:
            batch.autotune(1)                       # steps 2..10 try all 9 launch choices
        batch.step(depths, poses, active=active, tv_iterations=3, tv_lambda=0.1, use_graph=k >= 11)
        for i in range(len(specs)):
            if active[i]:
                rd, _, _ = batch.raycast(i)
                np.testing.assert_array_equal(rd.view(np.uint32), last[i].view(np.uint32))
    t = batch.tuning()
    assert t["ray_tile"] in ((16, 8), (8, 8), (32, 4))
    times = batch.tuning_times()
    assert all(v > 0 for v in times["integrate_ms"].values())
    tris = 0
    for i in range(len(specs)):
        ps, fs, (vs, ts) = _state(singles[i])
        pb, fb, (vb, tb) = _state(batched[i])
        assert pos_set(ps) == pos_set(pb)
        np.testing.assert_array_equal(ps, pb)
        for key in ("sdf", "w", "a", "b"):
            np.testing.assert_array_equal(fs[key].view(np.uint32), fb[key].view(np.uint32))
        assert set(vs) == set(vb) and ts == tb
        assert all(np.array_equal(vs[q], vb[q]) for q in vs)
        tris += len(ts)
        assert singles[i].stats()["error"] == 0 and batched[i].stats()["error"] == 0
    assert tris > 0
    batch.close()


def test_batch_device_inputs_and_graph_replay(built):
    """Depth frames resident on the device, every step replayed from the graph."""
    torch = pytest.importorskip("torch")
    specs = _scenes()[1:]
    singles = [Volume(p) for _, p, _ in specs]
    batched = [Volume(p) for _, p, _ in specs]
    batch = Batch(batched, raycast=True)
    for k in range(6):
        depths, poses = [], []
        for i, (wl, p, stride) in enumerate(specs):
            d, T = wl.frame(k), wl.pose(k)
            depths.append(torch.from_numpy(d).cuda())
            poses.append(T)
            singles[i].integrate_frame(d, T)
        batch.step(depths, poses, on_device=True, use_graph=True)
    torch.cuda.synchronize()
    for i in range(len(specs)):
        ps, fs, (vs, ts) = _state(singles[i])
        pb, fb, (vb, tb) = _state(batched[i])
        np.testing.assert_array_equal(ps, pb)
        np.testing.assert_array_equal(fs["sdf"].view(np.uint32), fb["sdf"].view(np.uint32))
        assert ts == tb
    batch.close()
