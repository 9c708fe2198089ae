"""Large-scene streaming (the 12 x 10 x 3 m floor plan): the generator on the
CPU, and on the GPU a long walk through several rooms with the full
MainEngine chain -- allocation far beyond any single view, garbage
collection returning blocks as the camera moves on, remeshing of the
frustum's blocks only, and a raycast every frame.
"""
import math

import numpy as np
import pytest

from meshhashing_gb300 import config, scene


def _inside_solid(sc, p):
    for cx, cy, cz, r in sc.spheres:
        if np.linalg.norm(p - np.array([cx, cy, cz])) < r + 0.05:
            return True
    for b in sc.boxes:
        if np.all(p > b[:3] - 0.05) and np.all(p < b[3:] + 0.05):
            return True
    return False


def test_floor_plan_walk_stays_in_free_space():
    wl = scene.floor_plan(2000, width=64, height=48)
    sc = wl.scene
    assert len(sc.spheres) + len(sc.boxes) == 17 + 40    # 17 wall slabs + 40 primitives
    pos = np.array([T[:3, 3] for T in wl.poses])
    assert np.all(pos > scene.PLAN_LO + 0.3) and np.all(pos < scene.PLAN_HI - 0.3)
    assert not any(_inside_solid(sc, p) for p in pos[::5])
    speed = np.linalg.norm(np.diff(pos, axis=0), axis=1) * 30.0
    assert speed.max() <= 0.5
    rooms = {(int(p[0] > -2) + int(p[0] > 2), int(p[1] > 0)) for p in pos}
    assert len(rooms) == 6
    a, b = wl.frame(700), wl.frame(700)
    assert np.array_equal(a, b) and 0.9 < (a > 0).mean() < 0.995


@pytest.mark.gpu
def test_streaming_walk_gc_and_remesh(built):
    from meshhashing_gb300 import Volume
    wl = scene.floor_plan(2000, width=160, height=120)
    p = config.params_for(wl, voxel_size=0.005, truncation=0.015, value_capacity=1 << 20, bucket_count=1 << 20,
                          max_vertex_count=1 << 21, max_triangle_count=1 << 21)
    v = Volume(p)
    rd = np.empty((p.rc_height, p.rc_width), np.float32)
    peak, hits = 0, []
    for k in range(0, 720, 3):                 # 24 s of walking: three rooms
        v.integrate_frame(wl.frame(k), wl.pose(k), ray_depth=rd)
        s = v.stats()
        peak = max(peak, s["blocks_allocated"])
        hits.append(np.isfinite(rd).mean())
    s = v.stats()
    assert s["error"] == 0 and s["dropped_inserts"] == 0, s
    assert s["frames"] == 240
    assert s["gc_freed_blocks"] > 0                     # blocks without surface are recycled as the walk goes on
    assert s["triangles_allocated"] > 1000, s
    # remeshing touched only the frustum's blocks: far fewer than the live set
    assert s["candidate_sum"] / s["mesh_passes"] < 0.8 * s["blocks_allocated"]
    assert np.median(hits[20:]) > 0.8


@pytest.mark.gpu
def test_floor_plan_walk_matches_oracle(built):
    """The floor-plan workload's settings (5 mm voxels, truncation 15 mm,
    2^22 buckets, PSDF, TV lambda 0.1 x 20) on a short walk at 160 x 120: the
    library's frame chain and the FP32 oracle's MainEngine loop side by side
    from an empty volume, through the recycle passes at frames 10, 20 and 30.
    After each pass the live block set (so the freed set), the voxel bits of
    every block, the mesh topology and the raycast bits are identical."""
    from meshhashing_gb300 import Volume
    from oracle.oracle import Oracle
    from tests._util import mesh_canon, tri_counts_per_block
    wl = scene.floor_plan(2000, width=160, height=120)
    p = config.params_for(wl, voxel_size=0.005, truncation=0.015, value_capacity=1 << 20, bucket_count=1 << 22,
                          max_vertex_count=1 << 21, max_triangle_count=1 << 21, linked_list_size=32)
    assert p.enable_bayesian_update == 1
    v = Volume(p)
    o = Oracle(p, fp64=False)
    rd = np.empty((p.rc_height, p.rc_width), np.float32)
    key = lambda q: ((q[:, 0].astype(np.int64) + (1 << 20)) << 42) + ((q[:, 1].astype(np.int64) + (1 << 20)) << 21) \
        + (q[:, 2].astype(np.int64) + (1 << 20))  # noqa: E731
    for i in range(30):
        k = 4 * i                                 # every 4th frame of the walk: 4 s of walking
        v.integrate_frame(wl.frame(k), wl.pose(k), tv_iterations=20, tv_lambda=0.1, ray_depth=rd)
        od = o.frame(wl.frame(k), wl.pose(k), raycast=True, tv_iterations=20, tv_lambda=0.1)
        if i % 10 != 9:
            continue
        gpos, gf = v.dump_blocks()
        opos, osdf, ow, oa, ob = o.blocks()
        assert np.array_equal(np.sort(key(gpos)), np.sort(key(opos))), f"frame {i}: block sets differ after GC"
        gi, oi = np.argsort(key(gpos)), np.argsort(key(opos))
        for name, of in (("sdf", osdf), ("w", ow), ("a", oa), ("b", ob)):
            np.testing.assert_array_equal(gf[name][gi].view(np.uint32), of[oi].view(np.uint32),
                                          err_msg=f"frame {i}: {name}")
        _, gt = mesh_canon(*v.dump_mesh())
        _, ot = mesh_canon(*o.dump_mesh())
        assert gt == ot and tri_counts_per_block(gt) == tri_counts_per_block(ot)
        hit = np.isfinite(od)
        assert np.array_equal(np.isfinite(rd), hit)
        np.testing.assert_array_equal(rd[hit].view(np.uint32), od[hit].view(np.uint32))
    s = v.stats()
    assert s["error"] == 0 and s["dropped_inserts"] == 0 and s["gc_freed_blocks"] > 0, s
