"""GPU parity tests: every stage through the C ABI against the oracle.

Stage-wise: before each stage the oracle is handed the GPU's own state, so a
float difference upstream cannot mask a discrete mismatch downstream.  The
FP32-faithful oracle (same operation order, IEEE single, no FMA) is the
reference for discrete results and exact values; the FP64 oracle gives the
error bounds stated in each test.
"""
import numpy as np
import pytest

from meshhashing_gb300 import Volume, config, scene
from oracle.oracle import Oracle
from tests._util import align, mesh_canon, pos_set, tri_counts_per_block, ulp_diff

pytestmark = pytest.mark.gpu


def small_workload(width=160, height=120, n=60):
    wl = scene.small_circle(n)
    f = 262.5 * width / 320
    wl.camera = scene.Camera(width, height, f, f, (width - 1) / 2, (height - 1) / 2)
    return wl


def psdf_workload(width=160, height=120, n=40):
    return scene.full_spline(n, width=width, height=height)


def make(wl, **over):
    kw = dict(value_capacity=1 << 18, bucket_count=1 << 16, max_vertex_count=1 << 20, max_triangle_count=1 << 20)
    kw.update(over)
    p = config.params_for(wl, **kw)
    return p, Volume(p)


def hand_over(v, o, with_mesh=False):
    """Load the GPU volume's state into the oracle."""
    pos, f = v.dump_blocks()
    o.set_blocks(pos, f["sdf"], f["w"], f["a"], f["b"])
    if with_mesh:
        vk, vd, tr = v.dump_mesh()
        o.load_mesh(vk, vd, tr)
        o.set_cubes(pos, v.cubes(pos))
        life, inner, bnd = v.block_meta(pos)
        o.set_block_meta(pos, life, inner, bnd)
    return pos, f


def test_alloc_and_collect_match_oracle(built):
    wl = small_workload()
    p, v = make(wl)
    o = Oracle(p, fp64=False)
    for i in range(0, 30, 3):
        d, T = wl.frame(i), wl.pose(i)
        v.set_frame(d, T)
        o.frame_set(d, T)
        v.alloc_block_array()
        o.allocate()
        gpos, _ = v.dump_blocks(fields=())
        opos = o.blocks()[0]
        assert pos_set(gpos) == pos_set(opos), f"frame {i}: block sets differ"
        assert len(gpos) == len(pos_set(gpos)), "duplicate blocks in the hash table"
        v.collect_blocks_in_frustum()
        o.collect_frustum()
        assert pos_set(v.candidates()) == pos_set(o.candidates()), f"frame {i}: candidates differ"
    st = v.stats()
    assert st["error"] == 0 and st["dropped_inserts"] == 0
    assert st["blocks_allocated"] == len(gpos)


def test_integrate_simple_exact(built):
    wl = small_workload()
    p, v = make(wl)
    o32 = Oracle(p, fp64=False)
    o64 = Oracle(p, fp64=True)
    worst_s, worst_w = 0.0, 0.0
    for i in range(0, 24, 2):
        d, T = wl.frame(i), wl.pose(i)
        v.set_frame(d, T)
        v.alloc_block_array()
        v.collect_blocks_in_frustum()
        cand = v.candidates()
        pos, f = hand_over(v, o32)
        o64.set_blocks(pos, f["sdf"], f["w"], f["a"], f["b"])
        for o in (o32, o64):
            o.frame_set(d, T)
            o.set_candidates(cand)
        v.update_blocks_simple()
        o32.integrate_simple()
        o64.integrate_simple()
        gpos, gf = v.dump_blocks()
        p32, s32, w32, _, _ = o32.blocks()
        p64, s64, w64, _, _ = o64.blocks()
        g, o, _ = align(gpos, gf["sdf"], p32, s32)
        gw, ow, _ = align(gpos, gf["w"], p32, w32)
        assert np.array_equal(gw, ow), f"frame {i}: weights differ from the FP32 oracle"
        assert ulp_diff(g, o).max() == 0, f"frame {i}: sdf differs from the FP32 oracle"
        g6, o6, _ = align(gpos, gf["sdf"], p64, s64)
        gw6, ow6, _ = align(gpos, gf["w"], p64, w64)
        m = ow6 > 0
        worst_s = max(worst_s, float(np.abs(g6 - o6)[m].max()))
        worst_w = max(worst_w, float((np.abs(gw6 - ow6)[m] / ow6[m]).max()))
    # against FP64: sdf within 1e-4 of the truncation distance (absolute error
    # is a few ulp of the 4 m camera depth), weights within 1e-5 relative
    assert worst_s < 1e-4 * p.truncation_distance, worst_s
    assert worst_w < 1e-5, worst_w
    print(f"simple update vs FP64: max |dsdf| = {worst_s:.3e} m, max rel dw = {worst_w:.3e}")


def _psdf_chain(v, o32, wl, frames, with_checks=True, o64=None):
    stats = {"inlier_max_ulp": 0, "sdf_rel": 0.0, "w_rel": 0.0, "sdf64_abs": 0.0, "w64_rel": 0.0, "ab64_rel": 0.0}
    for i in frames:
        d, T = wl.frame(i), wl.pose(i)
        v.set_frame(d, T)
        v.alloc_block_array()
        v.collect_blocks_in_frustum()
        cand = v.candidates()
        if with_checks:
            for o in (o32,) + ((o64,) if o64 is not None else ()):
                hand_over(v, o, with_mesh=True)
                o.frame_set(d, T)
                o.set_candidates(cand)
        v.predict_outlier_ratio()
        if with_checks:
            o32.predict_inlier()
            gi, oi = v.inlier(), o32.inlier()
            stats["inlier_max_ulp"] = max(stats["inlier_max_ulp"], int(ulp_diff(gi, oi).max()))
            o32.set_inlier(gi)
            if o64 is not None:
                o64.set_inlier(gi)
        v.update_blocks_bayesian()
        if with_checks and o64 is not None:
            # the same update in double from the same state and inlier ratios
            o64.integrate_psdf()
            gpos, gf = v.dump_blocks()
            p64, s64, w64, a64, b64 = o64.blocks()
            g, o, _ = align(gpos, gf["sdf"], p64, s64)
            stats["sdf64_abs"] = max(stats["sdf64_abs"], float(np.abs(g - o).max()) if g.size else 0.0)
            g, o, _ = align(gpos, gf["w"], p64, w64)
            m = o > 0
            stats["w64_rel"] = max(stats["w64_rel"], float((np.abs(g - o)[m] / o[m]).max()) if m.any() else 0.0)
            for key, ofield in (("a", a64), ("b", b64)):
                g, o, _ = align(gpos, gf[key], p64, ofield)
                m = np.abs(o) > 1e-3
                if m.any():
                    stats["ab64_rel"] = max(stats["ab64_rel"], float((np.abs(g - o)[m] / np.abs(o[m])).max()))
        if with_checks:
            o32.integrate_psdf()
            gpos, gf = v.dump_blocks()
            p32, s32, w32, a32, b32 = o32.blocks()
            for name, gfield, ofield in (("sdf", gf["sdf"], s32), ("w", gf["w"], w32)):
                g, o, _ = align(gpos, gfield, p32, ofield)
                scale = np.maximum(np.abs(o), 1e-3 if name == "sdf" else 1.0)
                rel = float((np.abs(g - o) / scale).max()) if g.size else 0.0
                key = "sdf_rel" if name == "sdf" else "w_rel"
                stats[key] = max(stats[key], rel)
        v.marching_cubes()
        v.collect_low_surfel_blocks()
    return stats


def test_psdf_predict_and_update(built):
    wl = psdf_workload()
    p, v = make(wl)
    o32 = Oracle(p, fp64=False)
    # build up a surface with meshed vertices first, then check stage-wise
    _psdf_chain(v, o32, wl, range(0, 12), with_checks=False)
    st = _psdf_chain(v, o32, wl, range(12, 18), with_checks=True, o64=Oracle(p, fp64=True))
    # expf differs by a few ulp between the CUDA and host math libraries
    assert st["inlier_max_ulp"] <= 64, st
    assert st["sdf_rel"] < 1e-4 and st["w_rel"] < 1e-4, st
    print(f"PSDF update vs FP64: max |dsdf| = {st['sdf64_abs']:.3e} m, max rel dw = {st['w64_rel']:.3e}, "
          f"max rel da/db = {st['ab64_rel']:.3e}")
    assert st["sdf64_abs"] < 1e-5 and st["w64_rel"] < 1e-4, st
    assert v.stats()["error"] == 0


def _mesh_compare(v, o, p, cand_pos):
    gvk, gvd, gtr = v.dump_mesh()
    ovk, ovd, otr = o.dump_mesh()
    gverts, gtris = mesh_canon(gvk, gvd, gtr)
    overts, otris = mesh_canon(ovk, ovd, otr)
    assert set(gverts) == set(overts), "vertex sets differ"
    assert gtris == otris, "triangle topology differs"
    assert tri_counts_per_block(gtris) == tri_counts_per_block(otris)
    keys = sorted(gverts)
    if keys:
        gp = np.stack([gverts[k] for k in keys])
        op = np.stack([overts[k] for k in keys])
        pos_err = np.abs(gp[:, :3] - op[:, :3]).max() / p.voxel_size
        assert pos_err < 1e-4, pos_err
        np.testing.assert_array_equal(gp[:, 7], op[:, 7])      # reference counts
        return len(keys), len(gtris), pos_err
    return 0, 0, 0.0


def test_marching_cubes_topology_exact(built):
    wl = small_workload()
    p, v = make(wl)
    o = Oracle(p, fp64=False)
    o64 = Oracle(p, fp64=True)
    total_tris = 0
    for i in range(0, 40):
        d, T = wl.frame(i), wl.pose(i)
        v.set_frame(d, T)
        v.alloc_block_array()
        v.collect_blocks_in_frustum()
        v.update_blocks_simple()
        if i % 8 == 7:
            cand = v.candidates()
            pos, f = hand_over(v, o, with_mesh=True)
            o.set_candidates(cand)
            o64.set_blocks(pos, f["sdf"], f["w"], f["a"], f["b"])
            vk, vd, tr = v.dump_mesh()
            o64.load_mesh(vk, vd, tr)
            o64.set_candidates(cand)
            v.marching_cubes()
            o.mesh()
            o64.mesh()
            # a cube with no surface (index 0 or 255) needs no mesh page, so a
            # block without one reports 0 for both
            gc, oc = v.cubes(cand), o.cubes(cand)
            np.testing.assert_array_equal(np.where(gc == 255, 0, gc), np.where(oc == 255, 0, oc))
            nv, nt, err = _mesh_compare(v, o, p, cand)
            total_tris = nt
            # FP64 vertex positions
            gverts, _ = mesh_canon(*v.dump_mesh())
            overts, _ = mesh_canon(*o64.dump_mesh())
            common = sorted(set(gverts) & set(overts))
            if common:
                e64 = max(float(np.abs(gverts[k][:3] - overts[k][:3]).max()) for k in common) / p.voxel_size
                assert e64 < 1e-4, e64
                print(f"vertex positions vs FP64: max error = {e64:.3e} voxel over {len(common)} vertices")
            life, inner, bnd = v.block_meta(cand)
            _, oin, obnd, _ = o.block_meta(cand)
            np.testing.assert_array_equal(inner, oin)
            np.testing.assert_array_equal(bnd, obnd)
        else:
            v.marching_cubes()
    assert total_tris > 0
    assert v.stats()["error"] == 0


def test_raycast_matches_oracle(built):
    wl = small_workload()
    p, v = make(wl)
    for i in range(0, 30):
        v.integrate_frame(wl.frame(i), wl.pose(i))
    o32 = Oracle(p, fp64=False)
    o64 = Oracle(p, fp64=True)
    hand_over(v, o32)
    hand_over(v, o64)
    for i in (5, 17, 29):
        cTw = np.linalg.inv(wl.poses[i]).astype(np.float32)
        gd, gv, gn = v.raycast(cTw)
        od, ov, on = o32.raycast(cTw)
        hit = np.isfinite(od)
        np.testing.assert_array_equal(np.isfinite(gd), hit)
        assert np.abs(gd[hit] - od[hit]).max() <= 1e-6
        nh = hit & np.isfinite(on[..., 0])
        assert np.abs(gn[nh] - on[nh]).max() < 1e-4
        # FP64: same discrete path (the oracle replays the single-precision
        # decisions), values in double -- depth within 1e-4 m everywhere
        d64, _, _ = o64.raycast(cTw)
        both = hit & np.isfinite(d64)
        assert both.sum() >= 0.999 * hit.sum()
        diff = np.abs(gd[both] - d64[both])
        assert diff.max() < 1e-4, diff.max()
        print(f"raycast vs FP64: max |ddepth| = {diff.max():.3e} m over {both.sum()} pixels")
        gt = scene.render_depth(wl.scene, wl.camera, wl.poses[i]).astype(np.float32)
        ok = hit & (gt > 0)
        assert np.median(np.abs(gd[ok] - gt[ok])) < 0.01


def test_gc_matches_oracle(built):
    wl = psdf_workload()
    p, v = make(wl)
    o = Oracle(p, fp64=False)
    for i in range(0, 12):
        v.integrate_frame(wl.frame(i), wl.pose(i))
    # one more frame stage by stage, with the oracle following on GPU state
    d, T = wl.frame(12), wl.pose(12)
    v.set_frame(d, T)
    v.alloc_block_array()
    v.collect_blocks_in_frustum()
    v.predict_outlier_ratio()
    v.update_blocks_bayesian()
    v.marching_cubes()
    cand = v.candidates()
    hand_over(v, o, with_mesh=True)
    o.set_candidates(cand)
    v.collect_low_surfel_blocks()
    o.gc_low_surfel()
    life, _, _ = v.block_meta(cand)
    olife, _, _, oflag = o.block_meta(cand)
    np.testing.assert_array_equal(life, olife)
    gflags = v.flags()
    gcand = v.candidates()
    gflag_set = set(tuple(c) for c, f in zip(gcand, gflags) if f)
    oflag_set = set(tuple(c) for c, f in zip(cand, oflag) if f)
    assert gflag_set == oflag_set
    before = pos_set(v.dump_blocks(fields=())[0])
    v.recycle_garbage_block_array()
    freed = o.gc_recycle()
    after = pos_set(v.dump_blocks(fields=())[0])
    assert after == pos_set(o.blocks()[0])
    assert len(before) - len(after) == freed
    assert v.stats()["error"] == 0


def test_full_chain_small_circle(built):
    """MainEngine frame loop (simple mode, with the 15-frame recycle) end to end."""
    wl = small_workload()
    p, v = make(wl)
    o = Oracle(p, fp64=False)
    for i in range(0, 20):
        d, T = wl.frame(i), wl.pose(i)
        v.integrate_frame(d, T)
        o.frame(d, T)
    gpos, gf = v.dump_blocks()
    opos, os_, ow, _, _ = o.blocks()
    assert pos_set(gpos) == pos_set(opos)
    g, oo, _ = align(gpos, gf["w"], opos, ow)
    assert np.array_equal(g, oo)
    _, gtris = mesh_canon(*v.dump_mesh())
    _, otris = mesh_canon(*o.dump_mesh())
    assert gtris == otris
    assert len(gtris) > 0


def test_error_paths(built):
    from meshhashing_gb300 import MeshHashError
    wl = small_workload()
    # invalid parameters
    p = config.params_for(wl, bucket_count=1000)
    with pytest.raises(MeshHashError):
        Volume(p)
    # stage before any frame
    p, v = make(wl)
    with pytest.raises(MeshHashError):
        v.alloc_block_array()
    # all-invalid frame allocates nothing
    v.set_frame(np.zeros((wl.camera.height, wl.camera.width), np.float32), wl.pose(0))
    v.alloc_block_array()
    assert v.stats()["blocks_allocated"] == 0
    # a block pool that is far too small reports MH_ERR_CAPACITY, no fault
    p, v = make(wl, value_capacity=64)
    v.integrate_frame(wl.frame(0), wl.pose(0))
    st = v.stats()
    assert st["error"] == 3 and st["blocks_allocated"] == 64 and st["dropped_inserts"] > 0
    v.clear_error()
    assert v.stats()["error"] == 0


def test_hash_overflow_chains(built):
    """Tiny bucket count forces overflow chains; the block set stays exact."""
    wl = small_workload()
    p, v = make(wl, bucket_count=1 << 8, overflow_capacity=1 << 15, linked_list_size=64)
    o = Oracle(p, fp64=False)
    for i in range(0, 6):
        d, T = wl.frame(i), wl.pose(i)
        v.set_frame(d, T)
        o.frame_set(d, T)
        v.alloc_block_array()
        o.allocate()
    st = v.stats()
    assert st["overflow_used"] > 0 and st["error"] == 0
    assert pos_set(v.dump_blocks(fields=())[0]) == pos_set(o.blocks()[0])
    # every block is found again (collect_all + set_candidates round trip)
    pos = v.dump_blocks(fields=())[0]
    v.set_candidates(pos)
    assert pos_set(v.candidates()) == pos_set(pos)
