"""Block checkpoint / resume (mh_save_volume, mh_load_volume): a map saved
after fusion and loaded into a fresh volume has the same blocks and voxel
bits and raycasts to the same bits; with the simple update it also fuses the
next frame to the same state (the Bayesian update reads inlier ratios
predicted from mesh vertices, which a resumed volume only has after its next
mesh pass)."""
import numpy as np
import pytest

from meshhashing_gb300 import Volume, config, scene

pytestmark = pytest.mark.gpu


def _state(v):
    pos, f = v.dump_blocks()
    order = np.lexsort((pos[:, 2], pos[:, 1], pos[:, 0]))
    return pos[order], {k: f[k][order] for k in ("sdf", "w", "a", "b")}


@pytest.mark.parametrize("psdf", [False, True])
def test_save_load_round_trip(built, tmp_path, psdf):
    if psdf:
        wl = scene.full_spline(40, width=128, height=96)
        p = config.params_for(wl, value_capacity=1 << 17, bucket_count=1 << 16)
    else:
        wl = scene.small_circle(60)
        f = 262.5 * 128 / 320
        wl.camera = scene.Camera(128, 96, f, f, 63.5, 47.5)
        p = config.params_for(wl, value_capacity=1 << 16, bucket_count=1 << 15)
    a = Volume(p)
    for i in range(0, 20):
        a.integrate_frame(wl.frame(i), wl.pose(i))
    path = tmp_path / "map.mhvol"
    a.save(path)
    b = Volume(p)
    n = b.load(path)
    pa, fa = _state(a)
    pb, fb = _state(b)
    assert n == len(pa) and np.array_equal(pa, pb)
    for k in ("sdf", "w") + (("a", "b") if psdf else ()):
        np.testing.assert_array_equal(fa[k].view(np.uint32), fb[k].view(np.uint32))
    cTw = np.linalg.inv(wl.pose(21)).astype(np.float32)
    da, _, na = a.raycast(cTw)
    db, _, nb = b.raycast(cTw)
    np.testing.assert_array_equal(da.view(np.uint32), db.view(np.uint32))
    np.testing.assert_array_equal(na.view(np.uint32), nb.view(np.uint32))
    if psdf:
        return
    # both fuse the next frame alike
    for v in (a, b):
        v.integrate_frame(wl.frame(20), wl.pose(20))
    pa, fa = _state(a)
    pb, fb = _state(b)
    assert np.array_equal(pa, pb)
    np.testing.assert_array_equal(fa["sdf"].view(np.uint32), fb["sdf"].view(np.uint32))
    assert a.stats()["error"] == 0 and b.stats()["error"] == 0


def test_load_refuses_mismatched_file(built, tmp_path):
    """A checkpoint whose update mode (field count), voxel size or truncation
    differs from the volume's is refused before any block is inserted."""
    from meshhashing_gb300 import MeshHashError
    wl = scene.full_spline(4, width=128, height=96)
    kw = dict(value_capacity=1 << 14, bucket_count=1 << 14, max_vertex_count=1 << 16, max_triangle_count=1 << 16)
    p = config.params_for(wl, **kw)
    a = Volume(p)
    for i in range(2):
        a.integrate_frame(wl.frame(i), wl.pose(i))
    path = tmp_path / "psdf.mhvol"
    a.save(path)
    others = [config.params_for(wl, bayesian=False, **kw),                 # 2-field volume, 4-field file
              config.params_for(wl, voxel_size=0.005, **kw),
              config.params_for(wl, truncation=0.016, **kw)]
    for q in others:
        b = Volume(q)
        with pytest.raises(MeshHashError):
            b.load(path)
        assert b.stats()["blocks_allocated"] == 0
    # and the other way round: a 2-field file into a PSDF volume
    s = Volume(config.params_for(wl, bayesian=False, **kw))
    s.integrate_frame(wl.frame(0), wl.pose(0))
    s.save(tmp_path / "simple.mhvol")
    b = Volume(p)
    with pytest.raises(MeshHashError):
        b.load(tmp_path / "simple.mhvol")
    assert b.stats()["blocks_allocated"] == 0
