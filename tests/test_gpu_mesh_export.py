"""Dense mesh export (mh_mesh_compact, mh_write_ply, mh_write_obj) against the
mesh held in the volume's pools (mh_dump_mesh): the same triangles, as
triples of vertex positions; only referenced vertices; the same arrays on a
second call; and the PLY and OBJ files hold exactly those arrays."""
import numpy as np
import pytest

from meshhashing_gb300 import Volume, config, scene

pytestmark = pytest.mark.gpu


def _volume():
    wl = scene.small_circle(60)
    f = 262.5 * 160 / 320
    wl.camera = scene.Camera(160, 120, f, f, 79.5, 59.5)
    p = config.params_for(wl, value_capacity=1 << 16, bucket_count=1 << 15, max_vertex_count=1 << 18,
                          max_triangle_count=1 << 18)
    v = Volume(p)
    for i in range(0, 60, 2):
        v.integrate_frame(wl.frame(i), wl.pose(i))
    return v


def _tri_key(a, b, c):
    # a triangle as its vertex positions, up to rotation of the corners
    k = [tuple(a), tuple(b), tuple(c)]
    i = k.index(min(k))
    return tuple(k[i:] + k[:i])


def test_compact_matches_pools_and_ply(built, tmp_path):
    v = _volume()
    pos, nrm, tri = v.compact_mesh()
    assert len(tri) > 1000
    vk, vd, tr = v.dump_mesh()
    keys = [tuple(int(c) for c in k) for k in vk]
    index = {k: i for i, k in enumerate(keys)}
    want = set()
    for t in tr:
        ids = [int(x) for x in t[4:7]]
        want.add(_tri_key(*[vd[i][:3] for i in ids]))
    got = {_tri_key(pos[a], pos[b], pos[c]) for a, b, c in tri}
    assert got == want
    assert len(index) >= len(pos)                        # only referenced vertices
    assert np.all(np.bincount(tri.reshape(-1), minlength=len(pos)) > 0)
    nn = np.linalg.norm(nrm, axis=1)        # unit, or zero where the gradient had no sample
    assert np.all((np.abs(nn - 1.0) < 1e-3) | (nn == 0.0)) and (nn > 0).mean() > 0.95
    pos2, nrm2, tri2 = v.compact_mesh()
    assert np.array_equal(pos, pos2) and np.array_equal(nrm, nrm2) and np.array_equal(tri, tri2)
    path = tmp_path / "mesh.ply"
    v.write_ply(path)
    raw = path.read_bytes()
    head, body = raw.split(b"end_header\n", 1)
    assert f"element vertex {len(pos)}".encode() in head and f"element face {len(tri)}".encode() in head
    vrec = np.frombuffer(body[:len(pos) * 24], np.float32).reshape(-1, 6)
    assert np.array_equal(vrec[:, :3], pos) and np.array_equal(vrec[:, 3:], nrm)
    frec = np.frombuffer(body[len(pos) * 24:], np.dtype([("n", "u1"), ("i", "<i4", (3,))]))
    assert np.all(frec["n"] == 3) and np.array_equal(frec["i"], tri)
    obj = tmp_path / "mesh.obj"
    v.write_obj(obj)
    lines = obj.read_text().splitlines()
    vl = np.array([[float(x) for x in ln.split()[1:]] for ln in lines if ln.startswith("v ")], np.float32)
    nl = np.array([[float(x) for x in ln.split()[1:]] for ln in lines if ln.startswith("vn ")], np.float32)
    fl = np.array([[int(x.split("//")[0]) for x in ln.split()[1:]] for ln in lines if ln.startswith("f ")])
    assert np.array_equal(vl, pos) and np.array_equal(nl, nrm) and np.array_equal(fl - 1, tri)


def test_compact_matches_oracle_mesh(built):
    """The dense mesh of a 30-frame map against the FP32 oracle's mesh of the
    same frames (its MainEngine loop from the same empty volume): the same
    triangles as triples of vertex-position bits, with multiplicity, and
    the same vertex count."""
    from collections import Counter
    from oracle.oracle import Oracle
    wl = scene.small_circle(60)
    f = 262.5 * 160 / 320
    wl.camera = scene.Camera(160, 120, f, f, 79.5, 59.5)
    p = config.params_for(wl, value_capacity=1 << 16, bucket_count=1 << 15, max_vertex_count=1 << 18,
                          max_triangle_count=1 << 18)
    v = Volume(p)
    o = Oracle(p, fp64=False)
    for i in range(0, 60, 2):
        v.integrate_frame(wl.frame(i), wl.pose(i))
        o.frame(wl.frame(i), wl.pose(i))
    pos, _, tri = v.compact_mesh()
    vk, vd, tr = o.dump_mesh()
    got = Counter(_tri_key(*[pos[k].view(np.uint32) for k in t]) for t in tri)
    want = Counter(_tri_key(*[vd[int(k)][:3].view(np.uint32) for k in t[4:7]]) for t in tr)
    assert len(tri) > 1000 and got == want
    assert len(pos) == len(np.unique(tr[:, 4:7].reshape(-1)))
