"""Shared helpers of the parity tests (comparison of GPU and oracle state)."""
import numpy as np


def rows_by_pos(pos):
    return {tuple(int(c) for c in p): i for i, p in enumerate(pos)}


def pos_set(pos):
    return set(tuple(int(c) for c in p) for p in pos)


def align(gpos, gfield, opos, ofield):
    """Return (g, o) field rows for the blocks present in both, in one order."""
    gi = rows_by_pos(gpos)
    oi = rows_by_pos(opos)
    common = sorted(set(gi) & set(oi))
    g = np.stack([gfield[gi[k]] for k in common]) if common else np.zeros((0, 512), np.float32)
    o = np.stack([ofield[oi[k]] for k in common]) if common else np.zeros((0, 512), np.float32)
    return g, o, common


def ulp_diff(a, b):
    a = np.ascontiguousarray(a, np.float32).view(np.int32).astype(np.int64)
    b = np.ascontiguousarray(b, np.float32).view(np.int32).astype(np.int64)
    a = np.where(a < 0, -(a & 0x7FFFFFFF), a)
    b = np.where(b < 0, -(b & 0x7FFFFFFF), b)
    return np.abs(a - b)


def mesh_canon(vkeys, vdata, tris):
    """Pool-independent mesh: {vertex key: data}, set of triangles as keys."""
    keys = [tuple(int(c) for c in k) for k in vkeys]
    verts = {k: vdata[i] for i, k in enumerate(keys)}
    tset = set()
    for t in tris:
        ids = [int(x) for x in t[4:7]]
        vk = tuple(keys[i] if i >= 0 else None for i in ids)
        tset.add((int(t[0]), int(t[1]), int(t[2]), int(t[3])) + vk)
    return verts, tset


def tri_counts_per_block(tset):
    out = {}
    for t in tset:
        b = (t[0] >> 3, t[1] >> 3, t[2] >> 3)
        out[b] = out.get(b, 0) + 1
    return out
