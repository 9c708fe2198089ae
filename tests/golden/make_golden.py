"""Generate the golden fixtures in tests/golden/ from the reference itself.

The reference has no tests or golden vectors, so its own device code, built
for the CPU (oracle/refcpu: the reference's kernels and headers compiled with
g++ against a CUDA-emulation shim), is run on small seeded inputs through
the MainEngine stage order, and its outputs are stored together with the
inputs.  Needs the reference tree (argument 1, else $MESHHASHING_REFERENCE,
else oracle/refcpu.py's default); the fixtures are
committed, so tests never need the tree.

  simple_room96.npz  plain TSDF chain, 96x72, 8 mm voxels, 6 frames of the
                     circle trajectory: block sets, candidates, voxel values
                     of sampled blocks, marching-cubes mesh, cube indices,
                     raycast depth and normals
  psdf_room96.npz    PSDF chain, 96x72, 4 mm voxels, 6 frames of the spline
                     trajectory (with outliers and missing pixels): block
                     set, voxel values of sampled blocks, inlier ratios
  huber_room96.npz   PrimalDualInit + 8 PrimalDualIterate calls
                     (optimize/primal_dual.cu) on a 48-block cluster of the
                     simple chain's last candidates: the cluster's and its
                     face neighbours' sdf and weight before, the cluster's
                     sdf after, the two error sums of every iteration
  track_room96.npz   PointToSurface (localizing/point_to_psdf.cu) on the
                     simple chain's map with frame 18's depth at two poses
                     off the true one: A, b, err and count
  compress_room96.npz MainEngine's mesh output on the simple chain's map:
                     CollectAllBlocks + CompressMesh
                     (visualization/compress_mesh.cu): compact vertex
                     positions and normals, triangles as compact indices,
                     and CompressMesh's stats (triangles, vertices, summed
                     vertex reference counts)

Both use params.compat_arithmetic = 1 (the reference's single-precision
formulas as written).  Allocation is repeated until no block is added, which
removes the reference's per-bucket insert drops (the comparison target is the
full touched set).

Usage: python tests/golden/make_golden.py [reference root]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from meshhashing_gb300 import config, scene  # noqa: E402

N_SAMPLE = 32


def simple_case():
    wl = scene.small_circle(60)
    f = 262.5 * 96 / 320
    wl.camera = scene.Camera(96, 72, f, f, 47.5, 35.5)
    frames = [0, 3, 6, 9, 12, 15]
    p = config.params_for(wl, value_capacity=1 << 14, bucket_count=1 << 14, max_vertex_count=1 << 16,
                          max_triangle_count=1 << 16, weight_sample=1000, compat_arithmetic=1)
    depth = np.stack([wl.frame(i) for i in frames])
    poses = np.stack([wl.pose(i) for i in frames])
    return p, depth, poses


def psdf_case():
    wl = scene.full_spline(40, width=96, height=72)
    frames = [0, 1, 2, 3, 4, 5]
    p = config.params_for(wl, value_capacity=1 << 15, bucket_count=1 << 17, max_vertex_count=1 << 16,
                          max_triangle_count=1 << 16, compat_arithmetic=1)
    depth = np.stack([wl.frame(i) for i in frames])
    poses = np.stack([wl.pose(i) for i in frames])
    return p, depth, poses


def sample_blocks(pos, w):
    """Deterministic sample: the blocks with the most observed voxels."""
    key = np.lexsort((pos[:, 2], pos[:, 1], pos[:, 0]))
    obs = (w[key] > 0).sum(axis=1)
    order = key[np.argsort(-obs, kind="stable")]
    return order[:N_SAMPLE]


def run_simple(ref_mod, p, depth, poses):
    r = ref_mod.RefCPU(p)
    counts = []
    for d, T in zip(depth, poses):
        r.frame_set(d, T)
        counts.append(r.alloc(True))
        r.collect()
        r.integrate_simple()
        r.mesh()
        r.gc_low_surfel()
    cand = r.candidates()
    pos, s, w, _, _ = r.blocks()
    idx = sample_blocks(pos, w)
    vk, vd, tr = r.dump_mesh()
    cTw = np.linalg.inv(poses[-1].astype(np.float64)).astype(np.float32)
    rd, rn = r.raycast(cTw)
    return dict(depth=depth, poses=poses, counts=np.array(counts, np.int32), blocks=pos, candidates=cand,
                sample_pos=pos[idx], sample_sdf=s[idx], sample_w=w[idx], cubes=r.cubes(pos[idx]),
                vkeys=vk, vpos=vd[:, :3], vref=vd[:, 7].astype(np.int32), tris=tr, ray_cTw=cTw, ray_depth=rd,
                ray_normal=rn[..., :3])


def run_psdf(ref_mod, p, depth, poses):
    r = ref_mod.RefCPU(p)
    counts = []
    for d, T in zip(depth, poses):
        r.frame_set(d, T)
        counts.append(r.alloc(True))
        r.collect()
        r.predict()
        r.integrate_psdf()
        r.mesh()
        r.gc_low_surfel()
    pos, s, w, a, b = r.blocks()
    idx = sample_blocks(pos, w)
    return dict(depth=depth, poses=poses, counts=np.array(counts, np.int32), blocks=pos, sample_pos=pos[idx],
                sample_sdf=s[idx], sample_w=w[idx], sample_a=a[idx], sample_b=b[idx], inlier=r.inlier())


HUBER = dict(lam=2.0, sigma=8.0, tau=0.01, iterations=8, blocks=48)
FACES = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)]


def huber_cluster(cand, pos, w, n):
    """The n candidates nearest (Chebyshev distance, then position) to the
    candidate with the most observed voxels."""
    idx = {tuple(q): i for i, q in enumerate(pos.tolist())}
    obs = np.array([(w[idx[tuple(q)]] > 0).sum() for q in cand.tolist()])
    c0 = cand[int(np.argmax(obs))]
    d = np.abs(cand - c0).max(axis=1)
    order = np.lexsort((cand[:, 2], cand[:, 1], cand[:, 0], d))
    return cand[order[:n]]


def run_huber(ref_mod, p, depth, poses):
    r = ref_mod.RefCPU(p)
    for d, T in zip(depth, poses):
        r.frame_set(d, T)
        r.alloc(True)
        r.collect()
        r.integrate_simple()
        r.mesh()
        r.gc_low_surfel()
    pos, s, w, _, _ = r.blocks()
    cl = huber_cluster(r.candidates(), pos, w, HUBER["blocks"])
    have = {tuple(q) for q in pos.tolist()}
    near = {tuple(q) for q in cl.tolist()}
    near |= {(q[0] + f[0], q[1] + f[1], q[2] + f[2]) for q in cl.tolist() for f in FACES}
    near = np.array(sorted(q for q in near if q in have), np.int32)
    assert r.set_candidates(cl) == len(cl)
    r.pd_init()
    errs = np.stack([r.pd_iterate(HUBER["lam"], HUBER["sigma"], HUBER["tau"]) for _ in range(HUBER["iterations"])])
    pos2, s2, _, _, _ = r.blocks()
    return dict(pre_pos=near, pre_sdf=rows(pos, s, near), pre_w=rows(pos, w, near), cand=cl,
                post_sdf=rows(pos2, s2, cl), errs=errs,
                hparams=np.array([HUBER["lam"], HUBER["sigma"], HUBER["tau"], HUBER["iterations"]], np.float32))


TRACK_FRAME = 18
TRACK_XI = [[0.01, -0.005, 0.008, 0.01, -0.008, 0.005], [-0.02, 0.012, -0.01, -0.015, 0.01, 0.02]]


def track_case():
    """Frame 18 of the simple trajectory and the poses the fixture uses."""
    from meshhashing_gb300.pose import left_update
    wl = scene.small_circle(60)
    f = 262.5 * 96 / 320
    wl.camera = scene.Camera(96, 72, f, f, 47.5, 35.5)
    T = wl.pose(TRACK_FRAME).astype(np.float64)
    poses = np.stack([left_update(T, np.array(x)).astype(np.float32) for x in TRACK_XI])
    return wl.frame(TRACK_FRAME), T.astype(np.float32), poses


def run_track(ref_mod, p, depth, poses):
    r = ref_mod.RefCPU(p)
    for d, T in zip(depth, poses):
        r.frame_set(d, T)
        r.alloc(True)
        r.collect()
        r.integrate_simple()
        r.mesh()
        r.gc_low_surfel()
    d18, T18, tp = track_case()
    out = {"A": [], "b": [], "err": [], "count": []}
    for T in tp:
        r.frame_set(d18, T)
        A, b, e, n = r.point_to_psdf(T)
        out["A"].append(A), out["b"].append(b), out["err"].append(e), out["count"].append(n)
    return dict(depth=d18, pose_true=T18, poses=tp, A=np.stack(out["A"]), b=np.stack(out["b"]),
                err=np.array(out["err"], np.float32), count=np.array(out["count"], np.int32))


def run_compress(ref_mod, p, depth, poses):
    r = ref_mod.RefCPU(p)
    for d, T in zip(depth, poses):
        r.frame_set(d, T)
        r.alloc(True)
        r.collect()
        r.integrate_simple()
        r.mesh()
        r.gc_low_surfel()
    pos, nrm, tri, stats = r.compress_mesh()
    return dict(depth=depth, poses=poses, pos=pos, normal=nrm, tris=tri, stats=stats)


def rows(pos, field, want):
    idx = {tuple(q): i for i, q in enumerate(pos.tolist())}
    return np.stack([field[idx[tuple(q)]] for q in np.asarray(want).tolist()])


def main():
    from oracle import refcpu
    ref_root = sys.argv[1] if len(sys.argv) > 1 else refcpu.reference_dir()
    refcpu.build(ref_root)
    p, depth, poses = simple_case()
    np.savez_compressed(os.path.join(HERE, "simple_room96.npz"), **run_simple(refcpu, p, depth, poses))
    p, depth, poses = psdf_case()
    np.savez_compressed(os.path.join(HERE, "psdf_room96.npz"), **run_psdf(refcpu, p, depth, poses))
    p, depth, poses = simple_case()
    np.savez_compressed(os.path.join(HERE, "huber_room96.npz"), **run_huber(refcpu, p, depth, poses))
    np.savez_compressed(os.path.join(HERE, "track_room96.npz"), **run_track(refcpu, p, depth, poses))
    np.savez_compressed(os.path.join(HERE, "compress_room96.npz"), **run_compress(refcpu, p, depth, poses))
    for f in ("simple_room96.npz", "psdf_room96.npz", "huber_room96.npz", "track_room96.npz", "compress_room96.npz"):
        print(f, os.path.getsize(os.path.join(HERE, f)), "bytes")


if __name__ == "__main__":
    main()
