#!/usr/bin/env python
"""Fused fusion-chain throughput at 640x480 (PSDF, 4 mm voxels) on one GB300.

One step = one MainEngine frame of the PSDF workload (640x480, fx=fy=525,
4 mm voxels, truncation 12 mm, 2^21 buckets): TV denoising (lambda 0.1,
20 iterations), block allocation, frustum collection, inlier-ratio
prediction, Bayesian update, marching cubes with low-surfel GC (recycling
every 10th frame) and a 640x480 raycast.  Input frames are seeded synthetic
renders of the room scene (scene.full_spline) with Gaussian noise
sigma = 0.0012 z^2, 5 % outliers and 2 % missing pixels; the map is
pre-fused for --prefuse frames before warm-up so the timed frames see a
populated volume.

Outputs one JSON line (rank 0):
  value  frames/s with all input frames resident in HBM (device-to-device);
  e2e    frames/s through the C ABI with host buffers: each frame's depth is
         copied from pinned host memory and its raycast depth read back; the
         timed region's frames, replayed on the volume after a reset and the
         same pre-fusion.
Under torchrun each rank fuses its own replica (no collective on the data
path); value is the aggregate over ranks with the max-over-ranks time.
``--impl reference`` times the reference path's CPU restatement (the FP64
oracle, all host threads) on the same workload instead.
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "640×480 frames/s (alloc+fuse+mesh+raycast) batched vs plain, %HBM peak"
_T0 = time.time()


def log(msg):
    """Progress on stderr (seconds since start); the result line is stdout."""
    sys.stderr.write(f"[bench {time.time() - _T0:7.1f} s] {msg}\n")
    sys.stderr.flush()
TV_ITERS, TV_LAMBDA = 20, 0.1


def _frame_job(args):
    i, n_total, w, h = args
    from meshhashing_gb300 import scene
    wl = scene.full_spline(n_total, width=w, height=h)
    return wl.frame(i), wl.pose(i)


def gen_frames(indices, n_total, w=640, h=480, procs=None):
    ctx = mp.get_context("spawn")
    procs = procs or min(len(indices), os.cpu_count() or 4, 16)
    with ctx.Pool(procs) as pool:
        out = pool.map(_frame_job, [(i, n_total, w, h) for i in indices])
    return [o[0] for o in out], [o[1] for o in out]


class ClockSampler:
    """nvidia-smi clock/throttle samples every 50 ms, each with its own
    timestamp, so the summary keeps exactly the samples taken inside the
    timed region."""

    Q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.rows, self.proc, self.thread = [], None, None

    def start(self, interval_ms=50):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                          "-lms", str(interval_ms)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        import datetime
        for line in self.proc.stdout:
            r = [c.strip() for c in line.split(",")]
            if len(r) < 10:
                continue
            ts = None
            for fmt in ("%Y/%m/%d %H:%M:%S.%f", "%Y/%m/%d %H:%M:%S"):
                try:
                    ts = datetime.datetime.strptime(r[0], fmt).timestamp()
                    break
                except ValueError:
                    pass
            self.rows.append([ts if ts is not None else time.time()] + r[1:])

    def stop(self, window, loaded):
        """Summary of the samples inside `window` (wall-clock seconds); when
        the timed region was shorter than the sampling interval, of those in
        `loaded` (the timed region and the same workload's passes after it)."""
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread is not None:
            self.thread.join(timeout=5)
        span = "timed region"
        rows = [r for r in self.rows if window[0] <= r[0] <= window[1]]
        if not rows:
            span = "timed region and the profiled pass of the same workload after it"
            rows = [r for r in self.rows if loaded[0] <= r[0] <= loaded[1]]
        if not rows:
            return None
        by_gpu = {}
        for r in rows:
            by_gpu.setdefault(r[1], []).append(r)

        def pw(rs):
            v = [float(r[4]) for r in rs if r[4].replace(".", "", 1).isdigit()]
            return float(np.median(v)) if v else 0.0
        gpu = max(by_gpu, key=lambda g: pw(by_gpu[g]))
        rows = by_gpu[gpu]
        sm = [float(r[2]) for r in rows if r[2].isdigit()]
        mx = [float(r[3]) for r in rows if r[3].isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[6 + k].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "gpu": gpu, "samples": len(rows), "interval_ms": 50, "span": span}


def workload_params(capacity_log2=22):
    from meshhashing_gb300 import config, scene
    wl = scene.full_spline(8)
    pools = 1 << min(23, capacity_log2 + 2)
    return config.params_for(wl, value_capacity=1 << capacity_log2, max_vertex_count=pools,
                             max_triangle_count=pools, overflow_capacity=1 << 20,
                             mesh_page_capacity=1 << (capacity_log2 - 3))


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def bytes_per_launch(stage, nb, px, rpx, vwork, cube_blocks=0, mesh_blocks=0, predict_blocks=0, ray_blocks=None):
    """Algorithmic bytes one launch of a stage must move (per-frame averages of
    the blocks each kernel actually visits, counted on the device)."""
    if stage == "integrate":       # sdf, inv_sigma2, a, b read+write; depth + inlier images
        return nb * 512 * 32 + px * 8
    if stage == "predict":         # vertex slots of blocks with vertices; the inlier image
        return predict_blocks * 512 * 12 + px * 4
    if stage == "raycast":         # 2 KB sdf + 16 B entry per block the rays touch; depth, vertex, normal out
        return (ray_blocks if ray_blocks is not None else nb) * (512 * 4 + 16) + rpx * 36
    if stage == "mesh":            # 9^3 corner tile of 4 fields + cube bytes for tiled blocks;
        # slots (12 + 20 B), cube and claim per voxel of paged blocks, twice; 32 B per vertex
        return cube_blocks * (729 * 16 + 512) + mesh_blocks * 512 * (12 + 20 + 1 + 4) * 2 + vwork * 32
    if stage == "tv":
        return TV_ITERS * px * 36 + px * 24
    if stage == "alloc":
        return px * 4
    if stage == "collect":
        return nb * 16 * 2
    return 0.0


# ---------------------------------------------------------------- batched scenes
BATCH_RES = ((160, 120), (320, 240), (640, 480))
BATCH_VOXEL = (0.004, 0.006, 0.008)


def batch_specs(n_scenes):
    """Scene s: room generator seed s, frame count U[20, 200], resolution and
    voxel size drawn from the batched-fusion workload's sets (seeded)."""
    rng = np.random.default_rng(12345)
    out = []
    for s in range(n_scenes):
        w, h = BATCH_RES[rng.integers(0, 3)]
        out.append(dict(seed=s, frames=int(rng.integers(20, 201)), width=w, height=h,
                        voxel=float(BATCH_VOXEL[rng.integers(0, 3)])))
    return out


def _batch_frame_job(args):
    spec, i = args
    from meshhashing_gb300 import scene
    wl = scene.full_spline(spec["frames"], seed=spec["seed"], width=spec["width"], height=spec["height"])
    return wl.frame(i), wl.pose(i)


def gen_batch_frames(specs):
    """Every frame of every scene's own sequence (spec["frames"] frames)."""
    ctx = mp.get_context("spawn")
    jobs = [(sp, i) for sp in specs for i in range(sp["frames"])]
    with ctx.Pool(min(os.cpu_count() or 4, 16)) as pool:
        out = pool.map(_batch_frame_job, jobs, chunksize=8)
    frames, poses, k = [], [], 0
    for sp in specs:
        frames.append([out[k + i][0] for i in range(sp["frames"])])
        poses.append([out[k + i][1] for i in range(sp["frames"])])
        k += sp["frames"]
    return frames, poses


# Block pool growth of the batched-fusion scenes, measured by fusing every
# scene through its whole sequence with a generous pool: the high-water block
# count follows about K * frames^0.62 for each (width, voxel mm) -- the 5 %
# outliers in [0.3, 5] m keep allocating free space until the swept volume
# fills.  K is the largest ratio seen in each group.
BATCH_GROWTH_EXP = 0.62
BATCH_GROWTH_K = {(160, 4): 9044, (160, 6): 6803, (160, 8): 4440,
                  (320, 4): 23822, (320, 6): 14067, (320, 8): 8878,
                  (640, 4): 53108, (640, 6): 19511, (640, 8): 12138}


def batch_params(spec):
    """Pools sized for the scene's whole sequence: 1.3 x the measured growth
    of its (resolution, voxel) group, mesh pages for a thirty-second of the
    blocks, vertex and triangle pools above the largest counts seen (286 k /
    550 k)."""
    from meshhashing_gb300 import config, scene
    wl = scene.full_spline(spec["frames"], seed=spec["seed"], width=spec["width"], height=spec["height"])
    vox = spec["voxel"]
    k = BATCH_GROWTH_K[(spec["width"], round(vox * 1000))]
    cap = int(1.3 * k * spec["frames"] ** BATCH_GROWTH_EXP) // 1024 * 1024 + 4096
    buckets = 1 << max(14, (cap - 1).bit_length())
    return config.params_for(wl, voxel_size=vox, truncation=3 * vox, value_capacity=cap,
                             bucket_count=buckets, max_vertex_count=1 << 19, max_triangle_count=1 << 20,
                             overflow_capacity=max(buckets // 4, 1024), mesh_page_capacity=max(cap // 32, 6144))


def run_pose_refinement(params, frames, poses, W, H, fused=100, refined=200, iterations=10):
    """Differentiable-raycast pose refinement as the workload states it: a
    fresh volume fuses frames 0..fused-1 (with the TV pre-filter), then each
    of the next `refined` frames starts from its true pose perturbed by sigma
    1 degree / 2 cm per axis (seeded) and runs `iterations` Gauss-Newton steps
    (mh_refine_pose); the reference's point-to-PSDF tracker runs from the same
    starts.  The map is not updated during refinement.  Also one full-frame
    raycast backward with voxel gradients."""
    import torch
    from meshhashing_gb300 import Volume
    from meshhashing_gb300.pose import left_update, pose_error
    vol = Volume(params)
    for i in range(fused):
        vol.integrate_frame(frames[i], poses[i], tv_iterations=TV_ITERS, tv_lambda=TV_LAMBDA)
    torch.cuda.synchronize()
    rng = np.random.default_rng(77)
    start, final, ms = [], [], []
    p2p = {"reference": ([], []), "fixed_jacobian": ([], [])}
    for d, T in zip(frames[fused:fused + refined], poses[fused:fused + refined]):
        T_true = np.asarray(T, np.float64)
        xi = np.concatenate([rng.standard_normal(3) * 0.02, rng.standard_normal(3) * np.radians(1.0)])
        T0 = left_update(T_true, xi)
        vol.set_frame(d, T0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        T_ref, cost, count = vol.refine_pose(T0, iterations=iterations, max_residual=0.05)
        ms.append((time.perf_counter() - t0) * 1000.0)
        start.append(pose_error(T0, T_true))
        final.append(pose_error(T_ref, T_true))
        # the reference's point-to-PSDF tracker from the same start: its own
        # damping and Jacobian, then Gauss-Newton with the corrected Jacobian
        for key, lam, ref_j in (("reference", 1e5, True), ("fixed_jacobian", 1.0, False)):
            vol.set_frame(d, T0)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            T_p, _, _ = vol.track_point_to_psdf(T0, iterations=iterations, lam=lam, reference_jacobian=ref_j)
            p2p[key][0].append((time.perf_counter() - t0) * 1000.0)
            p2p[key][1].append(pose_error(T_p, T_true))
    cTw = np.linalg.inv(np.asarray(poses[fused], np.float64)).astype(np.float32)
    dl = torch.randn((H, W), generator=torch.Generator().manual_seed(3)).cuda()
    grad = torch.zeros(vol.params.value_capacity * 512, dtype=torch.float32, device="cuda")
    vol.raycast_backward(cTw, dl, None, grad)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    vol.raycast_backward(cTw, dl, None, grad)
    bw_ms = (time.perf_counter() - t0) * 1000.0
    vol.close()
    del grad

    def summary(errs):
        mm = np.array([e[0] for e in errs]) * 1000.0
        deg = np.array([e[1] for e in errs])
        return {"median": {"mm": float(np.median(mm)), "deg": float(np.median(deg))},
                "p95": {"mm": float(np.percentile(mm, 95)), "deg": float(np.percentile(deg, 95))},
                "max": {"mm": float(mm.max()), "deg": float(deg.max())}}
    return {"fused_frames": fused, "refined_frames": len(ms), "iterations": iterations,
            "ms_per_frame": {"median": float(np.median(ms)), "p95": float(np.percentile(ms, 95))},
            "start_error": summary(start), "final_error": summary(final),
            "raycast_backward_ms": bw_ms,
            "point_to_psdf": {k: {"ms_per_frame": float(np.median(v[0])), "final_error": summary(v[1])}
                              for k, v in p2p.items()},
            "note": "frames 100..299 of the PSDF sequence on the map of frames 0..99; start poses perturbed by "
                    "sigma 1 deg / 2 cm per axis; ms_per_frame is host wall time of the 10 iterations "
                    "(synchronised); point_to_psdf: the reference's tracker (MainEngine::Localizing) from the same "
                    "starts, with its lambda 1e5 and J[2] = dD/dx, and with lambda 1 and the corrected Jacobian"}


def run_huber_tv(vol, peak, iterations=10):
    """Volumetric Huber-TV (mh_huber_tv_init / _iterate) over the last
    frame's candidate blocks of the fused map: one init, one untimed
    iteration, then `iterations` timed with CUDA events.  Algorithmic bytes
    per iteration, per observed voxel of the work list: the dual pass's 28 B
    read (list entry, sdf, sdf_bar, sdf0, p) + 12 B write (p) and the primal
    pass's 28 B read (list entry, p, sdf, sdf0, weight) + 8 B write (sdf,
    sdf_bar) = 76 B; face neighbours come from cache and are not counted.
    The per-call work list (one pass over the candidates' weight and mask)
    is inside the timed region."""
    import torch
    cand = vol.candidates()
    pos, f = vol.dump_blocks(("w",))
    key = lambda q: (q[:, 0].astype(np.int64) << 42) + (q[:, 1].astype(np.int64) << 21) + q[:, 2]  # noqa: E731
    sel = np.isin(key(pos), key(cand))
    observed = int(np.count_nonzero(f["w"][sel] >= np.float32(1e-6)))
    del f
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    torch.cuda.synchronize()
    e0.record()
    vol.huber_tv_init()
    e1.record()
    vol.huber_tv_iterate(2.0, 8.0, 0.01, 1)
    torch.cuda.synchronize()
    e1b = torch.cuda.Event(enable_timing=True)
    e1b.record()
    energy = vol.huber_tv_iterate(2.0, 8.0, 0.01, iterations)
    e2.record()
    torch.cuda.synchronize()
    ms = e1b.elapsed_time(e2) / iterations
    alg = observed * 76
    gbs = alg / (ms / 1000.0) / 1e9
    return {"candidate_blocks": int(len(cand)), "observed_voxels": observed, "iterations": iterations,
            "init_ms": e0.elapsed_time(e1), "ms_per_iteration": ms, "bytes_per_iteration": alg, "gbs": gbs,
            "frac": gbs / peak, "energy": [float(x) for x in energy],
            "params": {"lambda": 2.0, "sigma": 8.0, "tau": 0.01},
            "note": "CUDA events around the iterations; the energy read-back at the end is inside the timing"}


def run_batched(specs, frames, poses):
    """The batched-fusion schedule: every scene advances through its own
    frame count (U[20, 200]); aggregate frames/s over the whole schedule,
    first with the scenes one after another through the plain per-frame
    chain, then (same volumes, reset) as one batch: one launch per stage for
    all scenes still running (scenes whose sequence ended are retired through
    the step's active mask), autotuned on a separate pass, every step
    replayed from a CUDA graph."""
    import torch
    from meshhashing_gb300 import Batch, Volume
    n = len(specs)
    nfr = [sp["frames"] for sp in specs]
    total_frames = int(sum(nfr))
    steps = max(nfr)
    vols = [Volume(batch_params(sp)) for sp in specs]
    dev = [torch.from_numpy(np.stack(f)).cuda() for f in frames]
    outs = [torch.empty((sp["height"], sp["width"]), dtype=torch.float32, device="cuda") for sp in specs]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def plain_frame(s, i):
        vols[s].integrate_frame(dev[s][i], poses[s][i], on_device=True, tv_iterations=TV_ITERS,
                                tv_lambda=TV_LAMBDA, ray_depth=outs[s], outputs_on_device=True)

    # warm-up: three frames of every scene, then every volume starts empty
    for s in range(n):
        for i in range(3):
            plain_frame(s, i)
    torch.cuda.synchronize()
    for v in vols:
        v.reset()
    log(f"  {n} scenes created and warmed up; plain schedule")
    e0.record()
    for s in range(n):
        for i in range(nfr[s]):
            plain_frame(s, i)
    e1.record()
    torch.cuda.synchronize()
    plain_ms = e0.elapsed_time(e1)
    log(f"  plain schedule {plain_ms / 1000:.1f} s; batch tuning")
    err_plain = sum(v.stats()["error"] != 0 for v in vols)
    plain_blocks = [v.stats()["blocks_allocated"] for v in vols]

    batch = Batch(vols, raycast=True)
    for v in vols:
        v.reset()
    tune_steps = 9
    batch.autotune(1)

    def bstep(i, graph):
        act = [i < nfr[s] for s in range(n)]
        batch.step([dev[s][i] if act[s] else None for s in range(n)], [poses[s][i] if act[s] else None for s in range(n)],
                   active=act, on_device=True, tv_iterations=TV_ITERS, tv_lambda=TV_LAMBDA, use_graph=graph)

    # autotuning and graph capture on a pass over the first steps, then every
    # volume starts empty again
    for i in range(tune_steps):
        bstep(i, False)
    for i in range(tune_steps, tune_steps + 2):
        bstep(i, True)
    torch.cuda.synchronize()
    tuning, times, stage = batch.tuning(), batch.tuning_times(), batch.stage_times()
    for v in vols:
        v.reset()
    log("  batched schedule")
    e0.record()
    for i in range(steps):
        bstep(i, True)
    e1.record()
    torch.cuda.synchronize()
    batch_ms = e0.elapsed_time(e1)
    log(f"  batched schedule {batch_ms / 1000:.1f} s")
    err_batch = sum(v.stats()["error"] != 0 for v in vols)
    same_blocks = all(v.stats()["blocks_allocated"] == b for v, b in zip(vols, plain_blocks))
    batch.close()
    for v in vols:
        v.close()
    del dev
    res, vox = {}, {}
    for sp in specs:
        k = "%dx%d" % (sp["width"], sp["height"])
        res[k] = res.get(k, 0) + 1
        k = "%d" % round(sp["voxel"] * 1000)
        vox[k] = vox.get(k, 0) + 1
    return {"workload": "%d independent room scenes (seeds 0..%d), frame counts U[20, 200], PSDF, TV %d it, raycast"
                        % (n, n - 1, TV_ITERS),
            "scenes": n, "resolutions": res, "voxel_mm": vox, "frames_total": total_frames, "steps": steps,
            "value": total_frames / (batch_ms / 1000.0), "unit": "frames/s (all scenes)",
            "plain_value": total_frames / (plain_ms / 1000.0),
            "speedup_vs_plain": plain_ms / batch_ms, "batch_s": batch_ms / 1000.0, "plain_s": plain_ms / 1000.0,
            "form": "one launch per stage for the scenes still running (active mask), each step replayed from a "
                    "CUDA graph",
            "plain_form": "scenes one after another, each through its whole sequence, per-frame stream launches",
            "same_block_counts": bool(same_blocks),
            "tuning": {"chosen": {"ray_tile": list(tuning["ray_tile"]),
                                  "integrate_cta_per_sm": tuning["integrate_cta_per_sm"]},
                       "raycast_ms": {"%dx%d" % k: v for k, v in times["raycast_ms"].items()},
                       "integrate_ms": {str(k): v for k, v in times["integrate_ms"].items()},
                       "stage_ms_per_step": stage,
                       "note": "autotuning steps 0..8 of the schedule on a separate pass (small maps)"},
            "scenes_with_error": {"plain": int(err_plain), "batched": int(err_batch)}}


# ---------------------------------------------------------------- streaming
STREAM_FRAMES = 300


def _stream_job(i):
    from meshhashing_gb300 import scene
    wl = scene.floor_plan(2000)
    return wl.frame(i), wl.pose(i)


def gen_stream_frames(n):
    ctx = mp.get_context("spawn")
    with ctx.Pool(min(os.cpu_count() or 4, 16)) as pool:
        out = pool.map(_stream_job, list(range(n)), chunksize=2)
    return [o[0] for o in out], [o[1] for o in out]


def run_stream(frames, poses):
    """Large-scene streaming: the first frames of the 2000-frame walk through
    the 12 x 10 x 3 m floor plan (640x480, 5 mm voxels, PSDF, 2^22 buckets),
    the full MainEngine chain with a raycast every frame."""
    import torch
    from meshhashing_gb300 import Volume, config, scene
    wl = scene.floor_plan(2000)
    # 12 M blocks (98 GB of voxels): the walk's 5 % outliers, up to 5 m along
    # the rays, end up allocating most of the free space in and around the
    # building (7.7 M blocks live after the 2000 frames).  At 1.8 blocks per
    # bucket (2^22 buckets of 4 slots) the Teschner hash overfills some
    # buckets past 4 + 7 entries, so overflow chains may grow to 32 here
    # (linked_list_size, a HashParams knob; the reference's default is 7).
    p = config.params_for(wl, voxel_size=0.005, truncation=0.015, value_capacity=12_000_000, bucket_count=1 << 22,
                          max_vertex_count=1 << 23, max_triangle_count=1 << 23, overflow_capacity=1 << 22,
                          mesh_page_capacity=1 << 19, linked_list_size=32)
    vol = Volume(p)
    dev = torch.from_numpy(np.stack(frames)).cuda()
    rd = torch.empty((p.height, p.width), dtype=torch.float32, device="cuda")
    rn = torch.empty((p.height, p.width, 4), dtype=torch.float32, device="cuda")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    peak = 0
    torch.cuda.synchronize()
    e0.record()
    for i in range(len(frames)):
        vol.integrate_frame(dev[i], poses[i], on_device=True, tv_iterations=TV_ITERS, tv_lambda=TV_LAMBDA,
                            ray_depth=rd, ray_normal=rn, outputs_on_device=True)
        if i % 50 == 49:
            peak = max(peak, vol.stats()["blocks_allocated"])
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    s = vol.stats()
    vol.close()
    return {"workload": "floor plan 12x10x3 m, 6 rooms, 40 primitives; 640x480 walk at 0.4 m/s, 5 mm voxels, "
                        "PSDF, 2^22 buckets, TV %d it, raycast every frame" % TV_ITERS,
            "frames": len(frames), "value": len(frames) / (ms / 1000.0), "unit": "frames/s",
            "ms_per_frame": ms / len(frames), "blocks_allocated": s["blocks_allocated"], "blocks_peak": int(peak),
            "gc_freed_blocks": s["gc_freed_blocks"], "triangles": s["triangles_allocated"],
            "vertices": s["vertices_allocated"], "candidates_per_frame": s["candidate_sum"] / max(s["mesh_passes"], 1),
            "error": s["error"], "dropped_inserts": s["dropped_inserts"], "overflow_used": s["overflow_used"],
            "mesh_pages_used": s["mesh_pages_used"], "block_capacity": p.value_capacity,
            "note": "frames 0..%d of the 2000-frame walk, the map growing from empty; the stats() reads "
                    "every 50 frames are inside the timed region" % (len(frames) - 1)}


def max_over_ranks(x, world, device):
    """The largest x over the ranks: replicas run in lockstep between
    barriers, so the job takes as long as its slowest rank."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(world, steps, seconds):
    """Whole-job frames/s: every rank advances its own replica by `steps`
    frames in `seconds` (the max over ranks)."""
    return world * steps / seconds


def bench_config(prefuse, warmup, world=1):
    """The workload of both arms (ours and --impl reference), identical so the
    two lines describe the same frames."""
    return {"workload": "psdf_640x480_4mm_room_spline", "resolution": [640, 480], "voxel_mm": 4,
            "truncation_mm": 12, "buckets": 1 << 21, "tv_iterations": TV_ITERS, "prefuse_frames": prefuse,
            "timed_frames": f"from frame {prefuse + warmup} on, one frame per step, after {warmup} warm-up frames",
            "l2": "per-frame voxel working set (hundreds of thousands of 8 KB blocks) exceeds L2; no flush",
            "parallelism": "replicas" if world > 1 else "single"}


REF_MAX_FRAMES = 40
POSE_FUSED, POSE_REFINED = 100, 200
SEQ_FRAMES = 500   # the PSDF workload's sequence length


def run_cpu_baseline(params, frames, poses, threads=None):
    """FP64 oracle on all host threads, from an empty volume."""
    from oracle import oracle as O
    O.build()
    if threads:
        O.set_threads(threads)
    o = O.Oracle(params, fp64=True)
    t0 = time.perf_counter()
    for d, T in zip(frames, poses):
        o.frame(d, T, raycast=True, tv_iterations=TV_ITERS, tv_lambda=TV_LAMBDA)
    dt = time.perf_counter() - t0
    return len(frames) / dt, O.num_threads(), dt


def run_reference(args, rank, world):
    """The reference path's CPU implementation (the FP64 oracle restating the
    reference's rules; the reference itself has no CPU path) on the same
    frames as our arm: the map is pre-fused with the same prefuse + warm-up
    frames (untimed), then the timed window's frames follow, one per step, up
    to REF_MAX_FRAMES of them so the run stays within a few minutes."""
    if rank != 0:
        return
    import platform
    params = workload_params()
    P, W = args.prefuse, args.warmup
    n_time = max(1, min(args.steps, REF_MAX_FRAMES))
    frames, poses = gen_frames(list(range(P + W + n_time)), SEQ_FRAMES)
    from oracle import oracle as O
    O.build()
    o = O.Oracle(params, fp64=True)
    t_pre = time.perf_counter()
    for i in range(P + W):
        o.frame(frames[i], poses[i], raycast=True, tv_iterations=TV_ITERS, tv_lambda=TV_LAMBDA)
    t_pre = time.perf_counter() - t_pre
    t0 = time.perf_counter()
    for i in range(P + W, P + W + n_time):
        o.frame(frames[i], poses[i], raycast=True, tv_iterations=TV_ITERS, tv_lambda=TV_LAMBDA)
    dt = time.perf_counter() - t0
    fps = n_time / dt
    cores = O.num_threads()
    sample = (f"frames {P + W}..{P + W + n_time - 1} (the first {n_time} of the timed window) on the map pre-fused "
              f"from frames 0..{P + W - 1} ({t_pre:.0f} s, untimed); FP64 oracle, {cores} threads, "
              f"{platform.machine()}")
    out = {"metric": METRIC, "value": fps, "unit": "frames/s", "n_gpus": world, "steps": n_time,
           "warmup": W, "ms_per_step": 1000.0 * dt / n_time, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "impl": "reference",
           "config": bench_config(P, W, world),
           "cpu_baseline": {"value": fps, "unit": "frames/s", "cores": cores, "kind": "port", "sample": sample},
           "e2e": {"value": fps, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--prefuse", type=int, default=40)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-frames", type=int, default=16,
                    help="frames of the FP64 oracle CPU baseline (about 10 s on 16 cores)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batch-scenes", type=int, default=64,
                    help="scenes of the batched-vs-plain measurement (0: skip it)")
    ap.add_argument("--stream-frames", type=int, default=STREAM_FRAMES,
                    help="frames of the floor-plan streaming measurement (0: skip it)")
    ap.add_argument("--pose-refined", type=int, default=POSE_REFINED,
                    help="frames of the pose-refinement measurement after its 100 fused frames (0: skip it)")
    ap.add_argument("--capacity-log2", type=int, default=22,
                    help="block pool size (2^n blocks); smaller values for profiler captures")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    K, W, P = args.steps, args.warmup, args.prefuse
    # Every frame comes from the workload's 500-frame sequence: the timed pass
    # takes K frames, the per-stage pass up to 100 after it; the e2e pass
    # replays the timed pass's K frames after a reset; the pose-refinement
    # measurement uses frames 0..299.
    K2, K3 = min(K, 100), K
    if P + W + K + K2 > SEQ_FRAMES:
        raise SystemExit(f"--prefuse + --warmup + --steps + min(steps, 100) must be <= {SEQ_FRAMES}")
    n_total = SEQ_FRAMES
    # frames are rendered in a spawn pool before any CUDA call
    n_pose = POSE_FUSED + args.pose_refined if args.pose_refined > 0 else 0
    log("rendering the PSDF sequence")
    frames, poses = gen_frames(list(range(max(P + W + K + K2, n_pose))), SEQ_FRAMES)
    cpu_frames = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu_frames = (frames[:args.cpu_frames], poses[:args.cpu_frames])

    bspecs = batch_specs(args.batch_scenes) if (args.batch_scenes > 0 and world == 1) else []
    if bspecs:
        log(f"rendering the batched-fusion scenes ({sum(sp['frames'] for sp in bspecs)} frames)")
    bframes = gen_batch_frames(bspecs) if bspecs else None
    if args.stream_frames > 0 and world == 1:
        log(f"rendering {args.stream_frames} floor-plan frames")
    sframes = gen_stream_frames(args.stream_frames) if (args.stream_frames > 0 and world == 1) else None
    log("frames ready")

    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from meshhashing_gb300 import Volume, launch_count
    from meshhashing_gb300 import build as B
    B.build()
    params = workload_params(args.capacity_log2)
    vol = Volume(params)
    Hh, Ww = params.height, params.width
    dev_depth = torch.from_numpy(np.stack(frames[:P + W + K + K2])).cuda()
    rd = torch.empty((Hh, Ww), dtype=torch.float32, device="cuda")
    rv = torch.empty((Hh, Ww, 4), dtype=torch.float32, device="cuda")
    rn = torch.empty((Hh, Ww, 4), dtype=torch.float32, device="cuda")

    def step(i):
        vol.integrate_frame(dev_depth[i], poses[i], on_device=True, tv_iterations=TV_ITERS, tv_lambda=TV_LAMBDA,
                            ray_depth=rd, ray_vertex=rv, ray_normal=rn, outputs_on_device=True)

    for i in range(P + W):
        step(i)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    sampler = ClockSampler()
    log("map pre-fused; timed region")
    sampler.start()
    time.sleep(0.3)                     # nvidia-smi is sampling before the timed region starts
    barrier()
    l0 = launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    w0 = time.time()
    e0.record()
    for i in range(P + W, P + W + K):
        step(i)
    e1.record()
    barrier()
    w1 = time.time()
    launches = launch_count() - l0
    ms = e0.elapsed_time(e1)
    # per-stage times: a second pass over the next K frames with CUDA events
    # around every stage (kept out of the timed region above)
    s0 = vol.stats()
    vol.profile(True)
    vol.profile_read()
    for i in range(P + W + K, P + W + K + K2):
        step(i)
    prof = vol.profile_read()
    vol.profile(False)
    s1 = vol.stats()
    # the raycast's block footprint (distinct blocks its rays look up) at the
    # last profiled frame's pose, for the raycast byte model
    ray_blocks = vol.raycast_footprint(np.linalg.inv(np.asarray(poses[P + W + K + K2 - 1], np.float64))
                                       .astype(np.float32))
    clocks = sampler.stop((w0, w1), (w0, time.time()))
    ms = max_over_ranks(ms, world, "cuda")
    value = job_rate(world, K, ms / 1000.0)

    s2 = vol.stats()
    # e2e: the timed pass's K frames again, on the same map states: the
    # volume is reset and the same P + W frames are pre-fused (untimed); then
    # each frame's depth goes in from pinned host memory and its raycast depth
    # comes back to the host
    vol.reset()
    for i in range(P + W):
        step(i)
    host_in = [torch.from_numpy(f).pin_memory() for f in frames[P + W:P + W + K3]]
    host_out = torch.empty((Hh, Ww), dtype=torch.float32).pin_memory()
    step_e2e = lambda j: vol.integrate_frame(host_in[j], poses[P + W + j], on_device=False,
                                             tv_iterations=TV_ITERS, tv_lambda=TV_LAMBDA, ray_depth=host_out,
                                             outputs_on_device=False)
    barrier()
    t0 = time.perf_counter()
    for j in range(K3):
        step_e2e(j)
    barrier()
    e2e_s = max_over_ranks(time.perf_counter() - t0, world, "cuda")
    e2e = job_rate(world, K3, e2e_s)
    s3 = vol.stats()

    passes = max(s1["mesh_passes"] - s0["mesh_passes"], 1)
    nb = (s1["candidate_sum"] - s0["candidate_sum"]) / passes
    vwork = (s1["vertex_work_sum"] - s0["vertex_work_sum"]) / passes
    counts = {"cube_blocks": (s1["cube_blocks_sum"] - s0["cube_blocks_sum"]) / passes,
              "mesh_blocks": (s1["mesh_list_sum"] - s0["mesh_list_sum"]) / passes,
              "predict_blocks": (s1["predict_blocks_sum"] - s0["predict_blocks_sum"]) / passes,
              "ray_blocks": ray_blocks}
    px, rpx = Ww * Hh, params.rc_width * params.rc_height
    peak, peak_kind = peaks()
    stage_ms = {k: v[0] for k, v in prof.items()}
    dom = max(("integrate", "raycast", "predict", "alloc", "collect"), key=lambda k: stage_ms[k])
    calls = max(prof[dom][1], 1)
    per_launch_ms = stage_ms[dom] / calls
    alg = bytes_per_launch(dom, nb, px, rpx, vwork, **counts)
    achieved = alg / (per_launch_ms / 1000.0) / 1e9
    # DRAM bytes per launch measured by ncu (dram__bytes_read.sum + _write.sum,
    # --set full) on this workload's 10-frame map (frame 9: 274,742 candidate
    # blocks, 143,854 of them looked up by rays), scaled to this run by the
    # units the kernel's traffic follows: blocks the rays look up for the
    # raycast, candidate blocks for the integrate
    NCU_TRAFFIC = {"raycast": (116.87e6, 143854.0, "ray_blocks", "blocks looked up by rays"),
                   "integrate": (1780.52e6, 274742.0, "candidates", "candidate blocks")}
    traffic, traffic_src = None, None
    if dom in NCU_TRAFFIC:
        b0, n0, unit, what = NCU_TRAFFIC[dom]
        n1 = ray_blocks if unit == "ray_blocks" else nb
        traffic = b0 * n1 / n0
        traffic_src = ("ncu DRAM read+write of one launch at %d %s (frame 9 of this workload, 10-frame map), "
                       "scaled by %s" % (int(n0), what, what))
    stages = {}
    for k, (t_ms, c) in prof.items():
        if c:
            b = bytes_per_launch(k, nb, px, rpx, vwork, **counts)
            gbs = b / ((t_ms / c) / 1000.0) / 1e9 if t_ms > 0 else None
            stages[k] = {"ms_per_frame": t_ms / K2, "gbs": gbs, "frac": (gbs / peak) if gbs else None}

    log("Huber-TV")
    huber = run_huber_tv(vol, peak)
    vol.close()
    log("pose refinement")
    pose = run_pose_refinement(params, frames, poses, Ww, Hh, POSE_FUSED, args.pose_refined) \
        if args.pose_refined > 0 else None
    batched = None
    if bspecs:
        log("batched fusion, all scenes")
        batched = run_batched(bspecs, bframes[0], bframes[1])
        log("batched fusion, scenes below 640x480")
        small = [k for k, sp in enumerate(bspecs) if sp["width"] < 640]
        batched["below_640x480"] = run_batched([bspecs[k] for k in small], [bframes[0][k] for k in small],
                                               [bframes[1][k] for k in small])
    if sframes:
        log("streaming")
    stream = run_stream(*sframes) if sframes else None

    cpu = None
    if cpu_frames is not None:
        log("CPU baseline")
        fps, cores, dt = run_cpu_baseline(params, *cpu_frames)
        cpu = {"value": fps, "unit": "frames/s", "cores": cores, "kind": "port",
               "sample": f"frames 0..{len(cpu_frames[0]) - 1} from an empty volume (FP64 oracle), {dt:.1f} s"}

    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": "frames/s", "n_gpus": world, "steps": K, "warmup": W,
               "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
               "dtype": "f32", "data": "synthetic",
               "config": bench_config(P, W, world),
               "form": "plain (per-frame stream launches)",
               "e2e": {"value": e2e, "unit": "frames/s", "h2d_bytes_per_step": px * 4 + 64,
                       "d2h_bytes_per_step": rpx * 4,
                       "frames": f"{P + W}..{P + W + K3 - 1} (the timed frames), replayed after a volume reset "
                                 f"and the same {P + W}-frame pre-fusion"},
               "gpu_launches": int(launches),
               "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                            "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                            "bytes_per_launch": alg, "traffic_source": traffic_src},
               "stages": stages,
               "blocks": {"candidates_per_frame": nb, "vertices_per_frame": vwork, **counts,
                          "allocated": s2["blocks_allocated"], "mesh_pages": s2["mesh_pages_used"],
                          "error": s2["error"] or s3["error"]},
               "clocks": clocks,
               "pose_refinement": pose,
               "huber_tv": huber,
               "batched": batched,
               "stream": stream,
               "cpu_baseline": cpu}
        print(json.dumps(out), flush=True)
        log("done")
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
