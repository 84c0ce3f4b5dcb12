"""Benchmark of the per-frame TSDF path: allocate -> integrate -> extract.

Workload (default): the long synthetic stream - 640x480 uint16 depth + RGB of
a seeded 8x8x3 m room with 40 boxes/spheres/cylinders, spline trajectory at
0.5 m/s and 30 Hz, 5 mm voxels, 20 mm truncation, 2^22 hash slots; one step
is one frame through allocate -> integrate -> per-frame marching cubes,
launched as one CUDA graph.  The frames are generated by the seeded scene
generator (no dataset is needed or present).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference]

Prints one JSON line (rank 0).  `value` is frames/s with the frames already
in HBM (device time of each step, L2 flushed between steps); `e2e` is the
same through the C ABI with host buffers (pinned): each frame's depth and
colour uploaded and its whole mesh copied back to host memory as vertices
and faces (`e2e.triangle_soup`: the same triangles as a soup), frames
submitted back to back (`e2e.sync_per_frame`: one frame at a time;
`e2e.mesh_left_on_device`: without the mesh copy).
`--impl reference` times the CPU restatement of the reference's algorithm
(oracle/) on all host cores on the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "voxel-hashing-sdf_gb300")
for p in (REPO, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402

METRIC = "TSDF frames/s (allocate+integrate+extract per frame)"
UNIT = "frames/s"
WORKLOAD = {
    "workload": "long synthetic stream: 640x480 u16 depth + RGB, 8x8x3 m room with 40 objects, "
                "spline trajectory 0.5 m/s @ 30 Hz, 5 mm voxels, 20 mm truncation, 2^22 hash slots, "
                "per-frame allocate->integrate->extract as one CUDA graph",
    "width": 640, "height": 480, "voxel_m": 0.005, "trunc_m": 0.02, "table_log2": 22,
    "max_depth_m": 4.0, "scene_seed": 2,
}
ENGINE_PARAMS = dict(width=640, height=480, min_depth=0.1, max_depth=4.0, voxel_size=0.005,
                     trunc=0.02, table_log2=22, pool_blocks=1_500_000,
                     max_frame_blocks=200_000, max_triangles=8_000_000)
L2_BYTES = 129 * 1024 * 1024


def traffic_ratios():
    """DRAM traffic / algorithmic bytes per kernel launch from the committed
    ncu capture (profiles/traffic_per_kernel_long_stream.txt), or {}."""
    out = {}
    try:
        with open(os.path.join(REPO, "profiles", "traffic_per_kernel_long_stream.txt")) as f:
            for line in f:
                if line.startswith("traffic_ratio "):
                    _, k, v = line.split()
                    out[k] = float(v)
    except OSError:
        pass
    return out


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def peak_hbm():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""

    def __init__(self, gpu):
        self.gpu = gpu
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}", "--format=csv,noheader",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}

        def num(s):
            try:
                return float(s.split()[0])
            except Exception:
                return None
        sm = [num(r[1]) for r in self.rows if len(r) > 2 and num(r[1])]
        mx = [num(r[2]) for r in self.rows if len(r) > 2 and num(r[2])]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for i, n in enumerate(names):
                if len(r) > 5 + i and r[5 + i].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.rows)}


def make_frames(num, seed):
    from vhsdf import synth
    s = synth.Scene(kind=2, seed=seed, num_frames=max(num, 1))
    frames = [s.render(f) for f in range(num)]
    return s, frames


def cpu_leg(frames, scene, seconds=15.0, threads=None):
    """Times the oracle (all threads, or `threads`) on the first frames of
    the stream."""
    from oracle.oracle import Oracle
    all_threads = Oracle.max_threads()
    if threads:
        Oracle.set_threads(threads)
    cores = Oracle.max_threads()
    o = Oracle(640, 480, scene.fx, scene.fy, scene.cx, scene.cy, min_depth=0.1, max_depth=4.0,
               voxel_size=0.005, trunc=0.02, mc_min_weight=1.0, precision=64)
    t0 = time.perf_counter()
    n = 0
    for d, c, p in frames:
        o.integrate(d, c, p)
        o.marching_cubes("frame")
        n += 1
        if time.perf_counter() - t0 > seconds:
            break
    dt = time.perf_counter() - t0
    if threads:
        Oracle.set_threads(all_threads)
    return {"value": n / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"first {n} frames of the same stream (allocate+integrate+per-frame MC), "
                      f"FP64 oracle, {cores} thread{'' if cores == 1 else 's'}, {dt:.1f} s"}


def perturb_pose(pose, deg, metres, rng):
    """Rotates the camera by `deg` about a random axis through its centre and
    moves the centre by `metres` along a random direction."""
    axis = rng.normal(size=3)
    axis /= np.linalg.norm(axis)
    th = np.deg2rad(deg)
    K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    R = np.eye(3) + np.sin(th) * K + (1 - np.cos(th)) * K @ K
    dirn = rng.normal(size=3)
    dirn /= np.linalg.norm(dirn)
    out = pose.astype(np.float64).copy()
    out[:3, :3] = R @ out[:3, :3]
    out[:3, 3] = out[:3, 3] + metres * dirn
    return out.astype(np.float32)


def pose_error(a, b):
    dt = np.linalg.norm(a[:3, 3].astype(np.float64) - b[:3, 3])
    dR = a[:3, :3].astype(np.float64) @ b[:3, :3].T.astype(np.float64)
    return dt, float(np.degrees(np.arccos(np.clip((np.trace(dR) - 1) / 2, -1, 1))))


def volume_extras(vol, poses, local):
    """Ray casting and mesh export on a fused volume: 640x480 depth / normal /
    colour maps from each pose into device buffers (CUDA events on the
    volume's stream), and one full-volume extraction with the GPU vertex
    merge (host clock, including the copies of the indexed mesh)."""
    import torch
    from vhsdf import _native as N
    stream = torch.cuda.Stream(device=local)
    vol.set_stream(stream.cuda_stream)
    p = vol.params
    depth = torch.empty((p.height, p.width), dtype=torch.float32, device="cuda")
    normal = torch.empty((p.height, p.width, 3), dtype=torch.float32, device="cuda")
    rgb = torch.empty((p.height, p.width, 3), dtype=torch.uint8, device="cuda")
    hits = []

    def cast(c2w):
        pose = np.ascontiguousarray(np.asarray(c2w, np.float32).reshape(16))
        N.check(vol._L.vh_raycast(vol._h, pose.ctypes.data, depth.data_ptr(), normal.data_ptr(),
                                  rgb.data_ptr(), N.VH_MEM_DEVICE))

    for c2w in poses[:3]:
        cast(c2w)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2 * len(poses))]
    for k, c2w in enumerate(poses):
        ev[2 * k].record(stream)
        cast(c2w)
        ev[2 * k + 1].record(stream)
        hits.append(float((depth > 0).float().mean()))
    stream.synchronize()
    ms = [ev[2 * k].elapsed_time(ev[2 * k + 1]) for k in range(len(poses))]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    verts, cols, faces = vol.mesh_indexed()
    t_mesh = time.perf_counter() - t0
    return {"raycast_ms_640x480": float(np.median(ms)),
            "raycast_rays_per_s": p.width * p.height / (np.median(ms) / 1000.0),
            "raycast_hit_fraction_median": float(np.median(hits)),
            "mesh_indexed": {"faces": int(len(faces)), "vertices": int(len(verts)),
                             "s_incl_extract_and_copies": t_mesh}}


def adjoint_leg(num_frames, local, iterations=20):
    """Differentiable pose refinement: the 4x4x3 m room with 3 spheres, 100
    frames 640x480 fused at 5 mm (truncation 0.1 m); `num_frames` of its poses
    perturbed by a seeded 2 deg rotation about the camera centre and a 20 mm
    translation, then refined with 20 Gauss-Newton steps over all pixels by the
    sampling adjoint and by forward-only central differences (13 residual
    evaluations per pixel and step).  pose_steps_per_s counts the steps alone
    (device events around the graph of steps); call_steps_per_s the whole call
    (depth upload, pose upload, steps, download)."""
    from vhsdf import Volume, synth
    s = synth.Scene(kind=1, seed=0, num_frames=100)
    vol = Volume(width=640, height=480, fx=s.fx, fy=s.fy, cx=s.cx, cy=s.cy, min_depth=0.1,
                 max_depth=4.5, voxel_size=0.005, trunc=0.1, table_log2=22,
                 pool_blocks=400_000, max_frame_blocks=200_000, max_triangles=1 << 20,
                 device=local)
    frames = [s.render(f) for f in range(100)]
    for d, c, p in frames:
        vol.integrate(d, c, p)
    picks = np.linspace(0, 99, num_frames).astype(int)
    inits = {int(f): perturb_pose(frames[f][2], 2.0, 0.02, np.random.default_rng(1000 + int(f)))
             for f in picks}
    out, poses = {}, {}
    for method in ("adjoint", "fd"):
        vol.pose_refine(frames[0][0], inits[int(picks[0])], iterations=iterations, method=method)
        ms = ms_call = 0.0
        errs, res = [], []
        for f in picks:
            d, _, gt = frames[f]
            r, st = vol.pose_refine(d, inits[int(f)], iterations=iterations, stride=1,
                                    method=method)
            ms += st["ms_steps"]
            ms_call += st["ms"]
            errs.append(pose_error(r, gt))
            res.append(r)
        poses[method] = res
        steps = iterations * len(picks)
        e_mm = np.array([1000 * e[0] for e in errs])
        e_deg = np.array([e[1] for e in errs])
        ok = (e_mm <= 1.0) & (e_deg <= 0.05)
        out[method] = {"pose_steps_per_s": steps / (ms / 1000.0),
                       "call_steps_per_s": steps / (ms_call / 1000.0),
                       "us_per_step": 1000.0 * ms / steps,
                       "within_1mm_0.05deg": int(ok.sum()),
                       "within_2mm_0.1deg": int(((e_mm <= 2.0) & (e_deg <= 0.1)).sum()),
                       "err_mm_median": float(np.median(e_mm)),
                       "err_deg_median": float(np.median(e_deg)),
                       "err_mm_p90": float(np.percentile(e_mm, 90)),
                       "err_deg_p90": float(np.percentile(e_deg, 90))}
    gap = [pose_error(a, b) for a, b in zip(poses["adjoint"], poses["fd"])]
    # the data's floor: refinement started at the ground-truth pose
    floor, to_floor = [], []
    for f, r in zip(picks, poses["adjoint"]):
        d, _, gt = frames[f]
        r0, _ = vol.pose_refine(d, gt, iterations=iterations, stride=1, method="adjoint")
        floor.append(pose_error(r0, gt))
        to_floor.append(pose_error(r, r0))
    out["floor"] = {
        "from": "refinement started at the ground-truth pose (same steps, adjoint)",
        "err_mm_median": float(np.median([1000 * e[0] for e in floor])),
        "err_deg_median": float(np.median([e[1] for e in floor])),
        "adjoint_gap_to_floor_mm_median": float(np.median([1000 * e[0] for e in to_floor])),
        "adjoint_gap_to_floor_deg_median": float(np.median([e[1] for e in to_floor])),
        "adjoint_within_1mm_0.05deg_of_floor": int(sum(1 for e in to_floor
                                                        if 1000 * e[0] <= 1 and e[1] <= 0.05))}
    # the same poses through vh_pose_refine_batch, 16 per call (one launch per
    # Gauss-Newton step for all 16)
    vol.pose_refine_batch([frames[int(f)][0] for f in picks[:16]],
                          [inits[int(f)] for f in picks[:16]], iterations=iterations)
    ms_b, errs_b, res_b = 0.0, [], []
    for i in range(0, len(picks), 16):
        group = picks[i:i + 16]
        r, st = vol.pose_refine_batch([frames[int(f)][0] for f in group],
                                      [inits[int(f)] for f in group], iterations=iterations)
        ms_b += st[0]["ms_steps"]
        for k, f in enumerate(group):
            errs_b.append(pose_error(r[k], frames[int(f)][2]))
            res_b.append(r[k])
    eb_mm = np.array([1000 * e[0] for e in errs_b])
    eb_deg = np.array([e[1] for e in errs_b])
    out["adjoint_batched"] = {
        "poses_per_call": 16,
        "pose_steps_per_s": iterations * len(picks) / (ms_b / 1000.0),
        "within_1mm_0.05deg": int(((eb_mm <= 1.0) & (eb_deg <= 0.05)).sum()),
        "err_mm_median": float(np.median(eb_mm)),
        "err_deg_median": float(np.median(eb_deg)),
        "gap_to_one_at_a_time_mm_median": float(np.median(
            [1000 * pose_error(a, b)[0] for a, b in zip(res_b, poses["adjoint"])]))}
    extras = volume_extras(vol, [frames[int(f)][2] for f in picks], local)
    vol.close()
    return {"workload": "4x4x3 m room, 3 spheres, 100 frames 640x480 fused at 5 mm (T 0.1 m); "
                        f"{len(picks)} poses perturbed 2 deg about the camera centre + 20 mm "
                        f"(seeded); {iterations} Gauss-Newton steps, all 307200 pixels",
            "adjoint": out["adjoint"], "fd_jacobian": out["fd"],
            "adjoint_batched": out["adjoint_batched"],
            "floor": out["floor"],
            "adjoint_vs_fd_pose_gap_mm_median": float(np.median([1000 * g[0] for g in gap])),
            "speedup": out["adjoint"]["pose_steps_per_s"] / out["fd"]["pose_steps_per_s"],
            "same_volume": extras}


BATCH_RES = [(320, 240), (640, 480), (960, 720), (1280, 960)]


def batch_specs(num_scenes, small=False):
    """The batched-scenes workload: scene s (seed 100 + s) is a seeded room
    of extent U[1, 8] m with voxel U[4, 20] mm, truncation max(4 voxels,
    30 mm) (the depth noise reaches 1.5e-3 z^2 = 24 mm at 4 m), U[10, 200]
    frames and one of four depth resolutions; hash table and pool are sized
    from the room's surface (table 2^16 .. 2^22).  small: scenes of seeds
    1000 + s at 160x120 with voxels U[10, 20] mm (a launch-bound batch)."""
    from vhsdf import synth
    out = []
    for s in range(num_scenes):
        seed = (1000 if small else 100) + s
        rng = np.random.default_rng(seed)
        vox = float(rng.uniform(0.010, 0.020) if small else rng.uniform(0.004, 0.020))
        nf = int(rng.integers(10, 201))
        w, h = (160, 120) if small else BATCH_RES[int(rng.integers(0, 4))]
        sc = synth.Scene(kind=3, seed=seed, num_frames=nf, width=w, height=h)
        lo, hi = sc.bounds()
        ext = hi - lo
        area = 2 * ext[0] * ext[1] + 2 * (ext[0] + ext[1]) * ext[2]
        blocks = int(4 * area / (8 * vox) ** 2) + 4096
        tlog = int(min(22, max(16, np.ceil(np.log2(2 * blocks)))))
        prm = dict(width=w, height=h, fx=sc.fx, fy=sc.fy, cx=sc.cx, cy=sc.cy, min_depth=0.1,
                   max_depth=8.0, voxel_size=vox, trunc=max(4 * vox, 0.03), table_log2=tlog,
                   pool_blocks=min(blocks, (1 << tlog) - (1 << (tlog - 3))),
                   max_frame_blocks=min(blocks, 400_000), max_triangles=16 * w * h, flags=0)
        out.append((sc, nf, prm))
    return out


def _timed_batch(params, frames, prepared, with_mesh):
    """One batch over `params`: warm-up step (graph capture), volumes reset,
    then the prepared steps through the C ABI, timed by the host clock
    between device synchronisations.  Returns (seconds, status, stats)."""
    from vhsdf import Batch
    from vhsdf import _native as N
    L = N.lib()
    batch = Batch(params)
    batch.process([fr[0] for fr in frames], with_mesh=with_mesh, depth_format="u16")
    batch.sync()
    for i in range(len(params)):
        batch.scene(i).reset()
    batch.sync()
    t0 = time.perf_counter()
    for dp, cp, poses in prepared:
        N.check(L.vh_batch_process(batch._b, dp, N.VH_DEPTH_U16_MM, cp, poses.ctypes.data,
                                   N.VH_MEM_DEVICE, 1 if with_mesh else 0))
    status, bstats = batch.sync()
    t = time.perf_counter() - t0
    batch.close()
    return t, status, bstats


def batched_leg(num_scenes, steps, local, small=False):
    """Many uneven scenes in one persistent launch per stage (vh_batch) vs the
    same frames through one handle per scene (one per-frame graph each).
    Frames are resident on the device; both runs are timed by the host clock
    between device synchronisations, allocate -> integrate per frame (a
    single noisy frame at 4 mm voxels flips sign across the whole band, so
    per-frame meshes grow beyond 16 triangles per pixel: fusion is timed,
    extraction is not)."""
    import torch
    from vhsdf import Batch, Volume
    specs = batch_specs(num_scenes, small)
    frames = []
    for sc, nf, prm in specs:
        fr = []
        for f in range(min(nf, steps)):
            d, c, p = sc.render(f)
            fr.append((torch.from_numpy(d.astype(np.int16)).cuda(local),
                       torch.from_numpy(c).cuda(local), p))
        frames.append(fr)
    total = sum(len(fr) for fr in frames)
    pixels = sum(prm["width"] * prm["height"] * len(fr) for (_, _, prm), fr in zip(specs, frames))
    torch.cuda.synchronize()
    batch = Batch([dict(prm, device=local) for _, _, prm in specs])
    # warm-up (graph capture) on the first frames, then start from empty volumes
    batch.process([fr[0] for fr in frames], with_mesh=False, depth_format="u16")
    batch.sync()
    for i in range(num_scenes):
        batch.scene(i).reset()
    batch.sync()
    # the C ABI called directly with each step's arguments prepared before
    # the timed loop (the Python wrapper's per-tensor checks are not part of
    # the engine); the same for the per-scene arm below
    import ctypes as C
    from vhsdf import _native as N
    L = N.lib()
    prepared = []
    for k in range(steps):
        dp, cp = (C.c_void_p * num_scenes)(), (C.c_void_p * num_scenes)()
        poses = np.zeros((num_scenes, 16), np.float32)
        for i, fr in enumerate(frames):
            if k < len(fr):
                dp[i], cp[i] = fr[k][0].data_ptr(), fr[k][1].data_ptr()
                poses[i] = np.asarray(fr[k][2], np.float32).reshape(16)
        prepared.append((dp, cp, poses))
    t0 = time.perf_counter()
    for dp, cp, poses in prepared:
        N.check(L.vh_batch_process(batch._b, dp, N.VH_DEPTH_U16_MM, cp, poses.ctypes.data,
                                   N.VH_MEM_DEVICE, 0))
    status, bstats = batch.sync()
    t_batch = time.perf_counter() - t0
    # the same through the Python wrapper (per-tensor checks each step)
    for i in range(num_scenes):
        batch.scene(i).reset()
    batch.sync()
    t0 = time.perf_counter()
    for k in range(steps):
        batch.process([fr[k] if k < len(fr) else None for fr in frames], with_mesh=False,
                      depth_format="u16")
    batch.sync()
    t_batch_py = time.perf_counter() - t0
    batch.close()
    # the whole step as one persistent launch (VH_FLAG_BATCH_FUSED)
    t_fused, fstatus, fstats = _timed_batch(
        [dict(prm, device=local, flags=N.VH_FLAG_BATCH_FUSED) for _, _, prm in specs], frames,
        prepared, False)
    vols = [Volume(**dict(prm, device=local)) for _, _, prm in specs]
    for v, fr in zip(vols, frames):
        v.integrate(*fr[0], depth_format="u16")
    for v in vols:
        v.sync()
        v.reset()
    for v in vols:
        v.sync()
    single = []
    for k in range(steps):
        row = []
        for v, fr in zip(vols, frames):
            if k < len(fr):
                pose = np.ascontiguousarray(np.asarray(fr[k][2], np.float32).reshape(16))
                row.append((v._h, fr[k][0].data_ptr(), fr[k][1].data_ptr(), pose))
        single.append(row)
    t0 = time.perf_counter()
    for row in single:
        for h, dptr, cptr, pose in row:
            N.check(L.vh_integrate(h, dptr, N.VH_DEPTH_U16_MM, cptr, pose.ctypes.data,
                                   N.VH_MEM_DEVICE))
    for v in vols:
        v.sync()
    t_seq = time.perf_counter() - t0
    sstats = [v.stats() for v in vols]
    for v in vols:
        v.reset()
    for v in vols:
        v.sync()
    t0 = time.perf_counter()
    for k in range(steps):
        for v, fr in zip(vols, frames):
            if k < len(fr):
                v.integrate(*fr[k], depth_format="u16")
    for v in vols:
        v.sync()
    t_seq_py = time.perf_counter() - t0
    same = all(b["blocks_allocated"] == q["blocks_allocated"]
               and b["voxels_updated"] == q["voxels_updated"] for b, q in zip(bstats, sstats))
    same_fused = all(b["blocks_allocated"] == q["blocks_allocated"]
                     and b["voxels_updated"] == q["voxels_updated"]
                     for b, q in zip(fstats, sstats))
    for v in vols:
        v.close()
    extraction = None
    if small:
        try:
            extraction = _batched_extraction(specs, frames, steps, local)
        except Exception as e:  # a capacity error is reported, not fatal
            extraction = {"unavailable": f"{type(e).__name__}: {e}"}
    first = 1000 if small else 100
    shape = ("160x120, voxel U[10, 20] mm" if small else
             "320x240 .. 1280x960, voxel U[4, 20] mm")
    return {"workload": f"{num_scenes} seeded rooms (seeds {first}..{first + num_scenes - 1}): "
                        f"extent U[1, 8] m, {shape}, truncation max(4 voxels, 30 mm), "
                        "U[10, 200] frames, tables 2^16 .. 2^22; first "
                        f"{steps} frames of each, allocate -> integrate per frame",
            "frames": total, "megapixels": pixels / 1e6,
            "batched_frames_per_s": total / t_batch, "per_scene_graphs_frames_per_s": total / t_seq,
            "speedup": t_seq / t_batch, "status_ok": all(x == 0 for x in status),
            "calls": "C ABI with each step's arguments prepared before the timed loop",
            "through_python_wrappers": {"batched_frames_per_s": total / t_batch_py,
                                        "per_scene_graphs_frames_per_s": total / t_seq_py,
                                        "speedup": t_seq_py / t_batch_py},
            "counts_equal_per_scene": same,
            "one_persistent_launch": {
                "what": "VH_FLAG_BATCH_FUSED: the step's allocation, resolve and integration of "
                        "every scene in one persistent launch (after a one-CTA begin kernel)",
                "frames_per_s": total / t_fused, "speedup_vs_per_scene_graphs": t_seq / t_fused,
                "vs_staged_batch": t_batch / t_fused,
                "status_ok": all(x == 0 for x in fstatus),
                "counts_equal_per_scene": same_fused},
            "voxel_updates_per_s": sum(b["voxels_updated"] for b in bstats) / t_batch,
            "launches_per_step": {
                "batched": 4 * min(16, num_scenes),  # frame_begin, allocate, resolve, integrate per group
                "per_scene_graphs": sum(int(q["frame_kernels"]) for q in sstats)},
            "with_extraction": extraction}


def _batched_extraction(specs, frames, steps, local):
    """The same steps with per-frame marching cubes (meshes left on the
    device): one vh_process_frame per scene and frame against batched steps
    with the mesh flag; both through the C ABI with prepared arguments.
    Single noisy frames mesh the whole band (up to ~25 triangles per pixel
    on these scenes), so both arms get 64 triangles per pixel of room."""
    import ctypes as C
    from vhsdf import Batch, Volume
    from vhsdf import _native as N
    L = N.lib()
    n = len(specs)
    params = [dict(prm, device=local, max_triangles=64 * prm["width"] * prm["height"])
              for _, _, prm in specs]
    vols = [Volume(**prm) for prm in params]
    for v, fr in zip(vols, frames):
        v.process_frame(*fr[0], depth_format="u16")
    for v in vols:
        v.sync()
        v.reset()
    for v in vols:
        v.sync()
    rows = []
    for k in range(steps):
        row = []
        for v, fr in zip(vols, frames):
            if k < len(fr):
                pose = np.ascontiguousarray(np.asarray(fr[k][2], np.float32).reshape(16))
                row.append((v._h, fr[k][0].data_ptr(), fr[k][1].data_ptr(), pose))
        rows.append(row)
    t0 = time.perf_counter()
    for row in rows:
        for h, dptr, cptr, pose in row:
            N.check(L.vh_process_frame(h, dptr, N.VH_DEPTH_U16_MM, cptr, pose.ctypes.data,
                                       N.VH_MEM_DEVICE, None))
    for v in vols:
        v.sync()
    t_seq = time.perf_counter() - t0
    seq_tris = [int(v.stats()["triangles"]) for v in vols]
    for v in vols:
        v.close()
    batch = Batch(params)
    batch.process([fr[0] for fr in frames], with_mesh=True, depth_format="u16")
    batch.sync()
    for i in range(n):
        batch.scene(i).reset()
    batch.sync()
    prepared = []
    for k in range(steps):
        dp, cp = (C.c_void_p * n)(), (C.c_void_p * n)()
        poses = np.zeros((n, 16), np.float32)
        for i, fr in enumerate(frames):
            if k < len(fr):
                dp[i], cp[i] = fr[k][0].data_ptr(), fr[k][1].data_ptr()
                poses[i] = np.asarray(fr[k][2], np.float32).reshape(16)
        prepared.append((dp, cp, poses))
    t0 = time.perf_counter()
    for dp, cp, poses in prepared:
        N.check(L.vh_batch_process(batch._b, dp, N.VH_DEPTH_U16_MM, cp, poses.ctypes.data,
                                   N.VH_MEM_DEVICE, 1))
    status, bstats = batch.sync()
    t_batch = time.perf_counter() - t0
    batch.close()
    t_fused, fstatus, fstats = _timed_batch(
        [dict(prm, flags=N.VH_FLAG_BATCH_FUSED) for prm in params], frames, prepared, True)
    total = sum(len(fr) for fr in frames)
    return {"what": "allocate -> integrate -> per-frame marching cubes per frame, meshes left "
                    "on the device",
            "batched_frames_per_s": total / t_batch, "per_scene_graphs_frames_per_s": total / t_seq,
            "speedup": t_seq / t_batch, "status_ok": all(x == 0 for x in status),
            "last_mesh_triangles_equal_per_scene":
                [int(b["triangles"]) for b in bstats] == seq_tris,
            "one_persistent_launch": {
                "frames_per_s": total / t_fused, "speedup_vs_per_scene_graphs": t_seq / t_fused,
                "status_ok": all(x == 0 for x in fstatus),
                "last_mesh_triangles_equal_per_scene":
                    [int(b["triangles"]) for b in fstats] == seq_tris},
            "triangles_last_step": sum(seq_tris)}


def hbm_stress_leg(num_frames, local, keyframes=16, iterations=20):
    """HBM stress: a 20x20x4 m floor of 4x4 rooms, num_frames frames of
    1280x960 u16 depth walked through the rooms at 0.5 m/s, 30 Hz; voxel
    4 mm, truncation 16 mm, 2^24 hash slots.  Frames are rendered on a host
    thread while the GPU integrates; the fusion rate is the device time of
    allocate + integrate per frame (per-stage CUDA events).  Then one
    full-volume marching cubes, and Gauss-Newton refinement (adjoint) of
    `keyframes` keyframe poses perturbed by 0.25 deg / 5 mm (keyframe drift;
    with a 16 mm truncation band a larger error leaves the band)."""
    import queue
    import torch
    from vhsdf import Volume, synth, _native as N
    w, h = 1280, 960
    sc = synth.Scene(kind=4, seed=5, num_frames=num_frames, width=w, height=h)
    vol = Volume(width=w, height=h, fx=sc.fx, fy=sc.fy, cx=sc.cx, cy=sc.cy, min_depth=0.1,
                 max_depth=4.0, voxel_size=0.004, trunc=0.016, table_log2=24,
                 pool_blocks=8_000_000, max_frame_blocks=1_500_000, max_triangles=1 << 24,
                 flags=N.VH_FLAG_PROFILE, device=local)
    q = queue.Queue(maxsize=16)

    def producer():
        for f in range(num_frames):
            q.put(sc.render(f))

    th = threading.Thread(target=producer, daemon=True)
    t0 = time.perf_counter()
    th.start()
    dev_ms = updates = alg = 0.0
    peak_frame_blocks = 0
    for f in range(num_frames):
        d, c, p = q.get()
        vol.integrate(d, c, p)
        st = vol.stats()
        dev_ms += st["ms_allocate"] + st["ms_integrate"]
        updates += st["voxels_updated"]
        alg += 12 * 512 * st["frame_blocks"] + 12 * st["voxels_updated"] + 8 * w * h
        peak_frame_blocks = max(peak_frame_blocks, st["frame_blocks"])
    wall = time.perf_counter() - t0
    th.join()
    st = vol.stats()
    torch.cuda.synchronize(local)
    t1 = time.perf_counter()
    _, ntri = vol.extract("all")
    t_mc = time.perf_counter() - t1
    t1 = time.perf_counter()  # again, the triangle buffer already grown
    vol.extract("all")
    torch.cuda.synchronize(local)
    t_mc2 = time.perf_counter() - t1
    picks = np.linspace(0, num_frames - 1, keyframes).astype(int)
    kf = [sc.render(int(f)) for f in picks]
    depths = [d for d, _, _ in kf]
    gts = [gt for _, _, gt in kf]
    inits = [perturb_pose(gt, 0.25, 0.005, np.random.default_rng(2000 + int(f)))
             for gt, f in zip(gts, picks)]
    # batched: every keyframe in one launch per Gauss-Newton step
    vol.pose_refine_batch(depths, inits, iterations=iterations, stride=1)  # warm-up
    res_b, st_b = vol.pose_refine_batch(depths, inits, iterations=iterations, stride=1)
    ms_batch = st_b[0]["ms_steps"]
    # the cost's own minimum: refinement started at the ground truth
    res0_b, _ = vol.pose_refine_batch(depths, gts, iterations=iterations, stride=1)
    errs = [pose_error(r, gt) for r, gt in zip(res_b, gts)]
    floor = [pose_error(r, gt) for r, gt in zip(res0_b, gts)]
    gap = [pose_error(r, r0) for r, r0 in zip(res_b, res0_b)]
    # one keyframe at a time, for comparison
    ms_steps = 0.0
    for d, init in zip(depths, inits):
        _, rs = vol.pose_refine(d, init, iterations=iterations, stride=1, method="adjoint")
        ms_steps += rs["ms_steps"]
    peak, _ = peak_hbm()
    e_mm = np.array([1000 * e[0] for e in errs])
    e_deg = np.array([e[1] for e in errs])
    out = {"workload": f"20x20x4 m floor of 4x4 rooms (seed 5), {num_frames} frames 1280x960 u16 "
                       "depth at 0.5 m/s, 30 Hz; voxel 4 mm, truncation 16 mm, 2^24 hash slots",
           "frames": num_frames,
           "fusion_frames_per_s_device": num_frames / (dev_ms / 1000.0),
           "voxel_updates_per_s": updates / (dev_ms / 1000.0),
           "fusion_hbm_frac": alg / (dev_ms / 1000.0) / 1e9 / peak,
           "wall_s_incl_host_render": wall,
           "blocks_allocated": st["blocks_allocated"],
           "block_pool_gb": st["blocks_allocated"] * 6144 / 1e9,
           "table_load": st["blocks_allocated"] / float(1 << 24),
           "peak_frame_blocks": peak_frame_blocks,
           "full_volume_mc": {"triangles": int(ntri), "s": t_mc,
                              "triangles_per_s": ntri / t_mc,
                              "s_second_extraction": t_mc2,
                              "blocks_per_s_second_extraction": st["blocks_allocated"] / t_mc2},
           "keyframe_refinement": {"keyframes": int(keyframes), "iterations": iterations,
                                   "batched": "vh_pose_refine_batch: all keyframes in one "
                                              "launch per Gauss-Newton step",
                                   "pose_steps_per_s": keyframes * iterations / (ms_batch / 1000.0),
                                   "pose_steps_per_s_one_at_a_time":
                                       keyframes * iterations / (ms_steps / 1000.0),
                                   "err_mm_median": float(np.median(e_mm)),
                                   "err_deg_median": float(np.median(e_deg)),
                                   "perturbation": "0.25 deg about the camera centre + 5 mm",
                                   "floor_mm_median": float(np.median([1000 * e[0] for e in floor])),
                                   "floor_deg_median": float(np.median([e[1] for e in floor])),
                                   "gap_to_floor_mm_median": float(np.median([1000 * e[0] for e in gap])),
                                   "gap_to_floor_deg_median": float(np.median([e[1] for e in gap])),
                                   "within_1mm_0.05deg": int(((e_mm <= 1) & (e_deg <= 0.05)).sum()),
                                   "within_2mm_0.1deg": int(((e_mm <= 2) & (e_deg <= 0.1)).sum())}}
    vol.close()
    return out


def eviction_leg(params, tuning, stream, num=80, every=20):
    """Out-of-core streaming beside the frames: every `every`-th frame of the
    walk through the 20x20 m floor of 4x4 rooms (640x480; the camera covers
    ~27 m), device-resident, back to back - plainly, with vh_evict_async
    after every frame (blocks farther than the frame's reach from the camera
    leave HBM for the host store while the next frames run), and with the
    synchronous vh_stream_out at the same radius.  Volume parameters as the
    long stream's (5 mm, 20 mm, 2^22 slots).  Wall clock from the first
    submission to vh_sync (which waits for the last eviction's copy)."""
    import torch
    from vhsdf import Volume, synth
    sc = synth.Scene(kind=4, seed=5, num_frames=num * every, width=params["width"],
                     height=params["height"])
    params = dict(params, fx=sc.fx, fy=sc.fy, cx=sc.cx, cy=sc.cy,
                  pool_blocks=ENGINE_PARAMS["pool_blocks"])  # the walk needs ~300k blocks
    dev = []
    for f in range(0, num * every, every):
        d, c, p = sc.render(f)
        dev.append((torch.from_numpy(d.astype(np.int16)).cuda(), torch.from_numpy(c).cuda(), p))
    # every block a frame touches lies within (max depth + T) x the longest
    # pixel ray (1.25 at these intrinsics), plus a block diagonal for the halo
    radius = 1.3 * (params["max_depth"] + params["trunc"]) + 2 * 3 ** 0.5 * 8 * params["voxel_size"]
    out = {}
    for mode in ("off", "async", "sync"):
        vol = Volume(**params)
        vol.set_tuning(**tuning)
        vol.set_stream(stream.cuda_stream)
        with torch.cuda.stream(stream):
            vol.process_frame(*dev[0], depth_format="u16")  # graph capture
            if mode == "async":
                vol.evict_async(dev[0][2][:3, 3], 1e6)  # first call allocates its buffers
            vol.sync()
            vol.reset()
            t0 = time.perf_counter()
            for d, c, p in dev:
                vol.process_frame(d, c, p, depth_format="u16")
                if mode == "async":
                    vol.evict_async(p[:3, 3], radius)
                elif mode == "sync":
                    vol.stream_out(p[:3, 3], radius)
            vol.sync()
            dt = time.perf_counter() - t0
        st = vol.stats()
        out[mode] = {"frames_per_s": len(dev) / dt, "resident_blocks": st["blocks_allocated"],
                     "host_blocks": vol.host_blocks()}
        vol.close()
    out["radius_m"] = radius
    out["frames"] = f"{len(dev)} (every {every}th of a {num * every}-frame walk through the rooms)"
    out["evicted_blocks_per_frame"] = out["async"]["host_blocks"] / len(dev)
    out["async_vs_off"] = out["async"]["frames_per_s"] / out["off"]["frames_per_s"]
    out["async_vs_sync"] = out["async"]["frames_per_s"] / out["sync"]["frames_per_s"]
    return out


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    scene, frames = make_frames(args.warmup + args.steps, WORKLOAD["scene_seed"])
    from oracle.oracle import Oracle
    cores = Oracle.max_threads()
    o = Oracle(640, 480, scene.fx, scene.fy, scene.cx, scene.cy, min_depth=0.1, max_depth=4.0,
               voxel_size=0.005, trunc=0.02, mc_min_weight=1.0, precision=64)
    for d, c, p in frames[:args.warmup]:
        o.integrate(d, c, p)
        o.marching_cubes("frame")
    t0 = time.perf_counter()
    for d, c, p in frames[args.warmup:]:
        o.integrate(d, c, p)
        o.marching_cubes("frame")
    dt = time.perf_counter() - t0
    v = args.steps / dt
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": WORKLOAD,
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{args.steps} timed frames after {args.warmup} warm-up "
                                   f"frames: allocate + integrate + per-frame marching cubes "
                                   f"of the FP64 CPU port in oracle/, canonical band rule"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "reference_class": "cpu_port_of_reference_algorithm",
        "comparable_to_reference_cuda_build": False,
        "note": "CPU port (oracle/vh_oracle.cpp, FP64) of the engine's rule, which is the "
                "reference's camera math, integration update and marching cubes with the "
                "benchmark's canonical band allocation and old-weight sdf average (not the "
                "reference's DDA allocation or its w_new update).  The reference's CUDA build "
                "is not run: it cannot hold this workload (400k-block per-frame tables, "
                "1e6-block staging buffer), and on a shared GPU its table insert spins without "
                "bound and its allocator traps when full; the comparison with it is "
                "unmeasured",
    }), flush=True)


def run_engine(args):
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    from vhsdf import Volume, _native as N

    from vhsdf import replicas
    seed = replicas.stream_seed(WORKLOAD["scene_seed"], rank)  # independent stream per replica
    nframes = args.warmup + args.steps
    scene, frames = make_frames(nframes, seed)
    params = dict(ENGINE_PARAMS, fx=scene.fx, fy=scene.fy, cx=scene.cx, cy=scene.cy,
                  flags=N.VH_FLAG_PROFILE, device=local)
    if args.pool_blocks:
        params["pool_blocks"] = args.pool_blocks

    stream = torch.cuda.Stream()
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.int32, device="cuda")
    dev = [(torch.from_numpy(d.astype(np.int16)).cuda(), torch.from_numpy(c).cuda(), p)
           for d, c, p in frames]
    # uint16 depth lives in an int16 tensor: same bytes, passed as uint16
    torch.cuda.synchronize()

    def timed_pass(vol, host):
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        stage = []
        wall = []
        with torch.cuda.stream(stream):
            for i in range(nframes):
                timed = i >= args.warmup
                j = i - args.warmup
                if host:
                    d, c, p = pinned[i]
                else:
                    d, c, p = dev[i]
                if timed:
                    stream.synchronize()
                # L2 flush, outside the events.  In the device pass the GPU
                # runs it while the host submits the frame, so the frame's
                # interval holds no wait for the host; the host pass times
                # one frame at a time from an idle stream.
                flush.zero_()
                if timed:
                    if host:
                        stream.synchronize()
                    t0 = time.perf_counter()
                    starts[j].record(stream)
                if host:  # the frame's mesh comes back to pinned host memory
                    vol.process_frame_mesh(d, c, p, mesh_bufs[0], one_count, depth_format="u16")
                else:
                    vol.process_frame(d, c, p, depth_format="u16")
                if timed:
                    ends[j].record(stream)
                    if host:
                        vol.sync()  # the mesh copy-out is complete
                    st = vol.stats()  # synchronises; D2H of the frame's counters
                    wall.append(time.perf_counter() - t0)
                    stage.append(st)
                else:
                    vol.sync()
        stream.synchronize()
        ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
        return ms, stage, wall

    # ---- launch tuning (scratch volume, outside any timed region) ----
    tuner = Volume(**params)
    if args.tuning:
        iv, ic, mcs, mv = (int(x) for x in args.tuning.split(","))
        tuner.set_tuning(iv, ic, mcs, mv)
        tuning = tuner.tuning()
    else:
        tuning = tuner.tuning() if args.no_autotune else tuner.autotune(*frames[0])
    tuner.close()

    # ---- device-resident pass (value + roofline) ----
    vol = Volume(**params)
    vol.set_tuning(**tuning)
    vol.set_stream(stream.cuda_stream)
    pinned = None
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t_wall = time.perf_counter()
        ms, stage, _ = timed_pass(vol, host=False)
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall
    if world > 1:
        torch.distributed.barrier()
    dev_ms = sum(ms)
    vol.close()

    # ---- end-to-end pass through the C ABI with pinned host buffers ----
    pinned = []
    for d, c, p in frames:
        dp = torch.empty(d.shape, dtype=torch.int16, pin_memory=True).numpy().view(np.uint16)
        dp[...] = d
        cp = torch.empty(c.shape, dtype=torch.uint8, pin_memory=True).numpy()
        cp[...] = c
        pinned.append((dp, cp, p))
    cap = int(max(s["triangles"] for s in stage) * 1.25) + 4096
    mesh_bufs = [torch.empty((cap, 12), dtype=torch.float32, pin_memory=True).numpy()
                 for _ in range(3)]
    one_count = np.zeros(1, np.int64)
    vol = Volume(**dict(params, max_triangles=cap))
    vol.set_tuning(**tuning)
    vol.set_stream(stream.cuda_stream)
    _, _, wall = timed_pass(vol, host=True)  # one frame at a time: latency
    vol.close()
    e2e_sync_s = sum(wall)
    # Throughput with the product result on the host: frames submitted back
    # to back (the engine's asynchronous mode) through vh_process_frame_mesh,
    # each with its host->device upload (overlapping the previous frame's
    # kernels) and the device->host copy of its whole triangle mesh into
    # pinned host memory (overlapping the next frame's kernels), as the
    # reference's processFrame copies its triangles back every frame.
    mesh_counts = [np.zeros(1, np.int64) for _ in range(nframes)]
    vol = Volume(**dict(params, max_triangles=cap))
    vol.set_tuning(**tuning)
    vol.set_stream(stream.cuda_stream)
    with torch.cuda.stream(stream):
        for i in range(args.warmup):
            vol.process_frame_mesh(*pinned[i], mesh_bufs[i % 3], mesh_counts[i],
                                   depth_format="u16")
        vol.sync()
        t0 = time.perf_counter()
        for i in range(args.warmup, nframes):
            vol.process_frame_mesh(*pinned[i], mesh_bufs[i % 3], mesh_counts[i],
                                   depth_format="u16")
        vol.sync()
        e2e_s = time.perf_counter() - t0
    vol.close()
    e2e_soup_s = e2e_s
    e2e_tris = [int(c[0]) for c in mesh_counts[args.warmup:]]
    # the delivered counts are the device pass's, frame for frame
    mesh_counts_match = e2e_tris == [int(s["triangles"]) for s in stage]
    del mesh_bufs
    # The same frames with each frame's mesh delivered indexed
    # (vh_process_frame_indexed: vertices shared within a block, faces as
    # vertex numbers; the same triangles in about half the bytes).
    idx_bufs = [(torch.empty((cap, 4), dtype=torch.float32, pin_memory=True).numpy(),
                 torch.empty((cap, 3), dtype=torch.int32, pin_memory=True).numpy())
                for _ in range(3)]
    idx_counts = [np.zeros(2, np.int64) for _ in range(nframes)]
    vol = Volume(**dict(params, max_triangles=cap))
    vol.set_tuning(**tuning)
    vol.set_stream(stream.cuda_stream)
    with torch.cuda.stream(stream):
        for i in range(args.warmup):
            vol.process_frame_indexed(*pinned[i], *idx_bufs[i % 3], idx_counts[i],
                                      depth_format="u16")
        vol.sync()
        t0 = time.perf_counter()
        for i in range(args.warmup, nframes):
            vol.process_frame_indexed(*pinned[i], *idx_bufs[i % 3], idx_counts[i],
                                      depth_format="u16")
        vol.sync()
        e2e_idx_s = time.perf_counter() - t0
    idx_last = vol.stats()  # per-stage events of the last frame (k_mc_indexed)
    vol.close()
    del idx_bufs
    idx_verts = [int(c[0]) for c in idx_counts[args.warmup:]]
    idx_faces = [int(c[1]) for c in idx_counts[args.warmup:]]
    idx_counts_match = idx_faces == [int(s["triangles"]) for s in stage]
    # The same with the mesh left on the device (vh_process_frame; only the
    # 64-byte counters reach the host): what the copies cost.
    vol = Volume(**params)
    vol.set_tuning(**tuning)
    vol.set_stream(stream.cuda_stream)
    with torch.cuda.stream(stream):
        for i in range(args.warmup):
            vol.process_frame(*pinned[i], depth_format="u16")
        vol.sync()
        t0 = time.perf_counter()
        for i in range(args.warmup, nframes):
            vol.process_frame(*pinned[i], depth_format="u16")
        vol.sync()
        e2e_dev_s = time.perf_counter() - t0
    vol.close()

    eviction = (eviction_leg(params, tuning, stream, num=args.eviction_frames)
                if rank == 0 and args.eviction_frames > 0 else None)
    dev_ms, e2e_idx_s, e2e_soup_s, e2e_sync_s, e2e_dev_s = replicas.reduce_max(
        [dev_ms, e2e_idx_s, e2e_soup_s, e2e_sync_s, e2e_dev_s], device="cuda")
    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return

    frames_total = args.steps * world
    value = frames_total / (dev_ms / 1000.0)
    e2e = frames_total / e2e_idx_s
    e2e_soup = frames_total / e2e_soup_s
    e2e_sync = frames_total / e2e_sync_s
    e2e_dev = frames_total / e2e_dev_s
    # Rooflines.  Algorithmic bytes per launch:
    #   k_mc        12 B per voxel of every listed block (sdf, weight, rgb read
    #               once) + 45 B per output triangle (3 vertices of xyz f32
    #               and rgb u8; the kernel writes them as 3 x float4, 48 B,
    #               the colour packed in the fourth word)
    #   k_integrate 12 B per voxel of every listed block read + 12 B per
    #               updated voxel written + 8 B per pixel record
    # DRAM traffic per launch: the traffic / algorithmic ratio that the
    # committed warm-cache ncu capture of this stream measured per kernel
    # (frames 3-4, one kernel per capture), scaled to this run's launches.
    npx = 640 * 480
    blocks = [s["frame_blocks"] for s in stage]
    updated = [s["voxels_updated"] for s in stage]
    tris = [s["triangles"] for s in stage]
    mc_alg = [12 * 512 * b + 45 * t for b, t in zip(blocks, tris)]
    mc_stored = [12 * 512 * b + 48 * t for b, t in zip(blocks, tris)]  # the ratio's base
    in_alg = [12 * 512 * b + 12 * u + 8 * npx for b, u in zip(blocks, updated)]
    mc_ms = [s["ms_extract"] for s in stage]
    in_ms = [s["ms_integrate"] for s in stage]
    mc_ach = sum(mc_alg) / (sum(mc_ms) / 1000.0) / 1e9
    in_ach = sum(in_alg) / (sum(in_ms) / 1000.0) / 1e9
    peak, peak_src = peak_hbm()
    ratios = traffic_ratios()
    cpu = None
    if world == 1:  # the CPU baseline is rank 0's at N=1 only
        cpu = cpu_leg(frames, scene, seconds=args.cpu_seconds)
        one = cpu_leg(frames, scene, seconds=min(args.cpu_seconds, 5.0), threads=1)
        cpu["single_thread"] = {"value": one["value"], "cores": 1, "sample": one["sample"]}
    adjoint = (adjoint_leg(args.adjoint_frames, local, args.adjoint_iterations)
               if args.adjoint_frames > 0 and rank == 0 else None)
    batched = (batched_leg(args.batch_scenes, args.batch_steps, local)
               if args.batch_scenes > 0 and rank == 0 else None)
    batched_small = (batched_leg(4 * args.batch_scenes, args.batch_steps, local, small=True)
                     if args.batch_scenes > 0 and rank == 0 else None)
    # the HBM-stress configuration's first frames (its full 2000-frame run,
    # `--hbm-stress 2000`, renders minutes of 1280x960 frames on the host)
    hbm = (hbm_stress_leg(args.hbm_stress_frames, local)
           if args.hbm_stress_frames > 0 and rank == 0 else None)
    res = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": WORKLOAD,
        "l2": "flushed between steps (256 MiB memset), outside timing",
        "parallelism": "replicas" if world > 1 else "single",
        "voxel_updates_per_s": sum(updated) * world / (dev_ms / 1000.0),
        "e2e": {"value": e2e, "unit": UNIT,
                "h2d_bytes_per_step": 2 * npx + 3 * npx + 80,
                "d2h_bytes_per_step": (16 * statistics.mean(idx_verts)
                                       + 12 * statistics.mean(idx_faces) + 64),
                "mode": "vh_process_frame_indexed on pinned host frames submitted back to back "
                        "(asynchronous mode, one sync at the end): per frame the depth + RGB "
                        "upload and the copy of the frame's whole mesh into pinned host "
                        "memory as vertices (16 B: xyz f32 + rgb) and faces (3 int32 vertex "
                        "numbers), the same triangles as the soup below, plus the 64-byte "
                        "counters; no L2 flush, the per-frame working set (listed blocks "
                        "read, mesh written) exceeds L2",
                "vertices_per_step": statistics.mean(idx_verts),
                "faces_per_step": statistics.mean(idx_faces),
                "last_frame_stages_ms": {k: idx_last[k] for k in
                                         ("ms_allocate", "ms_integrate", "ms_extract",
                                          "ms_frame")},
                "mesh_counts_match_device_pass": idx_counts_match,
                "triangle_soup": {
                    "value": e2e_soup,
                    "mode": "vh_process_frame_mesh: the same frames with each frame's mesh "
                            "copied as a triangle soup (48 B per triangle), the layout of the "
                            "reference's per-frame triangle copy",
                    "d2h_bytes_per_step": 48 * statistics.mean(e2e_tris) + 64,
                    "triangles_per_step": statistics.mean(e2e_tris),
                    "mesh_counts_match_device_pass": mesh_counts_match},
                "sync_per_frame": e2e_sync,
                "mesh_left_on_device": e2e_dev},
        "roofline": {"bound": "hbm", "achieved": mc_ach, "peak": peak, "unit": "GB/s",
                     "frac": mc_ach / peak,
                     "traffic": (ratios["k_mc"] * statistics.mean(mc_stored)
                                 if "k_mc" in ratios else None),
                     "kernel": "k_mc", "peak_source": peak_src,
                     "algorithmic_bytes": statistics.mean(mc_alg)},
        "roofline_integrate": {"bound": "hbm", "achieved": in_ach, "peak": peak, "unit": "GB/s",
                               "frac": in_ach / peak,
                               "traffic": (ratios["k_integrate"] * statistics.mean(in_alg)
                                           if "k_integrate" in ratios else None),
                               "kernel": "k_integrate", "peak_source": peak_src,
                               "algorithmic_bytes": statistics.mean(in_alg)},
        "stages_ms": {k: statistics.mean(s[k] for s in stage)
                      for k in ("ms_allocate", "ms_integrate", "ms_extract", "ms_frame")},
        "per_frame": {"blocks": statistics.mean(blocks), "voxels_updated": statistics.mean(updated),
                      "triangles": statistics.mean(tris)},
        # kernels of the timed frames as the engine counted them when it
        # enqueued each frame (frame_begin, allocate, resolve, integrate, mc)
        "gpu_launches": sum(s["frame_kernels"] for s in stage),
        "tuning": tuning,
        "wall_s": t_wall,
        "clocks": clk.summary(),
        "cpu_baseline": cpu,
        "out_of_core": eviction,
        "pose_refinement": adjoint,
        "batched_scenes": batched,
        "batched_small_scenes": batched_small,
        "hbm_stress": hbm,
    }
    print(json.dumps(res), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--adjoint-frames", type=int, default=100,
                    help="poses refined in the pose-refinement leg (0 = skip)")
    ap.add_argument("--adjoint-iterations", type=int, default=20,
                    help="Gauss-Newton steps per pose in the pose-refinement leg")
    ap.add_argument("--batch-scenes", type=int, default=64,
                    help="scenes in the batched-scenes leg (0 = skip)")
    ap.add_argument("--eviction-frames", type=int, default=80,
                    help="frames of the out-of-core leg (0 = skip)")
    ap.add_argument("--batch-steps", type=int, default=12,
                    help="frames per scene in the batched-scenes leg")
    ap.add_argument("--only-batched", action="store_true",
                    help="run only the batched-scenes leg and print its JSON (profiling)")
    ap.add_argument("--hbm-stress", type=int, default=0,
                    help="run only the HBM-stress leg with this many frames (e.g. 2000)")
    ap.add_argument("--hbm-stress-frames", type=int, default=150,
                    help="frames of the HBM-stress leg in the default run (0 skips it)")
    ap.add_argument("--only-pose-refinement", action="store_true",
                    help="run only the pose-refinement leg and print its JSON (profiling)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="use the default launch configuration (for profiling runs)")
    ap.add_argument("--tuning", default="",
                    help="explicit launch configuration integrate_variant,integrate_ctas_per_sm,"
                         "mc_ctas_per_sm,mc_variant (0 = occupancy maximum; no autotuning)")
    ap.add_argument("--pool-blocks", type=int, default=0,
                    help="smaller block pool (for short profiling runs)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 0)
    if args.impl == "reference":
        run_reference(args)
    elif args.hbm_stress > 0:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps({"hbm_stress": hbm_stress_leg(args.hbm_stress, 0)}), flush=True)
    elif args.only_batched:
        import torch
        torch.cuda.set_device(0)
        n = max(args.batch_scenes, 1)
        print(json.dumps({"batched_scenes": batched_leg(n, args.batch_steps, 0),
                          "batched_small_scenes": batched_leg(4 * n, args.batch_steps, 0,
                                                              small=True)}), flush=True)
    elif args.only_pose_refinement:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps({"pose_refinement": adjoint_leg(max(args.adjoint_frames, 1), 0,
                                                         args.adjoint_iterations)}), flush=True)
    else:
        run_engine(args)


if __name__ == "__main__":
    main()
