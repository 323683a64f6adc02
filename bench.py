"""Benchmark of the registration cost path on the batched PSO workload.

Workload (one "step" = one frame registered): 3 bones (uint16 phantoms
160x96x96, 256x128x128, 200x200x120 at 0.4 mm), 2 views with 1024x1024 uint16
radiographs, the filter chain Contrast(2.5, 0.9) -> Sharpen(1) -> Gaussian(1.5)
-> Sobel on both the DRR and the radiograph lists, masked NCC, and a
synchronous PSO of 100 particles x 50 iterations per bone (w 0.7298,
c1 = c2 = 1.4962), every iteration scoring all 300 particles of the three
swarms in one graph-captured launch sequence.  Data are seeded synthetic
phantoms and radiographs rendered at a seeded ground truth.

Prints one JSON line (see the keys below).  `--impl reference` times the
CPU restatement of the path (the oracle) on the host cores instead.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "pose evals/s (DRR+filter+NCC, 2 views)"
CONFIG = {"workload": "batched PSO, 3 bones (160x96x96, 256x128x128, 200x200x120 u16 @0.4mm), 2 views, "
                      "1024x1024 u16 radiographs, Contrast->Sharpen->Gaussian(1.5)->Sobel, masked NCC, "
                      "100 particles x 50 iterations per bone",
          "bones": 3, "views": 2, "render": [1024, 1024], "particles": 100, "iterations": 50}
SHAPES = [(96, 96, 160), (128, 128, 256), (120, 200, 200)]  # (depth, height, width)


def make_scene(seed=0, landmark=False):
    from autoscoper_gb300 import scene as S
    return S.make_scene(SHAPES, 0.4, (1024, 1024), 0.3, filters="chain", seed=seed,
                        bone_offsets=[(0.0, 0.0, -45.0), (0.0, 0.0, 0.0), (0.0, 0.0, 45.0)], rot_range=10.0,
                        landmark=landmark)


def render_targets(sc):
    """Radiographs = 1 - sum of the bones' DRRs at the ground truth (GPU)."""
    from autoscoper_gb300 import api, scene as S
    vols = api.render_targets(sc)
    rng = np.random.Generator(np.random.PCG64(99))
    sc.poses = [S.perturb(t, rng, 5.0, 5.0) for t in sc.truth]
    return vols


class Clocks:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 3 + i and r[3 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_counts(kernel):
    """Per-launch counters of `kernel` from the committed ncu summary of the
    bench's roofline batch (profiles/<kernel>_counters_batch_300.json), or None."""
    p = os.path.join(ROOT, "profiles", f"{kernel}_counters_batch_300.json")
    return json.load(open(p)) if os.path.exists(p) else None


def launch_report(eng, reps=5):
    """The engine's launch shapes (the autotuner's table entry for its
    workload class, or the defaults) and the roofline batch's time with them
    and with the defaults (ms per evaluation, median of `reps`)."""
    import ctypes as C
    from autoscoper_gb300 import _lib as L, tune
    cls = (C.c_int * 3)()
    L.call("asc_engine_workload_class", eng.handle, cls)
    cur = L.LaunchConfig()
    L.call("asc_engine_get_launch", eng.handle, C.byref(cur), None)
    mine = (cur.ray_blocks_per_sm, cur.view_blocks_per_sm, cur.ray_shape)
    rng = np.random.default_rng(3)
    bones = np.repeat(np.arange(3), 100).astype(np.int32)
    man = np.concatenate([rng.uniform(-5, 5, (300, 3)), rng.uniform(-5, 5, (300, 3))], 1)
    t_default = tune.time_config(eng, bones, man, tune.DEFAULT, reps)
    t_tuned = tune.time_config(eng, bones, man, mine, reps)
    return {"class": list(cls), "tuned": list(mine), "default": list(tune.DEFAULT),
            "batch_ms_tuned": t_tuned["total"], "batch_ms_default": t_default["total"],
            "table": "autoscoper_gb300/tuning.txt" if os.path.exists(L.TUNING) else None}


def device_sms():
    import torch
    return torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count


def roofline(phase, samples, pixels, marched, slots, sm_mhz, nexact=0):
    """The dominant kernel (k_ray) against the limit it is bound by.

    k_ray marches FP32 samples whose taps come from L1/L2 (every volume is
    far below the 129 MB L2); ncu shows it bound by instruction issue.  So
    `frac` is the issue fraction: warp instructions per launch (ncu,
    profiles/k_ray_counters_batch_300.json, scaled to this launch by marched
    samples) over SMs x 4 schedulers x the sampled SM clock x the launch's
    CUDA-event time (the ray phase holds k_ray_fix too, whose instructions,
    scaled by the rays it marches, are added).  Beside it: the marched gather bytes (16 B per marched
    sample + 4 B per DRR pixel) against the L2 read bandwidth measured here
    (frac_l2), the DRAM traffic against the HBM copy peak (frac_hbm), and the
    algorithmic bytes of the reference's march (16 B per sample of the whole
    box + 4 B per pixel) under alg_* (above the L2 peak: empty-space skipping
    proves most of those samples add 0 and never loads them).  k_view's issue
    and DRAM fractions ride along."""
    from autoscoper_gb300 import _lib as L
    import ctypes as C
    hbm, peak_kind = peaks()
    g = C.c_double()
    L.call("asc_probe_read_bandwidth", 32 << 20, 400, C.byref(g), None)
    l2 = g.value
    sms = device_sms()
    clk = (sm_mhz or 2070.0) * 1e6
    out = {"bound": "issue", "kernel": "k_ray", "unit": "G warp-inst/s"}
    ray_s, view_s = phase[1] / 1e3, phase[2] / 1e3
    issue_peak = sms * 4 * clk
    kr = profile_counts("k_ray")
    if kr and kr.get("marched_per_launch"):
        inst = kr["inst_per_launch"] * marched / kr["marched_per_launch"]
        kf = profile_counts("k_ray_fix")
        if kf and kf.get("exact_cutoff_rays_per_launch"):
            inst += kf["inst_per_launch"] * nexact / kf["exact_cutoff_rays_per_launch"]
        out.update(achieved=inst / ray_s / 1e9, peak=issue_peak / 1e9, frac=inst / ray_s / issue_peak,
                   inst_per_launch=inst)
        traffic = kr["dram_bytes_per_launch"] * marched / kr["marched_per_launch"]
    else:
        out.update(achieved=None, peak=issue_peak / 1e9, frac=None)
        traffic = None
    out["frac_issue"] = out["frac"]
    marched_bytes = 16.0 * marched + 4.0 * pixels
    out.update(l2_peak_gbs=l2, achieved_marched_gbs=marched_bytes / ray_s / 1e9,
               frac_l2=marched_bytes / ray_s / 1e9 / l2, traffic=traffic, hbm_peak_gbs=hbm, peak_kind=peak_kind,
               frac_hbm=traffic / ray_s / 1e9 / hbm if traffic else None)
    alg = 16.0 * samples + 4.0 * pixels
    out.update(alg_bytes_per_launch=alg, alg_gbs=alg / ray_s / 1e9, alg_over_l2_peak=alg / ray_s / 1e9 / l2,
               marched_fraction=marched / max(samples, 1), simt_efficiency=marched / max(slots, 1),
               sm_mhz=clk / 1e6, sms=sms)
    kv = profile_counts("k_view")
    if kv and kv.get("pixels_per_launch"):
        vi = kv["inst_per_launch"] * pixels / kv["pixels_per_launch"]
        vt = kv["dram_bytes_per_launch"] * pixels / kv["pixels_per_launch"]
        out["k_view"] = {"ms": phase[2], "frac_issue": vi / view_s / issue_peak, "traffic": vt,
                         "frac_hbm": vt / view_s / 1e9 / hbm}
    out["note"] = ("frac = k_ray's issued warp instructions / (SMs x 4 x SM clock x time); the taps come from "
                   "L1/L2, so frac_l2 (marched gather bytes / measured L2 read bandwidth) and frac_hbm (DRAM traffic "
                   "/ HBM copy peak) show the memory side; alg_* is the reference march's algorithmic bytes")
    return out


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    return ws, rank, local, pg


def barrier(pg):
    if pg:
        pg.barrier()


def allmax(pg, x):
    if not pg:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def cpu_sample(sc, n_evals, seed=5):
    """Times the FP64 oracle's minimizationFunc on `n_evals` candidates."""
    from oracle import oracle as O
    tr = O.Tracker(sc)
    rng = np.random.default_rng(seed)
    t0 = time.perf_counter()
    for k in range(n_evals):
        b = k % len(sc.volumes)
        tr.minimization_func(b, rng.uniform(-2, 2, 6))
    dt = time.perf_counter() - t0
    return n_evals / dt, dt


def run_reference(args, ws, rank, pg):
    if rank != 0:
        return
    sc = make_scene()
    from autoscoper_gb300 import scene as S
    # radiographs from the oracle itself (no GPU on this arm)
    from oracle import oracle as O
    tr = O.Tracker(sc)
    for vi, v in enumerate(sc.views):
        cam = v.camera
        acc = np.zeros((cam.height, cam.width))
        for b in range(len(sc.volumes)):
            ok, m, _, _, _ = tr.view_setup(b, vi, sc.truth[b])
            rp = sc.ray[vi][b]
            acc += O.raycast(tr.vd[b], m, S.target_viewport(cam), rp.step, rp.intensity, rp.cutoff, cam.width,
                             cam.height)
        v.radiograph = S.radiograph_from_drr(acc, seed=vi)
    per_step = 3
    for _ in range(args.warmup):
        cpu_sample(sc, 1)
    times = []
    for _ in range(args.steps):
        _, dt = cpu_sample(sc, per_step)
        times.append(dt)
    v = per_step * args.steps / sum(times)
    cores = os.cpu_count()
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "pose-evals/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * sum(times) / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": CONFIG,
            "cpu_baseline": {"value": v, "unit": "pose-evals/s", "cores": cores, "kind": "port",
                             "sample": f"{per_step} minimizationFunc evaluations per step on the full workload "
                                       f"(FP64 oracle, OpenMP ray cast over {cores} threads)"},
            "e2e": {"value": v, "unit": "pose-evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline sample")
    ap.add_argument("--iters", type=int, default=50, help="PSO iterations per step")
    ap.add_argument("--particles", type=int, default=100, help="PSO particles per bone")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain per-pose sample")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end pass")
    args = ap.parse_args()
    ws, rank, local, pg = dist_setup()
    if args.impl == "reference":
        run_reference(args, ws, rank, pg)
        return
    import ctypes as C
    from autoscoper_gb300 import _lib as L
    from autoscoper_gb300 import api
    L.load()
    L.call("asc_set_device", local)
    sc = make_scene(seed=rank)
    vols = render_targets(sc)
    eng = api.Engine(sc, max_items=3 * args.particles, volumes=vols)
    lib = L.load()
    stream = C.c_void_p()
    L.call("asc_stream_create", C.byref(stream))
    ev0, ev1 = C.c_void_p(), C.c_void_p()
    L.call("asc_event_create", C.byref(ev0))
    L.call("asc_event_create", C.byref(ev1))
    flush = api.DeviceArray((256 << 20,), np.uint8)  # 256 MB > 129 MB L2
    nb, npart, iters = 3, args.particles, args.iters
    best = np.zeros((nb, 6))
    bcost = np.zeros(nb)
    ev = C.c_longlong()

    def step():
        L.call("asc_engine_pso", eng.handle, npart, iters, 0.7298, 1.4962, 1.4962, -6.0, 6.0, 7,
               best.ctypes.data_as(C.POINTER(C.c_double)), bcost.ctypes.data_as(C.POINTER(C.c_double)),
               C.byref(ev), stream)

    for _ in range(args.warmup):
        step()
    L.call("asc_stream_sync", stream)
    # ---- device-resident throughput: K steps, L2 flushed between steps
    ms_total = 0.0
    with Clocks(local) as clk:
        barrier(pg)
        L.call("asc_device_sync")
        for _ in range(args.steps):
            L.call("asc_memset", flush.ptr, 1, flush.nbytes, stream)
            L.call("asc_event_record", ev0, stream)
            step()
            L.call("asc_event_record", ev1, stream)
            ms = C.c_float()
            L.call("asc_event_elapsed", ev0, ev1, C.byref(ms))
            ms_total += ms.value
        L.call("asc_device_sync")
        barrier(pg)
    ms_step = allmax(pg, ms_total / args.steps)
    evals_per_step = nb * npart * iters
    value = ws * evals_per_step / (ms_step / 1000.0)
    # ---- end to end through the public API: per step, the frame's two
    # radiographs go host->device from pinned memory, the best poses come back
    pinned = []
    for v in sc.views:
        p = C.c_void_p()
        L.call("asc_host_alloc", C.byref(p), v.radiograph.nbytes)
        C.memmove(p, v.radiograph.ctypes.data, v.radiograph.nbytes)
        pinned.append(p)
    h2d = sum(v.radiograph.nbytes for v in sc.views)
    d2h = best.nbytes + bcost.nbytes
    barrier(pg)
    L.call("asc_device_sync")
    t0 = time.perf_counter()
    for _ in range(0 if args.no_e2e else args.steps):
        for vi, p in enumerate(pinned):
            L.call("asc_image_update", eng.rads[vi].handle, p, stream)
        step()  # returns after the D2H copy of best poses and costs
    L.call("asc_device_sync")
    e2e_s = allmax(pg, (time.perf_counter() - t0) / args.steps)
    e2e = ws * evals_per_step / e2e_s if not args.no_e2e else None
    # ---- launch shapes: the tuning table's choice for this workload class
    # against the defaults, on the roofline batch
    launch = launch_report(eng)
    # ---- roofline of the dominant kernel (ray cast) on one PSO-iteration batch
    L.call("asc_engine_profile", eng.handle, 1)
    rng = np.random.default_rng(3)
    bones = np.repeat(np.arange(nb), npart).astype(np.int32)
    man = np.concatenate([rng.uniform(-5, 5, (nb * npart, 3)), rng.uniform(-5, 5, (nb * npart, 3))], 1)
    phase = np.zeros(3)
    reps = 5
    samples = C.c_ulonglong()
    pixels = C.c_ulonglong()
    for r in range(reps + 1):
        L.call("asc_memset", flush.ptr, 1, flush.nbytes, stream)
        eng.eval(bones, man)
        t3 = (C.c_float * 3)()
        L.call("asc_engine_stats", eng.handle, t3, C.byref(samples), C.byref(pixels))
        if r:
            phase += np.array(t3[:])
    phase /= reps
    L.call("asc_engine_profile", eng.handle, 0)
    cnt = (C.c_ulonglong * 4)()
    L.call("asc_engine_counters", eng.handle, cnt)
    marched, slots = cnt[2], cnt[3]
    nexact = C.c_int()
    L.call("asc_engine_exact_rays", eng.handle, C.byref(nexact))
    rl = roofline(phase, samples.value, pixels.value, marched, slots, clk.summary().get("sm_mhz"), nexact.value)
    # ---- plain per-pose drop-in form on the same GPU (sampled)
    plain_v = None
    if not args.no_plain:
        nplain = 60
        pb, pm = bones[::5][:nplain], man[::5][:nplain]
        eng.eval(pb[:2], pm[:2], plain=True)
        t0 = time.perf_counter()
        eng.eval(pb, pm, plain=True)
        plain_v = nplain / (time.perf_counter() - t0)
    # ---- CPU baseline (oracle) on a bounded sample
    cpu = None
    if rank == 0 and not args.no_cpu:
        v, dt = cpu_sample(sc, 3)
        cpu = {"value": v, "unit": "pose-evals/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"3 minimizationFunc evaluations of this workload by the FP64 oracle ({dt:.1f} s)"}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "pose-evals/s", "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32 (u16 volumes, FP64 pose/NCC combine)", "data": "synthetic",
                "config": dict(CONFIG, l2="256 MB memset between timed steps", parallelism=f"replicas x{ws}"),
                "e2e": {"value": e2e, "unit": "pose-evals/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
                # per step: k_pso_init, then per iteration one graph of eight kernels (k_pso_update,
                # k_setup_iv, k_setup, k_tile_map, k_ray, k_ray_fix, k_view, k_pso_best)
                "gpu_launches": args.steps * (1 + 8 * iters),
                "roofline": rl,
                "kernel_ms": {"setup": phase[0], "ray": phase[1], "view": phase[2]},
                "launch": launch,
                "work": {"samples_per_batch": samples.value, "marched_per_batch": marched,
                         "pixels_per_batch": pixels.value, "batch": nb * npart,
                         "exact_cutoff_rays_per_batch": nexact.value},
                "plain": {"value": plain_v, "unit": "pose-evals/s",
                          "speedup": value / plain_v if plain_v else None},
                "cpu_baseline": cpu, "clocks": clk.summary(),
                "best_cost": bcost.tolist()}
        print(json.dumps(line), flush=True)


def sinusoid_trajectory(truth0, frames, fps=250.0, seed=0, rot_amp=20.0, trans_amp=10.0):
    """Per-axis sinusoids (rotations +-rot_amp deg, translations +-trans_amp mm)
    at frequencies U(0.5, 2) Hz with random phase, sampled at fps."""
    rng = np.random.default_rng(seed)
    f = rng.uniform(0.5, 2.0, 6)
    ph = rng.uniform(0, 2 * np.pi, 6)
    amp = np.array([trans_amp] * 3 + [rot_amp] * 3)
    t = np.arange(frames)[:, None] / fps
    return np.asarray(truth0)[None, :] + amp * np.sin(2 * np.pi * f * t + ph) - amp * np.sin(ph)


def run_tracking(args):
    """Sequence tracking: 2 bones (256x128x128, 192x192x160 u16 @0.4 mm), 2 views
    of 1024^2, sinusoidal ground truth at 250 fps; every frame starts from the
    previous frame's pose, PSO (64 x 30) then Downhill Simplex.  Radiographs and
    volumes stay resident on the GPU; frames/s end to end."""
    from autoscoper_gb300 import _lib as L, api, scene as S
    L.load()
    sc = S.make_scene([(128, 128, 256), (160, 192, 192)], 0.4, (1024, 1024), 0.3, filters="sobel", seed=4,
                      bone_offsets=[(0.0, 0.0, -30.0), (0.0, 0.0, 30.0)], rot_range=10.0, landmark=True)
    nf = args.frames
    traj = [sinusoid_trajectory(t, nf, seed=11 + b) for b, t in enumerate(sc.truth)]
    vols = [api.DeviceVolume(v) for v in sc.volumes]
    images = []
    for f in range(nf):
        sc.truth = [traj[b][f] for b in range(2)]
        api.render_targets(sc, volumes=vols)
        images.append([api.DeviceImage(v.radiograph) for v in sc.views])
    rng = np.random.default_rng(5)
    sc.poses = [S.perturb(traj[b][0], rng, 1.0, 1.0) for b in range(2)]
    eng = api.Engine(sc, max_items=2 * 64, volumes=vols, images=images[0])
    start = np.zeros((nf, 2, 6))
    start[0] = [np.asarray(p, np.float64) for p in sc.poses]
    L.call("asc_device_sync")
    t0 = time.perf_counter()
    # Tracker::optimize frame after frame, each from the previous frame's pose
    poses, cost, evals = eng.track(images, start, method=0, n_particles=64, n_iter=30, lo=-3.0, hi=3.0,
                                   seed=args.seed, guess=1, repeats=1)
    dt = time.perf_counter() - t0
    e = np.abs(poses - np.stack([traj[b] for b in range(2)], 1))  # frames x bones x 6
    fm, fd = e[:, :, :3].max(axis=(1, 2)), e[:, :, 3:].max(axis=(1, 2))  # per frame, worst bone and axis
    # Where a bone is off by more than 1 mm / 1 deg: does the cost prefer the
    # tracked pose over the truth (the cost's own minimum lies elsewhere: a
    # property of the phantom and filters) or the truth (the search missed it)?
    lost = [(f, b) for f in range(nf) for b in range(2)
            if e[f, b, :3].max() > 1.0 or e[f, b, 3:].max() > 1.0]
    prefers_tracked = 0
    worst_axes = np.zeros(6)
    for f, b in lost:
        for v in range(len(sc.views)):
            eng.set_radiograph(v, images[f][v])
        eng.set_base_pose(b, poses[f, b], exact=True)
        c_tr = eng.eval(np.array([b], np.int32), np.zeros((1, 6)))[0][0]
        eng.set_base_pose(b, traj[b][f], exact=True)
        c_gt = eng.eval(np.array([b], np.int32), np.zeros((1, 6)))[0][0]
        prefers_tracked += int(c_tr <= c_gt)
        worst_axes[int(np.argmax(e[f, b] / np.array([1, 1, 1, 1, 1, 1.0])))] += 1
    return {"workload": "sequence tracking", "metric": "frames/s (end to end, PSO 64x30 + simplex, 2 bones, 2 views)",
            "value": nf / dt, "unit": "frames/s", "frames": nf, "pose_evals": evals, "pose_evals_per_s": evals / dt,
            "mean_err_mm": float(e[:, :, :3].mean()), "max_err_mm": float(e[:, :, :3].max()),
            "mean_err_deg": float(e[:, :, 3:].mean()), "max_err_deg": float(e[:, :, 3:].max()),
            "frame_err_mm_p50_p95": [float(np.percentile(fm, 50)), float(np.percentile(fm, 95))],
            "frame_err_deg_p50_p95": [float(np.percentile(fd, 50)), float(np.percentile(fd, 95))],
            "frames_within_1mm_1deg": int(np.sum((fm <= 1.0) & (fd <= 1.0))),
            "lost_bone_frames": len(lost),
            "lost_where_cost_prefers_tracked_pose": prefers_tracked,
            "lost_worst_axis_counts_xyzypr": worst_axes.astype(int).tolist(),
            "first_lost_frame": int(min(f for f, _ in lost)) if lost else None, "seed": args.seed,
            "data": "synthetic sinusoidal trajectory, 250 fps"}


def run_serving(args):
    """Poisson stream (`--rate` jobs/s, `--jobs` jobs) of mixed registration
    jobs, served with continuous batching (up to `--max-jobs` jobs admitted at
    once, their candidates scored together in every engine launch; HBM
    budget 150 GB; subject volume cache) and by the FIFO loop (one job at a
    time) on the same engine.  Latency percentiles over all jobs and over the
    steady part of the stream (jobs arriving after the first quarter)."""
    from autoscoper_gb300 import _lib as L, api, serve
    L.load()

    def jobs():
        rng = np.random.default_rng(17)
        t, out = 0.0, []
        subjects = [f"subject{i}" for i in range(max(2, args.jobs // 2))]
        for i in range(args.jobs):
            t += rng.exponential(1.0 / args.rate)
            out.append(serve.make_job(i, rng, subjects[int(rng.integers(len(subjects)))], t,
                                      frames=(1, args.max_frames), particles=(32, 128), iterations=args.pso_iters,
                                      render_targets=api.render_targets))
        return out

    def steady(js):
        t_q = sorted(j.arrival for j in js)[len(js) // 4]
        lat = np.array([j.latency for j in js if j.arrival >= t_q and j.error is None])
        return {"p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
                "jobs": int(len(lat))}

    res = {}
    modes = [("continuous", args.max_jobs, None, 1), ("fifo", 1, None, 1)]
    if args.sat_items:
        modes.insert(1, ("capped", args.max_jobs, args.sat_items, 1))
    if args.min_backlog > 1:
        modes.insert(1, ("backlog", args.max_jobs, None, args.min_backlog))
    for name, mj, sat, mb in modes:
        js = jobs()
        srv = serve.Server(hbm_budget=150e9, max_jobs=mj, sat_items=sat, min_backlog=mb)
        summary = srv.serve(js, realtime=True)
        summary["steady"] = steady(js)
        summary["jobs_per_s"] = len(js) / summary["wall_s"]
        res[name] = summary
        del srv
    c, f = res["continuous"], res["fifo"]
    return {"workload": "serving", "metric": "sustained pose evals/s; p50/p99 job latency",
            "value": c["pose_evals_per_s"], "unit": "pose-evals/s", "rate_jobs_per_s": args.rate,
            "continuous": c, "fifo": f, "speedup_vs_fifo": c["pose_evals_per_s"] / max(f["pose_evals_per_s"], 1e-9),
            "capped": res.get("capped"), "backlog": res.get("backlog"),
            "data": f"synthetic mixed jobs: volumes 64^3-320^3 u16, viewports 256^2-1024^2, 1-4 bones, 1-3 views, "
                    f"1-{args.max_frames} frames, PSO 32-128 particles x {args.pso_iters} iterations then simplex"}


def run_precision(args):
    """Storage precision on the batched workload: u16, FP16 and BF16 volumes
    (FP32 sampling, compensated FP32 partials, FP64 combine).  Per storage:
    NCC error against the FP64 oracle on a sample of candidates, pose-evals/s
    on the 300-candidate batch, and the final pose error of `--frames` seeded
    registrations (start poses +-1.5 mm / +-1.5 deg, PSO 64 x 30 in +-6 then
    Downhill Simplex per frame) against the ground truth (phantoms with an
    off-axis landmark) and against the u16 result."""
    from autoscoper_gb300 import _lib as L, api, scene as S
    from oracle import oracle as O
    L.load()
    sc = make_scene(landmark=True)  # the landmark makes every rotation observable
    vols = render_targets(sc)
    tr = O.Tracker(sc)
    rng = np.random.default_rng(8)
    n = 300
    bones = np.repeat(np.arange(3), 100).astype(np.int32)
    man = np.concatenate([rng.uniform(-5, 5, (n, 3)), rng.uniform(-5, 5, (n, 3))], 1)
    sample = rng.choice(n, size=args.oracle_sample, replace=False)
    ref = {int(k): [1.0 - c for c in tr.track_frame(int(bones[k]), tr.compose(int(bones[k]), man[k]))]
           for k in sample}
    # start poses +-1.5 mm / +-1.5 deg: inside the chain-filtered cost's basin,
    # so that the pose differences measure the storage, not search failures
    # of the optimizer (from +-5 mm / +-5 deg the NCC is ~0 at the start)
    starts = []
    srng = np.random.default_rng(21)
    for _ in range(args.frames):
        starts.append([S.perturb(t, srng, 1.5, 1.5) for t in sc.truth])
    truth = np.array([np.asarray(t, np.float64) for t in sc.truth])
    out, poses_u16 = {}, None
    for name, st in (("u16", L.ASC_STORE_U16), ("f16", L.ASC_STORE_F16), ("bf16", L.ASC_STORE_BF16)):
        eng = api.Engine(sc, max_items=n, storage=st)
        cost, vcost = eng.eval(bones, man)
        errs = [abs((1.0 - vcost[k, v]) - ref[k][v]) / max(abs(ref[k][v]), 1e-12) for k in ref for v in range(2)]
        aerrs = [abs((1.0 - vcost[k, v]) - ref[k][v]) for k in ref for v in range(2)]
        nccs = [abs(ref[k][v]) for k in ref for v in range(2)]
        eng.eval(bones, man)
        L.call("asc_device_sync")
        t0 = time.perf_counter()
        for _ in range(3):
            eng.eval(bones, man)
        dt = (time.perf_counter() - t0) / 3
        finals = []
        for f, start in enumerate(starts):
            for b, p in enumerate(start):
                eng.set_base_pose(b, p)
            poses, _, _ = eng.optimize_frame(method=0, n_particles=64, n_iter=30, seed=300 + f)
            finals.append(poses)
        finals = np.array(finals)  # frames x bones x 6
        err = np.abs(finals - truth[None])
        row = {"ncc_rel_err_max": float(np.max(errs)), "ncc_rel_err_median": float(np.median(errs)),
               "ncc_abs_err_max": float(np.max(aerrs)), "ncc_abs_err_median": float(np.median(aerrs)),
               "ncc_abs_min": float(np.min(nccs)), "ncc_abs_median": float(np.median(nccs)),
               "pose_evals_per_s": n / dt, "frames": len(starts),
               "pose_err_vs_truth_mm": {"mean": float(err[..., :3].mean()), "max": float(err[..., :3].max())},
               "pose_err_vs_truth_deg": {"mean": float(err[..., 3:].mean()), "max": float(err[..., 3:].max())}}
        if poses_u16 is None:
            poses_u16 = finals
        else:
            d = np.abs(finals - poses_u16)
            row["pose_diff_vs_u16_mm_max"] = float(d[..., :3].max())
            row["pose_diff_vs_u16_deg_max"] = float(d[..., 3:].max())
        out[name] = row
    return {"workload": "precision", "metric": "NCC error vs FP64 oracle and final pose error per volume storage",
            "storage": out, "oracle_sample": int(args.oracle_sample),
            "data": "batched PSO workload (3 bones, 2 views 1024^2, chain filters), synthetic"}


def run_config1(args):
    """The plain method, small: one bone (128^3 u16 phantom at 0.5 mm), 2
    views of 512^2, Sobel, Downhill Simplex from +-2 mm / +-2 deg, one frame.
    Reports the plain per-pose form (the reference's launch sequence, one
    pose at a time), the batched engine on a 256-candidate batch, the
    simplex registration end to end, and the FP64 oracle on the host cores."""
    import ctypes as C
    from autoscoper_gb300 import _lib as L, api, scene as S
    L.load()
    sc = S.make_scene([(128, 128, 128)], 0.5, (512, 512), 0.4, filters="sobel", seed=1, bone_offsets=[(0, 0, 0)])
    vols = api.render_targets(sc)
    rng = np.random.Generator(np.random.PCG64(77))
    sc.poses = [S.perturb(t, rng, 2.0, 2.0) for t in sc.truth]
    eng = api.Engine(sc, max_items=256, volumes=vols)
    crng = np.random.default_rng(4)
    n = 256
    bones = np.zeros(n, np.int32)
    man = np.concatenate([crng.uniform(-2, 2, (n, 3)), crng.uniform(-2, 2, (n, 3))], 1)
    for _ in range(3):
        eng.eval(bones, man)
    L.call("asc_device_sync")
    t0 = time.perf_counter()
    reps = 10
    for _ in range(reps):
        eng.eval(bones, man)
    batched = reps * n / (time.perf_counter() - t0)
    eng.eval(bones[:4], man[:4], plain=True)
    lat = []
    for k in range(64):
        t1 = time.perf_counter()
        eng.eval(bones[k:k + 1], man[k:k + 1], plain=True)
        lat.append(time.perf_counter() - t1)
    lat = np.array(lat)
    regs = []
    srng = np.random.Generator(np.random.PCG64(78))
    for f in range(min(args.frames, 10)):
        eng.set_base_pose(0, S.perturb(sc.truth[0], srng, 2.0, 2.0))
        t1 = time.perf_counter()
        poses, cost, ev = eng.optimize_frame(method=1)
        dt = time.perf_counter() - t1
        err = np.abs(poses[0] - np.asarray(sc.truth[0]))
        regs.append({"s": dt, "evals": ev, "err_mm": float(err[:3].max()), "err_deg": float(err[3:].max())})
    from oracle import oracle as O
    tr = O.Tracker(sc)
    t1 = time.perf_counter()
    for k in range(3):
        tr.minimization_func(0, man[k])
    cpu = 3 / (time.perf_counter() - t1)
    return {"workload": "config 1: plain method, one 128^3 u16 bone at 0.5 mm, 2 views 512^2, Sobel, simplex",
            "metric": "pose evals/s (DRR+filter+NCC, 2 views)", "unit": "pose-evals/s",
            "plain": {"value": 1.0 / lat.mean(), "p50_ms": 1e3 * float(np.percentile(lat, 50)),
                      "p99_ms": 1e3 * float(np.percentile(lat, 99))},
            "batched": {"value": batched, "batch": n, "speedup_vs_plain": batched * lat.mean()},
            "simplex_registration": regs,
            "cpu_baseline": {"value": cpu, "unit": "pose-evals/s", "cores": os.cpu_count(), "kind": "port",
                             "sample": "3 minimizationFunc evaluations by the FP64 oracle"},
            "data": "synthetic phantom and radiographs rendered at a seeded ground truth"}


def run_roofline(args):
    """The roofline batch alone: `--particles` candidates per bone of the
    default workload at fixed random manipulators, evaluated `--reps` times
    (the profiling case for ncu: one k_ray/k_view launch per evaluation, the
    first after the targets are rendered).  Prints the per-launch work."""
    import ctypes as C
    from autoscoper_gb300 import _lib as L, api
    L.load()
    sc = make_scene()
    vols = render_targets(sc)
    nb, npart = 3, args.particles
    st = {"u16": L.ASC_STORE_U16, "f16": L.ASC_STORE_F16, "bf16": L.ASC_STORE_BF16, "f32": L.ASC_STORE_F32}[args.storage]
    eng = api.Engine(sc, max_items=nb * npart, volumes=vols if st == L.ASC_STORE_U16 else None, storage=st)
    L.call("asc_engine_profile", eng.handle, 1)
    rng = np.random.default_rng(3)
    bones = np.repeat(np.arange(nb), npart).astype(np.int32)
    man = np.concatenate([rng.uniform(-5, 5, (nb * npart, 3)), rng.uniform(-5, 5, (nb * npart, 3))], 1)
    ms = []
    for _ in range(args.reps):
        eng.eval(bones, man)
        t3 = (C.c_float * 3)()
        L.call("asc_engine_stats", eng.handle, t3, None, None)
        ms.append(list(t3))
    cnt = (C.c_ulonglong * 4)()
    L.call("asc_engine_counters", eng.handle, cnt)
    nexact = C.c_int()
    L.call("asc_engine_exact_rays", eng.handle, C.byref(nexact))
    ms = np.array(ms)
    return {"workload": "roofline batch", "storage": args.storage, "items": nb * npart, "views": 2, "reps": args.reps,
            "samples_per_launch": cnt[0], "pixels_per_launch": cnt[1], "marched_per_launch": cnt[2],
            "lane_slots_per_launch": cnt[3], "exact_cutoff_rays_per_launch": nexact.value, "setup_ms": float(ms[:, 0].mean()), "ray_ms": float(ms[:, 1].mean()),
            "view_ms": float(ms[:, 2].mean())}


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] in ("tracking", "serving", "precision", "roofline", "config1"):
        ap = argparse.ArgumentParser()
        ap.add_argument("workload")
        ap.add_argument("--frames", type=int, default=20)
        ap.add_argument("--jobs", type=int, default=24)
        ap.add_argument("--rate", type=float, default=2.0, help="mean job arrivals per second")
        ap.add_argument("--oracle-sample", type=int, default=12)
        ap.add_argument("--max-frames", type=int, default=5, help="serving: frames per job drawn from 1..max")
        ap.add_argument("--pso-iters", type=int, default=10, help="serving: PSO iterations per frame")
        ap.add_argument("--max-jobs", type=int, default=8, help="serving: jobs admitted at once")
        ap.add_argument("--seed", type=int, default=100, help="tracking: the swarms' random seed")
        ap.add_argument("--sat-items", type=int, default=0,
                        help="serving: also run the merged loop that admits a job only while the running jobs' "
                             "candidates per iteration stay below this")
        ap.add_argument("--min-backlog", type=int, default=0,
                        help="serving: also run the merged loop that admits a job beside running ones only while "
                             "this many jobs wait")
        ap.add_argument("--particles", type=int, default=100, help="roofline: candidates per bone")
        ap.add_argument("--reps", type=int, default=3, help="roofline: evaluations")
        ap.add_argument("--storage", default="u16", choices=["u16", "f16", "bf16", "f32"],
                        help="roofline: volume storage")
        a = ap.parse_args()
        fn = {"tracking": run_tracking, "serving": run_serving, "precision": run_precision,
              "roofline": run_roofline, "config1": run_config1}[a.workload]
        print(json.dumps(fn(a)), flush=True)
    else:
        main()
