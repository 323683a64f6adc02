"""Serving loop for registration jobs on one GPU.

A job registers 1..N frames of one subject: every frame is a PSO run of all
the job's bones at once on a device-resident engine (volumes, radiographs
and the swarm state stay on the GPU; each frame starts from the previous
frame's result, as Tracker::optimize's "previous pose" guess does).

Continuous batching: `slots` worker threads each take the next job that has
arrived and fits the HBM budget, build (or reuse from the subject cache) its
device volumes, and run it on the engine's own CUDA stream, so the work of
jobs admitted together overlaps on the device.  Jobs that do not fit wait
until running jobs release memory.  `slots=1` is the plain FIFO
one-job-at-a-time loop the continuous form is measured against.

Each job's computation depends only on its own inputs and seed (kernels are
deterministic and order-independent), so a job returns the same poses alone
and in any mix; tests/test_gpu_serve.py checks that.
"""
from __future__ import annotations

import ctypes as C
import threading
import time
import zlib
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

from . import _lib as L
from . import api
from . import geometry as G
from . import scene as S


@dataclass
class Job:
    job_id: int
    subject: str
    scene: S.Scene                   # cameras, volumes, radiographs, filters, start poses
    frames: int = 1
    particles: int = 64
    iterations: int = 20
    seed: int = 1
    arrival: float = 0.0             # seconds after the start of the stream
    # filled in by the server
    start: float = 0.0
    finish: float = 0.0
    poses: List[np.ndarray] = field(default_factory=list)   # per frame: (bones, 6)
    costs: List[np.ndarray] = field(default_factory=list)
    evals: int = 0
    error: Optional[str] = None

    @property
    def latency(self):
        return self.finish - self.arrival


PAD = 2          # edge voxels the device layout adds on every side
VOXEL_BYTES = 8  # two x-pair words (rows y and y+1) per padded voxel


def volume_bytes(vol: S.Volume) -> int:
    """Device bytes of a volume: the padded voxel words plus occupancy grids."""
    D, H, W = vol.data.shape
    cells = ((W + 7) // 8) * ((H + 7) // 8) * ((D + 7) // 8)
    return VOXEL_BYTES * (W + 2 * PAD) * (H + 2 * PAD) * (D + 2 * PAD) + 4 * cells


def engine_bytes(scene: S.Scene, max_items: int) -> int:
    """Device bytes asc_engine_create reserves (DRR crops, tile partials,
    plain-path buffers, swarm) plus the radiographs."""
    nv, rw, rh = len(scene.views), scene.render_width, scene.render_height
    n_iv = max_items * nv
    tiles = ((rw + 31) // 32) * ((rh + 31) // 32)
    b = n_iv * rw * rh * 4 + n_iv * tiles * 72 + 7 * rw * rh * 4 + n_iv * 160 + max_items * 200
    if scene.cf_model:  # SAD: f and g per crop pixel, tile sums, view means
        b += n_iv * rw * rh * 8 + n_iv * tiles * 4 + n_iv * 16
    b += sum(v.radiograph.nbytes for v in scene.views)
    return b


class VolumeCache:
    """Device volumes per subject id, shared by the jobs of that subject."""

    def __init__(self):
        self.lock = threading.Lock()
        self.entries: Dict[str, list] = {}
        self.refs: Dict[str, int] = {}
        self.hits = 0
        self.misses = 0

    def acquire(self, job: Job):
        with self.lock:
            if job.subject in self.entries:
                self.hits += 1
                self.refs[job.subject] += 1
                return self.entries[job.subject], False
            self.misses += 1
            vols = [api.DeviceVolume(v) for v in job.scene.volumes]
            self.entries[job.subject] = vols
            self.refs[job.subject] = 1
            return vols, True

    def release(self, job: Job):
        with self.lock:
            self.refs[job.subject] -= 1

    def evict_unused(self):
        """Frees subjects no running job holds; returns the bytes freed."""
        freed = 0
        with self.lock:
            for s in [s for s, r in self.refs.items() if r == 0]:
                freed += sum(VOXEL_BYTES * int(np.prod(np.asarray(v.dims) + 2 * PAD)) for v in self.entries[s])
                del self.entries[s]
                del self.refs[s]
        return freed


class Server:
    def __init__(self, hbm_budget: float = 150e9, slots: int = 4):
        self.budget = float(hbm_budget)
        self.slots = slots
        self.cache = VolumeCache()
        self.cond = threading.Condition()
        self.reserved = 0.0
        self.peak = 0.0
        self.cached_bytes: Dict[str, int] = {}

    # -- admission ---------------------------------------------------------
    def _need(self, job: Job) -> float:
        need = engine_bytes(job.scene, len(job.scene.volumes) * job.particles)
        if job.subject not in self.cached_bytes:
            need += sum(volume_bytes(v) for v in job.scene.volumes)
        return need

    def _admit(self, job: Job) -> bool:
        need = self._need(job)
        if self.reserved + need > self.budget:
            freed = self.cache.evict_unused()
            if freed:
                for s in [s for s in self.cached_bytes if s not in self.cache.entries]:
                    self.reserved -= self.cached_bytes.pop(s)
                need = self._need(job)
            if self.reserved + need > self.budget:
                return False
        self.reserved += need
        if job.subject not in self.cached_bytes:
            self.cached_bytes[job.subject] = sum(volume_bytes(v) for v in job.scene.volumes)
        self.peak = max(self.peak, self.reserved)
        return True

    def _release(self, job: Job):
        with self.cond:
            self.reserved -= engine_bytes(job.scene, len(job.scene.volumes) * job.particles)
            self.cond.notify_all()

    # -- one job -------------------------------------------------------------
    @staticmethod
    def run_job(job: Job, vols):
        sc = job.scene
        nb = len(sc.volumes)
        eng = api.Engine(sc, max_items=nb * job.particles, volumes=vols)
        try:
            for f in range(job.frames):
                best, cost, ev = eng.pso(job.particles, job.iterations, seed=job.seed + f)
                job.evals += ev
                poses = np.zeros((nb, 6))
                for b in range(nb):
                    base = G.from_xyzypr(np.asarray(sc.poses[b], np.float32).astype(np.float64))
                    V = sc.pivots[b]
                    fr = G.mul(G.mul(G.mul(base, G.inverse(V)), G.from_axis_angle(best[b])), V)
                    poses[b] = G.to_xyzypr(fr).astype(np.float32)
                    sc.poses[b] = poses[b].astype(np.float32)
                    eng.set_base_pose(b, poses[b])
                job.poses.append(poses)
                job.costs.append(cost)
        finally:
            del eng

    # -- the loop ------------------------------------------------------------
    def serve(self, jobs: List[Job], realtime: bool = True) -> dict:
        """Runs `jobs` (sorted by arrival); with realtime, a job becomes
        eligible at its arrival time.  Returns summary metrics."""
        queue = sorted(jobs, key=lambda j: j.arrival)
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0
        for j in list(queue):  # a job larger than the whole budget can never run
            if self._need(j) > self.budget:
                j.error = "job needs more device memory than the HBM budget"
                j.start = j.finish = j.arrival
                queue.remove(j)

        def worker():
            while True:
                with self.cond:
                    job = None
                    while job is None:
                        if not queue:
                            return
                        t = now()
                        for j in queue:
                            if (not realtime or j.arrival <= t) and self._admit(j):
                                job = j
                                break
                            if realtime and j.arrival > t:
                                break
                        if job is None:
                            wait = 0.01
                            if realtime and queue and queue[0].arrival > t:
                                wait = min(wait, queue[0].arrival - t)
                            self.cond.wait(timeout=max(wait, 1e-3))
                    queue.remove(job)
                job.start = now()
                try:
                    vols, _ = self.cache.acquire(job)
                    self.run_job(job, vols)
                except Exception as e:  # a failed job does not stop the loop
                    job.error = str(e)
                finally:
                    self.cache.release(job)
                    job.finish = now()
                    self._release(job)

        threads = [threading.Thread(target=worker, daemon=True) for _ in range(self.slots)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        wall = now()
        lat = np.array([j.latency for j in jobs if j.error is None])
        evals = sum(j.evals for j in jobs)
        errors = sorted({j.error for j in jobs if j.error is not None})
        return {"jobs": len(jobs), "failed": sum(j.error is not None for j in jobs), "errors": errors, "wall_s": wall,
                "pose_evals": evals, "pose_evals_per_s": evals / wall if wall > 0 else 0.0,
                "p50_latency_s": float(np.percentile(lat, 50)) if len(lat) else None,
                "p99_latency_s": float(np.percentile(lat, 99)) if len(lat) else None,
                "peak_reserved_gb": self.peak / 1e9, "cache_hits": self.cache.hits,
                "cache_misses": self.cache.misses, "slots": self.slots}


def device_memory():
    """(free, total) device bytes."""
    free, total = C.c_size_t(), C.c_size_t()
    L.call("asc_mem_info", C.byref(free), C.byref(total))
    return free.value, total.value


def make_job(job_id, rng, subject, arrival, vol_range=(64, 320), view_range=(256, 1024), bones=(1, 4), views=(1, 3),
             frames=(1, 50), particles=(32, 128), iterations=20, render_targets=None):
    """A seeded synthetic job of the mixed serving workload.  The subject id
    fixes the volumes (same subject = same phantoms)."""
    srng = np.random.default_rng(zlib.crc32(subject.encode()))  # stable across processes (str hash is salted)
    nb = int(srng.integers(bones[0], bones[1] + 1))
    shapes = []
    for _ in range(nb):
        n = int(srng.integers(vol_range[0] // 16, vol_range[1] // 16 + 1)) * 16
        shapes.append((n, n, n))
    res = int(rng.integers(view_range[0] // 64, view_range[1] // 64 + 1)) * 64
    nv = int(rng.integers(views[0], views[1] + 1))
    voxel = 0.4
    pitch = 0.3 * 1024 / res
    seed = int(srng.integers(0, 1 << 30))
    sc = S.make_scene(shapes, voxel, (res, res), pitch, filters="sobel", seed=seed,
                      bone_offsets=[(0.0, 0.0, 40.0 * (i - (nb - 1) / 2.0)) for i in range(nb)])
    if nv < 2:
        sc.views = sc.views[:nv]
        sc.ray = sc.ray[:nv]
    elif nv == 3:
        cams = S.biplane_cameras(res, res, pitch)
        extra = G.look_at_frame((424.26, 424.26, 0.0), (0, 0, 0), (0, 0, 1))
        cams.append(S.Camera(extra, res, res, res / 2.0, res / 2.0, 1200.0 / pitch, 1200.0 / pitch))
        sc.views.append(S.View(cams[2], np.zeros((res, res), np.uint16), S.config_filters("sobel"),
                               S.config_filters("sobel")))
        sc.ray.append([S.RayParams(r.step, r.intensity, r.cutoff) for r in sc.ray[0]])
    if render_targets:
        render_targets(sc)
    prng = np.random.default_rng(job_id + 7)
    sc.poses = [S.perturb(t, prng, 3.0, 3.0) for t in sc.truth]
    return Job(job_id, subject, sc, frames=int(rng.integers(frames[0], frames[1] + 1)),
               particles=int(rng.integers(particles[0] // 16, particles[1] // 16 + 1)) * 16, iterations=iterations,
               seed=job_id + 1, arrival=arrival)
