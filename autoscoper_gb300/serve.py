"""Serving loop for registration jobs on one GPU, batched at iteration
granularity.

A job registers 1..N frames of one subject (bones x views, volumes of uneven
size): per frame, Tracker::optimize's PSO then Downhill Simplex for all its
bones (Tracker.cpp:337-571), each frame starting from the previous frame's
result, as the "previous pose" guess does.

Continuous batching.  One engine (`SlotEngine`) holds up to 16 views and 64
bones as slots (asc_engine_set_view / asc_engine_set_bone).  Admission gives
an arrived job view and bone slots and device memory for its volumes and
radiographs under the HBM budget (volumes cached per subject id across
jobs).  Every step of the loop asks each admitted job for its next
candidates -- all particles of a PSO iteration, or the reflection,
expansion and contraction points of every bone's simplex -- scores them all
in ONE engine launch, and hands each job its costs, so the work of all
admitted jobs shares every launch; a job that finishes frees its slots and
memory for the next.  `max_jobs=1` is the plain FIFO one-job-at-a-time loop
the continuous form is measured against.

Each job's computation depends only on its own inputs and seeds (the
engine's costs do not depend on the batch or the slots, its optimizers run
their own random streams), so a job returns the same poses alone and in any
mix; tests/test_gpu_serve.py checks that.
"""
from __future__ import annotations

import ctypes as C
import time
import zlib
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

from . import _lib as L
from . import api
from . import geometry as G
from . import scene as S
from . import steppers as ST


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
    lo: float = -3.0                 # PSO range of the manipulator
    hi: float = 3.0
    offsets: float = 0.1             # initial simplex offsets (Trial::offsets)
    ftol: float = 1e-3
    # filled in by the server
    start: float = 0.0
    finish: float = 0.0
    poses: List[np.ndarray] = field(default_factory=list)   # per frame: (bones, 6) stored poses
    costs: List[np.ndarray] = field(default_factory=list)
    evals: int = 0
    error: Optional[str] = None

    @property
    def latency(self):
        return self.finish - self.arrival


PAD = 2          # edge voxels the device layout adds on every side
VOXEL_BYTES = 8  # two x-pair words (rows y and y+1) per padded voxel


def volume_bytes(vol: S.Volume) -> int:
    """Device bytes of a volume: the padded voxel words plus its occupancy
    grids (a byte and a 16-byte box per 8^3 cell, one grid per view)."""
    D, H, W = vol.data.shape
    cells = ((W + 7) // 8 + 4) * ((H + 7) // 8 + 4) * ((D + 7) // 8 + 4)
    return VOXEL_BYTES * (W + 2 * PAD) * (H + 2 * PAD) * (D + 2 * PAD) + 3 * 17 * cells


def job_bytes(job: Job) -> int:
    """Device bytes a job holds besides its volumes: its radiographs."""
    return sum(v.radiograph.nbytes for v in job.scene.views)


def engine_bytes(n_views: int, rw: int, rh: int, max_items: int, slots: int = 4) -> int:
    """Device bytes asc_engine_create reserves: DRR crops, tile partials,
    layouts, the plain-path buffers."""
    n_iv = max_items * min(slots, n_views)
    tiles = ((rw + 47) // 48) * ((rh + 47) // 48)
    return n_iv * rw * rh * 4 + n_iv * tiles * 72 + 7 * rw * rh * 4 + n_iv * 200 + max_items * 80


class VolumeCache:
    """Device volumes per subject id, shared by the jobs of that subject and
    kept after them until memory is needed."""

    def __init__(self):
        self.entries: Dict[str, list] = {}
        self.bytes: Dict[str, int] = {}
        self.refs: Dict[str, int] = {}
        self.hits = 0
        self.misses = 0

    def held(self) -> int:
        return sum(self.bytes.values())

    def need(self, job: Job) -> int:
        return 0 if job.subject in self.entries else sum(volume_bytes(v) for v in job.scene.volumes)

    def acquire(self, job: Job):
        if job.subject in self.entries:
            self.hits += 1
        else:
            self.misses += 1
            self.entries[job.subject] = [api.DeviceVolume(v) for v in job.scene.volumes]
            self.bytes[job.subject] = sum(volume_bytes(v) for v in job.scene.volumes)
            self.refs[job.subject] = 0
        self.refs[job.subject] += 1
        return self.entries[job.subject]

    def release(self, job: Job):
        self.refs[job.subject] -= 1

    def evict_unused(self) -> int:
        freed = 0
        for s in [s for s, r in self.refs.items() if r == 0]:
            freed += self.bytes.pop(s)
            del self.entries[s]
            del self.refs[s]
        return freed


class SlotEngine:
    """One engine whose views and bones are slots that jobs occupy in turn."""

    def __init__(self, n_views=16, n_bones=64, render=(1024, 1024), max_items=2048, coverage=L.ASC_SUM_TREE):
        self.n_views, self.n_bones, self.max_items = n_views, n_bones, max_items
        self.rw, self.rh = render
        # placeholders that the first job of each slot replaces
        self._vol = api.DeviceVolume(S.Volume(np.full((8, 8, 8), 1000, np.uint16)))
        self._img = api.DeviceImage(np.zeros((8, 8), np.uint16))
        cam = S.biplane_cameras(8, 8, 1.0)[0]
        ph = S.View(cam, np.zeros((8, 8), np.uint16))
        views = (L.ViewDesc * n_views)()
        for v in range(n_views):
            api.fill_view_desc(views[v], ph, self._img)
        bones = (L.BoneDesc * n_bones)()
        for b in range(n_bones):
            api.fill_bone_desc(bones[b], self._vol, G.identity(), np.zeros(6), [S.RayParams()] * 4)
        h = C.c_void_p()
        L.call("asc_engine_create", n_views, views, n_bones, bones, self.rw, self.rh, max_items, coverage, 0,
               C.byref(h))
        self.handle = h.value
        self.keep = {}  # device images a slot's view refers to

    def set_view(self, slot, view: S.View, radiograph: api.DeviceImage, rw, rh):
        d = api.fill_view_desc(L.ViewDesc(), view, radiograph)
        self.keep[slot] = radiograph
        L.call("asc_engine_set_view", self.handle, slot, C.byref(d), rw, rh)

    def set_bone(self, slot, volume: api.DeviceVolume, pivot, pose, rays, view_slots):
        d = api.fill_bone_desc(L.BoneDesc(), volume, pivot, pose, rays)
        vs = (C.c_int * len(view_slots))(*view_slots)
        L.call("asc_engine_set_bone", self.handle, slot, C.byref(d), len(view_slots), vs)

    def set_base_pose(self, slot, xyzypr):
        p = np.ascontiguousarray(xyzypr, np.float64)
        L.call("asc_engine_set_base_pose", self.handle, slot, p.ctypes.data_as(C.POINTER(C.c_double)))

    def eval(self, bones, manips) -> np.ndarray:
        """Costs of candidates (bone slot, manipulator), in launches of at
        most max_items."""
        b = np.ascontiguousarray(bones, dtype=np.int32)
        m = np.ascontiguousarray(manips, dtype=np.float64).reshape(-1, 6)
        out = np.zeros(len(b))
        for i in range(0, len(b), self.max_items):
            bb, mm = b[i:i + self.max_items], m[i:i + self.max_items]
            c = np.zeros(len(bb))
            L.call("asc_engine_eval_host", self.handle, len(bb), bb.ctypes.data_as(C.POINTER(C.c_int)),
                   mm.ctypes.data_as(C.POINTER(C.c_double)), c.ctypes.data_as(C.POINTER(C.c_double)), None, None)
            out[i:i + len(bb)] = c
        return out

    def __del__(self):
        try:
            if self.handle:
                L.load().asc_engine_destroy(self.handle)
        except Exception:
            pass


def keycurve_store(pose) -> np.ndarray:
    """The pose the key curves hold after storing `pose` (asc_keycurve_store)."""
    p = np.ascontiguousarray(pose, np.float64)
    out = np.zeros(6)
    L.call("asc_keycurve_store", p.ctypes.data_as(C.POINTER(C.c_double)), out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def compose(pivot, base, manip) -> np.ndarray:
    """minimizationFunc's pose: base . V^-1 . manip . V (Tracker.cpp:778-793)."""
    f = G.mul(G.mul(G.mul(G.from_xyzypr(base), G.inverse(pivot)), G.from_axis_angle(manip)), pivot)
    return G.to_xyzypr(f)


def register(job: Job, eng: SlotEngine, bone_slots: List[int]):
    """A job's frames as a generator of scoring requests: yields (bone slots,
    manipulators) and receives their costs.  Per frame, for all bones at
    once: the cost at the start pose, a synchronous PSO, the pose moved to the
    swarm's best (the curves keep the stored pose, which the simplex evaluates
    around, while the final composition starts from the unrounded one), the
    lock-step simplex, and the simplex result kept if it beats the start
    (Tracker.cpp:441-571, as asc_engine_optimize_frame does it)."""
    sc = job.scene
    nb = len(bone_slots)
    slots = np.array(bone_slots, np.int32)
    base = [keycurve_store(np.asarray(p, np.float64)) for p in sc.poses]
    for f in range(job.frames):
        for b in range(nb):
            eng.set_base_pose(slots[b], base[b])
        init = yield slots, np.zeros((nb, 6))
        swarms = [ST.SyncSwarm(job.particles, job.lo, job.hi, seed=(job.seed * 1000003 + f) * 64 + b)
                  for b in range(nb)]
        for it in range(job.iterations):
            costs = yield np.repeat(slots, job.particles), np.concatenate([s.points() for s in swarms])
            for b, s in enumerate(swarms):
                s.update(costs[b * job.particles:(b + 1) * job.particles], move=it + 1 < job.iterations)
        mid = [compose(sc.pivots[b], base[b], swarms[b].gb) for b in range(nb)]
        for b in range(nb):
            eng.set_base_pose(slots[b], keycurve_store(mid[b]))
        P = [np.zeros((7, 6)) for _ in range(nb)]
        for b in range(nb):
            for i in range(1, 7):
                P[b][i, i - 1] = job.offsets
        Y = [np.zeros(7) for _ in range(nb)]
        gens = [ST.amoeba_steps(P[b], Y[b], job.ftol, score_initial=True) for b in range(nb)]
        pending = {b: next(gens[b]) for b in range(nb)}
        while pending:
            order = sorted(pending)
            sl = np.concatenate([np.full(len(pending[b]), slots[b], np.int32) for b in order])
            pts = np.concatenate([np.asarray(pending[b]) for b in order])
            costs = yield sl, pts
            k = 0
            for b in order:
                n = len(pending[b])
                try:
                    pending[b] = gens[b].send(list(costs[k:k + n]))
                except StopIteration:
                    del pending[b]
                k += n
        fin = yield slots, np.array([P[b][0] for b in range(nb)])
        poses, out = np.zeros((nb, 6)), np.zeros(nb)
        for b in range(nb):
            take = fin[b] < init[b]
            poses[b] = keycurve_store(compose(sc.pivots[b], mid[b], P[b][0] if take else np.zeros(6)))
            out[b] = fin[b] if take else init[b]
            base[b] = poses[b]
        job.poses.append(poses)
        job.costs.append(out)


class Server:
    """Continuous batching of registration jobs on one SlotEngine.

    hbm_budget: device bytes the server may hold (engine scratch, cached
    volumes, radiographs); max_jobs: jobs admitted at once (1 = FIFO);
    sat_items: a job joins running ones only while their candidates per
    PSO iteration (particles x bones) stay below this (None: no limit).  A
    launch of that many candidates already fills the GPU, so a job admitted
    beyond it would only stretch the running jobs' iterations.
    min_backlog: a job joins running ones only while at least this many jobs
    wait (1: always).  Below the rate one GPU sustains the queue stays short
    and jobs then run one at a time, each at full speed; under a backlog
    they are merged."""

    def __init__(self, hbm_budget: float = 150e9, max_jobs: int = 8, n_views=16, n_bones=64, render=(1024, 1024),
                 max_items=2048, sat_items: Optional[int] = None, min_backlog: int = 1):
        self.budget = float(hbm_budget)
        self.max_jobs = max_jobs
        self.sat_items = sat_items
        self.min_backlog = min_backlog
        self.eng = SlotEngine(n_views, n_bones, render, max_items)
        self.base_bytes = engine_bytes(n_views, render[0], render[1], max_items)
        self.cache = VolumeCache()
        self.free_views = list(range(n_views))
        self.free_bones = list(range(n_bones))
        self.job_bytes = 0
        self.peak = 0.0
        self.occupancy = []  # (time, reserved bytes) after every change

    def reserved(self) -> float:
        return self.base_bytes + self.cache.held() + self.job_bytes

    def _fits(self, job: Job) -> bool:
        if len(job.scene.views) > len(self.free_views) or len(job.scene.volumes) > len(self.free_bones):
            return False
        if job.scene.render_width > self.eng.rw or job.scene.render_height > self.eng.rh:
            return False
        need = self.cache.need(job) + job_bytes(job)
        if self.reserved() + need > self.budget:
            self.cache.evict_unused()
            need = self.cache.need(job) + job_bytes(job)
        return self.reserved() + need <= self.budget

    def _start(self, job: Job, now: float):
        sc = job.scene
        vols = self.cache.acquire(job)
        vslots = [self.free_views.pop(0) for _ in sc.views]
        bslots = [self.free_bones.pop(0) for _ in sc.volumes]
        rads = [api.DeviceImage(v.radiograph) for v in sc.views]
        for i, v in enumerate(sc.views):
            self.eng.set_view(vslots[i], v, rads[i], sc.render_width, sc.render_height)
        for b in range(len(sc.volumes)):
            self.eng.set_bone(bslots[b], vols[b], sc.pivots[b], sc.poses[b],
                              [sc.ray[v][b] for v in range(len(sc.views))], vslots)
        self.job_bytes += job_bytes(job)
        job.start = now
        gen = register(job, self.eng, bslots)
        return {"job": job, "gen": gen, "req": next(gen), "views": vslots, "bones": bslots, "rads": rads}

    def _finish(self, run, now: float):
        job = run["job"]
        job.finish = now
        self.free_views = sorted(self.free_views + run["views"])
        self.free_bones = sorted(self.free_bones + run["bones"])
        self.job_bytes -= job_bytes(job)
        self.cache.release(job)

    def serve(self, jobs: List[Job], realtime: bool = True) -> dict:
        """Runs `jobs` (sorted by arrival); with realtime a job becomes
        eligible at its arrival time.  Returns summary metrics."""
        queue = sorted(jobs, key=lambda j: j.arrival)
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0
        for j in list(queue):  # a job that can never fit
            if (len(j.scene.views) > self.eng.n_views or len(j.scene.volumes) > self.eng.n_bones or
                    self.base_bytes + sum(volume_bytes(v) for v in j.scene.volumes) + job_bytes(j) > self.budget):
                j.error = "job needs more slots or device memory than the server has"
                j.start = j.finish = j.arrival
                queue.remove(j)
        running = []
        launches = 0
        batch_items = []
        while queue or running:
            t = now()
            # admission in arrival order while slots and memory allow
            while queue and len(running) < self.max_jobs and (not realtime or queue[0].arrival <= t):
                if not self._fits(queue[0]):
                    break
                if running and self.sat_items is not None and \
                        sum(r["job"].particles * len(r["job"].scene.volumes) for r in running) >= self.sat_items:
                    break
                if running and self.min_backlog > 1 and \
                        sum(1 for j in queue if not realtime or j.arrival <= t) < self.min_backlog:
                    break
                job = queue.pop(0)
                try:
                    running.append(self._start(job, now()))
                except Exception as e:  # a failed job does not stop the loop
                    job.error = str(e)
                    job.finish = now()
                self.peak = max(self.peak, self.reserved())
                self.occupancy.append((now(), self.reserved()))
            if not running:
                if queue and realtime:
                    time.sleep(max(0.0, min(queue[0].arrival - now(), 0.01)))
                continue
            # one launch for every admitted job's next candidates
            bones = np.concatenate([r["req"][0] for r in running])
            manips = np.concatenate([r["req"][1] for r in running])
            costs = self.eng.eval(bones, manips)
            launches += 1
            batch_items.append(len(bones))
            k = 0
            for r in list(running):
                n = len(r["req"][0])
                r["job"].evals += n
                try:
                    r["req"] = r["gen"].send(costs[k:k + n])
                except StopIteration:
                    running.remove(r)
                    self._finish(r, now())
                    self.occupancy.append((now(), self.reserved()))
                except Exception as e:
                    r["job"].error = str(e)
                    running.remove(r)
                    self._finish(r, now())
                k += n
        wall = now()
        lat = np.array([j.latency for j in jobs if j.error is None])
        evals = sum(j.evals for j in jobs)
        errors = sorted({j.error for j in jobs if j.error is not None})
        occ = self.occupancy + [(wall, self.reserved())]
        mean_occ = sum((occ[i + 1][0] - occ[i][0]) * occ[i][1] for i in range(len(occ) - 1)) / wall if wall else 0.0
        return {"jobs": len(jobs), "failed": sum(j.error is not None for j in jobs), "errors": errors, "wall_s": wall,
                "pose_evals": evals, "pose_evals_per_s": evals / wall if wall > 0 else 0.0,
                "p50_latency_s": float(np.percentile(lat, 50)) if len(lat) else None,
                "p99_latency_s": float(np.percentile(lat, 99)) if len(lat) else None,
                "launches": launches, "mean_batch": float(np.mean(batch_items)) if batch_items else 0.0,
                "peak_reserved_gb": self.peak / 1e9, "mean_reserved_gb": mean_occ / 1e9,
                "cache_hits": self.cache.hits, "cache_misses": self.cache.misses, "max_jobs": self.max_jobs,
                "sat_items": self.sat_items, "min_backlog": self.min_backlog}


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
