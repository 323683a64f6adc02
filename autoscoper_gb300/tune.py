"""The project's autotuner: launch shapes per workload class.

An engine evaluation launches the ray cast (persistent blocks per SM, and
the ray block each warp takes in a 16 x 16 ray tile) and the fused filter /
NCC kernel (persistent blocks per SM).  The best shapes depend on the
workload: crop sizes (render size, magnification), volume sizes (how long a
ray marches, how much of a tile's work is the walk) and the number of views.
For each workload class this module times every candidate shape on that
workload's own candidate batch with CUDA events (the engine's phase timers),
keeps the fastest, and writes the table that asc_engine_create reads
(tuning.txt beside the library: one line per class,
"rpx vox views ray_blocks view_blocks ray_shape", the timings as comments).
Results do not depend on the shapes; only their time does.

    python -m autoscoper_gb300.tune --out autoscoper_gb300/tuning.txt
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
from typing import Dict, List

import numpy as np

from . import _lib as L

DEFAULT = (4, 0, 3)
RAY_BLOCKS = (2, 3, 4)
VIEW_BLOCKS = (1, 2, 0)   # 0: as many as fit
RAY_SHAPES = (2, 3, 4)    # warp ray blocks 4 x 8, 8 x 4, 16 x 2


def _set(handle, cfg):
    c = L.LaunchConfig(*cfg)
    L.call("asc_engine_set_launch", handle, C.byref(c))


def time_config(eng, bones, manips, cfg, reps=3) -> Dict[str, float]:
    """Median phase times (ms) of `reps` evaluations of the batch with the
    launch shapes cfg (after one untimed evaluation)."""
    _set(eng.handle, cfg)
    L.call("asc_engine_profile", eng.handle, 1)
    eng.eval(bones, manips)
    rows = []
    for _ in range(reps):
        eng.eval(bones, manips)
        t3 = (C.c_float * 3)()
        L.call("asc_engine_stats", eng.handle, t3, None, None)
        rows.append(list(t3))
    L.call("asc_engine_profile", eng.handle, 0)
    m = np.median(np.array(rows), axis=0)
    return {"setup": float(m[0]), "ray": float(m[1]), "view": float(m[2]), "total": float(m.sum())}


def tune(eng, bones, manips, reps=3) -> dict:
    """Every candidate shape on one engine and batch: returns the workload
    class, the default's and the best shape's times and every timing.  The
    engine keeps the best shape."""
    cls = (C.c_int * 3)()
    L.call("asc_engine_workload_class", eng.handle, cls)
    before = L.LaunchConfig()
    L.call("asc_engine_get_launch", eng.handle, C.byref(before), None)
    runs: List[dict] = []
    for rb in RAY_BLOCKS:
        for vb in VIEW_BLOCKS:
            for sh in RAY_SHAPES:
                t = time_config(eng, bones, manips, (rb, vb, sh), reps)
                runs.append({"cfg": [rb, vb, sh], **t})
    best = min(runs, key=lambda r: r["total"])
    default = next(r for r in runs if tuple(r["cfg"]) == DEFAULT)
    _set(eng.handle, best["cfg"])
    return {"class": list(cls), "items": int(len(bones)), "best": best, "default": default,
            "gain": default["total"] / best["total"], "runs": runs,
            "loaded": [before.ray_blocks_per_sm, before.view_blocks_per_sm, before.ray_shape]}


def write_table(path, results: Dict[str, dict]):
    """The table asc_tuning_load reads: per class the best shape, with the
    workload it was tuned on and its times as comments."""
    lines = ["# Launch shapes per workload class, written by autoscoper_gb300/tune.py on a GB300.",
             "# rpx vox views ray_blocks_per_sm view_blocks_per_sm ray_shape",
             "#   rpx: ceil log2 of the render pixels; vox: ceil log2 of the largest volume's voxels;",
             "#   view_blocks 0: as many k_view blocks as fit; ray_shape: log2 of a warp's ray-block width"]
    for name, r in results.items():
        c, b, d = r["class"], r["best"], r["default"]
        lines.append(f"# {name}: {r['items']} candidates; default {d['cfg']} {d['total']:.3f} ms "
                     f"(ray {d['ray']:.3f}, view {d['view']:.3f}); best {b['total']:.3f} ms "
                     f"(ray {b['ray']:.3f}, view {b['view']:.3f}), {r['gain']:.3f}x")
        lines.append(f"{c[0]} {c[1]} {c[2]} {b['cfg'][0]} {b['cfg'][1]} {b['cfg'][2]}")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def _workloads():
    """(name, engine, bones, manipulators) of the classes the table covers:
    the headline batch (3 bones, 2 x 1024^2, chain filters, 300 candidates),
    the small plain-method case (one 128^3 bone, 2 x 512^2, Sobel), and a
    serving engine holding mixed jobs."""
    from . import api, scene as S
    out = []
    shapes = [(96, 96, 160), (128, 128, 256), (120, 200, 200)]
    sc = S.make_scene(shapes, 0.4, (1024, 1024), 0.3, filters="chain", seed=0,
                      bone_offsets=[(0.0, 0.0, -45.0), (0.0, 0.0, 0.0), (0.0, 0.0, 45.0)], rot_range=10.0)
    vols = api.render_targets(sc)
    rng = np.random.default_rng(3)
    bones = np.repeat(np.arange(3), 100).astype(np.int32)
    man = np.concatenate([rng.uniform(-5, 5, (300, 3)), rng.uniform(-5, 5, (300, 3))], 1)
    out.append(("headline: 3 bones, 2 x 1024^2, chain, 300 candidates", api.Engine(sc, 300, volumes=vols), bones, man))
    sc1 = S.make_scene([(128, 128, 128)], 0.5, (512, 512), 0.4, filters="sobel", seed=1, bone_offsets=[(0, 0, 0)])
    v1 = api.render_targets(sc1)
    b1 = np.zeros(256, np.int32)
    m1 = np.concatenate([rng.uniform(-2, 2, (256, 3)), rng.uniform(-2, 2, (256, 3))], 1)
    out.append(("plain method: 1 bone 128^3, 2 x 512^2, sobel, 256 candidates", api.Engine(sc1, 256, volumes=v1), b1,
                m1))
    return out


def _serving_workload():
    """A serving engine holding six mixed jobs, with one PSO iteration of
    each as the batch (the launches the serving loop makes while the jobs
    run their swarms)."""
    from . import api, serve
    rng = np.random.default_rng(31)
    srv = serve.Server(hbm_budget=150e9, max_jobs=6)
    jobs = [serve.make_job(i, rng, f"tune{i}", 0.0, frames=(1, 1), particles=(32, 128), iterations=1,
                           render_targets=api.render_targets) for i in range(6)]
    runs = [srv._start(j, 0.0) for j in jobs]
    bones = np.concatenate([np.repeat(r["bones"], j.particles).astype(np.int32) for r, j in zip(runs, jobs)])
    manips = np.concatenate([np.random.default_rng(j.job_id).uniform(-3, 3, (len(r["bones"]) * j.particles, 6))
                             for r, j in zip(runs, jobs)])
    return srv, bones, manips


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=L.TUNING)
    ap.add_argument("--reps", type=int, default=3)
    a = ap.parse_args(argv)
    L.load()
    results = {}
    for name, eng, bones, man in _workloads():
        results[name] = tune(eng, bones, man, a.reps)
    srv, b, m = _serving_workload()

    class _E:  # the serving engine through tune()'s interface
        handle = srv.eng.handle

        @staticmethod
        def eval(bones, manips):
            return srv.eng.eval(bones, manips)

    results["serving: 6 mixed jobs on a 16-view slot engine, one PSO iteration each"] = tune(_E, b, m, a.reps)
    write_table(a.out, results)
    out = {}
    for k, r in results.items():
        out[k] = {kk: v for kk, v in r.items() if kk != "runs"}
        out[k]["runs"] = sorted([[*x["cfg"], round(x["total"], 3)] for x in r["runs"]], key=lambda x: x[-1])
    print(json.dumps(out))


if __name__ == "__main__":
    main()
