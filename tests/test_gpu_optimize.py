"""Tracker::optimize on the engine: the lock-step speculative simplex gives
exactly the sequential AMOEBA's poses on the GPU cost, PSO + simplex
registers a perturbed frame back towards the ground truth, and a tracked
sequence (initial guesses, repeats, key-curve storage) follows the
reference's orchestration step for step."""
import numpy as np
import pytest

from autoscoper_gb300 import api, geometry as G, scene as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _scene(seed):
    from test_gpu_engine import make_targets
    sc = S.make_scene([(40, 48, 56), (36, 30, 44)], 1.0, (112, 112), 0.9, filters="sobel", seed=seed,
                      bone_offsets=[(0, 0, -12), (4, -3, 14)])
    make_targets(sc, O.Tracker(sc))
    rng = np.random.default_rng(seed + 50)
    sc.poses = [S.perturb(t, rng, 1.0, 1.0) for t in sc.truth]
    return sc


def _compose(sc, b, base, manip):
    V = sc.pivots[b]
    f = O.frame_mul(O.frame_mul(O.frame_mul(O.frame_from_xyzypr(base), O.frame_inverse(V)),
                                O.frame_from_axis_angle(manip)), V)
    return O.frame_to_xyzypr(f)


def _apply(sc, b, manip):
    base = np.asarray(sc.poses[b], np.float32).astype(np.float64)
    return O.keycurve_store(_compose(sc, b, base, manip))


def _simplex(eng, b, offsets=0.1, ftol=1e-3):
    P = np.zeros((7, 6))
    for i in range(1, 7):
        P[i, i - 1] = offsets
    cost = lambda x: float(eng.eval(np.array([b], np.int32), np.asarray(x).reshape(1, 6))[0][0])
    Y = np.array([cost(p) for p in P])
    Pf, _, _ = api.amoeba(cost, P, Y, ftol)
    return Pf[0]


def test_simplex_only_equals_sequential_amoeba():
    sc = _scene(21)
    eng = api.Engine(sc, max_items=64)
    # sequential reference flow per bone with single evaluations on the same engine
    want = []
    for b in range(2):
        P = np.zeros((7, 6))
        for i in range(1, 7):
            P[i, i - 1] = 0.1
        cost = lambda x, b=b: float(eng.eval(np.array([b], np.int32), np.asarray(x).reshape(1, 6))[0][0])
        Y = np.array([cost(p) for p in P])
        Pf, Yf, _ = api.amoeba(cost, P, Y, 1e-3)
        want.append(_apply(sc, b, Pf[0]))
    eng2 = api.Engine(sc, max_items=64)
    poses, cost, evals = eng2.optimize_frame(method=1)
    for b in range(2):
        # same trajectory: a diverging simplex would end >= 1e-4 away
        assert np.abs(poses[b] - want[b]).max() <= 2e-5, (poses[b], want[b])


def test_pso_plus_simplex_registers_frame():
    sc = _scene(22)
    eng = api.Engine(sc, max_items=2 * 64)
    tr = O.Tracker(sc)
    c0 = [tr.minimization_func(b, np.zeros(6)) for b in range(2)]
    poses, cost, evals = eng.optimize_frame(method=0, n_particles=64, n_iter=20, lo=-2, hi=2, seed=5)
    assert evals > 2 * 64 * 20
    for b in range(2):
        assert cost[b] <= c0[b] + 1e-12
        err_mm = np.abs(poses[b][:3] - sc.truth[b][:3]).max()
        start_mm = np.abs(np.asarray(sc.poses[b][:3], np.float64) - sc.truth[b][:3]).max()
        assert err_mm < start_mm


def test_track_sequence_follows_reference_orchestration():
    """Four frames of a linear motion, guess 2 (linear extrapolation from the
    third frame on; before that the key curve's value, i.e. the previous
    frame's pose), two repeats per frame, simplex only: asc_engine_track
    against the orchestration of Tracker::optimize (Tracker.cpp:388-571)
    written out on the host over the same engine's costs, with the oracle's
    frame algebra and key-curve storage."""
    sc = _scene(23)
    tr = O.Tracker(sc)
    from test_gpu_engine import make_targets
    truth0 = [np.asarray(t, np.float64) for t in sc.truth]
    step = np.array([0.3, -0.2, 0.15, 0.25, -0.15, 0.2])
    frames = []
    for f in range(4):
        sc.truth = [t + f * step for t in truth0]
        make_targets(sc, tr)
        frames.append([v.radiograph.copy() for v in sc.views])
    images = [[api.DeviceImage(r) for r in fr] for fr in frames]
    nb = len(sc.volumes)
    start = np.zeros((4, nb, 6))
    start[0] = np.array([O.keycurve_store(p) for p in sc.poses])
    eng = api.Engine(sc, max_items=64)
    got, cost, evals = eng.track(images, start, method=1, guess=2, repeats=2)
    # the reference's orchestration, step by step
    ref_eng = api.Engine(sc, max_items=64)
    want = start.copy()
    for f in range(4):
        for v in range(len(sc.views)):
            ref_eng.set_radiograph(v, images[f][v])
        for b in range(nb):
            if f > 1:
                x = O.frame_linear_extrap(O.frame_from_xyzypr(want[f - 2, b]), O.frame_from_xyzypr(want[f - 1, b]))
                want[f, b] = O.keycurve_store(O.frame_to_xyzypr(x))
            elif f > 0:
                want[f, b] = want[f - 1, b]
        for _ in range(2):
            for b in range(nb):
                ref_eng.set_base_pose(b, want[f, b])
                manip = _simplex(ref_eng, b)
                want[f, b] = O.keycurve_store(_compose(sc, b, want[f, b], manip))
    assert evals > 0
    assert np.abs(got - want).max() <= 2e-5, np.abs(got - want).max()


def test_optimize_curves_follow_tracker_optimize():
    """asc_engine_optimize_curves frame by frame over four frames of a linear
    motion (guess 2: linear extrapolation from frame 2 on, before that the
    curve's own value; one repeat, simplex only) against
    Tracker::optimize (Tracker.cpp:386-571) written out over the oracle's
    pose curves (pinned to KeyCurve.hpp) and the same engine's costs: the
    curves agree at every frame."""
    from autoscoper_gb300 import _lib as L
    from test_gpu_engine import make_targets
    sc = _scene(29)
    tr = O.Tracker(sc)
    truth0 = [np.asarray(t, np.float64) for t in sc.truth]
    step = np.array([0.25, -0.2, 0.1, 0.2, -0.1, 0.15])
    images = []
    for f in range(4):
        sc.truth = [t + f * step for t in truth0]
        make_targets(sc, tr)
        images.append([api.DeviceImage(v.radiograph.copy()) for v in sc.views])
    nb, nv = len(sc.volumes), len(sc.views)
    eng, ref_eng = api.Engine(sc, max_items=64), api.Engine(sc, max_items=64)
    curves, ocurves = [api.PoseCurve() for _ in range(nb)], [O.PoseCurves() for _ in range(nb)]
    for b in range(nb):
        curves[b].insert(0, np.asarray(sc.poses[b], np.float64))
        ocurves[b].insert(0, np.asarray(sc.poses[b], np.float64))
    for f in range(4):
        for v in range(nv):
            eng.set_radiograph(v, images[f][v])
            ref_eng.set_radiograph(v, images[f][v])
        cost, evals = eng.optimize_curves(curves, f, 4, method=1, repeats=1, guess=2, dframe=1)
        assert evals > 0 and np.all(np.isfinite(cost))
        for b in range(nb):
            if f > 1:
                x = O.frame_linear_extrap(O.frame_from_xyzypr(ocurves[b].eval(f - 2)),
                                          O.frame_from_xyzypr(ocurves[b].eval(f - 1)))
                ocurves[b].insert(f, O.frame_to_xyzypr(x))
            base = ocurves[b].eval(f)  # at frame 1: the curve holds frame 0's key beyond it
            ref_eng.set_base_pose(b, base)
            ocurves[b].insert(f, _compose(sc, b, base, _simplex(ref_eng, b)))
        for b in range(nb):
            for g in range(f + 1):
                assert np.abs(curves[b].eval(g) - ocurves[b].eval(g)).max() <= 2e-5, (f, b, g)
    with pytest.raises(L.AscError):
        eng.optimize_curves(curves, 4, 4)  # a frame outside the trial
