"""Tracker::optimize on the engine: the lock-step speculative simplex gives
exactly the sequential AMOEBA's poses on the GPU cost, and PSO + simplex
registers a perturbed frame back towards the ground truth."""
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


def _apply(sc, b, manip):
    base = G.from_xyzypr(np.asarray(sc.poses[b], np.float32).astype(np.float64))
    V = sc.pivots[b]
    f = G.mul(G.mul(G.mul(base, G.inverse(V)), G.from_axis_angle(manip)), V)
    return G.to_xyzypr(f).astype(np.float32).astype(np.float64)


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
