"""Final-pose parity of Tracker::optimize (Tracker.cpp:337-580) against the
reference's optimizers driven by the FP64 oracle's costs.

Downhill Simplex only: asc_engine_optimize_frame (the lock-step speculative
simplex on the engine's costs) against the reference's sequential AMOEBA
(DownhillSimplex.cpp:39-172) on oracle.Tracker.minimization_func.  PSO then
simplex: the reference's own asynchronous PSO (PSO.cpp:198-295, glibc
rand()) and AMOEBA with Tracker::optimize's pose handling, run once on the
engine's costs and once on the oracle's.  (The engine's batched PSO is a
synchronous swarm with its own random stream, so its trajectory is not the
reference's; its results are checked against the oracle's costs in
test_gpu_engine.py.)  The final poses must agree within 0.05 mm in every
translation and 0.05 degrees of rotation."""
import numpy as np
import pytest

from autoscoper_gb300 import api, scene as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu

MM, DEG = 0.05, 0.05


def _scene(seed, filters="sobel"):
    from test_gpu_engine import make_targets
    sc = S.make_scene([(40, 48, 56), (36, 30, 44)], 1.0, (112, 112), 0.9, filters=filters, seed=seed,
                      bone_offsets=[(0, 0, -12), (4, -3, 14)])
    make_targets(sc, O.Tracker(sc))
    rng = np.random.default_rng(seed + 50)
    sc.poses = [S.perturb(t, rng, 1.0, 1.0) for t in sc.truth]
    return sc


def _moved(sc, b, base, manip):
    """xyzypr of bone b moved by `manip` from `base` (Tracker.cpp:540-556)."""
    V = sc.pivots[b]
    f = O.frame_mul(O.frame_mul(O.frame_mul(O.frame_from_xyzypr(base), O.frame_inverse(V)),
                                O.frame_from_axis_angle(manip)), V)
    return O.frame_to_xyzypr(f)


def _pose_after(sc, b, base, manip):
    """The pose the key curves hold after the optimizer moves bone b by
    `manip` from `base` (Tracker.cpp:540-571)."""
    return O.keycurve_store(_moved(sc, b, base, manip))


def _rot_deg(p, q):
    """Angle of the rotation between two xyzypr poses, in degrees."""
    a, b = O.frame_from_xyzypr(p), O.frame_from_xyzypr(q)
    Ra, Rb = a[:9].reshape(3, 3), b[:9].reshape(3, 3)
    c = (np.trace(Ra.T @ Rb) - 1.0) / 2.0
    return float(np.degrees(np.arccos(np.clip(c, -1.0, 1.0))))


def _oracle_simplex(tr, b, offsets=0.1, ftol=1e-3):
    P = np.zeros((7, 6))
    for i in range(1, 7):
        P[i, i - 1] = offsets
    cost = lambda x: tr.minimization_func(b, np.asarray(x, np.float64))
    Y = np.array([cost(p) for p in P])
    O.amoeba(cost, P, Y, ftol)
    return P[0], Y[0]


def _check(got, want):
    assert np.abs(got[:3] - want[:3]).max() <= MM, (got, want)
    assert _rot_deg(got, want) <= DEG, (got, want, _rot_deg(got, want))


@pytest.mark.parametrize("seed,filters", [(31, "sobel"), (32, "chain")])
def test_simplex_matches_oracle_driven_amoeba(seed, filters):
    """Downhill Simplex only (Tracker.cpp:496-525): the engine's final poses
    against AMOEBA run on the oracle's costs from the same simplex."""
    sc = _scene(seed, filters)
    tr = O.Tracker(sc)
    eng = api.Engine(sc, max_items=64)
    got, _, _ = eng.optimize_frame(method=1)
    for b in range(len(sc.volumes)):
        base = np.asarray(sc.poses[b], np.float32).astype(np.float64)
        x, _ = _oracle_simplex(tr, b)
        _check(got[b], _pose_after(sc, b, base, x))


def _reference_optimize(sc, b, cost_at, set_pose, seed):
    """Tracker::optimize for bone b with PSO then Downhill Simplex
    (Tracker.cpp:441-571) over a cost cost_at(manip) about the bone's current
    pose: the reference's sequential PSO (PSO.cpp:198-295, 100 particles,
    glibc rand() from `seed`), the pose moved to the swarm's best (the curves
    keep the stored pose, which the simplex evaluates around, the final
    composition starts from the unrounded one, Tracker.cpp:445-491), AMOEBA
    from the offsets, and the initial pose kept unless the simplex improved
    on it (Tracker.cpp:516-525).  set_pose(p) moves the cost's base pose."""
    base = np.asarray(sc.poses[b], np.float32).astype(np.float64)
    c0 = cost_at(np.zeros(6))
    pos, _ = O.pso_reference(lambda x: cost_at(np.asarray(x, np.float64)), -2.0, 2.0, epochs=6, stall=3, seed=seed)
    mid = _moved(sc, b, base, np.asarray(pos, np.float64))
    set_pose(O.keycurve_store(mid))
    P = np.zeros((7, 6))
    for i in range(1, 7):
        P[i, i - 1] = 0.1
    Y = np.array([cost_at(p) for p in P])
    O.amoeba(cost_at, P, Y, 1e-3)
    final = cost_at(P[0])
    set_pose(base)
    return _pose_after(sc, b, mid, P[0]) if final < c0 else O.keycurve_store(base)


def test_reference_pso_and_simplex_on_engine_costs_match_oracle_costs():
    """The reference's own optimizers (sequential PSO, then AMOEBA, with
    Tracker::optimize's pose handling) run twice per bone: on the engine's
    costs and on the FP64 oracle's.  The final poses agree within 0.05 mm /
    0.05 degrees."""
    sc = _scene(33)
    eng = api.Engine(sc, max_items=8)
    for b in range(len(sc.volumes)):
        start = np.asarray(sc.poses[b], np.float32)

        def eng_cost(x, b=b):
            return float(eng.eval(np.array([b], np.int32), np.asarray(x, np.float64).reshape(1, 6))[0][0])

        def eng_pose(p, b=b):
            eng.set_base_pose(b, p)
            sc.poses[b] = np.asarray(p, np.float32)

        got = _reference_optimize(sc, b, eng_cost, eng_pose, seed=7 + b)
        sc.poses[b] = start
        eng.set_base_pose(b, start)
        holder = {"tr": O.Tracker(sc)}

        def orc_cost(x, b=b):
            return holder["tr"].minimization_func(b, np.asarray(x, np.float64))

        def orc_pose(p, b=b):
            sc.poses[b] = np.asarray(p, np.float32)
            holder["tr"] = O.Tracker(sc)

        want = _reference_optimize(sc, b, orc_cost, orc_pose, seed=7 + b)
        sc.poses[b] = start
        _check(got, want)
