"""The optimizers of the serving loop as step machines (host only): the
stepwise AMOEBA with speculative points follows the reference's AMOEBA
(DownhillSimplex.cpp:39-172, restated by the oracle) vertex for vertex, and
the synchronous swarm depends on its seed alone."""
import numpy as np
import pytest

from autoscoper_gb300 import steppers as ST
from oracle import oracle as O

TARGET = np.array([0.3, -0.2, 0.1, 0.5, -0.4, 0.25])


def bumpy(x):
    x = np.asarray(x)
    return float(np.sum((x - TARGET) ** 2 * np.arange(1, 7)) + 0.1 * np.sin(7 * x[0]) * np.cos(5 * x[3]))


@pytest.mark.parametrize("offset", [0.1, 0.5, 2.0])
def test_stepwise_amoeba_follows_reference_amoeba(offset):
    P = np.zeros((7, 6))
    for i in range(1, 7):
        P[i, i - 1] = offset
    Y = np.array([bumpy(p) for p in P])
    want_P, want_Y = P.copy(), Y.copy()
    want_it = O.amoeba(bumpy, want_P, want_Y, 1e-3)
    got_P, got_Y, got_it = ST.run_amoeba(bumpy, P, Y)
    assert got_it == want_it and np.array_equal(got_P, want_P) and np.array_equal(got_Y, want_Y)
    # scoring the initial vertices inside the generator changes nothing
    P2, Y2, it2 = ST.run_amoeba(bumpy, P)
    assert it2 == want_it and np.array_equal(P2, want_P)


def test_lockstep_simplices_match_each_alone():
    """Several simplices stepped together (their points scored in one batch)
    end where each ends alone."""
    starts = [np.eye(7, 6, -1) * s for s in (0.1, 0.3, 0.7)]
    alone = [ST.run_amoeba(bumpy, P.copy())[0] for P in starts]
    Ps = [P.copy() for P in starts]
    Ys = [np.zeros(7) for _ in starts]
    gens = [ST.amoeba_steps(P, Y, 1e-3, score_initial=True) for P, Y in zip(Ps, Ys)]
    pending = {i: next(g) for i, g in enumerate(gens)}
    while pending:
        batch = {i: [bumpy(p) for p in pts] for i, pts in pending.items()}
        for i in list(pending):
            try:
                pending[i] = gens[i].send(batch[i])
            except StopIteration:
                del pending[i]
    for P, want in zip(Ps, alone):
        assert np.array_equal(P, want)


def test_swarm_is_seeded():
    a, b = ST.SyncSwarm(32, -2, 2, seed=5), ST.SyncSwarm(32, -2, 2, seed=5)
    for _ in range(4):
        ca = [bumpy(p) for p in a.points()]
        cb = [bumpy(p) for p in b.points()]
        a.update(ca)
        b.update(cb)
    assert np.array_equal(a.gb, b.gb) and a.gbc == b.gbc
    assert a.gbc < bumpy(np.zeros(6))  # the swarm improved on its start
