"""Optimizers as step machines for batched serving.

The serving loop scores the candidates of many jobs in one engine launch, so
an optimizer cannot own its loop: each optimizer here hands out the points
it needs scored and takes their costs back, one step at a time.

* ``amoeba_steps`` -- Downhill Simplex with the decision rules of AMOEBA
  (DownhillSimplex.cpp:39-172: reflection alpha 1, expansion gamma 2,
  contraction beta 0.5, shrink towards the best vertex; stop when the mean
  distance of the vertices to the centroid falls below ftol).  Each step asks
  for the reflection and, speculatively, the expansion and both possible
  contraction points at once, then applies AMOEBA's rules to their costs, so
  the vertices follow the sequential AMOEBA exactly (a point's cost depends on
  the point alone); a shrink asks for its ndim new vertices in one step.
* ``SyncSwarm`` -- a synchronous particle swarm (the velocity rule of
  PSO.cpp:83-109 with runtime inertia and acceleration constants): all
  particles of an iteration are scored together, then the personal and global
  bests and the velocities move.  Particle 0 starts at the zero manipulator,
  the others uniform in [lo, hi]^6 (PSO.cpp:207-214); its random stream is
  its own seed's, so a swarm's trajectory does not depend on what else shares
  the launch.
"""
from __future__ import annotations

import math
from typing import Generator, List

import numpy as np

ALPHA, BETA, GAMMA = 1.0, 0.5, 2.0  # DownhillSimplex.cpp:47-49


def amoeba_steps(P: np.ndarray, Y: np.ndarray, ftol=1e-3, itmax=1000,
                 score_initial=False) -> Generator[List[np.ndarray], List[float], int]:
    """Generator of AMOEBA steps over the (ndim+1, ndim) float64 simplex P and
    its costs Y, both updated in place.  Yields a list of points to score and
    receives their costs (``gen.send(costs)``); returns the iteration count.
    With score_initial the first step scores the initial vertices into Y."""
    mpts, ndim = P.shape
    if score_initial:
        Y[:] = (yield [P[i].copy() for i in range(mpts)])
    it = 0
    while True:
        ilo = 0
        ihi, inhi = (0, 1) if Y[0] > Y[1] else (1, 0)
        for i in range(mpts):
            if Y[i] < Y[ilo]:
                ilo = i
            if Y[i] > Y[ihi]:
                inhi, ihi = ihi, i
            elif Y[i] > Y[inhi] and i != ihi:
                inhi = i
        cent = np.zeros(ndim)
        for j in range(ndim):
            for i in range(mpts):
                cent[j] += P[i, j]
            cent[j] /= mpts
        rtol = 0.0
        for i in range(mpts):
            ss = 0.0
            for j in range(ndim):
                ss += (cent[j] - P[i, j]) * (cent[j] - P[i, j])
            rtol += math.sqrt(ss)
        rtol /= mpts
        if rtol < ftol or it == itmax:
            return it
        it += 1
        pbar = np.zeros(ndim)
        for i in range(mpts):
            if i != ihi:
                for j in range(ndim):
                    pbar[j] += P[i, j]
        pr = np.zeros(ndim)
        for j in range(ndim):
            pbar[j] /= 1.0 * ndim
            pr[j] = (1.0 + ALPHA) * pbar[j] - ALPHA * P[ihi, j]
        expand = GAMMA * pr + (1.0 - GAMMA) * pbar
        con_new = BETA * pr + (1.0 - BETA) * pbar         # contraction after pr replaced the worst vertex
        con_old = BETA * P[ihi] + (1.0 - BETA) * pbar     # contraction from the worst vertex as it was
        ypr, yexp, ycn, yco = (yield [pr, expand, con_new, con_old])
        if ypr <= Y[ilo]:
            if yexp < Y[ilo]:
                P[ihi], Y[ihi] = expand, yexp
            else:
                P[ihi], Y[ihi] = pr, ypr
        elif ypr >= Y[inhi]:
            if ypr < Y[ihi]:
                P[ihi], Y[ihi] = pr, ypr
                prr, yprr = con_new, ycn
            else:
                prr, yprr = con_old, yco
            if yprr < Y[ihi]:
                P[ihi], Y[ihi] = prr, yprr
            else:
                idx = [i for i in range(mpts) if i != ilo]
                pts = [0.5 * (P[i] + P[ilo]) for i in idx]
                ys = yield pts
                for i, p, y in zip(idx, pts, ys):
                    P[i], Y[i] = p, y
        else:
            P[ihi], Y[ihi] = pr, ypr


def run_amoeba(cost, P, Y=None, ftol=1e-3):
    """amoeba_steps driven to the end by a plain cost function (one point at
    a time); returns (P, Y, iterations)."""
    P = np.array(P, dtype=np.float64)
    fresh = Y is None
    Y = np.zeros(len(P)) if fresh else np.array(Y, dtype=np.float64)
    g = amoeba_steps(P, Y, ftol, score_initial=fresh)
    try:
        pts = next(g)
        while True:
            pts = g.send([cost(p) for p in pts])
    except StopIteration as stop:
        return P, Y, stop.value


class SyncSwarm:
    """Synchronous PSO of one bone: ``points()`` gives the particles to score,
    ``update(costs)`` moves the bests and, unless it was the last iteration,
    the particles."""

    def __init__(self, n_particles, lo, hi, seed, w=0.7298, c1=1.4962, c2=1.4962):
        self.rng = np.random.Generator(np.random.PCG64(seed))
        self.w, self.c1, self.c2 = w, c1, c2
        x = self.rng.uniform(lo, hi, (n_particles, 6))
        x[0] = 0.0
        self.x = x
        self.v = np.zeros_like(x)
        self.pb = x.copy()
        self.pbc = np.full(n_particles, np.inf)
        self.gb = np.zeros(6)
        self.gbc = np.inf

    def points(self) -> np.ndarray:
        return self.x

    def update(self, costs, move=True):
        c = np.asarray(costs, dtype=np.float64)
        better = c < self.pbc
        self.pb[better] = self.x[better]
        self.pbc[better] = c[better]
        k = int(np.argmin(c))
        if c[k] < self.gbc:
            self.gbc = float(c[k])
            self.gb = self.x[k].copy()
        if move:
            r1 = self.rng.random(self.x.shape)
            r2 = self.rng.random(self.x.shape)
            self.v = self.w * self.v + self.c1 * r1 * (self.pb - self.x) + self.c2 * r2 * (self.gb - self.x)
            self.x = self.x + self.v
