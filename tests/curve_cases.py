"""Seeded operation sequences on a volume's pose curves (insert, erase,
clear; all curves or some), shared by the curve tests."""
import numpy as np

N_FRAMES = 48


def pose(rng):
    return np.concatenate([rng.uniform(-60, 60, 3), rng.uniform(-170, 170, 3)])


def ops(seed, n=60):
    """[(kind, frame, mask, pose)]: kind 0 insert, 1 erase, 2 clear."""
    rng = np.random.default_rng(seed)
    out, last = [], pose(rng)
    for _ in range(n):
        r = rng.uniform()
        f = int(rng.integers(0, N_FRAMES - 4))
        mask = 15 if rng.uniform() < 0.8 else int(rng.integers(1, 16))
        if r < 0.70:
            p = pose(rng)
            if rng.uniform() < 0.25:     # a key equal or close to the last one (slerp's nearly-equal branch)
                p = last + (0 if rng.uniform() < 0.5 else rng.normal(0, 1e-3, 6))
            last = p
            out.append((0, f, mask, p))
        elif r < 0.97:
            out.append((1, f, mask, np.zeros(6)))
        else:
            out.append((2, 0, 15, np.zeros(6)))
    return out


def eval_frames():
    return list(range(N_FRAMES))
