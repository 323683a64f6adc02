"""Exact cutoff decisions of the batched engine's ray cast
(RayCaster_kernels.cu:190: a sample counts when sample > cutoff).

A uniform volume of raw level 200 with the cutoff c = float32(200 / 65535):
in FP32 c / norm rounds to 200.0, so an FP32 test would leave out every
sample, while c x 65535 = 199.99999995 keeps them all, as the FP64 oracle
does.  Every sample lies in the cutoff's rounding band, so every ray of the
batch (over 2^18 of them, every ray tile on the fix list) is marched a
second time with exact decisions.  The costs must match the oracle's at the
NCC bar.  A cutoff of 0 drops the band (the samples it would decide add at
most rounding), so no ray is marched twice."""
import ctypes as C

import numpy as np
import pytest

from autoscoper_gb300 import _lib as L
from autoscoper_gb300 import api, scene as S
from oracle import oracle as O
from test_gpu_engine import _check, make_targets

pytestmark = pytest.mark.gpu


def _exact_rays(eng):
    n = C.c_int()
    L.call("asc_engine_exact_rays", eng.handle, C.byref(n))
    return n.value


def _plateau(cutoff):
    sc = S.make_scene([(40, 36, 44)], 1.0, (96, 96), 1.0, filters="none", seed=8)
    sc.volumes[0].data = np.full_like(sc.volumes[0].data, 200)
    for row in sc.ray:
        row[0].cutoff = cutoff
    tr = O.Tracker(sc)
    make_targets(sc, tr)
    return sc, tr


def test_every_ray_in_the_band_is_marched_again_and_matches_oracle():
    cut = float(np.float32(200.0 / 65535.0))
    assert np.float32(cut) / (np.float32(1) / np.float32(65535)) == np.float32(200.0)  # FP32 alone drops all
    sc, tr = _plateau(cut)
    n = 256
    eng = api.Engine(sc, max_items=n)
    rng = np.random.default_rng(9)
    bones = np.zeros(n, np.int32)
    man = np.concatenate([rng.uniform(-1.5, 1.5, (n, 3)), rng.uniform(-1.5, 1.5, (n, 3))], 1)
    man[0] = 0
    cost, _ = eng.eval(bones, man)
    assert _exact_rays(eng) > 1 << 18
    for k in range(0, n, 8):
        refv = tr.track_frame(0, tr.compose(0, man[k]))
        _check(cost[k], tr.minimization_func(0, man[k]), refv)
    # the DRR itself holds the plateau's samples
    ok, m, vp, w, h = tr.view_setup(0, 0, sc.truth[0])
    assert ok and O.raycast(tr.vd[0], m, np.float32(vp).astype(np.float64), float(np.float32(sc.ray[0][0].step)),
                            float(np.float32(sc.ray[0][0].intensity)), cut, w, h).max() > 0.05


def test_zero_cutoff_marks_no_ray():
    sc, tr = _plateau(0.0)
    eng = api.Engine(sc, max_items=8)
    man = np.array([[0, 0, 0, 0, 0, 0], [0.5, -0.4, 0.3, 1.0, -0.6, 0.8]], np.float64)
    cost, _ = eng.eval(np.zeros(2, np.int32), man)
    assert _exact_rays(eng) == 0
    for k in range(2):
        _check(cost[k], tr.minimization_func(0, man[k]), tr.track_frame(0, tr.compose(0, man[k])))
