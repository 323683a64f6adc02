"""NCC parity on the benchmark's own workload: 3 bones (160x96x96,
256x128x128, 200x200x120 u16 at 0.4 mm), 2 views of 1024x1024 u16
radiographs, Contrast(2.5, 0.9) -> Sharpen(1) -> Gaussian(1.5) -> Sobel on
both filter lists.  Twelve seeded candidates (+-5 mm / +-5 deg manipulators)
are scored by the batched engine and by the plain per-pose form and compared,
view by view, with the FP64 oracle's Tracker::trackFrame
(Tracker.cpp:583-773).

The bar is 1e-5 relative on each view's NCC, |dNCC| <= 1e-5 max(|NCC|,
NCC_FLOOR).  Below |NCC| = NCC_FLOOR the relative bar becomes the absolute
1e-7: the path samples, interpolates, filters and accumulates in FP32, whose
rounding leaves ~1e-8 of NCC per stage (DRR march, each filter chain, the
radiograph sampler; measured 4e-8 at most on this workload), so no FP32
implementation holds 1e-5 relative when |NCC| nears 0.  The reference's own
FP32 kernels miss the same candidates by ~4e-6."""
import numpy as np
import pytest

from autoscoper_gb300 import api, scene as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL_REL = 1e-5
NCC_FLOOR = 1e-2  # |NCC| below which the bar is the absolute TOL_REL * NCC_FLOOR = 1e-7


@pytest.fixture(scope="module")
def headline():
    import bench
    sc = bench.make_scene()
    vols = bench.render_targets(sc)  # radiographs at the ground truth, start poses +-5 mm / deg
    return sc, vols


def test_headline_ncc_within_bar(headline):
    sc, vols = headline
    tr = O.Tracker(sc)
    eng = api.Engine(sc, max_items=64, volumes=vols)
    rng = np.random.default_rng(2024)
    n = 12
    bones = (np.arange(n) % 3).astype(np.int32)
    man = np.concatenate([rng.uniform(-5, 5, (n, 3)), rng.uniform(-5, 5, (n, 3))], 1)
    _, vcost = eng.eval(bones, man)
    _, pvcost = eng.eval(bones, man, plain=True)
    worst = 0.0
    for k in range(n):
        ref = tr.track_frame(int(bones[k]), tr.compose(int(bones[k]), man[k]))
        for v in range(2):
            n_ref = 1.0 - ref[v]
            bar = TOL_REL * max(abs(n_ref), NCC_FLOOR)
            for name, got in (("batched", vcost[k, v]), ("plain", pvcost[k, v])):
                d = abs((1.0 - got) - n_ref)
                worst = max(worst, d / bar)
                assert d <= bar, (name, k, v, 1.0 - got, n_ref, d)
    print(f"worst |dNCC| / bar = {worst:.3f}")
