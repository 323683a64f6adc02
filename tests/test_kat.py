"""Analytic known answers of the path's arithmetic, independent of any build
of the reference: the DRR of a constant-density slab along an axis (closed
form: samples x step x value / intensity), NCC of affinely related images
(+1 / -1), Sobel of a linear ramp (8 |gradient| in the interior), and the
Gaussian, Sharpen and Contrast filters of a constant image.  The oracle is
checked on the CPU; the same cases run through the CUDA kernels on a GPU."""
import numpy as np
import pytest

from autoscoper_gb300 import scene as S
from oracle import oracle as O

N = 16                     # cube edge in voxels (1 mm), so inv_scale = 1/16 exactly
VALUE = 1000               # u16 voxel value everywhere (no crop)
STEP = 1.0 / 16            # the unit slab z in [-1, 0] holds exactly 16 samples
INTENSITY = 0.1
# camera -> normalized volume: origin (0.5, 0.5, 1) above the slab; the
# centre pixel's ray runs along -z, entering at t = 16 and leaving at t = 32
M12 = np.array([1, 0, 0, 0.5, 0, 1, 0, 0.5, 0, 0, 1, 1.0])
DRR_CENTRE = 16 * STEP * (VALUE / 65535.0) / INTENSITY

RAMP_A, RAMP_B = 0.01, 0.02
SOBEL_RAMP = 8.0 * np.hypot(RAMP_A, RAMP_B)


def cube():
    return S.Volume(np.full((N, N, N), VALUE, np.uint16), (1.0, 1.0, 1.0))


def ramp(h=32, w=40):
    y, x = np.mgrid[0:h, 0:w]
    return (RAMP_A * x + RAMP_B * y).astype(np.float32)


def affine_pair(n=5000, seed=4):
    rng = np.random.default_rng(seed)
    f = rng.uniform(0.0, 1.0, n).astype(np.float32)
    return f, (2.5 * f + 0.3).astype(np.float32), (-f).astype(np.float32), np.ones(n, np.float32)


FILTER_CASES = [
    (S.Filter.gaussian(radius=1.5), 0.3, 0.3, 4),
    (S.Filter.sharpen(radius=1.0, contrast=1.0), 0.3, 0.3, 3),
    (S.Filter.contrast_filter(alpha=2.5, beta=0.9), 0.5, 0.5 ** 2.5, 1),
]


# ---------------------------------------------------------------- oracle

def test_oracle_constant_slab_drr():
    vd = O.VolumeDesc(cube())
    assert tuple(vd.inv_scale) == (1.0 / 16,) * 3 and tuple(vd.inv_trans) == (0.0, 0.0, 0.0)
    drr, ns = O.raycast(vd, M12, [0.0, 0.0, 1.0, 1.0], STEP, INTENSITY, 0.0, 1, 1, want_samples=True)
    assert ns[0, 0] == 16
    assert drr[0, 0] == pytest.approx(DRR_CENTRE, rel=1e-12)
    miss = O.raycast(vd, M12, [10.0, 10.0, 1.0, 1.0], STEP, INTENSITY, 0.0, 1, 1)
    assert miss[0, 0] == 0.0


def test_oracle_ncc_of_affine_images():
    f, g, neg, m = affine_pair()
    assert O.ncc(f, g, m, tree=False) == pytest.approx(1.0, abs=1e-12)
    assert O.ncc(f, neg, m, tree=False) == pytest.approx(-1.0, abs=1e-12)


def test_oracle_sobel_of_ramp():
    out = O.apply_filter(S.Filter.sobel(scale=1.0, blend=0.0), ramp())
    assert np.allclose(out[1:-1, 1:-1], SOBEL_RAMP, rtol=1e-6)


@pytest.mark.parametrize("flt,c,expect,margin", FILTER_CASES)
def test_oracle_filter_of_constant(flt, c, expect, margin):
    out = O.apply_filter(flt, np.full((30, 34), c, np.float32))
    assert np.allclose(out[margin:-margin, margin:-margin], expect, rtol=1e-6)


# ---------------------------------------------------------------- CUDA kernels

@pytest.mark.gpu
def test_gpu_constant_slab_drr():
    from autoscoper_gb300 import api
    vol = api.DeviceVolume(cube())
    assert tuple(vol.inv_scale) == (1.0 / 16,) * 3 and tuple(vol.inv_trans) == (0.0, 0.0, 0.0)
    # inverse model-view whose fold with inv_scale = 1/16 is exactly M12
    imv = np.zeros(16)
    imv[:12] = M12 * 16.0
    imv[15] = 1.0
    drr = api.raycast(vol, imv, [0.0, 0.0, 1.0, 1.0], STEP, INTENSITY, 0.0, 1, 1).to_host()
    assert drr[0, 0] == pytest.approx(DRR_CENTRE, rel=2e-6)
    miss = api.raycast(vol, imv, [10.0, 10.0, 1.0, 1.0], STEP, INTENSITY, 0.0, 1, 1).to_host()
    assert miss[0, 0] == 0.0


@pytest.mark.gpu
def test_gpu_ncc_of_affine_images():
    from autoscoper_gb300 import _lib as L, api
    f, g, neg, m = (api.DeviceArray.from_host(a) for a in affine_pair())
    assert api.ncc(f, g, m, coverage=L.ASC_SUM_FULL) == pytest.approx(1.0, abs=2e-6)
    assert api.ncc(f, neg, m, coverage=L.ASC_SUM_FULL) == pytest.approx(-1.0, abs=2e-6)


@pytest.mark.gpu
def test_gpu_sobel_of_ramp():
    from autoscoper_gb300 import api
    out = api.apply_filter(S.Filter.sobel(scale=1.0, blend=0.0), api.DeviceArray.from_host(ramp())).to_host()
    assert np.allclose(out[1:-1, 1:-1], SOBEL_RAMP, rtol=1e-5)


@pytest.mark.gpu
@pytest.mark.parametrize("flt,c,expect,margin", FILTER_CASES)
def test_gpu_filter_of_constant(flt, c, expect, margin):
    from autoscoper_gb300 import api
    src = api.DeviceArray.from_host(np.full((30, 34), c, np.float32))
    out = api.apply_filter(flt, src).to_host()
    assert np.allclose(out[margin:-margin, margin:-margin], expect, rtol=1e-5)
