"""GPU parity of the plain per-operator kernels against the FP64 oracle
(and, through the oracle pin, the reference).  Tolerances are stated per
test: the kernels compute in FP32, the oracle in FP64."""
import numpy as np
import pytest

from autoscoper_gb300 import _lib as L
from autoscoper_gb300 import api, scene as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small():
    sc = S.make_scene([(48, 40, 56)], 1.0, (128, 128), 0.8, filters="sobel", seed=3)
    return sc, O.Tracker(sc)


def _imv(sc, vi, pose):
    xc = O.frame_from_xyzypr(pose)
    mv = O.frame_mul(O.frame_inverse(sc.views[vi].camera.frame), xc)
    return O.frame_row_matrix(O.frame_inverse(mv))


def test_volume_description_matches_oracle(small):
    sc, tr = small
    rng = np.random.default_rng(5)
    data = np.zeros((20, 17, 23), np.uint16)
    data[3:15, 2:16, 5:20] = rng.integers(1, 4000, size=(12, 14, 15))
    for flip in ((0, 0, 0), (1, 0, 1)):
        vol = S.Volume(data, (0.4, 0.5, 0.6), flip)
        a, b = api.DeviceVolume(vol), O.VolumeDesc(vol)
        assert a.dims == b.dims
        assert np.array_equal(a.inv_scale, b.inv_scale) and np.array_equal(a.inv_trans, b.inv_trans)
        assert np.array_equal(a.trans_center, b.trans_center)
        assert np.float32(a.min_value) == np.float32(b.min_value)


def test_empty_volume_is_an_error_status():
    with pytest.raises(L.AscError) as e:
        api.DeviceVolume(S.Volume(np.zeros((4, 4, 4), np.uint16)))
    assert e.value.status == -3


@pytest.mark.parametrize("storage", [L.ASC_STORE_U16, L.ASC_STORE_F16, L.ASC_STORE_BF16])
def test_raycast_matches_oracle(small, storage):
    sc, tr = small
    dv = api.DeviceVolume(sc.volumes[0], storage)
    rng = np.random.default_rng(1)
    for k in range(3):
        pose = S.perturb(sc.truth[0], rng, 3.0, 5.0).astype(np.float64)
        for vi in range(2):
            ok, m, vp, w, h = tr.view_setup(0, vi, pose)
            rp = sc.ray[vi][0]
            got = api.raycast(dv, _imv(sc, vi, pose), vp, rp.step, rp.intensity, rp.cutoff, w, h).to_host()
            ref = O.raycast(tr.vd[0], m, np.float32(vp).astype(np.float64), float(np.float32(rp.step)),
                            float(np.float32(rp.intensity)), float(np.float32(rp.cutoff)), w, h)
            d = np.abs(got - ref)
            if storage == L.ASC_STORE_U16:
                # FP32 march vs FP64: samples within rounding of the cutoff may flip
                assert np.mean(d > 2e-5) < 2e-3, np.sort(d.ravel())[-10:]
                assert d.max() <= 2.5 * rp.step * rp.cutoff / rp.intensity + 2e-5
            elif storage == L.ASC_STORE_F16:
                # phantom values < 2048 are exact in half; the few above round
                assert np.mean(d > 1e-4) < 5e-3
            else:
                assert np.abs(got - ref).mean() < 2e-3  # bfloat16 keeps 8 mantissa bits


def test_raycast_invisible_and_empty(small):
    sc, tr = small
    dv = api.DeviceVolume(sc.volumes[0])
    out = api.DeviceArray((8, 8))
    out.upload(np.ones((8, 8), np.float32))
    api.raycast(dv, np.eye(4).reshape(-1), [-1, -1, 2, 2], 0.5, 1.0, 0.0, 8, 8, visible=False, out=out)
    assert np.all(out.to_host() == 0)
    # a ray set-up that misses the box everywhere
    imv = np.eye(4).reshape(-1).copy()
    imv[3] = 5000.0
    got = api.raycast(dv, imv, [-1, -1, 2, 2], 0.5, 1.0, 0.0, 8, 8).to_host()
    assert np.all(got == 0)


@pytest.mark.parametrize("bps", [8, 16])
def test_rad_render(bps):
    rng = np.random.default_rng(2)
    hi = 255 if bps == 8 else 65535
    img = rng.integers(0, hi, size=(96, 112)).astype(np.uint8 if bps == 8 else np.uint16)
    di = api.DeviceImage(img)
    ip = np.array([0.01, -0.02, 0.5, 0.45])
    for vp in (np.array([-0.2, -0.2, 0.4, 0.4]), np.array([-0.1, 0.0, 0.13, 0.2])):
        got = api.rad_render(di, ip, vp, 61, 47).to_host()
        ref = O.image_render(img, np.float32(ip).astype(np.float64), np.float32(vp).astype(np.float64), 61, 47)
        assert np.abs(got - ref).max() < 2e-5


def test_background_render():
    rng = np.random.default_rng(3)
    bg = rng.uniform(0, 1, size=(96, 112)).astype(np.float32)
    di = api.DeviceImage(bg)
    ip, vp = np.array([0.01, -0.02, 0.5, 0.45]), np.array([-0.2, -0.2, 0.4, 0.4])
    got = api.background_render(di, ip, vp, 0.5, 61, 47).to_host()
    ref = O.image_render(bg, np.float32(ip).astype(np.float64), np.float32(vp).astype(np.float64), 61, 47, mode=1,
                         threshold=0.5)
    assert np.mean(got != ref) < 2e-3


SHAPES = [(1, 1), (1, 9), (9, 1), (37, 53), (64, 64), (3, 1100)]


@pytest.mark.parametrize("shape", SHAPES)
def test_filters(shape):
    rng = np.random.default_rng(4)
    x = rng.uniform(0, 1, size=shape).astype(np.float32)
    dx = api.DeviceArray.from_host(x)
    cases = [S.Filter.sobel(1.0, 0.0), S.Filter.sobel(0.43, 3.0), S.Filter.sobel(2.0, 0.2),
             S.Filter.contrast_filter(2.5, 0.9), S.Filter.contrast_filter(1.0, 1.0),
             S.Filter.contrast_filter(1.0, 1.0, size=5), S.Filter.gaussian(1.5), S.Filter.gaussian(0.5),
             S.Filter.gaussian(0.2), S.Filter.sharpen(1.0, 1.0, 0.0), S.Filter.sharpen(2.0, 2.0, 0.05)]
    for f in cases:
        got = api.apply_filter(f, dx).to_host()
        ref = O.apply_filter(f, x)
        d = np.abs(got - ref)
        if f.kind == S.SHARPEN:
            assert np.mean(d > 1e-5) < 3e-3  # |f - blur| == threshold ties
        elif f.kind == S.CONTRAST:
            assert d.max() < 3e-5 * max(1.0, np.abs(ref).max())
        else:
            assert d.max() < 3e-6, (f, d.max())


def test_elementwise():
    rng = np.random.default_rng(5)
    a = rng.uniform(0, 1, size=(13, 17)).astype(np.float32)
    a[a < 0.3] = 0
    b = rng.uniform(0, 1, size=(13, 17)).astype(np.float32)
    c = (rng.uniform(size=(13, 17)) > 0.5).astype(np.float32)
    da, db, dc = (api.DeviceArray.from_host(v) for v in (a, b, c))
    assert np.array_equal(api.elementwise("asc_drr_background", da).to_host(), O.drr_background(a))
    assert np.abs(api.elementwise("asc_multiply", da, db).to_host() - O.multiply(a, b)).max() < 1e-7
    assert np.abs(api.elementwise("asc_merge", da, db).to_host() - O.merge(a, b)).max() < 1e-7
    comp = api.elementwise("asc_composite", da, db, dc).to_host().reshape(-1)
    assert np.abs(comp - O.composite(a, b, c)).max() < 1e-7
    f = api.DeviceArray((1000,))
    L.call("asc_fill", f.ptr, 1000, 0.25, None)
    assert np.all(f.to_host() == 0.25)


@pytest.mark.parametrize("n", [2, 7, 100, 256, 257, 768, 4099, 65536, 153600, 230001])
@pytest.mark.parametrize("coverage", [L.ASC_SUM_TREE, L.ASC_SUM_FULL])
def test_ncc_hdist(n, coverage):
    rng = np.random.default_rng(n)
    f = rng.uniform(0, 1, n).astype(np.float32)
    g = (0.6 * f + 0.3 * rng.uniform(0, 1, n)).astype(np.float32)
    m = (rng.uniform(size=n) > 0.3).astype(np.float32)
    f *= m
    g *= m
    df, dg, dm = (api.DeviceArray.from_host(v) for v in (f, g, m))
    tree = coverage == L.ASC_SUM_TREE
    got, ref = api.ncc(df, dg, dm, coverage), O.ncc(f, g, m, tree)
    assert abs(got - ref) <= 1e-5 * max(1.0, abs(ref)), (got, ref)
    got, ref = api.hdist(df, dg, dm, coverage), O.hdist(f, g, m, tree)
    assert abs(got - ref) <= 1e-5 * max(1.0, abs(ref)), (got, ref)


@pytest.mark.parametrize("storage", [L.ASC_STORE_U16, L.ASC_STORE_BF16])
def test_empty_space_skip_is_exact(small, storage):
    """Skipping cells whose voxels are all <= cutoff leaves every DRR pixel
    bit-identical (the skipped samples add nothing)."""
    sc, tr = small
    dv = api.DeviceVolume(sc.volumes[0], storage)
    rng = np.random.default_rng(8)
    try:
        for k in range(3):
            pose = S.perturb(sc.truth[0], rng, 3.0, 20.0).astype(np.float64)
            for vi in range(2):
                ok, m, vp, w, h = tr.view_setup(0, vi, pose)
                rp = sc.ray[vi][0]
                for cut in (rp.cutoff, 0.0, 0.02):
                    L.call("asc_set_option", 1, 1)
                    a = api.raycast(dv, _imv(sc, vi, pose), vp, rp.step, rp.intensity, cut, w, h).to_host()
                    L.call("asc_set_option", 1, 0)
                    b = api.raycast(dv, _imv(sc, vi, pose), vp, rp.step, rp.intensity, cut, w, h).to_host()
                    assert np.array_equal(a, b)
    finally:
        L.call("asc_set_option", 1, 1)


def test_ncc_degenerate():
    z = api.DeviceArray.from_host(np.zeros(64, np.float32))
    one = api.DeviceArray.from_host(np.ones(64, np.float32))
    assert api.ncc(z, z, one) == 1e5


def test_cutoff_at_a_voxel_level_decides_as_fp64():
    """A cutoff exactly at a tissue level (c = float32(200 / 65535), which FP32
    alone would round to the level itself): the plain ray caster and the
    batched engine count every sample of the uniform 200 soft tissue, as the
    FP64 oracle does (RayCaster_kernels.cu:189), and the engine's costs stay
    within the NCC bar.  No filters: on a noise-free phantom a Sobel image is
    exactly 0 over flat regions in FP64 but ~1e-9 in FP32, which moves the
    DRR mask (Tracker.cpp:722-735) by whole pixels, whatever the march does."""
    sc = S.make_scene([(40, 36, 44)], 1.0, (96, 96), 1.0, filters="none", seed=4)
    sc.volumes[0].data = S.phantom((40, 36, 44), seed=4, noise=0.0)
    cut = float(np.float32(200.0 / 65535.0))
    for row in sc.ray:
        row[0].cutoff = cut
    tr = O.Tracker(sc)
    for vi, v in enumerate(sc.views):
        ok, m, _, _, _ = tr.view_setup(0, vi, sc.truth[0])
        drr = O.raycast(tr.vd[0], m, S.target_viewport(v.camera), sc.ray[vi][0].step, sc.ray[vi][0].intensity, cut,
                        96, 96)
        v.radiograph = S.radiograph_from_drr(drr, seed=vi)
    dv = api.DeviceVolume(sc.volumes[0])
    rng = np.random.default_rng(6)
    pose = S.perturb(sc.truth[0], rng, 2.0, 10.0).astype(np.float64)
    for vi in range(2):
        ok, m, vp, w, h = tr.view_setup(0, vi, pose)
        rp = sc.ray[vi][0]
        got = api.raycast(dv, _imv(sc, vi, pose), vp, rp.step, rp.intensity, cut, w, h).to_host()
        ref = O.raycast(tr.vd[0], m, np.float32(vp).astype(np.float64), float(np.float32(rp.step)),
                        float(np.float32(rp.intensity)), cut, w, h)
        assert ref.max() > 0.1 and np.abs(got - ref).max() < 1e-6
    eng = api.Engine(sc, max_items=8, volumes=[dv])
    man = np.array([[0, 0, 0, 0, 0, 0], [0.4, -0.3, 0.2, 1.0, -0.5, 0.6]], np.float64)
    _, vcost = eng.eval(np.zeros(2, np.int32), man)
    for k in range(2):
        refv = tr.track_frame(0, tr.compose(0, man[k]))
        for v in range(2):
            assert abs(vcost[k, v] - refv[v]) <= 1e-5 * max(abs(1.0 - refv[v]), 1e-2), (k, v, vcost[k, v], refv[v])
