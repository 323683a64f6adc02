"""Pins the FP64 oracle to the reference's own sources compiled for the CPU
(oracle/_ref, built from libautoscoper/src by oracle/build_ref.sh).  Skipped
where the reference sources are absent; the committed fixtures in
tests/golden/ carry the same pin everywhere (test_oracle_golden.py)."""
import numpy as np
import pytest

from autoscoper_gb300 import geometry as G
from autoscoper_gb300 import scene as S
from oracle import oracle as O


@pytest.fixture(scope="module")
def small_scene():
    return S.make_scene([(48, 40, 56)], 1.0, (128, 128), 0.8, filters="sobel", seed=3)


def test_frames_bit_exact(ref_lib):
    rng = np.random.default_rng(0)
    for _ in range(50):
        x = np.concatenate([rng.uniform(-50, 50, 3), rng.uniform(-180, 180, 3)])
        y = np.concatenate([rng.uniform(-50, 50, 3), rng.uniform(-30, 30, 3)])
        for n in ("from_xyzypr", "from_axis_angle"):
            assert np.array_equal(getattr(O, "frame_" + n)(x), ref_lib.frame_op("ref_frame_" + n, x))
        f1, f2 = O.frame_from_xyzypr(x), O.frame_from_axis_angle(y)
        assert np.array_equal(O.frame_mul(f1, f2), ref_lib.frame_op("ref_frame_mul", f1, f2))
        assert np.array_equal(O.frame_inverse(f1), ref_lib.frame_op("ref_frame_inverse", f1))
        assert np.array_equal(O.frame_to_xyzypr(f1), ref_lib.frame_op("ref_frame_to_xyzypr", f1, n_out=6))
        assert np.array_equal(O.frame_row_matrix(f1), ref_lib.frame_op("ref_frame_row_matrix", f1, n_out=16))
        assert np.array_equal(O.keycurve_store(x), ref_lib.frame_op("ref_keycurve_store", x, n_out=6))
        assert np.array_equal(O.frame_linear_extrap(f1, O.frame_mul(f1, f2)),
                              ref_lib.frame_op("ref_frame_linear_extrap", f1, O.frame_mul(f1, f2)))
        # the host-side numpy mirror agrees to rounding
        assert np.allclose(G.from_xyzypr(x), O.frame_from_xyzypr(x), atol=1e-14)
        assert np.allclose(G.mul(f1, f2), O.frame_mul(f1, f2), atol=1e-12)


@pytest.mark.parametrize("flip", [(0, 0, 0), (1, 0, 1), (0, 1, 0)])
def test_volume_description(ref_lib, flip):
    rng = np.random.default_rng(5)
    data = np.zeros((20, 17, 23), np.uint16)
    data[3:15, 2:16, 5:20] = rng.integers(1, 4000, size=(12, 14, 15))
    vol = S.Volume(data, (0.4, 0.5, 0.6), flip)
    a, b = O.VolumeDesc(vol), ref_lib.RefVolume(vol)
    assert a.dims == b.dims
    assert np.array_equal(a.data, b.data)
    assert np.array_equal(a.inv_scale, b.inv_scale) and np.array_equal(a.inv_trans, b.inv_trans)
    assert np.array_equal(a.trans_center, b.trans_center)
    assert a.min_value == b.min_value and a.max_value == b.max_value


def _setup(tr, sc, vi, pose):
    xc = O.frame_from_xyzypr(pose)
    mv = O.frame_mul(O.frame_inverse(sc.views[vi].camera.frame), xc)
    imv = O.frame_row_matrix(O.frame_inverse(mv))
    return imv, tr.view_setup(0, vi, pose)


def test_raycast(ref_lib, small_scene):
    sc = small_scene
    tr = O.Tracker(sc)
    rv = ref_lib.RefVolume(sc.volumes[0])
    rng = np.random.default_rng(1)
    for k in range(4):
        pose = S.perturb(sc.truth[0], rng, 3.0, 5.0).astype(np.float64)
        for vi in range(2):
            imv, (ok, m, vp, w, h) = _setup(tr, sc, vi, pose)
            assert ok
            rp = sc.ray[vi][0]
            a = rv.raycast(imv, vp, rp.step, rp.intensity, rp.cutoff, w, h)
            b = O.raycast(tr.vd[0], m, np.float32(vp).astype(np.float64), float(np.float32(rp.step)),
                          float(np.float32(rp.intensity)), float(np.float32(rp.cutoff)), w, h)
            d = np.abs(a - b)
            # FP32 vs FP64 march: samples within rounding of the cutoff may flip,
            # each flip moving one pixel by about step*cutoff.
            assert np.mean(d > 1e-5) < 1e-3
            assert d.max() <= 2.5 * rp.step * rp.cutoff / rp.intensity + 1e-5


def test_rad_and_background(ref_lib, small_scene):
    sc = small_scene
    rng = np.random.default_rng(2)
    img16 = rng.integers(0, 65535, size=(96, 112), dtype=np.uint16)
    img8 = rng.integers(0, 255, size=(96, 112), dtype=np.uint8)
    bg = rng.uniform(0, 1, size=(96, 112)).astype(np.float32)
    ip = np.array([0.01, -0.02, 0.5, 0.45])
    for vp in (np.array([-0.2, -0.2, 0.4, 0.4]), np.array([-0.1, 0.0, 0.13, 0.2])):
        for img in (img16, img8):
            a = ref_lib.rad_render(img, ip, vp, 61, 47)
            b = O.image_render(img, np.float32(ip).astype(np.float64), np.float32(vp).astype(np.float64), 61, 47)
            assert np.abs(a - b).max() < 2e-5  # FP32 vs FP64 texel coordinates on a noise image
        a = ref_lib.background_render(bg, ip, vp, 0.5, 61, 47)
        b = O.image_render(bg, np.float32(ip).astype(np.float64), np.float32(vp).astype(np.float64), 61, 47,
                           mode=1, threshold=0.5)
        assert np.mean(a != b) < 2e-3  # threshold ties under FP32 interpolation


def _img(rng, h, w):
    return rng.uniform(0, 1, size=(h, w)).astype(np.float32)


@pytest.mark.parametrize("shape", [(1, 1), (1, 9), (9, 1), (37, 53)])
def test_filters(ref_lib, shape):
    rng = np.random.default_rng(3)
    h, w = shape
    x = _img(rng, h, w)
    for scale, blend in ((1.0, 0.0), (0.43, 3.0), (0.1, 1.7), (1.0, 0.5), (2.0, 0.2)):
        assert np.abs(ref_lib.sobel(x, scale, blend) - O.apply_filter(S.Filter.sobel(scale, blend), x)).max() < 3e-6
    for al, be in ((1.0, 1.0), (2.5, 0.9), (0.7, 1.3)):
        a = ref_lib.contrast(x, al, be)
        b = O.apply_filter(S.Filter.contrast_filter(al, be), x)
        assert np.abs(a - b).max() < 2e-5 * max(1.0, np.abs(b).max())
    for r in (0.5, 1.0, 1.5, 2.0):
        a = ref_lib.gaussian(x, r)
        b = O.apply_filter(S.Filter.gaussian(r), x)
        assert np.abs(a - b).max() < 3e-6
        for c, t in ((1.0, 0.0), (2.0, 0.05)):
            a = ref_lib.sharpen(x, r, c, t)
            b = O.apply_filter(S.Filter.sharpen(r, c, t), x)
            assert np.mean(np.abs(a - b) > 1e-5) < 2e-3  # threshold ties


def test_elementwise(ref_lib):
    rng = np.random.default_rng(4)
    a, b = _img(rng, 13, 17), _img(rng, 13, 17)
    a[a < 0.3] = 0.0
    c = (rng.uniform(size=(13, 17)) > 0.5).astype(np.float32)
    assert np.array_equal(ref_lib.drr_background(a), O.drr_background(a))
    assert np.abs(ref_lib.multiply(a, b) - O.multiply(a, b)).max() < 1e-7
    assert np.abs(ref_lib.merge(a, b) - O.merge(a, b)).max() < 1e-7
    assert np.abs(ref_lib.composite(a, b, c) - O.composite(a, b, c)).max() < 1e-7


def test_fill_ignores_value_in_reference(ref_lib):
    # gpu::fill writes 1.0 whatever value it is given (Compositor_kernels.cu:64-68).
    assert np.all(ref_lib.fill(10, 0.25) == 1.0)


@pytest.mark.parametrize("n", [2, 7, 100, 256, 257, 768, 4099])
def test_ncc_hdist(ref_lib, n):
    rng = np.random.default_rng(n)
    f = rng.uniform(0, 1, n).astype(np.float32)
    g = (0.6 * f + 0.3 * rng.uniform(0, 1, n)).astype(np.float32)
    m = (rng.uniform(size=n) > 0.3).astype(np.float32)
    f *= m
    g *= m
    a, b = ref_lib.ncc(f, g, m), O.ncc(f, g, m)
    assert abs(a - b) <= 2e-5 * max(1.0, abs(b))
    a, b = ref_lib.hdist(f, g, m), O.hdist(f, g, m)
    assert abs(a - b) <= 2e-5 * max(1.0, abs(b))


def test_ncc_tree_coverage(ref_lib):
    """The reference's sum() drops whole partials at levels whose thread
    count is not a power of two: with n = 768 (3 blocks -> 3 partials, folded
    with s = 1) the last 256 pixels never reach the NCC; with n = 153600
    (600 -> 3 partials) the last 22528.  The oracle's tree mode models it."""
    keep = O.tree_keep_mask(153600)
    assert keep[:131072].all() and not keep[131072:].any()
    n, cut = 768, 512
    keep = O.tree_keep_mask(n)
    assert keep[:cut].all() and not keep[cut:].any()
    rng = np.random.default_rng(9)
    f = rng.uniform(0, 1, n).astype(np.float32)
    g = f.copy()
    g[cut:] = rng.uniform(0, 1, n - cut)   # perfect match where the sum looks
    m = np.ones(n, np.float32)
    assert abs(ref_lib.ncc(f, g, m) - 1.0) < 1e-5
    assert abs(O.ncc(f, g, m, tree=True) - 1.0) < 1e-9
    assert O.ncc(f, g, m, tree=False) < 0.95


def test_ncc_degenerate(ref_lib):
    f = np.zeros(64, np.float32)
    m = np.ones(64, np.float32)
    assert ref_lib.ncc(f, f, m) == 1e5 and O.ncc(f, f, m) == 1e5


def _quadratic(x):
    t = np.array([0.3, -0.2, 0.1, 1.0, -0.5, 0.25])
    return float(np.sum((np.asarray(x, dtype=np.float64) - t) ** 2) + 0.01)


def test_pso_sequential_matches_reference(ref_lib):
    a_pos, a_val = ref_lib.pso(_quadratic, -1.0, 1.0, 6, 25, 1234)
    b_pos, b_val = O.pso_reference(_quadratic, -1.0, 1.0, 6, 25, 1234)
    assert np.array_equal(a_pos, b_pos) and a_val == b_val


def test_amoeba_matches_reference(ref_lib):
    P = np.zeros((7, 6))
    for i in range(1, 7):
        P[i, i - 1] = 0.1
    Y = np.array([_quadratic(p) for p in P])
    Pa, Ya, ita = ref_lib.amoeba(_quadratic, P, Y, 1e-3)
    Pb, Yb = P.copy(), Y.copy()
    itb = O.amoeba(_quadratic, Pb, Yb, 1e-3)
    assert ita == itb and np.array_equal(Pa, Pb) and np.array_equal(Ya, Yb)


@pytest.mark.parametrize("seed", range(6))
def test_pose_curves_bit_exact(ref_lib, seed):
    """The oracle's pose curves (every tangent and segment recomputed from the
    final keys) against the reference's KeyCurve.hpp updated key by key, after
    every prefix of a seeded insert/erase/clear sequence: bit-identical
    (NaN where the reference's slerp gives NaN)."""
    import curve_cases
    ops = curve_cases.ops(seed)
    frames = curve_cases.eval_frames()
    o = O.PoseCurves()
    for i, (kind, f, mask, p) in enumerate(ops):
        if kind == 0:
            o.insert(f, p, mask)
        elif kind == 1:
            o.erase(f, mask)
        else:
            o.clear()
        if i % 5 == 4 or i == len(ops) - 1:
            ref = ref_lib.pose_curve_run(ops[:i + 1], frames)
            got = np.array([o.eval(g) for g in frames])
            assert np.array_equal(got, ref, equal_nan=True), (seed, i)
