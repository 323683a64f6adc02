"""The kernels' own ray march (asc_march.cuh), compiled as host C++ with
g++, against the FP64 oracle: the double-float ray set-up reproduces the
oracle's sample counts and positions, the DRR agrees to ~1e-7, and skipping
empty cells changes no bit.  Runs on any machine (no GPU)."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from autoscoper_gb300 import scene as S
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def hm(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("hm") / "libhost_march.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", "-o", so,
                    os.path.join(ROOT, "tests", "cpp", "host_march.cpp")], check=True)
    lib = C.CDLL(so)
    lib.hm_raycast.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                               C.c_float, C.c_float, C.c_float, C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    lib.hm_occupancy.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_float, C.c_void_p]
    lib.hm_band.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_float, C.c_float,
                            C.c_int, C.c_int, C.c_void_p]
    return lib


def run(hm, vd, m, vp, rp, w, h, storage=0, skip=1, cutoff=None):
    out = np.zeros(w * h, np.float32)
    ns = np.zeros(w * h, np.int32)
    mf = np.ascontiguousarray(m, np.float32)
    vpf = np.ascontiguousarray(vp, np.float32)
    vol = np.ascontiguousarray(vd.data, np.uint16)
    cut = rp.cutoff if cutoff is None else cutoff
    hm.hm_raycast(vol.ctypes.data, vd.dims[0], vd.dims[1], vd.dims[2], storage, skip, mf.ctypes.data, vpf.ctypes.data,
                  rp.step, rp.intensity, cut, out.ctypes.data, w, h, ns.ctypes.data)
    return out.reshape(h, w), ns.reshape(h, w)


@pytest.fixture(scope="module")
def small():
    sc = S.make_scene([(48, 40, 56)], 1.0, (128, 128), 0.8, filters="sobel", seed=3)
    return sc, O.Tracker(sc)


def test_host_march_matches_oracle(hm, small):
    sc, tr = small
    rng = np.random.default_rng(1)
    for _ in range(3):
        pose = S.perturb(sc.truth[0], rng, 3.0, 20.0).astype(np.float64)
        for vi in range(2):
            ok, m, vp, w, h = tr.view_setup(0, vi, pose)
            rp = sc.ray[vi][0]
            got, ns = run(hm, tr.vd[0], m, vp, rp, w, h)
            ref, rns = O.raycast(tr.vd[0], m, np.float32(vp).astype(np.float64), float(np.float32(rp.step)),
                                 float(np.float32(rp.intensity)), float(np.float32(rp.cutoff)), w, h, want_samples=True)
            assert np.array_equal(ns, rns)            # same samples on every ray
            assert np.abs(got - ref).max() < 1e-6     # FP32 sums of FP64-placed samples


def test_host_march_skip_is_exact(hm, small):
    sc, tr = small
    # the grid holds all three kinds of cell: empty, trimmed to its box, and
    # covered by its box (whose trim the walk skips)
    vd = tr.vd[0]
    vol = np.ascontiguousarray(vd.data, np.uint16)
    counts = np.zeros(3, np.int64)
    hm.hm_occupancy(vol.ctypes.data, vd.dims[0], vd.dims[1], vd.dims[2], sc.ray[0][0].cutoff, counts.ctypes.data)
    assert counts.min() > 0, counts
    rng = np.random.default_rng(2)
    for _ in range(3):
        pose = S.perturb(sc.truth[0], rng, 3.0, 30.0).astype(np.float64)
        for vi in range(2):
            ok, m, vp, w, h = tr.view_setup(0, vi, pose)
            rp = sc.ray[vi][0]
            for cut in (rp.cutoff, 0.0, 0.02):
                a, _ = run(hm, tr.vd[0], m, vp, rp, w, h, skip=1, cutoff=cut)
                b, _ = run(hm, tr.vd[0], m, vp, rp, w, h, skip=0, cutoff=cut)
                assert np.array_equal(a, b)


@pytest.mark.parametrize("angles", [(0.0, 0.0, 0.0), (90.0, 0.0, 0.0), (0.0, 90.0, 90.0)])
def test_host_march_skip_is_exact_axis_aligned(hm, small, angles):
    """Rays along the grid axes: coordinates that stay on a cell plane or a
    voxel centre, and axes with no bound (NaN trim)."""
    sc, tr = small
    pose = np.array(sc.truth[0], np.float64)
    pose[3:] = angles
    for vi in range(2):
        ok, m, vp, w, h = tr.view_setup(0, vi, pose)
        if not ok:
            continue
        rp = sc.ray[vi][0]
        a, ns = run(hm, tr.vd[0], m, vp, rp, w, h, skip=1)
        b, _ = run(hm, tr.vd[0], m, vp, rp, w, h, skip=0)
        assert ns.sum() > 0 and np.array_equal(a, b)
        ref = O.raycast(tr.vd[0], m, np.float32(vp).astype(np.float64), float(np.float32(rp.step)),
                        float(np.float32(rp.intensity)), float(np.float32(rp.cutoff)), w, h)
        assert np.abs(a - ref).max() < 1e-6


def test_host_march_bf16_matches_oracle_on_rounded_volume(hm, small):
    sc, tr = small
    vd = tr.vd[0]
    # the oracle on the volume rounded to bfloat16 (round to nearest even)
    bits = vd.data.astype(np.float32).view(np.uint32)
    bits = (bits + 0x7FFF + ((bits >> 16) & 1)) & 0xFFFF0000
    rounded = bits.view(np.float32).astype(np.uint16)

    class VD:
        pass
    v2 = VD()
    v2.data, v2.bps, v2.dims = rounded, 16, vd.dims
    ok, m, vp, w, h = tr.view_setup(0, 0, sc.truth[0])
    rp = sc.ray[0][0]
    got, _ = run(hm, vd, m, vp, rp, w, h, storage=2)
    ref = O.raycast(v2, m, np.float32(vp).astype(np.float64), float(np.float32(rp.step)),
                    float(np.float32(rp.intensity)), float(np.float32(rp.cutoff)), w, h)
    assert np.abs(got - ref).max() < 1e-6


def test_host_march_f32_storage_equals_u16(hm, small):
    """FP32 voxels hold the same values as the u16 halves, and the march's
    interpolation is the same arithmetic on them: identical DRRs."""
    sc, tr = small
    rng = np.random.default_rng(4)
    pose = S.perturb(sc.truth[0], rng, 2.0, 10.0).astype(np.float64)
    ok, m, vp, w, h = tr.view_setup(0, 1, pose)
    rp = sc.ray[1][0]
    a, na = run(hm, tr.vd[0], m, vp, rp, w, h, storage=0)
    b, nb = run(hm, tr.vd[0], m, vp, rp, w, h, storage=3)
    assert np.array_equal(na, nb)
    assert np.array_equal(a, b)


def test_cutoff_at_a_voxel_level_decides_as_fp64(hm):
    """A cutoff at a tissue level exactly (c = float32(200 / 65535)): a sample
    of a uniform 200 region is 200 raw in FP32, while c / norm rounds to
    200.0 but c x 65535 is 199.99999995.  The march decides such samples
    exactly (RayCaster_kernels.cu:189: s > cutoff), as the FP64 oracle does,
    so every sample of the soft tissue counts and the DRRs agree."""
    sc = S.make_scene([(40, 36, 44)], 1.0, (96, 96), 1.0, filters="sobel", seed=4)
    sc.volumes[0].data = S.phantom((40, 36, 44), seed=4, noise=0.0)  # levels exactly 200, 900, 1800
    tr = O.Tracker(sc)
    cut = float(np.float32(200.0 / 65535.0))
    assert np.float32(cut) / (np.float32(1) / np.float32(65535)) == np.float32(200.0)  # FP32 alone would exclude 200
    rng = np.random.default_rng(6)
    for _ in range(2):
        pose = S.perturb(sc.truth[0], rng, 2.0, 10.0).astype(np.float64)
        for vi in range(2):
            ok, m, vp, w, h = tr.view_setup(0, vi, pose)
            rp = sc.ray[vi][0]
            got, _ = run(hm, tr.vd[0], m, vp, rp, w, h, cutoff=cut)
            ref = O.raycast(tr.vd[0], m, np.float32(vp).astype(np.float64), float(np.float32(rp.step)),
                            float(np.float32(rp.intensity)), cut, w, h)
            assert ref.max() > 0.1
            assert np.abs(got - ref).max() < 1e-6


@pytest.mark.parametrize("level,noise", [(200, 0.0), (200, 20.0)])
def test_cutoff_band_holds_every_fp32_misdecision(hm, level, noise):
    """The march decides a sample in FP32 only outside its ray's band
    (Cutoff: the bound on the FP32 value's error).  For every sample of every
    ray, with the cutoff at a voxel level (c = float32(level / 65535), where
    FP32 and exact decisions part), on a noise-free phantom (a plateau at the
    cutoff) and a noisy one: each sample whose FP32 decision (v > raw)
    differs from the exact one lies inside the band."""
    shape = (40, 36, 44)
    sc = S.make_scene([shape], 1.0, (96, 96), 1.0, filters="sobel", seed=4)
    sc.volumes[0].data = S.phantom(shape, seed=4, noise=noise)
    if noise == 0.0:
        assert (sc.volumes[0].data == level).any()
    tr = O.Tracker(sc)
    cut = float(np.float32(level / 65535.0))
    rng = np.random.default_rng(12)
    tot = np.zeros(4, np.int64)
    for _ in range(2):
        pose = S.perturb(sc.truth[0], rng, 2.0, 10.0).astype(np.float64)
        for vi in range(2):
            ok, m, vp, w, h = tr.view_setup(0, vi, pose)
            vd = tr.vd[0]
            vol = np.ascontiguousarray(vd.data, np.uint16)
            mf = np.ascontiguousarray(m, np.float32)
            vpf = np.ascontiguousarray(vp, np.float32)
            c = np.zeros(4, np.int64)
            hm.hm_band(vol.ctypes.data, vd.dims[0], vd.dims[1], vd.dims[2], mf.ctypes.data, vpf.ctypes.data,
                       float(np.float32(sc.ray[vi][0].step)), cut, w, h, c.ctypes.data)
            tot += c
    assert tot[0] > 10 ** 5, tot
    assert tot[2] == 0, tot                       # every misdecision inside the band
    if noise:
        assert 0 < tot[3] < 1e-2 * tot[0], tot    # a narrow band that samples do meet
    else:  # the soft tissue is a plateau at the cutoff: FP32 drops all of it, and all of it is in the band
        assert tot[1] > 0.5 * tot[0], tot
