"""The reference's C++ operator interface (include/autoscoper_gb300.hpp):
a trackFrame view written against xromm::gpu classes -- the operators
directly (dropin_trackframe.cpp) and through xromm::gpu::View
(dropin_view.cpp) -- compiles and links on the CPU; on the GPU it reproduces
the oracle's masked images and cost."""
import os
import subprocess

import numpy as np
import pytest

from autoscoper_gb300 import scene as S
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "dropin_trackframe.cpp")
SRC_VIEW = os.path.join(ROOT, "tests", "cpp", "dropin_view.cpp")
LIBDIR = os.path.join(ROOT, "autoscoper_gb300")


def compile_dropin(tmp_path, src=SRC):
    from autoscoper_gb300 import build
    build.build()
    exe = str(tmp_path / os.path.splitext(os.path.basename(src))[0])
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-I" + os.path.join(ROOT, "include"), src, "-o", exe,
           "-L" + LIBDIR, "-lautoscoper_gb300", "-Wl,-rpath," + LIBDIR]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.mark.parametrize("src", [SRC, SRC_VIEW])
def test_dropin_compiles_and_links(tmp_path, src):
    assert os.path.exists(compile_dropin(tmp_path, src))


def _fmt(x):
    if isinstance(x, str):
        return x
    if isinstance(x, (int, np.integer)):
        return str(int(x))
    return repr(float(x))


def _filters_spec(filters):
    out = [len(filters)]
    for f in filters:
        p = {S.SOBEL: (f.scale, f.blend, 0.0), S.CONTRAST: (f.alpha, f.beta, 0.0), S.GAUSSIAN: (f.radius, 0.0, 0.0),
             S.SHARPEN: (f.radius, f.contrast, f.threshold)}[f.kind]
        out += [f.kind, int(f.enabled), *p]
    return out


@pytest.mark.gpu
def test_dropin_view_matches_oracle(tmp_path):
    """Tracker::trackFrame's per-view sequence through View (renderDrrSingle,
    renderRad, renderBackground with a threshold, renderDRRMask, the
    multiplies, ncc) with the four-filter chain on both lists and a disabled
    filter that View::filter copies through, against the oracle's
    render_view / track_frame: images within FP32 rounding, the cost within
    the NCC bar."""
    exe = compile_dropin(tmp_path, SRC_VIEW)
    sc = S.make_scene([(40, 48, 56)], 1.0, (96, 96), 1.0, filters="chain", seed=12)
    tr = O.Tracker(sc)
    v = sc.views[0]
    ok, m, _, _, _ = tr.view_setup(0, 0, sc.truth[0])
    rp = sc.ray[0][0]
    drr = O.raycast(tr.vd[0], m, S.target_viewport(v.camera), rp.step, rp.intensity, rp.cutoff, 96, 96)
    v.radiograph = S.radiograph_from_drr(drr, seed=1)
    v.rad_filters.insert(2, S.Filter(S.GAUSSIAN, radius=2.0, enabled=False))
    yy, xx = np.mgrid[0:96, 0:96]
    v.background = (0.5 + 0.5 * np.sin(xx / 9.0) * np.cos(yy / 13.0)).astype(np.float32)
    v.bg_threshold = 0.3
    pose = np.asarray(sc.truth[0]) + np.array([0.5, -0.4, 0.3, 1.0, 0.5, -0.5])
    ok, m, vp, w, h = tr.view_setup(0, 0, pose)
    xc = O.frame_from_xyzypr(pose)
    mv = O.frame_mul(O.frame_inverse(v.camera.frame), xc)
    imv = O.frame_row_matrix(O.frame_inverse(mv))
    vol = sc.volumes[0]
    vol.data.tofile(tmp_path / "vol.raw")
    v.radiograph.tofile(tmp_path / "rad.raw")
    v.background.tofile(tmp_path / "bg.raw")
    D, H, W = vol.data.shape
    spec = [W, H, D, 16, *vol.scale, str(tmp_path / "vol.raw"), *imv, *np.float32(vp), rp.step, rp.intensity,
            rp.cutoff, 96, 96, 16, str(tmp_path / "rad.raw"), *np.float32(v.camera.viewport), w, h, 96, 96,
            str(tmp_path / "bg.raw"), v.bg_threshold, *_filters_spec(v.drr_filters), *_filters_spec(v.rad_filters)]
    (tmp_path / "spec.txt").write_text(" ".join(_fmt(x) for x in spec))
    subprocess.run([exe, str(tmp_path / "spec.txt"), str(tmp_path / "out.bin")], check=True)
    raw = np.fromfile(tmp_path / "out.bin", np.uint8)
    n = w * h
    a, b, mk = (raw[4 * n * i:4 * n * (i + 1)].view(np.float32).reshape(h, w) for i in range(3))
    cost = raw[12 * n:].view(np.float64)[0]
    r = tr.render_view(0, 0, pose)
    assert 0 < mk.sum() < r["mask"].size, "the background threshold must cut the mask"
    assert np.mean(mk != r["mask"]) < 1e-3  # a pixel within FP32 rounding of a mask edge may flip
    assert np.abs(a - r["drr"]).max() < 1e-5
    assert np.abs(b - r["rad"]).max() < 1e-5
    ref = tr.track_frame(0, pose)[0]
    assert abs(cost - ref) <= 1e-5 * max(abs(1.0 - ref), 1e-2)  # the NCC bar


@pytest.mark.gpu
def test_dropin_matches_oracle(tmp_path):
    exe = compile_dropin(tmp_path)
    sc = S.make_scene([(40, 48, 56)], 1.0, (96, 96), 1.0, filters="sobel", seed=8)
    tr = O.Tracker(sc)
    v = sc.views[0]
    ok, m, _, _, _ = tr.view_setup(0, 0, sc.truth[0])
    rp = sc.ray[0][0]
    drr = O.raycast(tr.vd[0], m, S.target_viewport(v.camera), rp.step, rp.intensity, rp.cutoff, 96, 96)
    v.radiograph = S.radiograph_from_drr(drr, seed=1)
    pose = np.asarray(sc.truth[0]) + np.array([0.5, -0.4, 0.3, 1.0, 0.5, -0.5])
    ok, m, vp, w, h = tr.view_setup(0, 0, pose)
    xc = O.frame_from_xyzypr(pose)
    mv = O.frame_mul(O.frame_inverse(v.camera.frame), xc)
    imv = O.frame_row_matrix(O.frame_inverse(mv))
    vol = sc.volumes[0]
    vol.data.tofile(tmp_path / "vol.raw")
    v.radiograph.tofile(tmp_path / "rad.raw")
    D, H, W = vol.data.shape
    spec = [W, H, D, 16, *vol.scale, str(tmp_path / "vol.raw"), *imv, *np.float32(vp), rp.step, rp.intensity,
            rp.cutoff, 96, 96, 16, str(tmp_path / "rad.raw"), *np.float32(v.camera.viewport), w, h, 1.0, 0.0]
    def fmt(x):
        if isinstance(x, str):
            return x
        if isinstance(x, (int, np.integer)):
            return str(int(x))
        return repr(float(x))

    (tmp_path / "spec.txt").write_text(" ".join(fmt(x) for x in spec))
    subprocess.run([exe, str(tmp_path / "spec.txt"), str(tmp_path / "out.bin")], check=True)
    raw = np.fromfile(tmp_path / "out.bin", np.uint8)
    n = w * h
    a = raw[:4 * n].view(np.float32).reshape(h, w)
    b = raw[4 * n:8 * n].view(np.float32).reshape(h, w)
    cost = raw[8 * n:].view(np.float64)[0]
    r = tr.render_view(0, 0, pose)
    assert np.mean(np.abs(a - r["drr"]) > 1e-4) < 2e-3
    assert np.mean(np.abs(b - r["rad"]) > 1e-4) < 2e-3
    ref = tr.track_frame(0, pose)[0]
    assert abs(cost - ref) <= 1e-5 * max(abs(1.0 - ref), 1e-2)  # the NCC bar
