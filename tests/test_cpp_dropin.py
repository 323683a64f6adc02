"""The reference's C++ operator interface (include/autoscoper_gb300.hpp):
a trackFrame view written against xromm::gpu classes compiles and links on
the CPU; on the GPU it reproduces the oracle's masked images and cost."""
import os
import subprocess

import numpy as np
import pytest

from autoscoper_gb300 import scene as S
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "dropin_trackframe.cpp")
LIBDIR = os.path.join(ROOT, "autoscoper_gb300")


def compile_dropin(tmp_path):
    from autoscoper_gb300 import build
    build.build()
    exe = str(tmp_path / "dropin_trackframe")
    cmd = ["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"), SRC, "-o", exe, "-L" + LIBDIR,
           "-lautoscoper_gb300", "-Wl,-rpath," + LIBDIR]
    subprocess.run(cmd, check=True, capture_output=True)
    return exe


def test_dropin_compiles_and_links(tmp_path):
    assert os.path.exists(compile_dropin(tmp_path))


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
    assert abs(cost - ref) < 1e-5 * max(1, abs(ref)) + 2e-6
