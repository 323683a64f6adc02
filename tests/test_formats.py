"""Autoscoper's input files on the host: TIFF pages (uncompressed, PackBits,
LZW, horizontal predictor, both byte orders, multi-page volumes), MayaCam
1.0 / 2.0 and VTK camera calibrations, .vie view settings and .cfg trials,
down to a Scene that the oracle scores.  The reference's sample files are
read too where its tree is present."""
import json
import os

import numpy as np
import pytest

from autoscoper_gb300 import formats as F, geometry as G, scene as S
import trial_files
from oracle.ref import REFERENCE_ROOT

SAMPLE = os.path.join(REFERENCE_ROOT, "sample_data")


@pytest.mark.parametrize("compression", ["none", "packbits", "lzw"])
@pytest.mark.parametrize("dtype", [np.uint8, np.uint16])
@pytest.mark.parametrize("byteorder", ["<", ">"])
def test_tiff_round_trip(tmp_path, compression, dtype, byteorder):
    rng = np.random.default_rng(3)
    hi = np.iinfo(dtype).max
    pages = [rng.integers(0, hi, (37, 53), endpoint=True).astype(dtype),
             np.full((37, 53), 7, dtype),                                   # long runs
             (np.arange(37 * 53) % 251).astype(dtype).reshape(37, 53)]      # repeats for LZW
    p = str(tmp_path / "v.tif")
    F.write_tiff(p, pages, compression, rows_per_strip=8, byteorder=byteorder)
    got = F.read_tiff(p)
    assert len(got) == 3
    for a, b in zip(got, pages):
        assert (a.width, a.height, a.bits) == (53, 37, 8 * np.dtype(dtype).itemsize)
        assert a.data.dtype == dtype and np.array_equal(a.data, b)


def test_tiff_lzw_long_stream_and_predictor(tmp_path):
    rng = np.random.default_rng(5)
    img = rng.integers(0, 65535, (300, 400)).astype(np.uint16)  # > 4096 codes: width growth and table resets
    p = str(tmp_path / "big.tif")
    F.write_tiff(p, [img], "lzw", rows_per_strip=300, predictor=True)
    assert np.array_equal(F.read_tiff(p)[0].data, img)


def test_volume_from_pages_and_pivot(tmp_path):
    rng = np.random.default_rng(1)
    vol = np.zeros((6, 9, 11), np.uint16)
    vol[1:5, 2:8, 3:10] = rng.integers(1, 4000, (4, 6, 7))
    p = str(tmp_path / "bone.tif")
    F.write_tiff(p, list(vol), "packbits")
    v = F.read_volume(p, (0.4, 0.5, 0.6), (1, 0, 0))
    assert np.array_equal(v.data, vol) and v.scale == (0.4, 0.5, 0.6) and v.flip == (1, 0, 0)
    # transCenter of the non-zero box after the x flip (x 3..9 -> 1..7)
    pv = S.pivot_matrix(v)
    want = [-np.float32(0.4) * 0.5 * (1 + 7), -np.float32(0.5) * 0.5 * (2 + 7), np.float32(0.6) * 0.5 * (1 + 4)]
    assert np.allclose(pv[9:12], want)


def test_mayacam2_round_trip_and_vtk(tmp_path):
    frame = G.look_at_frame((420.0, -80.0, 35.0), (0.0, 5.0, -3.0), (0.0, 0.0, 1.0))
    p = str(tmp_path / "cam.txt")
    trial_files.write_mayacam2(p, frame, 1024, 960, 515.5, 470.25, 4000.0, 4010.0)
    cam = F.read_camera(p)
    assert np.allclose(cam.frame, frame, atol=1e-12)
    assert (cam.width, cam.height, cam.cx, cam.cy, cam.fx, cam.fy) == (1024, 960, 515.5, 470.25, 4000.0, 4010.0)
    assert np.allclose(cam.viewport, G.camera_viewport(515.5, 470.25, 4000.0, 4010.0, 1024, 960))
    assert np.allclose(cam.image_plane, G.camera_image_plane(frame, 515.5, 470.25, -4005.0, 1024, 960))
    vj = str(tmp_path / "cam.json")
    json.dump({"@schema": F.VTK_CAMERA_SCHEMA, "version": 1.0, "image-width": 800, "image-height": 600,
               "camera-position": [420.0, -80.0, 35.0], "focal-point": [0.0, 5.0, -3.0], "view-up": [0, 0, 1],
               "view-angle": 30.0}, open(vj, "w"))
    vc = F.read_camera(vj)
    assert np.allclose(vc.frame, frame) and (vc.cx, vc.cy) == (400.0, 300.0)
    assert np.isclose(vc.fx, 800 / (2 * np.tan(np.radians(15.0))))


def test_mayacam1(tmp_path):
    p = str(tmp_path / "cam1.csv")
    open(p, "w").write("100,-20,30\n10,20,30\n0,0,0\n513,500,-3000\n0.1,0,0\n")
    cam = F.read_camera(p)
    assert np.allclose(cam.frame, G.from_xyzypr([100, -20, 30, 30, 20, 10]))
    assert (cam.width, cam.height, cam.cx, cam.cy, cam.fx) == (1024, 1024, 512.0, 499.0, 3000.0)
    assert cam.plane_z == -3000.0


def test_vie_settings(tmp_path):
    p = str(tmp_path / "v.vie")
    open(p, "w").write("RadFilters_begin\nSobelFilter_begin\nScale 0.43\nBlend 3\nSobelFilter_end\n"
                       "ContrastFilter_begin\nAlpha 2.5\nBeta 0.9\nContrastFilter_end\nRadFilters_end\n"
                       "DrrRenderer_begin\nSampleDistance 0.62\nRayIntensity 0.35\nCutoff 0\nDrrRenderer_end\n"
                       "DrrFilters_begin\nGaussianFilter_begin\nRadius 1.5\nGaussianFilter_end\n"
                       "SharpenFilter_begin\nRadius 2\nContrast 1.2\nSharpenFilter_end\nDrrFilters_end\n")
    vs = F.read_vie(p)
    assert [(f.kind, f.scale, f.blend) for f in vs.rad_filters[:1]] == [(S.SOBEL, 0.43, 3.0)]
    assert (vs.rad_filters[1].kind, vs.rad_filters[1].alpha, vs.rad_filters[1].beta) == (S.CONTRAST, 2.5, 0.9)
    assert (vs.ray.step, vs.ray.intensity, vs.ray.cutoff) == (0.62, 0.35, 0.0)
    assert [f.kind for f in vs.drr_filters] == [S.GAUSSIAN, S.SHARPEN]
    assert vs.drr_filters[1].radius == 2.0 and vs.drr_filters[1].contrast == 1.2


def test_cfg_and_trial_to_scene(tmp_path):
    from oracle import oracle as O
    sc, cfg = trial_files.synthetic_trial(tmp_path)
    t = F.read_cfg(cfg)
    assert t.version == (1, 1) and (t.render_width, t.render_height) == (64, 64)
    assert t.offsets == (0.2, 0.2, 0.2, 0.1, 0.1, 0.1) and t.flips == [(0, 0, 0)]
    loaded = F.load_trial(cfg, frame=1)
    assert np.array_equal(loaded.volumes[0].data, sc.volumes[0].data)
    for a, b in zip(loaded.views, sc.views):
        assert np.allclose(a.camera.viewport, b.camera.viewport)
        assert np.allclose(a.camera.image_plane, b.camera.image_plane)
        assert int(a.radiograph[0, 0]) == 30100
    loaded.poses = [np.asarray(sc.truth[0], np.float32)]
    cost = O.Tracker(loaded).minimization_func(0, np.zeros(6))
    assert np.isfinite(cost)
    with pytest.raises(ValueError):
        (tmp_path / "bad.cfg").write_text("VolumeFile bone.tif\n")
        F.read_cfg(str(tmp_path / "bad.cfg"))


@pytest.mark.skipif(not os.path.isdir(SAMPLE), reason="the reference's sample data is not on this machine")
def test_reference_sample_files():
    vol = F.read_volume(os.path.join(SAMPLE, "Models", "rad_dcm_cropped.tif"))
    assert vol.data.dtype == np.uint16 and vol.data.ndim == 3 and vol.data.max() > 0
    frames = F.video_frames(os.path.join(SAMPLE, "XMA_UND", "xr_data_wrist_cam01"))
    img = F.read_frame(frames[0])
    assert img.ndim == 2 and img.std() > 0
    cam = F.read_camera(os.path.join(SAMPLE, "Calibration", "xr_calib_wrist_cam01.txt"))
    R = np.asarray(cam.frame[:9]).reshape(3, 3)
    assert np.allclose(R @ R.T, np.eye(3), atol=1e-6)
    vs = F.read_vie(os.path.join(SAMPLE, "xParameters", "control_settings.vie"))
    assert (vs.ray.step, vs.ray.intensity) == (0.62, 0.35)
    assert [f.kind for f in vs.rad_filters] == [S.SOBEL, S.CONTRAST]


@pytest.mark.gpu
def test_trial_from_files_on_the_engine(tmp_path):
    """A trial read from its files scores on the engine as on the oracle."""
    from autoscoper_gb300 import api
    from oracle import oracle as O
    sc, cfg = trial_files.synthetic_trial(tmp_path)
    loaded = F.load_trial(cfg, frame=0)
    loaded.poses = [np.asarray(sc.truth[0], np.float32)]
    tr = O.Tracker(loaded)
    eng = api.Engine(loaded, max_items=8)
    man = np.array([[0, 0, 0, 0, 0, 0], [0.5, -0.3, 0.2, 1.0, 0.5, -0.5]], np.float64)
    cost, vcost = eng.eval(np.zeros(2, np.int32), man)
    for k in range(2):
        want = tr.track_frame(0, tr.compose(0, man[k]))
        for got, c in zip(vcost[k], want):  # the NCC bar per view
            assert abs(got - c) <= 1e-5 * max(abs(1.0 - c), 1e-2), (got, c)
