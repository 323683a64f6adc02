"""Image outputs of a view against the oracle: the merged multi-bone DRR of
View::renderDrr, the three images of Tracker::getImageData, and the
background image of Video::create_background_image."""
import numpy as np
import pytest

from autoscoper_gb300 import api, scene as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scene():
    from test_gpu_engine import make_targets
    sc = S.make_scene([(40, 48, 56), (36, 30, 44)], 1.0, (96, 96), 1.05, filters="sobel", seed=9,
                      bone_offsets=[(0, 0, -12), (4, -3, 14)])
    tr = O.Tracker(sc)
    make_targets(sc, tr)
    return sc, tr


def _full_vp(cam):
    return np.array([-cam.viewport[2] / 2, -cam.viewport[3] / 2, cam.viewport[2], cam.viewport[3]])


def _oracle_drr(sc, tr, vi, b, pose, vp, w, h):
    v = sc.views[vi]
    xc = O.frame_from_xyzypr(pose)
    mv = O.frame_mul(O.frame_inverse(v.camera.frame), xc)
    m = O.fold_inv_model_view(O.frame_row_matrix(O.frame_inverse(mv)), tr.vd[b].inv_scale, tr.vd[b].inv_trans)
    m = m.astype(np.float32).astype(np.float64)
    rp = sc.ray[vi][b]
    return O.raycast(tr.vd[b], m, np.float32(vp).astype(np.float64), float(np.float32(rp.step)),
                     float(np.float32(rp.intensity)), float(np.float32(rp.cutoff)), w, h)


def test_render_drr_merges_bones_then_filters(scene):
    sc, tr = scene
    eng = api.Engine(sc, max_items=8)
    poses = np.array([np.asarray(p, np.float32).astype(np.float64) for p in sc.poses])
    for vi, v in enumerate(sc.views):
        got = eng.render_drr(vi, poses)
        h, w = got.shape
        vp = _full_vp(v.camera)
        merged = np.zeros((h, w))
        for b in range(len(sc.volumes)):
            merged = O.merge(merged, _oracle_drr(sc, tr, vi, b, poses[b], vp, w, h))
        want = O.filter_chain(v.drr_filters, merged)
        assert np.abs(got - want).max() < 1e-5


def test_image_data_matches_oracle_chain(scene):
    sc, tr = scene
    eng = api.Engine(sc, max_items=8)
    pose = np.asarray(sc.poses[1], np.float32).astype(np.float64)
    vi = 0
    v = sc.views[vi]
    rad, drr, mask = eng.image_data(vi, 1, pose)
    h, w = drr.shape
    vp = np.float32(_full_vp(v.camera)).astype(np.float64)
    d = O.filter_chain(v.drr_filters, _oracle_drr(sc, tr, vi, 1, pose, _full_vp(v.camera), w, h))
    ipf = np.asarray(v.camera.viewport, np.float32).astype(np.float64)
    r = O.filter_chain(v.rad_filters, O.image_render(v.radiograph, ipf, vp, w, h, mode=0))
    m = O.drr_background(d)
    assert np.abs(mask - m).max() == 0.0
    assert np.abs(drr - O.multiply(d, m)).max() < 1e-5
    assert np.abs(rad - O.multiply(r, m)).max() < 1e-5
    assert api.to_u8(drr).dtype == np.uint8


def test_background_from_frames_is_the_pixelwise_max():
    rng = np.random.default_rng(2)
    frames = [rng.integers(0, 65536, (40, 52)).astype(np.uint16) for _ in range(4)]
    got = api.background_from_frames(frames)
    want = np.max(np.stack(frames).astype(np.float32) / np.float32(65535.0), axis=0)
    assert np.array_equal(got, want)
