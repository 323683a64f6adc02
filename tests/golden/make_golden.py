"""Regenerates tests/golden/reference_small.npz from the reference's own
sources built for the CPU (oracle/build_ref.sh).  Run from the repo root:

    python tests/golden/make_golden.py

The fixture holds the inputs and the reference's outputs for one small
seeded scene (one 40x48x56 u16 phantom, two cameras, 96x96 radiographs):
the VolumeDescription constants, the folded ray-caster matrices and
viewports, DRRs (exact-weight texture emulation), radiograph crops, each
filter on a seeded image, the masks, and NCC / SAD of the masked pair.
tests/test_oracle_golden.py checks the oracle against it on any machine.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from autoscoper_gb300 import scene as S  # noqa: E402
from oracle import oracle as O  # noqa: E402
from oracle import ref as R  # noqa: E402


def small_scene():
    sc = S.make_scene([(40, 48, 56)], 1.0, (96, 96), 1.0, filters="sobel", seed=11)
    # radiograph: 1 - DRR at the ground truth (reference ray caster), u16
    rv = R.RefVolume(sc.volumes[0])
    for vi, v in enumerate(sc.views):
        cam = v.camera
        xc = O.frame_from_xyzypr(sc.truth[0])
        mv = O.frame_mul(O.frame_inverse(cam.frame), xc)
        imv = O.frame_row_matrix(O.frame_inverse(mv))
        rp = sc.ray[vi][0]
        drr = rv.raycast(imv, S.target_viewport(cam), rp.step, rp.intensity, rp.cutoff, cam.width, cam.height)
        v.radiograph = S.radiograph_from_drr(drr.astype(np.float64), seed=vi)
    return sc


def main():
    assert R.available(), "reference sources not present"
    sc = small_scene()
    rv = R.RefVolume(sc.volumes[0])
    out = {"volume": sc.volumes[0].data, "scale": np.array(sc.volumes[0].scale),
           "inv_scale": rv.inv_scale, "inv_trans": rv.inv_trans, "trans_center": rv.trans_center,
           "minmax": np.array([rv.min_value, rv.max_value], np.float32)}
    rng = np.random.default_rng(12)
    poses = [np.asarray(sc.truth[0], np.float64)] + [S.perturb(sc.truth[0], rng, 2.0, 2.0).astype(np.float64)
                                                    for _ in range(2)]
    out["poses"] = np.array(poses)
    tr = O.Tracker(sc)
    for vi, v in enumerate(sc.views):
        out[f"cam{vi}_frame"] = v.camera.frame
        out[f"cam{vi}_K"] = np.array([v.camera.width, v.camera.height, v.camera.cx, v.camera.cy, v.camera.fx,
                                      v.camera.fy])
        out[f"rad{vi}"] = v.radiograph
        rp = sc.ray[vi][0]
        out[f"ray{vi}"] = np.array([rp.step, rp.intensity, rp.cutoff], np.float32)
        for k, pose in enumerate(poses):
            xc = O.frame_from_xyzypr(pose)
            mv = O.frame_mul(O.frame_inverse(v.camera.frame), xc)
            imv = O.frame_row_matrix(O.frame_inverse(mv))
            ok, m, vp, w, h = tr.view_setup(0, vi, pose)
            drr = rv.raycast(imv, vp, rp.step, rp.intensity, rp.cutoff, w, h)
            drr_f = R.sobel(drr, 1.0, 0.0)
            rad = R.rad_render(v.radiograph, v.camera.viewport, vp, w, h)
            rad_f = R.sobel(rad, 1.0, 0.0)
            mask = R.drr_background(drr_f)
            radm = R.multiply(rad_f, mask)
            drrm = R.multiply(drr_f, mask)
            key = f"v{vi}p{k}"
            out[key + "_imv"] = imv
            out[key + "_vp"] = vp
            out[key + "_drr"] = drr
            out[key + "_rad"] = rad
            out[key + "_ncc"] = np.array(R.ncc(drrm, radm, mask))
            out[key + "_hdist"] = np.array(R.hdist(drrm, radm, mask))
    img = rng.uniform(0, 1, size=(37, 41)).astype(np.float32)
    out["filter_in"] = img
    out["sobel"] = R.sobel(img, 0.43, 3.0)
    out["contrast"] = R.contrast(img, 2.5, 0.9)
    out["gaussian"] = R.gaussian(img, 1.5)
    out["sharpen"] = R.sharpen(img, 1.0, 2.0, 0.01)
    np.savez_compressed(os.path.join(ROOT, "tests", "golden", "reference_small.npz"), **out)
    print("wrote tests/golden/reference_small.npz")


if __name__ == "__main__":
    main()
