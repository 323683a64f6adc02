"""Trial files on disk for the tests: a volume TIFF, MayaCam 2.0 camera
files, per-camera videos of TIFF frames and the .cfg that ties them."""
import os

import numpy as np

from autoscoper_gb300 import formats as F
from autoscoper_gb300 import scene as S


def write_mayacam2(path, frame, W, H, cx, cy, fx, fy):
    """The file read_mayacam2 turns into this camera (its conversion run
    backwards)."""
    R = np.asarray(frame[:9]).reshape(3, 3).copy()   # rows = stored columns of CoordFrame
    t = np.asarray(frame[9:12]).copy()
    R[0, :] = -R[0, :]
    R[1, :] = -R[1, :]
    t_wc = -(R @ t)  # R is orthonormal: undo t' = -R^T t (as rows)
    Rf = R.T.copy()
    Rf[:, 0] = -Rf[:, 0]
    Rf[:, 2] = -Rf[:, 2]
    t_wc = np.array([-t_wc[0], t_wc[1], -t_wc[2]])
    K = np.array([[fx, 0, 0], [0, fy, 0], [cx, (H - 1) - cy, 1.0]])
    lines = ["image size", f"{W},{H}", "", "camera matrix"]
    lines += [",".join(repr(float(K[j, i])) for j in range(3)) for i in range(3)]
    lines += ["", "rotation"]
    lines += [",".join(repr(float(Rf[j, i])) for j in range(3)) for i in range(3)]
    lines += ["", "translation"] + [repr(float(x)) for x in t_wc]
    open(path, "w").write("\n".join(lines) + "\n")



def synthetic_trial(tmp_path, frames=None, shape=(24, 28, 32), size=(64, 64), seed=2):
    """A one-volume, two-camera trial; frames: per frame, one image per
    camera (default: two flat frames)."""
    sc = S.make_scene([shape], 1.0, size, 1.6, filters="sobel", seed=seed)
    F.write_tiff(str(tmp_path / "bone.tif"), list(sc.volumes[0].data), "lzw")
    W, H = size
    if frames is None:
        frames = [[np.full((H, W), 30000 + 100 * f, np.uint16) for _ in sc.views] for f in range(2)]
    for i, v in enumerate(sc.views):
        c = v.camera
        write_mayacam2(str(tmp_path / f"cam{i}.txt"), c.frame, c.width, c.height, c.cx, c.cy, c.fx, c.fy)
        os.makedirs(tmp_path / f"video{i}", exist_ok=True)
        for f, imgs in enumerate(frames):
            F.write_tiff(str(tmp_path / f"video{i}" / f"frame_{f:03d}.tif"), [imgs[i]], "packbits")
    cfg = tmp_path / "trial.cfg"
    cfg.write_text("# synthetic trial\nVersion 1.1\nmayaCam_csv cam0.txt\nmayaCam_csv cam1.txt\n"
                   "CameraRootDir video0\nCameraRootDir video1\nVolumeFile bone.tif\nVoxelSize 1 1 1\n"
                   f"VolumeFlip 0 0 0\nRenderResolution {W} {H}\nOptimizationOffsets 0.2 0.2 0.2 0.1 0.1 0.1\n")
    return sc, str(cfg)


def render_targets(sc):
    """Radiographs of the scene's bones at their true poses, rendered by the
    oracle over each whole camera image (u16, with noise)."""
    from oracle import oracle as O
    tr = O.Tracker(sc)
    for vi, v in enumerate(sc.views):
        drr_sum = np.zeros((v.camera.height, v.camera.width))
        for b in range(len(sc.volumes)):
            ok, m, _, _, _ = tr.view_setup(b, vi, sc.truth[b])
            rp = sc.ray[vi][b]
            drr_sum += O.raycast(tr.vd[b], m, S.target_viewport(v.camera), rp.step, rp.intensity, rp.cutoff,
                                 v.camera.width, v.camera.height)
        v.radiograph = S.radiograph_from_drr(drr_sum, seed=vi)
    return [v.radiograph for v in sc.views]
