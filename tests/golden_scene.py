"""Rebuilds the small golden scene from tests/golden/reference_small.npz."""
import os

import numpy as np

from autoscoper_gb300 import scene as S

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_small.npz")


def load():
    z = np.load(GOLDEN)
    vol = S.Volume(z["volume"], tuple(float(s) for s in z["scale"]))
    views = []
    ray = []
    for vi in range(2):
        W, H, cx, cy, fx, fy = z[f"cam{vi}_K"]
        cam = S.Camera(z[f"cam{vi}_frame"], int(W), int(H), cx, cy, fx, fy)
        views.append(S.View(cam, z[f"rad{vi}"], S.config_filters("sobel"), S.config_filters("sobel")))
        st, it, cu = (float(x) for x in z[f"ray{vi}"])
        ray.append([S.RayParams(st, it, cu)])
    poses = z["poses"]
    sc = S.Scene(views, [vol], ray, 96, 96, [S.pivot_matrix(vol)], [poses[0].astype(np.float32)], 0, [poses[0]])
    return sc, z
