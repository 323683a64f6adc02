"""FP64 rigid-frame and camera algebra used to describe scenes on the host.

A frame is a float64 array of 12: the rotation stored as three columns
(``f[0:3]`` is the image of the x axis, ``f[3:6]`` of y, ``f[6:9]`` of z)
followed by the translation ``f[9:12]``.  This is the storage order of
Autoscoper's ``xromm::CoordFrame`` (libautoscoper/src/CoordFrame.cpp:356-370),
so frames pass unchanged to the C ABI.  Angles are in degrees, as there.
"""
from __future__ import annotations

import math

import numpy as np


def identity() -> np.ndarray:
    f = np.zeros(12)
    f[0] = f[4] = f[8] = 1.0
    return f


def rotate(f: np.ndarray, axis, angle: float) -> np.ndarray:
    """Right-multiplies f's rotation by a rotation of `angle` degrees about
    `axis` (CoordFrame::rotate, CoordFrame.cpp:262-320)."""
    a = np.asarray(axis, dtype=np.float64).copy()
    c = math.cos(math.pi * angle / 180.0)
    s = math.sin(math.pi * angle / 180.0)
    mag = math.sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2])
    out = f.copy()
    if mag == 0:
        return out
    a /= mag
    oc = 1.0 - c
    x, y, z = a
    R = np.array([oc * x * x + c, oc * x * y + s * z, oc * x * z - s * y,
                  oc * x * y - s * z, oc * y * y + c, oc * y * z + s * x,
                  oc * x * z + s * y, oc * y * z - s * x, oc * z * z + c]).reshape(3, 3)
    M = f[:9].reshape(3, 3)
    out[:9] = (M @ R).reshape(9)
    return out


def from_xyzypr(v) -> np.ndarray:
    """CoordFrame::from_xyzypr (CoordFrame.cpp:100-108): yaw about z, then
    pitch about the new y, then roll about the new x."""
    f = identity()
    f = rotate(f, f[6:9].copy(), v[3])
    f = rotate(f, f[3:6].copy(), v[4])
    f = rotate(f, f[0:3].copy(), v[5])
    f[9:12] += np.asarray(v[:3], dtype=np.float64)
    return f


def from_axis_angle(v) -> np.ndarray:
    """CoordFrame::from_xyzAxis_angle (CoordFrame.cpp:163-175): translation
    v[0:3]; rotation about v[3:6] by |v[3:6]| degrees."""
    f = identity()
    ang = math.sqrt(v[3] * v[3] + v[4] * v[4] + v[5] * v[5])
    if ang != 0:
        f = rotate(f, np.asarray(v[3:6], dtype=np.float64), ang)
    f[9:12] += np.asarray(v[:3], dtype=np.float64)
    return f


def to_xyzypr(f) -> np.ndarray:
    """CoordFrame::to_xyzypr (CoordFrame.cpp:177-189)."""
    return np.array([f[9], f[10], f[11],
                     180.0 * math.atan2(f[1], f[0]) / math.pi,
                     180.0 * math.atan2(-f[2], math.sqrt(f[5] * f[5] + f[8] * f[8])) / math.pi,
                     180.0 * math.atan2(f[5], f[8]) / math.pi])


def mul(a, b) -> np.ndarray:
    """CoordFrame::operator* (CoordFrame.cpp:478-528): a then b (a . b)."""
    A = np.asarray(a[:9]).reshape(3, 3)  # rows = columns of the rotation
    B = np.asarray(b[:9]).reshape(3, 3)
    out = np.empty(12)
    # column c of the product = Rot(a) @ column c of Rot(b)
    out[:9] = (B @ A).reshape(9)
    out[9:12] = A.T @ np.asarray(b[9:12]) + np.asarray(a[9:12])
    return out


def inverse(a) -> np.ndarray:
    """CoordFrame::inverse (CoordFrame.cpp:335-353)."""
    A = np.asarray(a[:9]).reshape(3, 3)
    out = np.empty(12)
    out[:9] = A.T.reshape(9)
    R = A.T  # rotation matrix (columns = A rows)
    out[9:12] = -(R.T @ np.asarray(a[9:12]))
    return out


def point(f, p) -> np.ndarray:
    """CoordFrame::point_to_world_space (CoordFrame.cpp:356-370)."""
    A = np.asarray(f[:9]).reshape(3, 3)
    return A.T @ np.asarray(p, dtype=np.float64) + np.asarray(f[9:12])


def row_matrix(f) -> np.ndarray:
    """CoordFrame::to_matrix_row_order (CoordFrame.cpp:223-241)."""
    return np.array([f[0], f[3], f[6], f[9], f[1], f[4], f[7], f[10],
                     f[2], f[5], f[8], f[11], 0.0, 0.0, 0.0, 1.0])


def translate(f, v) -> np.ndarray:
    out = np.asarray(f, dtype=np.float64).copy()
    out[9:12] += np.asarray(v, dtype=np.float64)
    return out


def look_at_frame(eye, center, up) -> np.ndarray:
    """Camera->world frame of a pinhole at `eye` looking at `center`; the
    camera looks down its -z axis with +y up (the gluLookAt convention of
    Camera::calculateLookAtMatrix, Camera.cpp:497-513)."""
    eye = np.asarray(eye, dtype=np.float64)
    fwd = np.asarray(center, dtype=np.float64) - eye
    fwd /= np.linalg.norm(fwd)
    side = np.cross(fwd, np.asarray(up, dtype=np.float64))
    side /= np.linalg.norm(side)
    upp = np.cross(side, fwd)
    f = np.empty(12)
    f[0:3] = side
    f[3:6] = upp
    f[6:9] = -fwd
    f[9:12] = eye
    return f


def camera_viewport(cx, cy, fx, fy, W, H) -> np.ndarray:
    """Camera::calculateViewport (Camera.cpp:424-438): (centre x, centre y,
    width, height) of the image on the film plane z = -2."""
    if fx == 0 or fy == 0:
        raise ValueError("Invalid camera parameters (fx or fy is zero)")
    return np.array([-(2.0 * cx - W) / fx, -(2.0 * cy - H) / fy, 2.0 * W / fx, 2.0 * H / fy])


def camera_image_plane(cam, cx, cy, z, W, H) -> np.ndarray:
    """Camera::calculateImagePlane (Camera.cpp:440-484): the 4 world-space
    corners (TL, BL, BR, TR) of the image plane, 12 doubles."""
    dist = math.sqrt(cam[9] ** 2 + cam[10] ** 2 + cam[11] ** 2)
    scale = -1.5 * dist / z
    c = point(cam, [scale * (W / 2.0 - cx), scale * (H / 2.0 - cy), scale * z])
    hw, hh = scale * W / 2.0, scale * H / 2.0
    right, up = np.asarray(cam[0:3]), np.asarray(cam[3:6])
    return np.concatenate([c - hw * right + hh * up, c - hw * right - hh * up,
                           c + hw * right - hh * up, c + hw * right + hh * up])
