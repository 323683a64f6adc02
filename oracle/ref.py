"""ctypes access to the reference's own sources built for the CPU
(oracle/build_ref.sh -> oracle/_ref/libascref.so) -- TEST INFRASTRUCTURE.

Used only to pin the oracle (tests/test_oracle_pin.py) and to regenerate the
committed fixtures (tests/golden/make_golden.py).  The library exists only
where the reference sources are present; callers skip when `available()` is
False.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SO = os.path.join(HERE, "_ref", "libascref.so")
# Where the reference checkout lies on the machine that builds the pin: the
# ASC_REFERENCE_ROOT environment variable, else the build container's copy.
REFERENCE_ROOT = os.environ.get("ASC_REFERENCE_ROOT", "/root/reference")
_LIB = None

_d = C.POINTER(C.c_double)
_f = C.POINTER(C.c_float)
_i = C.POINTER(C.c_int)
COST_FN = C.CFUNCTYPE(C.c_double, _d, C.c_void_p)


def build() -> bool:
    """Builds libascref.so when the reference sources are present (again
    when the harness or its recipe changed)."""
    deps = [os.path.join(HERE, "build_ref.sh")] + [os.path.join(HERE, "ref_shim", f)
                                                   for f in os.listdir(os.path.join(HERE, "ref_shim"))]
    fresh = os.path.exists(SO) and all(os.path.getmtime(d) <= os.path.getmtime(SO) for d in deps)
    if fresh:
        return True
    if not os.path.isdir(os.path.join(REFERENCE_ROOT, "libautoscoper")):
        return os.path.exists(SO)
    subprocess.run([os.path.join(HERE, "build_ref.sh"), REFERENCE_ROOT], check=True,
                   stdout=subprocess.DEVNULL)
    return os.path.exists(SO)


def available() -> bool:
    try:
        return build()
    except Exception:
        return False


def lib():
    global _LIB
    if _LIB is None:
        if not build():
            raise RuntimeError("reference CPU build unavailable")
        L = C.CDLL(SO)
        L.ref_volume_create.restype = C.c_void_p
        L.ref_volume_create.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, _d, _i]
        L.ref_volume_info.argtypes = [C.c_void_p, _i, _f, _f, _d, _f, C.c_void_p]
        L.ref_volume_destroy.argtypes = [C.c_void_p]
        L.ref_raycast.argtypes = [C.c_void_p, _d, _f, C.c_float, C.c_float, C.c_float, _f, C.c_int, C.c_int]
        L.ref_rad_render.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, _f, _f, _f, C.c_int, C.c_int]
        L.ref_background_render.argtypes = [_f, C.c_int, C.c_int, _f, _f, C.c_float, _f, C.c_int, C.c_int]
        L.ref_drr_background.argtypes = [_f, _f, C.c_int, C.c_int]
        for n in ("ref_multiply", "ref_merge"):
            getattr(L, n).argtypes = [_f, _f, _f, C.c_int, C.c_int]
        L.ref_composite.argtypes = [_f, _f, _f, _f, _f, C.c_int, C.c_int]
        L.ref_fill.argtypes = [_f, C.c_uint, C.c_float]
        L.ref_sobel.argtypes = [_f, _f, C.c_int, C.c_int, C.c_float, C.c_float]
        L.ref_contrast.argtypes = [_f, _f, C.c_int, C.c_int, C.c_float, C.c_float]
        L.ref_gaussian.argtypes = [_f, _f, C.c_int, C.c_int, C.c_float]
        L.ref_sharpen.argtypes = [_f, _f, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float]
        for n in ("ref_ncc", "ref_hdist"):
            getattr(L, n).argtypes = [_f, _f, _f, C.c_uint]
            getattr(L, n).restype = C.c_float
        for n in ("ref_frame_from_xyzypr", "ref_frame_from_axis_angle", "ref_frame_to_xyzypr", "ref_frame_inverse",
                  "ref_frame_row_matrix"):
            getattr(L, n).argtypes = [_d, _d]
        for n in ("ref_frame_mul", "ref_frame_linear_extrap"):
            getattr(L, n).argtypes = [_d, _d, _d]
        L.ref_pose_curve_run.argtypes = [C.c_int, _i, _i, _i, _d, C.c_int, _i, _d]
        L.ref_pso.argtypes = [COST_FN, C.c_void_p, C.c_float, C.c_float, C.c_uint, C.c_uint, C.c_uint, _f, _f]
        L.ref_amoeba.argtypes = [COST_FN, C.c_void_p, _d, _d, C.c_int, C.c_double]
        L.ref_amoeba.restype = C.c_int
        L.ref_set_tex_weight_bits.argtypes = [C.c_int]
        _LIB = L
    return _LIB


def _fp(a):
    return a.ctypes.data_as(_f)


def _dp(a):
    return a.ctypes.data_as(_d)


def f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def frame_op(name, *args, n_out=12):
    out = np.zeros(n_out)
    getattr(lib(), name)(*[_dp(f64(a)) for a in args], _dp(out))
    return out


def pose_curve_run(ops, eval_frames):
    """The reference's KeyCurve<float> x, y, z and KeyCurve<Quatf> driven by
    ops [(kind, frame, mask, pose)], read at eval_frames: (len, 6) poses."""
    n = len(ops)
    kinds = np.array([o[0] for o in ops], np.int32)
    frames = np.array([o[1] for o in ops], np.int32)
    masks = np.array([o[2] for o in ops], np.int32)
    poses = f64(np.array([o[3] for o in ops]).reshape(n, 6))
    ev = np.array(eval_frames, np.int32)
    out = np.zeros((len(ev), 6))
    lib().ref_pose_curve_run(n, kinds.ctypes.data_as(_i), frames.ctypes.data_as(_i), masks.ctypes.data_as(_i),
                             _dp(poses), len(ev), ev.ctypes.data_as(_i), _dp(out))
    return out


class RefVolume:
    def __init__(self, vol):
        data = np.ascontiguousarray(vol.data)
        D, H, W = data.shape
        self.h = lib().ref_volume_create(data.ctypes.data, W, H, D, 8 * data.dtype.itemsize, _dp(f64(vol.scale)),
                                         np.ascontiguousarray(vol.flip, dtype=np.int32).ctypes.data_as(_i))
        dims = np.zeros(3, np.int32)
        self.inv_scale = np.zeros(3, np.float32)
        self.inv_trans = np.zeros(3, np.float32)
        self.trans_center = np.zeros(3)
        mm = np.zeros(2, np.float32)
        out = np.empty_like(data).reshape(-1)
        lib().ref_volume_info(self.h, dims.ctypes.data_as(_i), _fp(self.inv_scale), _fp(self.inv_trans),
                              _dp(self.trans_center), _fp(mm), out.ctypes.data)
        self.dims = tuple(int(d) for d in dims)
        self.data = out[:int(dims.prod())].reshape(self.dims[2], self.dims[1], self.dims[0]).copy()
        self.min_value, self.max_value = float(mm[0]), float(mm[1])

    def __del__(self):
        try:
            lib().ref_volume_destroy(self.h)
        except Exception:
            pass

    def raycast(self, imv16, vp, step, intensity, cutoff, w, h):
        out = np.zeros(w * h, np.float32)
        lib().ref_raycast(self.h, _dp(f64(imv16)), _fp(f32(vp)), step, intensity, cutoff, _fp(out), w, h)
        return out.reshape(h, w)


def rad_render(img, ip, vp, w, h):
    img = np.ascontiguousarray(img)
    out = np.zeros(w * h, np.float32)
    lib().ref_rad_render(img.ctypes.data, img.shape[1], img.shape[0], 8 * img.dtype.itemsize, _fp(f32(ip)),
                         _fp(f32(vp)), _fp(out), w, h)
    return out.reshape(h, w)


def background_render(img, ip, vp, threshold, w, h):
    img = f32(img)
    out = np.zeros(w * h, np.float32)
    lib().ref_background_render(_fp(img), img.shape[1], img.shape[0], _fp(f32(ip)), _fp(f32(vp)), threshold,
                                _fp(out), w, h)
    return out.reshape(h, w)


def _img_op(name, *imgs, extra=()):
    imgs = [f32(a) for a in imgs]
    h, w = imgs[0].shape
    out = np.zeros((h, w), np.float32)
    getattr(lib(), name)(*[_fp(a) for a in imgs], _fp(out), w, h, *extra)
    return out


def drr_background(a):
    return _img_op("ref_drr_background", a)


def multiply(a, b):
    return _img_op("ref_multiply", a, b)


def merge(a, b):
    return _img_op("ref_merge", a, b)


def composite(a, b, c):
    a, b, c = f32(a), f32(b), f32(c)
    h, w = a.shape
    out = np.zeros(3 * w * h, np.float32)
    lib().ref_composite(_fp(a), _fp(b), _fp(c), _fp(c), _fp(out), w, h)
    return out


def fill(n, val):
    out = np.full(n, -7.0, np.float32)
    lib().ref_fill(_fp(out), n, val)
    return out


def sobel(img, scale, blend):
    return _img_op("ref_sobel", img, extra=(scale, blend))


def contrast(img, alpha, beta):
    return _img_op("ref_contrast", img, extra=(alpha, beta))


def gaussian(img, radius):
    return _img_op("ref_gaussian", img, extra=(radius,))


def sharpen(img, radius, contrast_, threshold):
    return _img_op("ref_sharpen", img, extra=(radius, contrast_, threshold))


def ncc(f, g, m):
    f, g, m = f32(f).reshape(-1), f32(g).reshape(-1), f32(m).reshape(-1)
    return float(lib().ref_ncc(_fp(f), _fp(g), _fp(m), f.size))


def hdist(f, g, m):
    f, g, m = f32(f).reshape(-1), f32(g).reshape(-1), f32(m).reshape(-1)
    return float(lib().ref_hdist(_fp(f), _fp(g), _fp(m), f.size))


def pso(cost, lo, hi, epochs, stall, seed):
    cb = COST_FN(lambda p, ctx: float(cost([p[i] for i in range(6)])))
    pos = np.zeros(6, np.float32)
    val = np.zeros(1, np.float32)
    lib().ref_pso(cb, None, lo, hi, epochs, stall, seed, _fp(pos), _fp(val))
    return pos, float(val[0])


def amoeba(cost, P, Y, ftol):
    P = f64(P).copy()
    Y = f64(Y).copy()
    ndim = P.shape[1]
    cb = COST_FN(lambda p, ctx: float(cost(np.array([p[i] for i in range(ndim)]))))
    it = lib().ref_amoeba(cb, None, _dp(P), _dp(Y), ndim, ftol)
    return P, Y, it
