"""FP64 CPU oracle for the registration cost path -- TEST INFRASTRUCTURE.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's cpu_baseline leg may
import this module; the product (autoscoper_gb300) never does.  The per-pixel
math lives in oracle.c (liboracle.so, built by ``make -C oracle``); this file
restates the per-view orchestration of the reference in Python:

* ``track_frame``       -- Tracker::trackFrame        (Tracker.cpp:583-773)
* ``minimization_func`` -- Tracker::minimizationFunc  (Tracker.cpp:775-827)
* ``filter_chain``      -- View::filter               (View.cpp:475-555)
* ``pso_reference``     -- pso()                      (PSO.cpp:198-295)
* ``amoeba``            -- AMOEBA                     (DownhillSimplex.cpp:39-172)

Parity pin: tests/test_oracle_pin.py checks this oracle against the
reference's own sources built for the CPU (oracle/_ref) and against the
committed fixtures in tests/golden/.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

_d = C.POINTER(C.c_double)
_f = C.POINTER(C.c_float)
_i = C.POINTER(C.c_int)


def build() -> str:
    """Compiles liboracle.so with gcc (make) if it is missing or stale."""
    so = os.path.join(HERE, "liboracle.so")
    src = os.path.join(HERE, "oracle.c")
    if not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    return so


def lib():
    global _LIB
    if _LIB is None:
        _LIB = C.CDLL(build())
        L = _LIB
        L.orc_raycast.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, _d, _d, C.c_double, C.c_double,
                                  C.c_double, _d, C.c_int, C.c_int, C.POINTER(C.c_int32)]
        L.orc_image_render.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, _d, _d, C.c_int, C.c_double, _d,
                                       C.c_int, C.c_int]
        for n in ("orc_drr_background",):
            getattr(L, n).argtypes = [_d, _d, C.c_size_t]
        for n in ("orc_multiply", "orc_merge"):
            getattr(L, n).argtypes = [_d, _d, _d, C.c_size_t]
        L.orc_composite.argtypes = [_d, _d, _d, _d, C.c_size_t]
        L.orc_sobel.argtypes = [_d, _d, C.c_int, C.c_int, C.c_double, C.c_double]
        L.orc_contrast.argtypes = [_d, _d, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int]
        L.orc_gauss_weights.argtypes = [C.c_double, _d, C.c_int]
        L.orc_gauss_weights.restype = C.c_int
        L.orc_gaussian.argtypes = [_d, _d, C.c_int, C.c_int, _d, C.c_int]
        L.orc_sharpen.argtypes = [_d, _d, C.c_int, C.c_int, _d, C.c_int, C.c_double, C.c_double]
        for n in ("orc_ncc", "orc_hdist"):
            getattr(L, n).argtypes = [_d, _d, _d, C.c_size_t, C.c_int]
            getattr(L, n).restype = C.c_double
        L.orc_tree_keep.argtypes = [C.c_size_t, C.c_size_t]
        L.orc_tree_keep.restype = C.c_int
        L.orc_calculate_viewport.argtypes = [_d, _d, _d, _f, _f, _d]
        L.orc_calculate_viewport.restype = C.c_int
        L.orc_fold_inv_model_view.argtypes = [_d, _f, _f, _d]
        L.orc_volume_describe.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, _d, _i, C.c_void_p, _i,
                                          _f, _f, _d, _f, _f]
        L.orc_volume_describe.restype = C.c_int
        for n in ("orc_frame_from_xyzypr", "orc_frame_from_axis_angle", "orc_frame_to_xyzypr", "orc_frame_inverse",
                  "orc_frame_row_matrix"):
            getattr(L, n).argtypes = [_d, _d]
        for n in ("orc_frame_mul", "orc_frame_linear_extrap"):
            getattr(L, n).argtypes = [_d, _d, _d]
        L.orc_camera_viewport.argtypes = [C.c_double] * 6 + [_d]
        L.orc_quat_from_ypr.argtypes = [C.c_float, C.c_float, C.c_float, _f]
        L.orc_quat_to_ypr.argtypes = [_f, _d]
        L.orc_curve_eval.argtypes = [C.c_int, _i, _f, C.c_int]
        L.orc_curve_eval.restype = C.c_float
        L.orc_quat_curve_eval.argtypes = [C.c_int, _i, _f, C.c_int, _f]
        L.orc_camera_image_plane.argtypes = [_d] + [C.c_double] * 5 + [_d]
    return _LIB


def _dp(a):
    return a.ctypes.data_as(_d)


def _arr(x, n=None):
    a = np.ascontiguousarray(x, dtype=np.float64)
    return a


# ---------------------------------------------------------------- geometry

def frame_from_xyzypr(v):
    out = np.zeros(12)
    lib().orc_frame_from_xyzypr(_dp(_arr(v)), _dp(out))
    return out


def frame_from_axis_angle(v):
    out = np.zeros(12)
    lib().orc_frame_from_axis_angle(_dp(_arr(v)), _dp(out))
    return out


def frame_to_xyzypr(f):
    out = np.zeros(6)
    lib().orc_frame_to_xyzypr(_dp(_arr(f)), _dp(out))
    return out


def frame_mul(a, b):
    out = np.zeros(12)
    lib().orc_frame_mul(_dp(_arr(a)), _dp(_arr(b)), _dp(out))
    return out


def frame_inverse(a):
    out = np.zeros(12)
    lib().orc_frame_inverse(_dp(_arr(a)), _dp(out))
    return out


def frame_row_matrix(a):
    out = np.zeros(16)
    lib().orc_frame_row_matrix(_dp(_arr(a)), _dp(out))
    return out


def frame_linear_extrap(a, b):
    out = np.zeros(12)
    lib().orc_frame_linear_extrap(_dp(_arr(a)), _dp(_arr(b)), _dp(out))
    return out


def keycurve_store(v):
    """The pose a trial's key curves hold after Tracker::optimize stores v
    (float translation, rotation through a float quaternion)."""
    out = np.zeros(6)
    lib().orc_keycurve_store(_dp(_arr(v)), _dp(out))
    return out


class PoseCurves:
    """A volume's pose curves (x, y, z KeyCurve<float>, rotation
    KeyCurve<Quatf>): the keys of each curve as frame -> stored value, and
    the value at a frame computed afresh from the final keys
    (orc_curve_eval, orc_quat_curve_eval)."""

    def __init__(self):
        self.keys = [{}, {}, {}, {}]   # x, y, z: float32; rotation: float32 (w, x, y, z)

    def clear(self):
        self.keys = [{}, {}, {}, {}]

    def insert(self, frame, pose, mask=15):
        for c in range(3):
            if mask >> c & 1:
                self.keys[c][frame] = np.float32(pose[c])
        if mask & 8:
            q = np.zeros(4, np.float32)
            lib().orc_quat_from_ypr(*(float(np.float32(pose[k])) for k in (3, 4, 5)), q.ctypes.data_as(_f))
            self.keys[3][frame] = q

    def erase(self, frame, mask=15):
        for c in range(4):
            if mask >> c & 1:
                self.keys[c].pop(frame, None)

    def eval(self, frame):
        out = np.zeros(6)
        for c in range(3):
            t = np.array(sorted(self.keys[c]), np.int32)
            v = np.array([self.keys[c][f] for f in t], np.float32)
            out[c] = lib().orc_curve_eval(len(t), t.ctypes.data_as(_i), v.ctypes.data_as(_f), int(frame))
        t = np.array(sorted(self.keys[3]), np.int32)
        q = np.array([self.keys[3][f] for f in t], np.float32).reshape(-1)
        r = np.zeros(4, np.float32)
        lib().orc_quat_curve_eval(len(t), t.ctypes.data_as(_i), q.ctypes.data_as(_f), int(frame), r.ctypes.data_as(_f))
        ypr = np.zeros(3)
        lib().orc_quat_to_ypr(r.ctypes.data_as(_f), _dp(ypr))
        out[3:] = ypr
        return out


def camera_viewport(cx, cy, fx, fy, W, H):
    out = np.zeros(4)
    lib().orc_camera_viewport(cx, cy, fx, fy, W, H, _dp(out))
    return out


def camera_image_plane(cam, cx, cy, z, W, H):
    out = np.zeros(12)
    lib().orc_camera_image_plane(_dp(_arr(cam)), cx, cy, z, W, H, _dp(out))
    return out


def calculate_viewport(modelview, cam_frame, image_plane, inv_scale, inv_trans):
    vp = np.zeros(4)
    isc = np.ascontiguousarray(inv_scale, dtype=np.float32)
    itr = np.ascontiguousarray(inv_trans, dtype=np.float32)
    ok = lib().orc_calculate_viewport(_dp(_arr(modelview)), _dp(_arr(cam_frame)), _dp(_arr(image_plane)),
                                      isc.ctypes.data_as(_f), itr.ctypes.data_as(_f), _dp(vp))
    return bool(ok), vp


def fold_inv_model_view(imv16, inv_scale, inv_trans):
    m = np.zeros(12)
    isc = np.ascontiguousarray(inv_scale, dtype=np.float32)
    itr = np.ascontiguousarray(inv_trans, dtype=np.float32)
    lib().orc_fold_inv_model_view(_dp(_arr(imv16)), isc.ctypes.data_as(_f), itr.ctypes.data_as(_f), _dp(m))
    return m


# ---------------------------------------------------------------- volumes

class VolumeDesc:
    """VolumeDescription (VolumeDescription.cpp:152-305) without the upload."""

    def __init__(self, vol):
        data = np.ascontiguousarray(vol.data)
        D, H, W = data.shape
        bps = 8 * data.dtype.itemsize
        out = np.empty_like(data).reshape(-1)
        dims = np.zeros(3, np.int32)
        isc = np.zeros(3, np.float32)
        itr = np.zeros(3, np.float32)
        tc = np.zeros(3)
        mn = np.zeros(1, np.float32)
        mx = np.zeros(1, np.float32)
        rc = lib().orc_volume_describe(data.ctypes.data, W, H, D, bps, _dp(_arr(vol.scale)),
                                       np.ascontiguousarray(vol.flip, dtype=np.int32).ctypes.data_as(_i),
                                       out.ctypes.data, dims.ctypes.data_as(_i), isc.ctypes.data_as(_f),
                                       itr.ctypes.data_as(_f), _dp(tc), mn.ctypes.data_as(_f), mx.ctypes.data_as(_f))
        if rc != 0:
            raise ValueError("unsupported bit depth" if rc == -1 else "empty volume")
        n = int(dims.prod())
        self.dims = tuple(int(d) for d in dims)  # (x, y, z)
        self.data = out[:n].reshape(self.dims[2], self.dims[1], self.dims[0]).copy()
        self.bps = bps
        self.inv_scale = isc
        self.inv_trans = itr
        self.trans_center = tc
        self.min_value = float(mn[0])
        self.max_value = float(mx[0])


# ---------------------------------------------------------------- kernels

def raycast(vd: VolumeDesc, m12, vp, step, intensity, cutoff, w, h, want_samples=False):
    out = np.zeros(w * h)
    ns = np.zeros(w * h, np.int32)
    lib().orc_raycast(vd.data.ctypes.data, vd.bps, vd.dims[0], vd.dims[1], vd.dims[2], _dp(_arr(m12)), _dp(_arr(vp)),
                      step, intensity, cutoff, _dp(out), w, h, ns.ctypes.data_as(C.POINTER(C.c_int32)))
    out = out.reshape(h, w)
    return (out, ns.reshape(h, w)) if want_samples else out


def image_render(img, image_plane, vp, w, h, mode=0, threshold=0.0):
    img = np.ascontiguousarray(img)
    vt = 32 if img.dtype == np.float32 else 8 * img.dtype.itemsize
    out = np.zeros(w * h)
    lib().orc_image_render(img.ctypes.data, vt, img.shape[1], img.shape[0], _dp(_arr(image_plane)), _dp(_arr(vp)),
                           mode, threshold, _dp(out), w, h)
    return out.reshape(h, w)


def drr_background(src):
    src = _arr(src)
    out = np.zeros_like(src)
    lib().orc_drr_background(_dp(src), _dp(out), src.size)
    return out


def multiply(a, b):
    a, b = _arr(a), _arr(b)
    out = np.zeros_like(a)
    lib().orc_multiply(_dp(a), _dp(b), _dp(out), a.size)
    return out


def merge(a, b):
    a, b = _arr(a), _arr(b)
    out = np.zeros_like(a)
    lib().orc_merge(_dp(a), _dp(b), _dp(out), a.size)
    return out


def composite(s1, s2, s3):
    s1, s2, s3 = _arr(s1), _arr(s2), _arr(s3)
    out = np.zeros(3 * s1.size)
    lib().orc_composite(_dp(s1), _dp(s2), _dp(s3), _dp(out), s1.size)
    return out


def gauss_weights(radius):
    buf = np.zeros(4096)
    K = lib().orc_gauss_weights(radius, _dp(buf), buf.size)
    return buf[:K * K].reshape(K, K) if K > 1 else np.ones((1, 1)), K


def apply_filter(flt, img):
    """One enabled filter (the `apply` of each xromm::gpu filter class)."""
    from autoscoper_gb300 import scene as S
    img = _arr(img)
    h, w = img.shape
    out = np.zeros_like(img)
    L = lib()
    if flt.kind == S.SOBEL:
        L.orc_sobel(_dp(img), _dp(out), w, h, flt.scale, flt.blend)
    elif flt.kind == S.CONTRAST:
        L.orc_contrast(_dp(img), _dp(out), w, h, flt.alpha, flt.beta, flt.size)
    elif flt.kind in (S.GAUSSIAN, S.SHARPEN):
        wts, K = gauss_weights(flt.radius)
        wts = np.ascontiguousarray(wts)
        if flt.kind == S.GAUSSIAN:
            L.orc_gaussian(_dp(img), _dp(out), w, h, _dp(wts), K)
        else:
            L.orc_sharpen(_dp(img), _dp(out), w, h, _dp(wts), K, flt.contrast, flt.threshold)
    else:
        raise ValueError(f"unsupported filter kind {flt.kind}")
    return out


def filter_chain(filters, img):
    """View::filter (View.cpp:475-555): enabled filters in order; a
    disabled filter copies; an empty list copies."""
    out = _arr(img).copy()
    for f in filters:
        if f.enabled:
            out = apply_filter(f, out)
    return out


def ncc(f, g, mask, tree=True):
    """tree=True: the reference's sum() coverage (see orc_tree_keep);
    tree=False: every pixel."""
    f, g, m = _arr(f), _arr(g), _arr(mask)
    return lib().orc_ncc(_dp(f.reshape(-1)), _dp(g.reshape(-1)), _dp(m.reshape(-1)), f.size, int(tree))


def hdist(f, g, mask, tree=True):
    f, g, m = _arr(f), _arr(g), _arr(mask)
    return lib().orc_hdist(_dp(f.reshape(-1)), _dp(g.reshape(-1)), _dp(m.reshape(-1)), f.size, int(tree))


def tree_keep_mask(n):
    """0/1 array: which of n elements the reference's sum() adds up."""
    L = lib()
    return np.array([L.orc_tree_keep(i, n) for i in range(n)], dtype=np.uint8)


# ---------------------------------------------------------------- tracker

class Tracker:
    """Host orchestration of Tracker::trackFrame / minimizationFunc over a
    scene (autoscoper_gb300.scene.Scene)."""

    def __init__(self, scene, f32_matrix=True, tree=True):
        self.scene = scene
        self.tree = tree
        self.vd = [VolumeDesc(v) for v in scene.volumes]
        # The reference folds the matrix into float32 (RayCaster.hpp:91);
        # f32_matrix=True reproduces that rounding before the FP64 march.
        self.f32_matrix = f32_matrix

    def view_setup(self, vol_id, view_id, xyzypr):
        """Steps (1a)-(1c) of trackFrame for one view: returns
        (ok, folded matrix, viewport, render_w, render_h)."""
        sc = self.scene
        v = sc.views[view_id]
        cam = v.camera
        vd = self.vd[vol_id]
        xc = frame_from_xyzypr(xyzypr)
        mv = frame_mul(frame_inverse(cam.frame), xc)
        imv = frame_row_matrix(frame_inverse(mv))
        m = fold_inv_model_view(imv, vd.inv_scale, vd.inv_trans)
        if self.f32_matrix:
            m = m.astype(np.float32).astype(np.float64)
        ok, vp = calculate_viewport(mv, cam.frame, cam.image_plane, vd.inv_scale, vd.inv_trans)
        if not ok:
            return False, m, vp, 0, 0
        cvp = cam.viewport
        rw = int(vp[2] * sc.render_width / cvp[2])
        rh = int(vp[3] * sc.render_height / cvp[3])
        if rw > sc.render_width or rh > sc.render_height:
            raise RuntimeError("Rendered image is larger than the viewport buffer")
        return True, m, vp, rw, rh

    def render_view(self, vol_id, view_id, xyzypr):
        """Images of steps (1e)-(1f): dict with drr, rad, mask (all masked)."""
        sc = self.scene
        v = sc.views[view_id]
        ok, m, vp, w, h = self.view_setup(vol_id, view_id, xyzypr)
        if not ok:
            return None
        vpf = np.asarray(vp, np.float32).astype(np.float64)   # set_viewport takes floats
        rp = sc.ray[view_id][vol_id]
        drr = raycast(self.vd[vol_id], m, vpf, float(np.float32(rp.step)), float(np.float32(rp.intensity)),
                      float(np.float32(rp.cutoff)), w, h)
        drr = filter_chain(v.drr_filters, drr)
        ipf = np.asarray(v.camera.viewport, np.float32).astype(np.float64)
        rad = image_render(v.radiograph, ipf, vpf, w, h, mode=0)
        rad = filter_chain(v.rad_filters, rad)
        if v.bg_threshold >= 0 and v.background is not None:
            bg = image_render(v.background, ipf, vpf, w, h, mode=1, threshold=float(np.float32(v.bg_threshold)))
        else:
            bg = np.ones((h, w))
        mask = multiply(bg, drr_background(drr))
        rad = multiply(rad, mask)
        drr = multiply(drr, mask)
        return {"drr": drr, "rad": rad, "mask": mask, "viewport": vp, "w": w, "h": h}

    def track_frame(self, vol_id, xyzypr):
        out = []
        for i in range(len(self.scene.views)):
            r = self.render_view(vol_id, i, xyzypr)
            if r is None:
                out.append(9999.0)
            elif self.scene.cf_model:
                out.append(hdist(r["drr"], r["rad"], r["mask"], self.tree))
            else:
                out.append(1.0 - ncc(r["drr"], r["rad"], r["mask"], self.tree))
        return out

    def compose(self, vol_id, manip):
        """Pose of minimizationFunc (Tracker.cpp:778-793): pose . V^-1 .
        manip . V, returned as xyzypr."""
        sc = self.scene
        base = np.asarray(sc.poses[vol_id], np.float32).astype(np.float64)
        xc = frame_from_xyzypr(base)
        V = sc.pivots[vol_id]
        xc = frame_mul(frame_mul(frame_mul(xc, frame_inverse(V)), frame_from_axis_angle(manip)), V)
        return frame_to_xyzypr(xc)

    def minimization_func(self, vol_id, manip):
        xyzypr = self.compose(vol_id, manip)
        c = self.track_frame(vol_id, xyzypr)
        total = float(sum(c))
        return 9999.0 if total < 0 else total


# ---------------------------------------------------------------- optimizers

def _libc():
    return C.CDLL(None)


def pso_reference(cost, lo, hi, epochs, stall, seed, n_particles=100):
    """pso() of PSO.cpp:198-295 with glibc rand() seeded by `seed`.
    `cost(x6: list of float) -> float`.  Returns (position float32[6], ncc)."""
    libc = _libc()
    libc.srand(C.c_uint(seed))
    RAND_MAX = np.float32(2147483647)

    def rnd():
        return np.float32(libc.rand()) / RAND_MAX

    f32 = np.float32
    FLT_MAX = f32(3.4028234663852886e38)
    pos = [np.zeros(6, f32)]
    for _ in range(1, n_particles):
        p = np.zeros(6, f32)
        for d in range(6):
            p[d] = f32(lo) + rnd() * (f32(hi) - f32(lo))
        pos.append(p)
    vel = [np.zeros(6, f32) for _ in range(n_particles)]
    ncc = [FLT_MAX] * n_particles
    pb_pos = [p.copy() for p in pos]
    pb_ncc = [FLT_MAX] * n_particles
    g_pos, g_ncc = np.zeros(6, f32), FLT_MAX
    omega = f32(0.8)
    c1 = c2 = f32(1.5)
    stall_iter, counter, go = 0, 0, True
    while go:
        if counter >= epochs:
            go = False
        cur = g_ncc
        for k in range(n_particles):
            for d in range(6):
                rp = rnd()
                rg = rnd()
                vel[k][d] = omega * vel[k][d] + c1 * rp * (pb_pos[k][d] - pos[k][d]) + c2 * rg * (g_pos[d] - pos[k][d])
                pos[k][d] = pos[k][d] + vel[k][d]
            ncc[k] = f32(cost([float(x) for x in pos[k]]))
            if ncc[k] < pb_ncc[k]:
                pb_pos[k], pb_ncc[k] = pos[k].copy(), ncc[k]
            if ncc[k] < g_ncc:
                g_pos, g_ncc = pos[k].copy(), ncc[k]
        omega = f32(omega * f32(0.9))
        dd = abs(f32(g_ncc - cur))
        if dd < f32(1e-4):
            stall_iter += 1
        elif dd > f32(0.001):
            stall_iter = 0
        if stall_iter == stall:
            go = False
        counter += 1
    return g_pos, float(g_ncc)


def amoeba(cost, P, Y, ftol, itmax=1000):
    """AMOEBA of DownhillSimplex.cpp:39-172 (Nelder-Mead, alpha 1, beta 0.5,
    gamma 2; stop when the mean vertex distance to the centroid < ftol).
    P: (ndim+1, ndim) array, Y: (ndim+1,) values; both updated in place.
    Returns the iteration count."""
    P = np.asarray(P, dtype=np.float64)
    Y = np.asarray(Y, dtype=np.float64)
    mpts, ndim = P.shape
    it = 0
    while True:
        ilo = 0
        ihi, inhi = (0, 1) if Y[0] > Y[1] else (1, 0)
        for i in range(mpts):
            if Y[i] < Y[ilo]:
                ilo = i
            if Y[i] > Y[ihi]:
                inhi, ihi = ihi, i
            elif Y[i] > Y[inhi] and i != ihi:
                inhi = i
        cent = np.zeros(ndim)
        for j in range(ndim):
            for i in range(mpts):
                cent[j] += P[i, j]
            cent[j] /= mpts
        rtol = 0.0
        for i in range(mpts):
            ss = 0.0
            for j in range(ndim):
                ss += (cent[j] - P[i, j]) * (cent[j] - P[i, j])
            rtol += math.sqrt(ss)
        rtol /= mpts
        if rtol < ftol or it == itmax:
            return it
        it += 1
        pbar = np.zeros(ndim)
        for i in range(mpts):
            if i != ihi:
                for j in range(ndim):
                    pbar[j] += P[i, j]
        pr = np.zeros(ndim)
        for j in range(ndim):
            pbar[j] /= 1.0 * ndim
            pr[j] = 2.0 * pbar[j] - 1.0 * P[ihi, j]
        ypr = cost(pr.copy())
        if ypr <= Y[ilo]:
            prr = 2.0 * pr + (1.0 - 2.0) * pbar
            yprr = cost(prr.copy())
            if yprr < Y[ilo]:
                P[ihi], Y[ihi] = prr, yprr
            else:
                P[ihi], Y[ihi] = pr, ypr
        elif ypr >= Y[inhi]:
            if ypr < Y[ihi]:
                P[ihi], Y[ihi] = pr, ypr
            prr = 0.5 * P[ihi] + (1.0 - 0.5) * pbar
            yprr = cost(prr.copy())
            if yprr < Y[ihi]:
                P[ihi], Y[ihi] = prr, yprr
            else:
                for i in range(mpts):
                    if i != ilo:
                        pr = 0.5 * (P[i] + P[ilo])
                        P[i] = pr
                        Y[i] = cost(pr.copy())
        else:
            P[ihi], Y[ihi] = pr, ypr
