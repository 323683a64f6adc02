"""Python face of the C ABI: device buffers, volumes, images, the plain
operators and the batched engine.  Thin wrappers only; all work runs in
libautoscoper_gb300.so on the GPU.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from . import geometry as G
from . import scene as S


def lib():
    return L.load()


class DeviceArray:
    """A cudaMalloc'd buffer holding a numpy-shaped array."""

    def __init__(self, shape, dtype=np.float32):
        self.shape = tuple(shape) if not isinstance(shape, int) else (shape,)
        self.dtype = np.dtype(dtype)
        self.nbytes = int(np.prod(self.shape)) * self.dtype.itemsize
        p = C.c_void_p()
        L.call("asc_malloc", C.byref(p), max(self.nbytes, 1))
        self.ptr = p.value

    @classmethod
    def from_host(cls, a, stream=None):
        a = np.ascontiguousarray(a)
        d = cls(a.shape, a.dtype)
        if a.nbytes:
            L.call("asc_memcpy_h2d", d.ptr, a.ctypes.data, a.nbytes, stream)
            L.call("asc_stream_sync", stream)
        return d

    def to_host(self, stream=None):
        a = np.empty(self.shape, self.dtype)
        if a.nbytes:
            L.call("asc_memcpy_d2h", a.ctypes.data, self.ptr, a.nbytes, stream)
        return a

    def upload(self, a, stream=None):
        a = np.ascontiguousarray(a, dtype=self.dtype)
        assert a.nbytes <= self.nbytes
        L.call("asc_memcpy_h2d", self.ptr, a.ctypes.data, a.nbytes, stream)

    def free(self):
        if getattr(self, "ptr", None):
            lib().asc_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def _d(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(C.POINTER(C.c_double))


def _f(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a, a.ctypes.data_as(C.POINTER(C.c_float))


class DeviceVolume:
    """VolumeDescription on the device (asc_volume_create)."""

    def __init__(self, vol: S.Volume, storage=L.ASC_STORE_U16):
        data = np.ascontiguousarray(vol.data)
        D, H, W = data.shape
        sc, scp = _d(vol.scale)
        fl = (C.c_int * 3)(*[int(x) for x in vol.flip])
        h = C.c_void_p()
        L.call("asc_volume_create", data.ctypes.data, W, H, D, 8 * data.dtype.itemsize, scp, fl, storage, C.byref(h))
        self.handle = h.value
        self.storage = storage
        isc = (C.c_float * 3)()
        itr = (C.c_float * 3)()
        tc = (C.c_double * 3)()
        mn, mx = C.c_float(), C.c_float()
        dims = (C.c_int * 3)()
        L.call("asc_volume_info", self.handle, isc, itr, tc, C.byref(mn), C.byref(mx), dims)
        self.inv_scale = np.array(isc[:], np.float32)
        self.inv_trans = np.array(itr[:], np.float32)
        self.trans_center = np.array(tc[:])
        self.min_value, self.max_value = mn.value, mx.value
        self.dims = tuple(dims[:])

    def __del__(self):
        try:
            if self.handle:
                lib().asc_volume_destroy(self.handle)
        except Exception:
            pass


class DeviceImage:
    """A radiograph (u8/u16) or background (float32) on the device."""

    def __init__(self, img):
        img = np.ascontiguousarray(img)
        bps = 32 if img.dtype == np.float32 else 8 * img.dtype.itemsize
        h = C.c_void_p()
        L.call("asc_image_create", img.ctypes.data, img.shape[1], img.shape[0], bps, C.byref(h))
        self.handle = h.value
        self.shape = img.shape

    def __del__(self):
        try:
            if self.handle:
                lib().asc_image_destroy(self.handle)
        except Exception:
            pass


# ---------------------------------------------------------------- plain operators (host arrays in/out)

def raycast(vol: DeviceVolume, imv16, viewport, step, intensity, cutoff, w, h, visible=True, out=None):
    o = out or DeviceArray((h, w))
    _, mp = _d(imv16)
    _, vpp = _f(viewport)
    L.call("asc_raycast", vol.handle, mp, vpp, step, intensity, cutoff, int(visible), o.ptr, w, h, None)
    return o


def rad_render(img: DeviceImage, image_plane, viewport, w, h, out=None):
    o = out or DeviceArray((h, w))
    _, ipp = _f(image_plane)
    _, vpp = _f(viewport)
    L.call("asc_rad_render", img.handle, ipp, vpp, o.ptr, w, h, None)
    return o


def background_render(img: DeviceImage, image_plane, viewport, threshold, w, h, out=None):
    o = out or DeviceArray((h, w))
    _, ipp = _f(image_plane)
    _, vpp = _f(viewport)
    L.call("asc_background_render", img.handle, ipp, vpp, threshold, o.ptr, w, h, None)
    return o


def apply_filter(flt: S.Filter, src: DeviceArray, out=None):
    h, w = src.shape
    o = out or DeviceArray((h, w))
    if flt.kind == S.SOBEL:
        L.call("asc_sobel", src.ptr, o.ptr, w, h, flt.scale, flt.blend, None)
    elif flt.kind == S.CONTRAST:
        L.call("asc_contrast", src.ptr, o.ptr, w, h, flt.alpha, flt.beta, flt.size, None)
    elif flt.kind == S.GAUSSIAN:
        L.call("asc_gaussian", src.ptr, o.ptr, w, h, flt.radius, None)
    elif flt.kind == S.SHARPEN:
        L.call("asc_sharpen", src.ptr, o.ptr, w, h, flt.radius, flt.contrast, flt.threshold, None)
    else:
        raise ValueError(flt.kind)
    return o


def ncc(f: DeviceArray, g: DeviceArray, mask: DeviceArray, coverage=L.ASC_SUM_TREE) -> float:
    r = C.c_double()
    L.call("asc_ncc_host", f.ptr, g.ptr, mask.ptr, int(np.prod(f.shape)), coverage, C.byref(r), None)
    return r.value


def hdist(f: DeviceArray, g: DeviceArray, mask: DeviceArray, coverage=L.ASC_SUM_TREE) -> float:
    r = C.c_double()
    L.call("asc_hdist_host", f.ptr, g.ptr, mask.ptr, int(np.prod(f.shape)), coverage, C.byref(r), None)
    return r.value


def elementwise(name, *srcs, out=None):
    h, w = srcs[0].shape
    o = out or DeviceArray((h, w) if name != "asc_composite" else (h, w, 3))
    args = [s.ptr for s in srcs]
    if name == "asc_composite":
        args.append(srcs[2].ptr)
    L.call(name, *args, o.ptr, w, h, None)
    return o


def render_targets(sc: S.Scene, volumes=None, noise=0.01):
    """Synthetic radiographs on the GPU: for every view, 1 - (sum of the
    bones' DRRs at their ground-truth poses), rendered at the radiograph's
    texel centres, plus N(0, noise), quantised to u16.  Returns the device
    volumes so callers can reuse them."""
    vols = volumes or [DeviceVolume(v) for v in sc.volumes]
    for vi, v in enumerate(sc.views):
        cam = v.camera
        acc = np.zeros((cam.height, cam.width))
        for b, dv in enumerate(vols):
            xc = G.from_xyzypr(sc.truth[b])
            mv = G.mul(G.inverse(cam.frame), xc)
            imv = G.row_matrix(G.inverse(mv))
            rp = sc.ray[vi][b]
            acc += raycast(dv, imv, S.target_viewport(cam), rp.step, rp.intensity, rp.cutoff, cam.width,
                           cam.height).to_host()
        v.radiograph = S.radiograph_from_drr(acc, seed=vi, noise=noise)
    return vols


# ---------------------------------------------------------------- engine

def _filters(lst, arr):
    n = 0
    for f in lst:
        if f.kind == S.SOBEL:
            p = (f.scale, f.blend, 0.0)
        elif f.kind == S.CONTRAST:
            p = (f.alpha, f.beta, float(f.size))
        elif f.kind == S.GAUSSIAN:
            p = (f.radius, 0.0, 0.0)
        elif f.kind == S.SHARPEN:
            p = (f.radius, f.contrast, f.threshold)
        else:
            raise ValueError(f.kind)
        arr[n] = L.FilterDesc(f.kind, int(f.enabled), *p)
        n += 1
    return n


def fill_view_desc(d, v: S.View, radiograph: "DeviceImage", background: "DeviceImage" = None):
    """An asc_view_desc of a scene view (camera, radiograph, background and
    the two filter lists)."""
    d.frame[:] = list(v.camera.frame)
    d.viewport[:] = list(v.camera.viewport)
    d.image_plane[:] = list(v.camera.image_plane)
    d.radiograph = radiograph.handle
    d.background = background.handle if background else None
    d.bg_threshold = v.bg_threshold
    d.n_drr_filters = _filters(v.drr_filters, d.drr_filters)
    d.n_rad_filters = _filters(v.rad_filters, d.rad_filters)
    return d


def fill_bone_desc(d, volume: "DeviceVolume", pivot, base_pose, rays):
    """An asc_bone_desc: the volume, its pivot, the base pose (rounded to
    float as the key curves hold it) and the RayCaster settings of each of
    its views in order (rays: list of S.RayParams)."""
    d.volume = volume.handle
    d.pivot[:] = list(pivot)
    d.base_pose[:] = [float(x) for x in np.asarray(base_pose, np.float32)]
    for j, rp in enumerate(rays):
        d.step[j], d.intensity[j], d.cutoff[j] = rp.step, rp.intensity, rp.cutoff
    return d


class Engine:
    """A scene resident on the device (asc_engine_create) that scores
    (bone, manipulator) candidates with Tracker::minimizationFunc semantics."""

    def __init__(self, scene: S.Scene, max_items=256, coverage=L.ASC_SUM_TREE, storage=L.ASC_STORE_U16,
                 volumes=None, images=None):
        self.scene = scene
        self.vols = volumes or [DeviceVolume(v, storage) for v in scene.volumes]
        self.rads = images or [DeviceImage(v.radiograph) for v in scene.views]
        self.bgs = [DeviceImage(v.background) if v.background is not None else None for v in scene.views]
        nv, nb = len(scene.views), len(scene.volumes)
        views = (L.ViewDesc * nv)()
        for i, v in enumerate(scene.views):
            fill_view_desc(views[i], v, self.rads[i], self.bgs[i])
        bones = (L.BoneDesc * nb)()
        for b in range(nb):
            fill_bone_desc(bones[b], self.vols[b], scene.pivots[b], scene.poses[b],
                           [scene.ray[v][b] for v in range(min(nv, 4))])
        h = C.c_void_p()
        L.call("asc_engine_create", nv, views, nb, bones, scene.render_width, scene.render_height, max_items,
               coverage, scene.cf_model, C.byref(h))
        self.handle = h.value
        self.n_views = nv
        self.max_items = max_items

    def set_base_pose(self, bone, xyzypr, exact=False):
        """The bone's pose; rounded to float as the key curves hold poses
        unless `exact` (a pose given in double, as getNCC's)."""
        v = np.asarray(xyzypr, np.float64) if exact else np.asarray(xyzypr, np.float32).astype(np.float64)
        _, p = _d(v)
        L.call("asc_engine_set_base_pose", self.handle, bone, p)

    def set_visible(self, bone, visible):
        L.call("asc_engine_set_visible", self.handle, bone, int(bool(visible)))

    def set_radiograph(self, view, img: DeviceImage):
        L.call("asc_engine_set_radiograph", self.handle, view, img.handle)
        self.rads[view] = img

    def eval(self, bones, manips, plain=False):
        """Costs (n,) and per-view costs (n, n_views) of candidates."""
        b = np.ascontiguousarray(bones, dtype=np.int32)
        m = np.ascontiguousarray(manips, dtype=np.float64).reshape(-1, 6)
        n = len(b)
        cost = np.zeros(n)
        vcost = np.zeros((n, self.n_views))
        fn = "asc_engine_eval_plain" if plain else "asc_engine_eval_host"
        L.call(fn, self.handle, n, b.ctypes.data_as(C.POINTER(C.c_int)), m.ctypes.data_as(C.POINTER(C.c_double)),
               cost.ctypes.data_as(C.POINTER(C.c_double)), vcost.ctypes.data_as(C.POINTER(C.c_double)), None)
        return cost, vcost

    def eval_device(self, n, bone_dev: DeviceArray, manip_dev: DeviceArray, cost_dev: DeviceArray, stream=None):
        L.call("asc_engine_eval", self.handle, n, bone_dev.ptr, manip_dev.ptr, cost_dev.ptr, None, stream)

    def pso(self, n_particles=100, n_iter=50, w=0.7298, c1=1.4962, c2=1.4962, lo=-6.0, hi=6.0, seed=1, max_stall=0):
        """Batched PSO of every bone (asc_engine_pso_stall).  Returns (gBest
        manipulators (n_bones, 6), their costs, evaluations); the iterations
        run are left in `last_pso_iterations`."""
        nb = len(self.scene.volumes)
        best = np.zeros((nb, 6))
        cost = np.zeros(nb)
        ev = C.c_longlong()
        its = C.c_int()
        L.call("asc_engine_pso_stall", self.handle, n_particles, n_iter, max_stall, w, c1, c2, lo, hi, seed,
               best.ctypes.data_as(C.POINTER(C.c_double)), cost.ctypes.data_as(C.POINTER(C.c_double)),
               C.byref(ev), C.byref(its), None)
        self.last_pso_iterations = its.value
        return best, cost, ev.value

    def optimize_frame(self, method=0, n_particles=64, n_iter=30, w=0.7298, c1=1.4962, c2=1.4962, lo=-6.0, hi=6.0,
                       seed=1, offsets=(0.1,) * 6, ftol=1e-3, max_stall=0):
        """Tracker::optimize for one frame, all bones (asc_engine_optimize_frame).
        Returns (poses (n_bones, 6), costs (n_bones,), evaluations)."""
        nb = len(self.scene.volumes)
        p = L.OptParams(method, n_particles, n_iter, w, c1, c2, lo, hi, seed, (C.c_double * 6)(*offsets), ftol,
                        max_stall)
        poses = np.zeros((nb, 6))
        raw = np.zeros((nb, 6))
        cost = np.zeros(nb)
        ev = C.c_longlong()
        L.call("asc_engine_optimize_frame_ex", self.handle, C.byref(p), poses.ctypes.data_as(C.POINTER(C.c_double)),
               raw.ctypes.data_as(C.POINTER(C.c_double)), cost.ctypes.data_as(C.POINTER(C.c_double)), C.byref(ev),
               None)
        self.last_raw_poses = raw  # before the key curves store them
        return poses, cost, ev.value

    def track(self, frames, poses, method=0, n_particles=64, n_iter=30, w=0.7298, c1=1.4962, c2=1.4962, lo=-6.0,
              hi=6.0, seed=1, offsets=(0.1,) * 6, ftol=1e-3, repeats=1, guess=1, dframe=1, keyed=None, max_stall=0):
        """A sequence of Tracker::optimize calls (asc_engine_track).  frames:
        per frame, one DeviceImage per view; poses: (n_frames, n_bones, 6) key
        curve values (the first tracked frame's is the start; `keyed` marks
        other frames that hold a key).  Returns (poses, costs, evals)."""
        nf, nb = len(frames), len(self.scene.volumes)
        rads = (C.c_void_p * (nf * self.n_views))(*[img.handle for fr in frames for img in fr])
        kf = None if keyed is None else np.ascontiguousarray(keyed, dtype=np.int32)
        p = L.TrackParams(L.OptParams(method, n_particles, n_iter, w, c1, c2, lo, hi, seed, (C.c_double * 6)(*offsets),
                                      ftol, max_stall), repeats, guess, dframe,
                          None if kf is None else kf.ctypes.data_as(C.POINTER(C.c_int)))
        out = np.ascontiguousarray(np.array(poses, dtype=np.float64).reshape(nf, nb, 6))
        cost = np.zeros((nf, nb))
        ev = C.c_longlong()
        L.call("asc_engine_track", self.handle, nf, rads, C.byref(p), out.ctypes.data_as(C.POINTER(C.c_double)),
               cost.ctypes.data_as(C.POINTER(C.c_double)), C.byref(ev), None)
        self.rads = list(frames[-1] if dframe > 0 else frames[0])  # the views' radiographs now
        return out, cost, ev.value

    def optimize_curves(self, curves, frame, n_frames, method=0, n_particles=64, n_iter=30, w=0.7298, c1=1.4962,
                        c2=1.4962, lo=-6.0, hi=6.0, seed=1, offsets=(0.1,) * 6, ftol=1e-3, repeats=1, guess=1, dframe=1,
                        max_stall=0):
        """Tracker::optimize at `frame` against each bone's PoseCurve
        (asc_engine_optimize_curves): the guess and the optimized poses are
        inserted into the curves.  Returns (costs per bone, evaluations)."""
        nb = len(self.scene.volumes)
        hs = (C.c_void_p * nb)(*[c.handle for c in curves])
        p = L.TrackParams(L.OptParams(method, n_particles, n_iter, w, c1, c2, lo, hi, seed, (C.c_double * 6)(*offsets),
                                      ftol, max_stall), repeats, guess, dframe, None)
        cost = np.zeros(nb)
        ev = C.c_longlong()
        L.call("asc_engine_optimize_curves", self.handle, hs, int(frame), int(n_frames), C.byref(p),
               cost.ctypes.data_as(C.POINTER(C.c_double)), C.byref(ev), None)
        return cost, ev.value

    def render_drr(self, view, poses, viewport=None):
        """View::renderDrr: all bones at `poses` (n_bones x 6), merged and
        filtered, over `viewport` (None: the whole image).  Returns (h, w)."""
        cam = self.scene.views[view].camera
        vp = np.array([-cam.viewport[2] / 2, -cam.viewport[3] / 2, cam.viewport[2], cam.viewport[3]]) \
            if viewport is None else np.asarray(viewport, np.float64)
        cvp = cam.viewport
        w = min(int(vp[2] * self.scene.render_width / cvp[2]), self.scene.render_width)
        h = min(int(vp[3] * self.scene.render_height / cvp[3]), self.scene.render_height)
        out = DeviceArray((max(h, 1), max(w, 1)))
        p = np.ascontiguousarray(poses, np.float64).reshape(-1)
        vpa = np.ascontiguousarray(vp, np.float64)
        L.call("asc_engine_render_drr", self.handle, view, p.ctypes.data_as(C.POINTER(C.c_double)),
               vpa.ctypes.data_as(C.POINTER(C.c_double)), out.ptr, None)
        return out.to_host()[:h, :w] if w > 0 and h > 0 else np.zeros((0, 0), np.float32)

    def image_data(self, view, bone, pose):
        """Tracker::getImageData: (rad, drr, mask) of the whole image at the
        render size, as float arrays (to_u8 gives the reference's bytes)."""
        h, w = self.scene.render_height, self.scene.render_width
        rad, drr, mask = DeviceArray((h, w)), DeviceArray((h, w)), DeviceArray((h, w))
        p = np.ascontiguousarray(pose, np.float64)
        ww, hh = C.c_int(), C.c_int()
        L.call("asc_engine_image_data", self.handle, view, bone, p.ctypes.data_as(C.POINTER(C.c_double)), rad.ptr,
               drr.ptr, mask.ptr, C.byref(ww), C.byref(hh), None)
        return rad.to_host(), drr.to_host(), mask.to_host()

    def debug_layout(self, n):
        d, lay = C.c_void_p(), C.c_void_p()
        L.call("asc_engine_debug", self.handle, C.byref(d), C.byref(lay))
        return d.value, lay.value

    def __del__(self):
        try:
            if self.handle:
                lib().asc_engine_destroy(self.handle)
        except Exception:
            pass


def pso_sequential(cost, n_particles=100, lo=-1.0, hi=1.0, epochs=50, stall=25, seed=0):
    """Reference-sequential PSO on the host (asc_pso_sequential)."""
    cb = L.COST_FN(lambda p, ctx: float(cost([p[i] for i in range(6)])))
    pos = (C.c_float * 6)()
    val = C.c_float()
    L.call("asc_pso_sequential", cb, None, n_particles, lo, hi, epochs, stall, seed, pos, C.byref(val))
    return np.array(pos[:], np.float32), float(val.value)


def amoeba_batch(batch_cost, P, Y, ftol=1e-3):
    """Lock-step speculative AMOEBA over ns simplices (asc_amoeba_batch).
    batch_cost(who: int array, X: (n, ndim)) -> (n,) values."""
    P = np.ascontiguousarray(P, dtype=np.float64).copy()
    Y = np.ascontiguousarray(Y, dtype=np.float64).copy()
    ns, mp, ndim = P.shape

    def cb(n, who, x, y, ctx):
        w = np.array([who[i] for i in range(n)])
        X = np.array([x[i] for i in range(n * ndim)]).reshape(n, ndim)
        v = batch_cost(w, X)
        for i in range(n):
            y[i] = float(v[i])
        return 0
    fn = L.BATCH_COST_FN(cb)
    it = (C.c_int * ns)()
    L.call("asc_amoeba_batch", fn, None, ns, P.ctypes.data_as(C.POINTER(C.c_double)),
           Y.ctypes.data_as(C.POINTER(C.c_double)), ndim, ftol, it)
    return P, Y, np.array(it[:])


def amoeba(cost, P, Y, ftol=1e-3):
    P = np.ascontiguousarray(P, dtype=np.float64).copy()
    Y = np.ascontiguousarray(Y, dtype=np.float64).copy()
    ndim = P.shape[1]
    cb = L.COST_FN(lambda p, ctx: float(cost(np.array([p[i] for i in range(ndim)]))))
    it = C.c_int()
    L.call("asc_amoeba", cb, None, P.ctypes.data_as(C.POINTER(C.c_double)),
           Y.ctypes.data_as(C.POINTER(C.c_double)), ndim, ftol, C.byref(it))
    return P, Y, it.value


class PoseCurve:
    """A volume's pose curves (asc_pose_curve: x, y, z KeyCurve<float> and
    the rotation KeyCurve<Quatf>).  insert/erase take a mask of curves
    (L.ASC_CURVE_X ... L.ASC_CURVE_ROT; all by default); eval reads the pose
    at a frame as AutoscoperMainWindow::getPose does."""

    def __init__(self):
        h = C.c_void_p()
        L.call("asc_pose_curve_create", C.byref(h))
        self.handle = h.value

    def clear(self):
        L.call("asc_pose_curve_clear", self.handle)

    def insert(self, frame, xyzypr, mask=L.ASC_CURVE_ALL):
        p = np.ascontiguousarray(xyzypr, np.float64)
        L.call("asc_pose_curve_insert", self.handle, int(frame), p.ctypes.data_as(C.POINTER(C.c_double)), mask)

    def erase(self, frame, mask=L.ASC_CURVE_ALL):
        L.call("asc_pose_curve_erase", self.handle, int(frame), mask)

    def keys(self, frame) -> int:
        m = C.c_int()
        L.call("asc_pose_curve_keys", self.handle, int(frame), C.byref(m))
        return m.value

    def eval(self, frame) -> np.ndarray:
        out = np.zeros(6)
        L.call("asc_pose_curve_eval", self.handle, int(frame), out.ctypes.data_as(C.POINTER(C.c_double)))
        return out

    def __del__(self):
        try:
            if self.handle:
                lib().asc_pose_curve_destroy(self.handle)
        except Exception:
            pass


def to_u8(img):
    """The bytes Tracker::getImageData returns for a float image
    (Tracker.cpp:844-863): (unsigned char)(255 * v)."""
    return (255.0 * np.asarray(img, np.float32)).astype(np.float32).astype(np.int64).astype(np.uint8)


def background_from_frames(frames):
    """Video::create_background_image: per pixel the largest normalized value
    of the frames (arrays or DeviceImages of one size)."""
    imgs = [f if isinstance(f, DeviceImage) else DeviceImage(f) for f in frames]
    h, w = imgs[0].shape
    out = DeviceArray((h, w))
    arr = (C.c_void_p * len(imgs))(*[i.handle for i in imgs])
    L.call("asc_background_from_frames", arr, len(imgs), out.ptr, None)
    return out.to_host()
