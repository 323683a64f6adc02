"""Scene description and seeded synthetic inputs for the registration cost path.

A *scene* is what Autoscoper's ``Tracker::load`` assembles from a trial
(libautoscoper/src/Tracker.cpp:244-335): cameras, bone volumes, one
radiograph per camera for the current frame, per-camera DRR and radiograph
filter chains, per-(camera, volume) ray-caster settings, the render
resolution, each volume's pivot matrix and the current pose of each volume.

There is no public dataset for this path; the phantoms, cameras and target
radiographs here are seeded synthetic stand-ins with the shapes, sizes and
value ranges of the workloads this project measures.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import geometry as G

# Filter kinds, in the numbering of xromm::gpu::Filter's type enum (Filter.hpp:59-66);
# the CUDA backend has no median filter.
CONTRAST, SOBEL, MEDIAN, GAUSSIAN, SHARPEN = 0, 1, 2, 3, 4


@dataclass
class Filter:
    """One entry of a View's DRR or radiograph filter list (View.cpp:475-555)."""
    kind: int
    scale: float = 1.0      # Sobel (SobelFilter.cpp:52-57 defaults 1.0 / 0.5)
    blend: float = 0.5
    alpha: float = 1.0      # Contrast (ContrastFilter.cpp:53-58 defaults 1 / 1 / 3)
    beta: float = 1.0
    size: int = 3
    radius: float = 1.0     # Gaussian / Sharpen (GaussianFilter.cpp:63, SharpenFilter.cpp:60-64)
    contrast: float = 1.0   # Sharpen
    threshold: float = 0.0  # Sharpen
    enabled: bool = True

    @staticmethod
    def sobel(scale=1.0, blend=0.5):
        return Filter(SOBEL, scale=scale, blend=blend)

    @staticmethod
    def contrast_filter(alpha=1.0, beta=1.0, size=3):
        return Filter(CONTRAST, alpha=alpha, beta=beta, size=size)

    @staticmethod
    def gaussian(radius=1.0):
        return Filter(GAUSSIAN, radius=max(radius, 0.0))

    @staticmethod
    def sharpen(radius=1.0, contrast=1.0, threshold=0.0):
        # SharpenFilter::set_contrast clamps below 1 (SharpenFilter.cpp:85-91)
        return Filter(SHARPEN, radius=max(radius, 0.0), contrast=max(contrast, 1.0), threshold=threshold)


@dataclass
class Camera:
    frame: np.ndarray          # camera -> world, 12 doubles
    width: int
    height: int
    cx: float
    cy: float
    fx: float
    fy: float

    @property
    def viewport(self) -> np.ndarray:
        return G.camera_viewport(self.cx, self.cy, self.fx, self.fy, self.width, self.height)

    @property
    def image_plane(self) -> np.ndarray:
        # MayaCam 2.0 convention: z = -(fx + fy) / 2 (Camera.cpp:355-358)
        return G.camera_image_plane(self.frame, self.cx, self.cy, -0.5 * (self.fx + self.fy),
                                    self.width, self.height)


@dataclass
class Volume:
    data: np.ndarray                      # (depth, height, width) uint16 or uint8
    scale: tuple = (1.0, 1.0, 1.0)        # voxel size in mm (x, y, z)
    flip: tuple = (0, 0, 0)
    subject: str = ""

    @property
    def bps(self) -> int:
        return 8 * self.data.dtype.itemsize


@dataclass
class RayParams:
    """RayCaster settings (RayCaster.cpp:57-64 defaults 0.5 / 10 / 0)."""
    step: float = 0.5
    intensity: float = 10.0
    cutoff: float = 0.0


@dataclass
class View:
    camera: Camera
    radiograph: np.ndarray                # (H, W) uint8/uint16
    drr_filters: List[Filter] = field(default_factory=list)
    rad_filters: List[Filter] = field(default_factory=list)
    background: Optional[np.ndarray] = None   # (H, W) float32
    bg_threshold: float = -1.0            # View.cpp:93: < 0 disables the mask

    @property
    def bps(self) -> int:
        return 8 * self.radiograph.dtype.itemsize


@dataclass
class Scene:
    views: List[View]
    volumes: List[Volume]
    ray: List[List[RayParams]]            # [view][volume]
    render_width: int
    render_height: int
    pivots: List[np.ndarray]              # volume matrices (frame = translate(transCenter))
    poses: List[np.ndarray]               # current pose per volume, xyzypr as float32 values
    cf_model: int = 0                     # 0 = 1-NCC, 1 = SAD ("hdist")
    truth: List[np.ndarray] = field(default_factory=list)  # ground-truth xyzypr per volume


# ---------------------------------------------------------------------------
# Synthetic inputs
# ---------------------------------------------------------------------------

def phantom(shape, semi_axes=None, seed=0, noise=20.0, soft=200, cortex=1800, core=900, shell=3.0,
            dtype=np.uint16, landmark=False) -> np.ndarray:
    """Bone phantom of shape (depth, height, width): soft tissue `soft`, an
    ellipsoidal cortical shell `cortex` of thickness `shell` voxels around a
    trabecular core `core`, plus Gaussian noise of sigma `noise` from
    numpy PCG64(seed), rounded and clamped to the integer range.  The
    ellipsoid is symmetric about an axis, so rotations about that axis do not
    change its DRRs; `landmark` adds a dense sphere off the axes inside the
    core, which makes every rotation observable."""
    D, H, W = shape
    if semi_axes is None:
        semi_axes = (0.31 * W, 0.31 * H, 0.31 * D)
    a, b, c = semi_axes
    z, y, x = np.meshgrid(np.arange(D) - (D - 1) / 2.0, np.arange(H) - (H - 1) / 2.0,
                          np.arange(W) - (W - 1) / 2.0, indexing="ij")
    outer = (x / a) ** 2 + (y / b) ** 2 + (z / c) ** 2 <= 1.0
    inner = (x / (a - shell)) ** 2 + (y / (b - shell)) ** 2 + (z / (c - shell)) ** 2 <= 1.0
    v = np.full(shape, float(soft))
    v[outer] = cortex
    v[inner] = core
    if landmark:
        r = 0.06 * min(D, H, W)
        blob = (x - 0.12 * W) ** 2 + (y - 0.10 * H) ** 2 + (z - 0.08 * D) ** 2 <= r * r
        v[blob & inner] = cortex
    rng = np.random.Generator(np.random.PCG64(seed))
    v += rng.normal(0.0, noise, size=shape)
    hi = np.iinfo(dtype).max
    return np.clip(np.rint(v), 0, hi).astype(dtype)


def biplane_cameras(width, height, pitch_mm, sid_mm=1200.0, sod_mm=600.0) -> List[Camera]:
    """Two pinholes 90 degrees apart (sources on +X and +Y), source-to-image
    `sid_mm`, source-to-isocentre `sod_mm`, principal point at the image centre,
    fx = fy = SID / pixel pitch."""
    f = sid_mm / pitch_mm
    cams = []
    for eye in ((sod_mm, 0.0, 0.0), (0.0, sod_mm, 0.0)):
        frame = G.look_at_frame(eye, (0.0, 0.0, 0.0), (0.0, 0.0, 1.0))
        cams.append(Camera(frame, width, height, width / 2.0, height / 2.0, f, f))
    return cams


def volume_center_object(vol: Volume) -> np.ndarray:
    """Centre of a volume's box in its object coordinates: x in [0, W*sx],
    y in [0, H*sy], z in [-D*sz, 0] (RayCaster.cpp:88-114 with
    VolumeDescription.cpp:240-252)."""
    D, H, W = vol.data.shape
    sx, sy, sz = vol.scale
    return np.array([W * sx / 2.0, H * sy / 2.0, -D * sz / 2.0])


def pose_centered_at(vol: Volume, center_world, ypr) -> np.ndarray:
    """xyzypr pose that rotates the volume by `ypr` and puts its box centre at
    `center_world`."""
    f = G.from_xyzypr([0, 0, 0, ypr[0], ypr[1], ypr[2]])
    t = np.asarray(center_world, dtype=np.float64) - G.point(f, volume_center_object(vol))
    return np.array([t[0], t[1], t[2], ypr[0], ypr[1], ypr[2]])


def pivot_matrix(vol: Volume) -> np.ndarray:
    """Volume matrix after Tracker::load's "center pivot" translate by
    VolumeDescription::transCenter (Tracker.cpp:286-290,
    VolumeDescription.cpp:152-305): the centre of the box of non-zero voxels
    of the flipped volume, scaled (the phantoms have no zero voxel, so theirs
    is the whole volume)."""
    d = vol.data
    fx, fy, fz = (bool(f) for f in vol.flip)
    d = d[::-1 if fz else 1, ::-1 if fy else 1, ::-1 if fx else 1]
    mn, mx = [], []
    for axis in (2, 1, 0):  # x, y, z
        other = tuple(a for a in range(3) if a != axis)
        idx = np.nonzero(np.any(d != 0, axis=other))[0]
        if idx.size == 0:
            raise ValueError("empty volume")
        mn.append(int(idx[0]))
        mx.append(int(idx[-1]))
    sx, sy, sz = (float(np.float32(s)) for s in vol.scale)
    tc = [-sx * 0.5 * (mn[0] + mx[0]), -sy * 0.5 * (mn[1] + mx[1]), sz * 0.5 * (mn[2] + mx[2])]
    return G.translate(G.identity(), tc)


def config_filters(kind: str) -> List[Filter]:
    if kind == "sobel":
        return [Filter.sobel(scale=1.0, blend=0.0)]
    if kind == "chain":
        return [Filter.contrast_filter(alpha=2.5, beta=0.9), Filter.sharpen(radius=1.0, contrast=1.0),
                Filter.gaussian(radius=1.5), Filter.sobel(scale=1.0, blend=0.0)]
    if kind == "none":
        return []
    raise ValueError(kind)


def make_scene(vol_shapes, voxel_mm, render, pitch_mm, filters="sobel", seed=0, bone_offsets=None,
               rot_range=10.0, cutoff_frac=0.1, landmark=False) -> Scene:
    """Scene skeleton without radiographs (see `render_targets`).

    vol_shapes: list of (depth, height, width); render: (w, h) of both the
    radiographs and the render buffer; pitch_mm: detector pixel pitch."""
    rng = np.random.Generator(np.random.PCG64(seed + 1000))
    vols = []
    for i, shp in enumerate(vol_shapes):
        semi = (40, 25, 25) if tuple(shp) == (128, 128, 128) else None
        vols.append(Volume(phantom(shp, semi, seed=seed + i, landmark=landmark), (voxel_mm,) * 3,
                           subject=f"s{seed}_{i}"))
    if bone_offsets is None:
        n = len(vols)
        bone_offsets = [(0.0, 0.0, 45.0 * (i - (n - 1) / 2.0)) for i in range(n)]
    cams = biplane_cameras(render[0], render[1], pitch_mm)
    views = [View(c, np.zeros((render[1], render[0]), np.uint16), config_filters(filters),
                  config_filters(filters)) for c in cams]
    ray = []
    for _ in views:
        row = []
        for v in vols:
            lo, hi = float(v.data.min()) / 65535.0, float(v.data.max()) / 65535.0
            row.append(RayParams(step=0.5 * voxel_mm, intensity=1.0, cutoff=lo + cutoff_frac * (hi - lo)))
        ray.append(row)
    truth = []
    for i, v in enumerate(vols):
        ypr = rng.uniform(-rot_range, rot_range, size=3)
        truth.append(pose_centered_at(v, bone_offsets[i], ypr))
    pivots = [pivot_matrix(v) for v in vols]
    poses = [t.astype(np.float32) for t in truth]
    return Scene(views, vols, ray, render[0], render[1], pivots, poses, 0, truth)


def target_viewport(cam: Camera) -> np.ndarray:
    """DRR viewport whose pixel (x, y) is the centre of radiograph texel
    (x, H-1-y) under RadRenderer's mapping (RadRenderer_kernels.cu:103-107)."""
    u0, v0, u1, v1 = cam.viewport
    W, H = cam.width, cam.height
    return np.array([u0 - u1 / 2.0 + u1 * 0.5 / W, v0 - v1 / 2.0 + v1 * 0.5 / H, u1, v1])


def radiograph_from_drr(drr_sum: np.ndarray, seed: int, noise=0.01, dtype=np.uint16) -> np.ndarray:
    """Target radiograph: 1 - min(sum of DRRs, 1), rows flipped to image
    order, plus N(0, noise) from PCG64(seed), quantised to `dtype`."""
    rng = np.random.Generator(np.random.PCG64(seed + 7))
    img = 1.0 - np.minimum(drr_sum, 1.0)[::-1, :]
    img = img + rng.normal(0.0, noise, size=img.shape)
    hi = np.iinfo(dtype).max
    return np.clip(np.rint(img * hi), 0, hi).astype(dtype)


def perturb(pose, rng, mm, deg) -> np.ndarray:
    d = np.concatenate([rng.uniform(-mm, mm, 3), rng.uniform(-deg, deg, 3)])
    return (np.asarray(pose, dtype=np.float64) + d).astype(np.float32)
