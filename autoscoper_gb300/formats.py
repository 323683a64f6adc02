"""Autoscoper's input files on the host: trial configurations (.cfg), camera
calibrations (MayaCam 1.0 / 2.0 text, VTK camera JSON), view settings
(.vie: filters and ray-caster settings) and TIFF images (volumes as
multi-page stacks, radiograph videos as directories of frames), so that a
reference trial drives the GB300 engine.

Parsing follows the reference's readers (file:line cited per function); the
TIFF decoder is written from the public TIFF 6.0 specification (strips,
uncompressed / PackBits / LZW, horizontal predictor) for the 8- and 16-bit
grayscale images those files hold.  ``write_tiff`` makes test images with
the same encodings.
"""
from __future__ import annotations

import json
import math
import os
import struct
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Tuple

import numpy as np

from . import geometry as G
from . import scene as S

# ---------------------------------------------------------------- TIFF

_TYPE_SIZE = {1: 1, 2: 1, 3: 2, 4: 4, 5: 8, 6: 1, 7: 1, 8: 2, 9: 4, 10: 8, 11: 4, 12: 8}
_TYPE_FMT = {1: "B", 3: "H", 4: "I", 6: "b", 8: "h", 9: "i", 11: "f", 12: "d"}


def _packbits_decode(data: bytes, expected: int) -> bytes:
    out = bytearray()
    i, n = 0, len(data)
    while i < n and len(out) < expected:
        c = data[i]
        i += 1
        if c < 128:          # copy the next c + 1 bytes
            out += data[i:i + c + 1]
            i += c + 1
        elif c > 128:        # repeat the next byte 257 - c times
            out += bytes([data[i]]) * (257 - c)
            i += 1
        # 128 is a no-op
    return bytes(out[:expected])


def _lzw_decode(data: bytes, expected: int) -> bytes:
    """TIFF LZW: MSB-first codes of 9-12 bits, Clear 256, EOI 257, the code
    width growing one code early (TIFF 6.0, section 13)."""
    out = bytearray()
    table: List[bytes] = [bytes([i]) for i in range(256)] + [b"", b""]
    width, bitpos, nbits = 9, 0, 8 * len(data)
    prev: Optional[bytes] = None
    while bitpos + width <= nbits:
        byte, off = bitpos >> 3, bitpos & 7
        chunk = int.from_bytes(data[byte:byte + 3].ljust(3, b"\0"), "big")
        code = (chunk >> (24 - off - width)) & ((1 << width) - 1)
        bitpos += width
        if code == 256:
            table = table[:258]
            width, prev = 9, None
            continue
        if code == 257:
            break
        if prev is None:
            entry = table[code]
        elif code < len(table):
            entry = table[code]
            table.append(prev + entry[:1])
        else:                # the code being defined now
            entry = prev + prev[:1]
            table.append(entry)
        out += entry
        prev = entry
        if len(table) + 1 >= (1 << width) and width < 12:
            width += 1
        if len(out) >= expected:
            break
    return bytes(out[:expected])


@dataclass
class TiffPage:
    width: int
    height: int
    bits: int
    data: np.ndarray  # (height, width), uint8 / uint16 / uint32


def read_tiff(path: str) -> List[TiffPage]:
    """Every page (IFD) of a TIFF file: one grayscale sample per pixel, 8, 16
    or 32 unsigned bits, in strips; compression none (1), LZW (5) or
    PackBits (32773), horizontal predictor (2) allowed."""
    with open(path, "rb") as fh:
        buf = fh.read()
    if buf[:2] == b"II":
        e = "<"
    elif buf[:2] == b"MM":
        e = ">"
    else:
        raise ValueError(f"{path}: not a TIFF file")
    if struct.unpack(e + "H", buf[2:4])[0] != 42:
        raise ValueError(f"{path}: unsupported TIFF variant")
    ifd = struct.unpack(e + "I", buf[4:8])[0]
    pages = []
    seen = set()
    while ifd and ifd not in seen:
        seen.add(ifd)
        (count,) = struct.unpack(e + "H", buf[ifd:ifd + 2])
        tags: Dict[int, List] = {}
        for k in range(count):
            p = ifd + 2 + 12 * k
            tag, typ, n = struct.unpack(e + "HHI", buf[p:p + 8])
            size = _TYPE_SIZE.get(typ, 1) * n
            raw = buf[p + 8:p + 12] if size <= 4 else buf[struct.unpack(e + "I", buf[p + 8:p + 12])[0]:][:size]
            if typ in _TYPE_FMT:
                tags[tag] = list(struct.unpack(e + _TYPE_FMT[typ] * n, raw[:size]))
            elif typ == 5:
                vals = struct.unpack(e + "I" * (2 * n), raw[:size])
                tags[tag] = [vals[2 * i] / max(vals[2 * i + 1], 1) for i in range(n)]
            else:
                tags[tag] = raw[:size]
        w, h = tags[256][0], tags[257][0]
        bits = tags.get(258, [1])[0]
        if tags.get(277, [1])[0] != 1:
            raise ValueError(f"{path}: only one sample per pixel is supported")
        if tags.get(339, [1])[0] != 1:
            raise ValueError(f"{path}: only unsigned integer samples are supported")
        if bits not in (8, 16, 32):
            raise ValueError(f"{path}: {bits} bits per sample is not supported")
        if 324 in tags:
            raise ValueError(f"{path}: tiled images are not supported")
        comp = tags.get(259, [1])[0]
        pred = tags.get(317, [1])[0]
        rps = tags.get(278, [h])[0]
        offs, cnts = tags[273], tags[279]
        bpr = w * bits // 8
        rows = []
        for s, (o, c) in enumerate(zip(offs, cnts)):
            nrow = min(rps, h - s * rps)
            raw = buf[o:o + c]
            if comp == 1:
                strip = raw[:nrow * bpr]
            elif comp == 32773:
                strip = _packbits_decode(raw, nrow * bpr)
            elif comp == 5:
                strip = _lzw_decode(raw, nrow * bpr)
            else:
                raise ValueError(f"{path}: compression {comp} is not supported")
            if len(strip) != nrow * bpr:
                raise ValueError(f"{path}: strip {s} decodes to {len(strip)} bytes, not {nrow * bpr}")
            rows.append(strip)
        dt = {8: np.uint8, 16: np.uint16, 32: np.uint32}[bits]
        img = np.frombuffer(b"".join(rows), dtype=np.dtype(dt).newbyteorder(e)).reshape(h, w).astype(dt)
        if pred == 2:  # horizontal differencing, modulo the sample width
            img = np.cumsum(img, axis=1, dtype=dt)
        pages.append(TiffPage(w, h, bits, img))
        ifd = struct.unpack(e + "I", buf[ifd + 2 + 12 * count:ifd + 6 + 12 * count])[0]
    return pages


def _packbits_encode(data: bytes) -> bytes:
    out = bytearray()
    i, n = 0, len(data)
    while i < n:
        j = i
        while j + 1 < n and data[j + 1] == data[i] and j - i < 127:
            j += 1
        if j > i:            # a run of j - i + 1 bytes
            out += bytes([257 - (j - i + 1), data[i]])
            i = j + 1
            continue
        j = i
        while j + 1 < n and (j + 2 >= n or data[j + 1] != data[j + 2]) and j - i < 127:
            j += 1
        out += bytes([j - i]) + data[i:j + 1]
        i = j + 1
    return bytes(out)


def _lzw_encode(data: bytes) -> bytes:
    """TIFF LZW encoder: a new table entry per emitted code; the width grows
    once the next free code passes the width's range (the decoder, one entry
    behind, grows one code early); Clear when the table is full."""
    table = {bytes([i]): i for i in range(256)}
    nxt, width = 258, 9
    codes = [(256, width)]
    cur = b""
    for b in data:
        cand = cur + bytes([b])
        if cand in table:
            cur = cand
            continue
        codes.append((table[cur], width))
        table[cand] = nxt
        nxt += 1
        if nxt == 4094:
            codes.append((256, width))
            table = {bytes([i]): i for i in range(256)}
            nxt, width = 258, 9
        elif nxt >= (1 << width):
            width += 1
        cur = bytes([b])
    if cur:
        codes.append((table[cur], width))
        nxt += 1
        if nxt < 4094 and nxt >= (1 << width):
            width += 1
    codes.append((257, width))
    acc, nacc, out = 0, 0, bytearray()
    for code, w in codes:
        acc = (acc << w) | code
        nacc += w
        while nacc >= 8:
            out.append((acc >> (nacc - 8)) & 0xFF)
            nacc -= 8
        acc &= (1 << nacc) - 1
    if nacc:
        out.append((acc << (8 - nacc)) & 0xFF)
    return bytes(out)


def write_tiff(path: str, pages: List[np.ndarray], compression: str = "none", rows_per_strip: int = 16,
               byteorder: str = "<", predictor: bool = False) -> None:
    """Writes grayscale uint8/uint16 pages (for tests and exports):
    compression 'none', 'packbits' or 'lzw', optionally with the horizontal
    differencing predictor."""
    code = {"none": 1, "lzw": 5, "packbits": 32773}[compression]
    e = byteorder
    body = bytearray(b"II" if e == "<" else b"MM")
    body += struct.pack(e + "HI", 42, 0)
    first_ifd_pos = 4
    prev_next_pos = first_ifd_pos
    for img in pages:
        img = np.ascontiguousarray(img)
        h, w = img.shape
        bits = 8 * img.dtype.itemsize
        strips = []
        stored = img
        if predictor:  # each sample minus its left neighbour, modulo the sample width
            stored = img.copy()
            stored[:, 1:] = img[:, 1:] - img[:, :-1]
        for r0 in range(0, h, rows_per_strip):
            raw = stored[r0:r0 + rows_per_strip].astype(img.dtype.newbyteorder(e)).tobytes()
            strips.append(raw if code == 1 else _packbits_encode(raw) if code == 32773 else _lzw_encode(raw))
        offs = []
        for s in strips:
            offs.append(len(body))
            body += s
            if len(body) % 2:
                body += b"\0"
        entries = [(256, 4, [w]), (257, 4, [h]), (258, 3, [bits]), (259, 3, [code]), (262, 3, [1]),
                   (273, 4, offs), (277, 3, [1]), (278, 4, [rows_per_strip]), (279, 4, [len(s) for s in strips])]
        if predictor:
            entries.append((317, 3, [2]))
        extra = bytearray()
        ifd_pos = len(body)
        ifd_size = 2 + 12 * len(entries) + 4
        blob_pos = ifd_pos + ifd_size
        ifd = bytearray(struct.pack(e + "H", len(entries)))
        for tag, typ, vals in entries:
            fmt = e + _TYPE_FMT[typ] * len(vals)
            raw = struct.pack(fmt, *vals)
            if len(raw) <= 4:
                ifd += struct.pack(e + "HHI", tag, typ, len(vals)) + raw.ljust(4, b"\0")
            else:
                ifd += struct.pack(e + "HHII", tag, typ, len(vals), blob_pos + len(extra))
                extra += raw
        next_pos = ifd_pos + len(ifd)
        ifd += struct.pack(e + "I", 0)
        body[prev_next_pos:prev_next_pos + 4] = struct.pack(e + "I", ifd_pos)
        body += ifd + extra
        prev_next_pos = next_pos
    with open(path, "wb") as fh:
        fh.write(bytes(body))


def read_volume(path: str, voxel_size=(1.0, 1.0, 1.0), flip=(0, 0, 0), subject: str = "") -> S.Volume:
    """A volume as Volume::Volume reads it (Volume.cpp:51-140): every page
    of a multi-page TIFF is one slice (depth = pages), 8 or 16 bits."""
    pages = read_tiff(path)
    if any(p.bits not in (8, 16) for p in pages):
        raise ValueError(f"{path}: volumes must be 8 or 16 bits per sample")
    if len({(p.width, p.height, p.bits) for p in pages}) != 1:
        raise ValueError(f"{path}: slices differ in size or depth")
    data = np.stack([p.data for p in pages])
    return S.Volume(data, tuple(float(v) for v in voxel_size), tuple(int(f) for f in flip), subject or path)


def video_frames(dirname: str) -> List[str]:
    """The frames of a radiograph video (Video.cpp:66-105): the directory's
    files with a .tif* extension, hidden files skipped, in sorted order."""
    names = []
    for n in os.listdir(dirname):
        if n.startswith("."):
            continue
        ext = n[n.rfind(".") + 1:] if "." in n else ""
        if ext[:3] != "tif":
            continue
        names.append(dirname + "/" + n)
    if not names:
        raise ValueError(f"No TIFF files found in directory: {dirname}")
    return sorted(names)


def read_frame(path: str) -> np.ndarray:
    page = read_tiff(path)[0]
    return page.data


# ---------------------------------------------------------------- cameras

@dataclass
class CameraFile(S.Camera):
    """A camera read from a calibration file: the Camera fields plus the
    film-plane z its image plane was computed with (MayaCam 1.0 keeps the
    file's sign; the other formats use -(fx + fy) / 2)."""
    plane_z: float = 0.0

    @property
    def image_plane(self) -> np.ndarray:
        return G.camera_image_plane(self.frame, self.cx, self.cy, self.plane_z, self.width, self.height)


def _csv_numbers(line: str, n: int, what: str, path: str, lineno: int) -> List[float]:
    vals = []
    for tok in line.split(",")[:n]:
        try:
            vals.append(float(tok))
        except ValueError:
            break
    if len(vals) != n:
        raise ValueError(f"{path}:{lineno}: there was an error reading {what} values")
    return vals


def read_mayacam1(path: str) -> CameraFile:
    """Camera::loadMayaCam1 (Camera.cpp:139-227): camera position; rotations
    about x, y, z; film-plane translation; u0, v0, Z (1-based); scale, width,
    height (0 means 1024)."""
    with open(path) as fh:
        lines = [ln.rstrip("\r\n") for ln in fh][:5]
    if len(lines) < 5:
        raise ValueError(f"{path}: a MayaCam 1.0 file has 5 lines")
    v = [_csv_numbers(lines[i], 3, "camera", path, i + 1) for i in range(5)]
    t, rot = v[0], v[1]
    u0, v0, z = v[3][0] - 1.0, v[3][1] - 1.0, v[3][2]
    w = v[4][1] or 1024.0
    h = v[4][2] or 1024.0
    frame = G.from_xyzypr([t[0], t[1], t[2], rot[2], rot[1], rot[0]])
    f = abs(z)
    return CameraFile(frame, int(w), int(h), u0, v0, f, f, plane_z=z)


def read_mayacam2(path: str) -> CameraFile:
    """Camera::loadMayaCam2 (Camera.cpp:229-362): image size (line 2), the
    camera matrix K (lines 5-7, by columns), the rotation R (lines 10-12, by
    columns) and translation t (lines 15-17) of a world->camera transform
    with image y down; converted to the camera->world frame with y up."""
    with open(path) as fh:
        lines = [ln.rstrip("\r\n") for ln in fh][:17]
    if len(lines) < 17:
        raise ValueError(f"{path}: a MayaCam 2.0 file has 17 lines")
    size = _csv_numbers(lines[1], 2, "'image size'", path, 2)
    K = np.zeros((3, 3))
    R = np.zeros((3, 3))
    for i in range(3):
        K[:, i] = _csv_numbers(lines[4 + i], 3, "'camera matrix'", path, 5 + i)
        R[:, i] = _csv_numbers(lines[9 + i], 3, "'rotation'", path, 10 + i)
    t = np.zeros(3)
    for i in range(3):
        try:
            t[i] = float(lines[14 + i].split()[0])
        except (ValueError, IndexError):
            raise ValueError(f"{path}:{15 + i}: there was an error reading 'translation' values")
    # invert the y axis, then the rotation and translation
    t[0], t[2] = -t[0], -t[2]
    R[:, 0] = -R[:, 0]
    R[:, 2] = -R[:, 2]
    K[2, 1] = (size[1] - 1) - K[2, 1]
    R = R.T.copy()
    t = -np.array([t[0] * R[0, i] + t[1] * R[1, i] + t[2] * R[2, i] for i in range(3)])
    R[0, :] = -R[0, :]
    R[1, :] = -R[1, :]
    frame = np.concatenate([R.reshape(-1), t])
    fx, fy = K[0, 0], K[1, 1]
    return CameraFile(frame, int(size[0]), int(size[1]), K[2, 0], K[2, 1], fx, fy, plane_z=-0.5 * (fx + fy))


VTK_CAMERA_SCHEMA = "https://autoscoperm.slicer.org/vtkCamera-schema-1.0.json"


def read_vtk_camera(path: str) -> CameraFile:
    """Camera::loadVTKCamera (Camera.cpp:364-422): position, focal point,
    view-up and view angle of a VTK camera (schema 1.0); principal point at
    the image centre."""
    with open(path) as fh:
        cal = json.load(fh)
    if cal.get("@schema") != VTK_CAMERA_SCHEMA:
        raise ValueError(f"{path}: unsupported schema {cal.get('@schema')}")
    if float(cal.get("version", 0)) != 1.0:
        raise ValueError(f"{path}: unsupported version {cal.get('version')}")
    w, h = float(cal["image-width"]), float(cal["image-height"])
    frame = G.look_at_frame(cal["camera-position"], cal["focal-point"], cal["view-up"])
    ang = float(cal["view-angle"]) * (math.pi / 180)
    fx, fy = w / (2 * math.tan(ang / 2)), h / (2 * math.tan(ang / 2))
    return CameraFile(frame, int(w), int(h), w / 2.0, h / 2.0, fx, fy, plane_z=-0.5 * (fx + fy))


def read_camera(path: str) -> CameraFile:
    """Camera::Camera (Camera.cpp:111-137): .json is a VTK camera; a file
    whose first line is 'image size' is MayaCam 2.0; else MayaCam 1.0."""
    ext = path[path.rfind(".") + 1:] if "." in path else ""
    if not ext:
        raise ValueError("Invalid MayaCam file")
    if ext == "json":
        return read_vtk_camera(path)
    with open(path) as fh:
        first = fh.readline().rstrip("\r\n")
    return read_mayacam2(path) if first == "image size" else read_mayacam1(path)


# ---------------------------------------------------------------- view settings (.vie)

@dataclass
class ViewSettings:
    drr_filters: List[S.Filter] = field(default_factory=list)
    rad_filters: List[S.Filter] = field(default_factory=list)
    ray: Optional[S.RayParams] = None


_FILTER_KEYS = {"SobelFilter": ("Scale", "Blend"), "ContrastFilter": ("Alpha", "Beta"),
                "GaussianFilter": ("Radius",), "SharpenFilter": ("Radius", "Contrast")}


def _filter(kind: str, vals: Dict[str, float]) -> S.Filter:
    if kind == "SobelFilter":
        return S.Filter.sobel(scale=vals.get("Scale", 1.0), blend=vals.get("Blend", 0.5))
    if kind == "ContrastFilter":
        return S.Filter.contrast_filter(alpha=vals.get("Alpha", 1.0), beta=vals.get("Beta", 1.0))
    if kind == "GaussianFilter":
        return S.Filter.gaussian(radius=vals.get("Radius", 1.0))
    return S.Filter.sharpen(radius=vals.get("Radius", 1.0), contrast=vals.get("Contrast", 1.0))


def read_vie(path: str) -> ViewSettings:
    """A view's settings file as the GUI writes and reads it
    (ModelViewTreeWidgetItem.cpp:96-190, FilterTreeWidgetItem.cpp:120-190):
    RadFilters / DrrFilters blocks of Sobel, Contrast, Gaussian and Sharpen
    filter blocks, and a DrrRenderer block (SampleDistance, RayIntensity,
    Cutoff)."""
    vs = ViewSettings()
    with open(path) as fh:
        lines = [ln.strip() for ln in fh]
    i = 0
    while i < len(lines):
        ln = lines[i]
        if ln in ("RadFilters_begin", "DrrFilters_begin"):
            target = vs.rad_filters if ln.startswith("Rad") else vs.drr_filters
            end = ln.replace("_begin", "_end")
            i += 1
            while i < len(lines) and lines[i] != end:
                key = lines[i].split()[0] if lines[i] else ""
                if key.endswith("_begin") and key[:-6] in _FILTER_KEYS:
                    kind = key[:-6]
                    vals = {}
                    i += 1
                    while i < len(lines) and lines[i] != kind + "_end":
                        parts = lines[i].split()
                        if len(parts) >= 2 and parts[0] in _FILTER_KEYS[kind]:
                            vals[parts[0]] = float(parts[1])
                        i += 1
                    target.append(_filter(kind, vals))
                i += 1
        elif ln == "DrrRenderer_begin":
            ray = S.RayParams()
            i += 1
            while i < len(lines) and lines[i] != "DrrRenderer_end":
                parts = lines[i].split()
                if len(parts) >= 2:
                    if parts[0] == "SampleDistance":
                        ray.step = float(parts[1])
                    elif parts[0] == "RayIntensity":
                        ray.intensity = float(parts[1])
                    elif parts[0] == "Cutoff":
                        ray.cutoff = float(parts[1])
                i += 1
            vs.ray = ray
        i += 1
    return vs


# ---------------------------------------------------------------- trials (.cfg)

@dataclass
class TrialFile:
    path: str
    version: Tuple[int, int]
    cameras: List[str]
    videos: List[str]
    volumes: List[str]
    voxel_sizes: List[Tuple[float, float, float]]
    flips: List[Tuple[int, int, int]]
    render_width: int
    render_height: int
    offsets: Tuple[float, ...]
    meshes: List[str]


def read_cfg(path: str) -> TrialFile:
    """Trial::parse / validate / load* (Trial.cpp:202-400): one key per line
    (mayaCam_csv, CameraRootDir, VolumeFile, VolumeFlip, VoxelSize,
    RenderResolution, OptimizationOffsets, MeshFile, Version); '#' comments;
    RenderResolution defaults to 512 x 512 and the offsets to 0.1."""
    keys: Dict[str, List[str]] = {k: [] for k in ("mayaCam_csv", "CameraRootDir", "VolumeFile", "VolumeFlip",
                                                   "VoxelSize", "RenderResolution", "OptimizationOffsets",
                                                   "MeshFile")}
    version = (1, 0)
    with open(path) as fh:
        for line in fh:
            line = line.rstrip("\r\n")
            if not line or line[0] == "#":
                continue
            key, _, value = line.partition(" ")
            if key in keys:
                keys[key].append(value.replace("\\", "/") if key in ("mayaCam_csv", "CameraRootDir", "VolumeFile")
                                 else value)
            elif key == "Version":
                parts = (value.split(".") + ["0", "0"])[:2]
                version = (int(parts[0] or 0), int(parts[1] or 0))
    if len(keys["mayaCam_csv"]) < 1:
        raise ValueError(f"{path}: There must be at least one mayacam files.")
    if len(keys["mayaCam_csv"]) != len(keys["CameraRootDir"]):
        raise ValueError(f"{path}: The number of cameras and videos must match.")
    if len(keys["VolumeFile"]) < 1:
        raise ValueError(f"{path}: There must be at least one volume file.")
    if len(keys["VolumeFile"]) != len(keys["VoxelSize"]):
        raise ValueError(f"{path}: Each volume must be associated with its corresponding voxel sizes.")
    if keys["MeshFile"] and len(keys["MeshFile"]) != len(keys["VolumeFile"]):
        raise ValueError(f"{path}: You must specify a mesh file for each volume or none at all.")
    base = os.path.dirname(os.path.abspath(path))

    def resolve(p):
        return p if os.path.isabs(p) else os.path.normpath(os.path.join(base, p))

    flips = []
    for i in range(len(keys["VolumeFile"])):
        f = keys["VolumeFlip"][i].split() if i < len(keys["VolumeFlip"]) else []
        flips.append(tuple(int(x) for x in (f + ["0", "0", "0"])[:3]))
    rw = rh = 512
    if keys["RenderResolution"]:
        r = keys["RenderResolution"][-1].split()
        rw, rh = int(r[0]), int(r[1])
    offsets = (0.1,) * 6
    if keys["OptimizationOffsets"]:
        offsets = tuple(float(x) for x in keys["OptimizationOffsets"][-1].split()[:6])
    return TrialFile(path, version, [resolve(p) for p in keys["mayaCam_csv"]],
                     [resolve(p) for p in keys["CameraRootDir"]], [resolve(p) for p in keys["VolumeFile"]],
                     [tuple(float(x) for x in v.split()[:3]) for v in keys["VoxelSize"]], flips, rw, rh, offsets,
                     [resolve(p) for p in keys["MeshFile"]])


def load_trial(path: str, frame: int = 0, vie: Optional[List[str]] = None,
               ray: Optional[S.RayParams] = None) -> S.Scene:
    """A Scene of a trial at one frame: its cameras, volumes (pivot at the
    volume centre, as Tracker::load's centre pivot), the frame's radiograph of
    each camera, per-view settings from .vie files (one per camera, optional)
    and the render resolution.  Poses start at the identity."""
    t = read_cfg(path)
    cams = [read_camera(c) for c in t.cameras]
    vols = [read_volume(v, s, f, subject=os.path.basename(v)) for v, s, f in zip(t.volumes, t.voxel_sizes, t.flips)]
    views = []
    rays = []
    for i, (cam, vdir) in enumerate(zip(cams, t.videos)):
        frames = video_frames(vdir)
        rad = read_frame(frames[min(frame, len(frames) - 1)])
        settings = read_vie(vie[i]) if vie and i < len(vie) and vie[i] else ViewSettings()
        views.append(S.View(cam, rad, settings.drr_filters, settings.rad_filters))
        r = settings.ray or ray or S.RayParams()
        rays.append([S.RayParams(r.step, r.intensity, r.cutoff) for _ in vols])
    pivots = [S.pivot_matrix(v) for v in vols]
    poses = [np.zeros(6, np.float32) for _ in vols]
    return S.Scene(views, vols, rays, t.render_width, t.render_height, pivots, poses, 0,
                   [np.zeros(6) for _ in vols])
