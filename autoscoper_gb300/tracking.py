"""Tracking files (.tra): one line per frame, per volume either 16 matrix
values (CoordFrame::to_matrix, written row by row or column by column) or
six xyzypr values, separated by commas or spaces, "NaN" where a frame holds
no key -- AutoscoperMainWindow::save_tracking_results and
load_tracking_results (autoscoper/src/ui/AutoscoperMainWindow.cpp:736-1106).
"""
from __future__ import annotations

import ctypes as C
import math
import re
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import _lib as L

_P = C.POINTER(C.c_double)
# the longest leading decimal number of a token, as `istream >> double` reads it
_NUM = re.compile(r"\s*([+-]?(?:\d+\.?\d*(?:[eE][+-]?\d+)?|\.\d+(?:[eE][+-]?\d+)?))")
# to_matrix index order of a row-by-row line (AutoscoperMainWindow.cpp:816-818)
ROW_ORDER = (0, 4, 8, 12, 1, 5, 9, 13, 2, 6, 10, 14, 3, 7, 11, 15)


def pose_to_matrix(xyzypr) -> np.ndarray:
    """CoordFrame::from_xyzypr(...).to_matrix (column-major 4 x 4)."""
    v = np.ascontiguousarray(xyzypr, np.float64)
    m = np.zeros(16)
    L.call("asc_pose_to_matrix", v.ctypes.data_as(_P), m.ctypes.data_as(_P))
    return m


def pose_from_matrix(m) -> np.ndarray:
    """CoordFrame::from_matrix(m).to_xyzypr."""
    a = np.ascontiguousarray(m, np.float64)
    v = np.zeros(6)
    L.call("asc_pose_from_matrix", a.ctypes.data_as(_P), v.ctypes.data_as(_P))
    return v


def _fixed16(v: float) -> str:
    return "%.16f" % v  # std::fixed with precision 16


def write_tracking(path: str, rows: Sequence[Sequence[Optional[np.ndarray]]], as_matrix: bool = True,
                   as_rows: bool = True, commas: bool = True, cm: bool = False, rad: bool = False) -> None:
    """rows[frame][volume]: the pose (xyzypr) to write, or None for a frame
    without keys (written as NaN)."""
    s = "," if commas else " "
    with open(path, "w") as fh:
        for frame in rows:
            cells = []
            for pose in frame:
                if pose is None:
                    cells.append(s.join(["NaN"] * (16 if as_matrix else 6)))
                    continue
                x = np.array(pose, np.float64)
                if as_matrix:
                    m = pose_to_matrix(x)
                    if cm:
                        m[12:15] /= 10.0
                    vals = [m[i] for i in ROW_ORDER] if as_rows else list(m)
                else:
                    if cm:
                        x[:3] /= 10.0
                    if rad:
                        x[3:] *= math.pi / 180.0
                    vals = list(x)
                cells.append(s.join(_fixed16(v) for v in vals))
            fh.write(s.join(cells) + "\n")


def _read_double(token: str) -> float:
    m = _NUM.match(token)
    return float(m.group(1)) if m else 0.0  # a failed extraction stores 0


def read_tracking(path: str, n_frames: int, n_volumes: int, as_matrix: bool = True, as_rows: bool = True,
                  commas: bool = True, cm: bool = False, rad: bool = False) -> List[Tuple[int, int, np.ndarray]]:
    """The keys a tracking file inserts, in order: (frame, volume offset,
    xyzypr).  As the reference reads it: at most n_frames lines; per volume
    the next 16 (matrix) or 6 values split at the separator, values missing
    from a short line keep the previous ones, and a volume whose last value
    read starts with "NaN" inserts nothing.  The pose inserted is the
    stored one the reference builds: xyzypr as given, or of the matrix."""
    sep = "," if commas else " "
    n = 16 if as_matrix else 6
    m = np.zeros(16)
    value = ""
    out = []
    with open(path, newline="") as fh:
        lines = fh.read().split("\n")
    if lines and lines[-1] == "":
        lines.pop()
    lines = [ln[:-1] if ln.endswith("\r") else ln for ln in lines]
    for i, line in enumerate(lines[:n_frames]):
        pos, eof = 0, False
        for k in range(n_volumes):
            for j in range(n):
                # std::getline(lineStream, value, sep)
                if eof:
                    break
                end = line.find(sep, pos)
                if end < 0:
                    value, pos, eof = line[pos:], len(line), True
                    if not value:
                        break
                else:
                    value, pos = line[pos:end], end + 1
                m[j] = _read_double(value)
            if value[:3] == "NaN":
                continue
            # the values are converted in place, so a short line later reads
            # what this one left behind
            if as_matrix and as_rows:
                m[:] = m[list(ROW_ORDER)]  # the transpose
            if cm:
                if as_matrix:
                    m[12:15] *= 10.0
                else:
                    m[:3] *= 10.0
            if rad and not as_matrix:
                m[3:6] *= 180.0 / math.pi
            if as_matrix:
                m[:6] = pose_from_matrix(m)  # CoordFrame::from_matrix(m).to_xyzypr(m)
            out.append((i, k, m[:6].copy()))
    return out
