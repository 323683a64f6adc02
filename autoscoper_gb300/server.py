"""The socket front door of the reference (autoscoper/src/net/Socket.cpp,
protocol version 2) over this library.

`Session` holds what AutoscoperMainWindow keeps for a socket client -- the
trial (cameras, videos, volumes), each volume's pose curves, the current
frame, per-camera view settings (filters, ray-caster settings), the
background threshold and volume visibility -- and answers the window's calls
(AutoscoperMainWindow.cpp: openTrial, load/save_tracking_results,
loadFilterSettings, setFrame, getPose, setPose, getNCC, setBackground,
getImageData, optimizeFrame, saveFullDRR, getNumVolumes, getNumFrames,
setVolumeVisibility) with the batched engine: one engine per (volume, cost
model) over that volume alone, as Tracker::trackFrame renders one volume.

`Server` is a TCP server on 127.0.0.1 speaking the reference's binary
protocol: a message is one type byte followed by little-endian int32 and
float64 fields and, for the file commands, a trailing UTF-8 path; the answer
starts with the type byte (0 on failure) followed by its payload
(Socket.cpp:77-443).  Messages are handled one at a time, as the reference's
event loop does.

    python -m autoscoper_gb300.server [--port 30007]
"""
from __future__ import annotations

import argparse
import os
import select
import socket
import socketserver
import stat
import struct
import sys
import threading
from typing import Dict, List, Optional, Tuple

import numpy as np

from . import _lib as L
from . import api
from . import formats as F
from . import geometry as G
from . import scene as S
from . import tracking as T

VERSION = 2          # AUTOSCOPER_SOCKET_VERSION
PORT = 30007         # the port PyAutoscoper connects to
N_PARTICLES = 100    # NUM_OF_PARTICLES of the reference's PSO


class SessionError(RuntimeError):
    pass


class Session:
    """A trial open for a client, with the engines that score it."""

    def __init__(self, storage: int = L.ASC_STORE_U16, coverage: int = L.ASC_SUM_TREE, drr_dir: Optional[str] = None,
                 seed: int = 1, frame_cache: int = 4):
        self.storage, self.coverage, self.seed = storage, coverage, seed
        self.drr_dir = drr_dir
        self.frame_cache = frame_cache
        self.trial: Optional[F.TrialFile] = None
        self._drr_count = 0

    # ------------------------------------------------------------ trial
    def open_trial(self, path: str) -> None:
        """AutoscoperMainWindow::openTrial (:1140-1230): the trial, the
        default view settings (xParameters/control_settings.vie beside the
        trial, for every camera) and tracking files (Tracking/<task>_<volume>.tra,
        matrix by rows with commas), then a key at frame 0 for volume 0."""
        t = F.read_cfg(path)
        cams = [F.read_camera(c) for c in t.cameras]
        vols = [F.read_volume(v, s, f, subject=os.path.basename(v)) for v, s, f in zip(t.volumes, t.voxel_sizes,
                                                                                       t.flips)]
        videos = [F.video_frames(d) for d in t.videos]
        if any(len(v) == 0 for v in videos):
            raise SessionError("a camera's video holds no frames")
        self.trial, self.cams, self.volumes, self.videos = t, cams, vols, videos
        self.num_frames = max(len(v) for v in videos)
        self.pivots = [S.pivot_matrix(v) for v in vols]
        self.settings = [F.ViewSettings() for _ in cams]
        self.curves = [api.PoseCurve() for _ in vols]
        self.visible = [True] * len(vols)
        self.backgrounds: Optional[List[np.ndarray]] = None
        self.bg_threshold = -1.0
        self.cf_model = 0
        self.current_volume = 0
        self.frame = 0
        self._host_frames: Dict[Tuple[int, int], np.ndarray] = {}
        self._dev_frames: Dict[int, List[api.DeviceImage]] = {}
        self._engines: Dict[Tuple[int, int], api.Engine] = {}
        self.dev_volumes = [api.DeviceVolume(v, self.storage) for v in vols]
        root = os.path.dirname(os.path.abspath(path))
        vie = os.path.join(root, "xParameters", "control_settings.vie")
        if os.path.exists(vie):
            for c in range(len(cams)):
                self.load_filter_settings(c, vie)
        task = os.path.basename(path)
        task = task[:task.find(".cfg")] if ".cfg" in task else task
        for v, vf in enumerate(t.volumes):
            name = os.path.splitext(os.path.basename(vf))[0]  # QFileInfo::completeBaseName
            tra = os.path.join(root, "Tracking", f"{task}_{name}.tra")
            if os.path.exists(tra):
                self.load_tracking_results(tra, True, True, True, False, False, False, v)
        # on_actionInsert_Key_triggered (:1874-1886): the manipulator's pose,
        # the curve value where volume 0 has keys, else the volume matrix
        c0, V = self.curves[0], self.pivots[0]
        manip = G.identity()
        if any(c0.keys(f) & L.ASC_CURVE_X for f in range(self.num_frames)):
            manip = G.mul(G.from_xyzypr(c0.eval(0)), G.inverse(V))  # update_xyzypr_and_coord_frame (:400-424)
        c0.insert(0, G.to_xyzypr(G.mul(manip, V)))

    def _need_trial(self):
        if self.trial is None:
            raise SessionError("no trial loaded")

    def _check_volume(self, v: int):
        self._need_trial()
        if not 0 <= v < len(self.volumes):
            raise SessionError(f"volume {v} out of range")

    # ------------------------------------------------------------ frames
    def _host_frame(self, cam: int, frame: int) -> np.ndarray:
        files = self.videos[cam]
        key = (cam, min(frame, len(files) - 1))  # Video::set_frame clamps (Video.cpp:220-224)
        img = self._host_frames.get(key)
        if img is None:
            if len(self._host_frames) >= self.frame_cache * len(self.cams):
                self._host_frames.pop(next(iter(self._host_frames)))
            img = self._host_frames[key] = F.read_frame(files[key[1]])
        return img

    def _device_frame(self, frame: int) -> List[api.DeviceImage]:
        imgs = self._dev_frames.get(frame)
        if imgs is None:
            if len(self._dev_frames) >= self.frame_cache:
                self._dev_frames.pop(next(iter(self._dev_frames)))
            imgs = self._dev_frames[frame] = [api.DeviceImage(self._host_frame(c, frame))
                                              for c in range(len(self.cams))]
        return imgs

    def set_frame(self, frame: int) -> None:
        self._need_trial()
        self.frame = frame

    # ------------------------------------------------------------ engines
    def _engine(self, v: int) -> api.Engine:
        """The engine of volume v under the current cost model, with the
        current frame's radiographs."""
        self._check_volume(v)
        rads = self._device_frame(self.frame)
        key = (v, self.cf_model)
        eng = self._engines.get(key)
        if eng is None:
            views = []
            for c, cam in enumerate(self.cams):
                st = self.settings[c]
                bg = self.backgrounds[c] if self.backgrounds is not None else None
                views.append(S.View(cam, self._host_frame(c, self.frame), list(st.drr_filters), list(st.rad_filters),
                                    bg, self.bg_threshold if bg is not None else -1.0))
            rays = [[self.settings[c].ray or S.RayParams()] for c in range(len(self.cams))]
            sc = S.Scene(views, [self.volumes[v]], rays, self.trial.render_width, self.trial.render_height,
                         [self.pivots[v]], [np.zeros(6, np.float32)], self.cf_model, [np.zeros(6)])
            eng = api.Engine(sc, max_items=N_PARTICLES, coverage=self.coverage, volumes=[self.dev_volumes[v]],
                             images=list(rads))
            self._engines[key] = eng
        for c, img in enumerate(rads):
            if eng.rads[c] is not img:
                eng.set_radiograph(c, img)
        eng.set_visible(0, self.visible[v])
        return eng

    def _drop_engines(self):
        self._engines.clear()

    # ------------------------------------------------------------ settings
    def load_filter_settings(self, camera: int, path: str) -> None:
        """loadFilterSettings: a camera's filters and ray-caster settings."""
        self._need_trial()
        if not 0 <= camera < len(self.cams):
            raise SessionError(f"camera {camera} out of range")
        self.settings[camera] = F.read_vie(path)
        self._drop_engines()

    def set_background(self, threshold: float) -> None:
        """setBackground (:879-896): the first time, each video's background
        image (Video::create_background_image); then the views' threshold."""
        self._need_trial()
        if self.bg_threshold < 0:
            self.backgrounds = [api.background_from_frames([F.read_frame(f) for f in files])
                                for files in self.videos]
        self.bg_threshold = float(threshold)
        self._drop_engines()

    def set_volume_visibility(self, volume: int, visible: bool) -> None:
        self._check_volume(volume)
        self.visible[volume] = bool(visible)

    # ------------------------------------------------------------ poses
    def _frame_arg(self, frame: int) -> int:
        return self.frame if frame == -1 else frame  # getPose/setPose: -1 is the current frame

    def get_pose(self, volume: int, frame: int) -> np.ndarray:
        self._check_volume(volume)
        return self.curves[volume].eval(self._frame_arg(frame))

    def set_pose(self, volume: int, frame: int, pose) -> None:
        self._check_volume(volume)
        self.curves[volume].insert(self._frame_arg(frame), np.asarray(pose, np.float64))

    def load_tracking_results(self, path: str, as_matrix: bool, as_rows: bool, commas: bool, cm: bool, rad: bool,
                              interpolate: bool, volume: int) -> bool:
        """load_tracking_results (:984-1106): the curves of `volume` (-1: all)
        cleared, then the file's keys inserted."""
        self._need_trial()
        if not os.path.exists(path):
            return False
        vols = range(len(self.volumes)) if volume == -1 else [volume]
        for v in vols:
            self._check_volume(v)
            self.curves[v].clear()
        for frame, k, pose in T.read_tracking(path, self.num_frames, len(vols), as_matrix, as_rows, commas, cm, rad):
            self.curves[vols[k]].insert(frame, pose)
        return True

    def save_tracking_results(self, path: str, as_matrix: bool, as_rows: bool, commas: bool, cm: bool, rad: bool,
                              interpolate: bool, volume: int) -> bool:
        """Socket case 3 and save_tracking_results (:736-840): the parent
        directory is created and must be writable; frames without a key in
        any of a volume's curves are NaN unless `interpolate`."""
        self._need_trial()
        if os.path.isdir(path):
            return False
        parent = os.path.dirname(path) or "."
        try:
            os.makedirs(parent, exist_ok=True)
        except OSError:
            return False
        if not os.stat(parent).st_mode & (stat.S_IWUSR | stat.S_IWGRP | stat.S_IWOTH):
            return False
        vols = range(len(self.volumes)) if volume == -1 else [volume]
        for v in vols:
            self._check_volume(v)
        rows = []
        for f in range(self.num_frames):
            rows.append([self.curves[v].eval(f) if interpolate or self.curves[v].keys(f) else None for v in vols])
        T.write_tracking(path, rows, as_matrix, as_rows, commas, cm, rad)
        return True

    # ------------------------------------------------------------ scoring
    def get_ncc(self, volume: int, pose) -> List[float]:
        """getNCC -> Tracker::trackFrame (Tracker.cpp:583-773): per view the
        cost of the volume at `pose` against the current frame."""
        eng = self._engine(volume)
        eng.set_base_pose(0, pose, exact=True)
        _, vcost = eng.eval(np.zeros(1, np.int32), np.zeros((1, 6)))
        return [float(c) for c in vcost[0]]

    def get_image_data(self, volume: int, camera: int, pose) -> Tuple[int, int, bytes]:
        """getImageData -> Tracker::getImageData (Tracker.cpp:865-921): the
        radiograph, DRR and mask of the whole image as bytes (255 v)."""
        eng = self._engine(volume)
        if not 0 <= camera < len(self.cams):
            raise SessionError(f"camera {camera} out of range")
        rad, drr, mask = eng.image_data(camera, 0, np.asarray(pose, np.float64))
        h, w = rad.shape
        return w, h, b"".join(api.to_u8(a).tobytes() for a in (rad, drr, mask))

    def optimize_frame(self, volume: int, frame: int, repeats: int, max_iter: int, min_limit: float,
                       max_limit: float, stall_iter: int, dframe: int, opt_method: int, cf_model: int,
                       guess: int) -> Tuple[float, int]:
        """optimizeFrame -> Tracker::optimize (Tracker.cpp:337-580) of one
        volume at one frame: PSO (the reference's 100 particles, max_iter + 1
        epochs at most, stopped by max_stall_iter stalls) then Downhill
        Simplex, or the simplex alone; the result goes into the curves.
        Returns (cost, evaluations)."""
        self._check_volume(volume)
        if opt_method not in (0, 1) or cf_model not in (0, 1):
            raise SessionError("opt_method and cf_model are 0 or 1")
        self.current_volume = volume
        self.cf_model = cf_model
        if frame < 0 or frame >= self.num_frames:
            print(f"optimize: invalid frame {frame}", file=sys.stderr)  # Tracker::optimize returns (:363-366)
            return 0.0, 0
        self.frame = frame
        eng = self._engine(volume)
        cost, ev = eng.optimize_curves([self.curves[volume]], frame, self.num_frames, method=opt_method,
                                       n_particles=N_PARTICLES, n_iter=max_iter + 1, lo=min_limit, hi=max_limit,
                                       seed=self.seed + frame, offsets=self.trial.offsets, repeats=repeats,
                                       guess=guess, dframe=dframe, max_stall=stall_iter)
        return float(cost[0]), ev

    def save_full_drr(self) -> List[str]:
        """saveFullDRR -> Tracker::getFullDRR (Tracker.cpp:1035-1081): per
        view the current volume's masked DRR over the whole image at its
        pose in the curves, written as an ASCII PGM (save_full_drr,
        Tracker.cpp:155-205: min-max scaled, 255 - v, rows as rendered)."""
        self._need_trial()
        eng = self._engine(self.current_volume)
        pose = self.curves[self.current_volume].eval(self.frame)
        out_dir = self.drr_dir or os.path.join(os.path.dirname(os.path.abspath(self.trial.path)), "my_drr")
        os.makedirs(out_dir, exist_ok=True)
        paths = []
        for c in range(len(self.cams)):
            _, drr, _ = eng.image_data(c, 0, pose)
            img = drr.astype(np.float32).reshape(-1)
            lo = np.float32(min(np.float32(np.finfo(np.float32).max), img.min()))
            hi = np.float32(max(np.float32(np.finfo(np.float32).tiny), img.max()))  # numeric_limits<float>::min()
            with np.errstate(divide="ignore", invalid="ignore"):
                scaled = (np.float32(255) * (img - lo)) / (hi - lo)
            u8 = np.where(np.isfinite(scaled), scaled, 0).astype(np.int64).astype(np.uint8)
            p = os.path.join(out_dir, "image_cam%02d.pgm" % self._drr_count)
            self._drr_count += 1
            h, w = drr.shape
            with open(p, "w") as fh:
                fh.write(f"P2\n{w} {h}\n255\n")
                fh.write("".join(f"{255 - int(v)} " for v in u8))
            paths.append(p)
        return paths

    def num_volumes(self) -> int:
        self._need_trial()
        return len(self.volumes)

    def num_frames_(self) -> int:
        self._need_trial()
        return self.num_frames


# ---------------------------------------------------------------- protocol

# fixed message lengths (type byte included); the file commands are variable
FIXED = {0: 1, 5: 5, 6: 9, 7: 57, 8: 53, 9: 9, 10: 57, 11: 53, 12: 1, 13: 1, 14: 1, 15: 1, 16: 1, 17: 9}
FILE_HEAD = {1: 1, 2: 29, 3: 29, 4: 5}


def _i(data: bytes, off: int) -> int:
    return struct.unpack_from("<i", data, off)[0]


def _d6(data: bytes, off: int) -> np.ndarray:
    return np.array(struct.unpack_from("<6d", data, off))


def handle_message(session: Session, data: bytes, log=sys.stderr) -> Optional[bytes]:
    """The answer to one message (Socket::handleMessage, Socket.cpp:77-443);
    None closes the connection."""
    t = data[0]
    try:
        if t == 0:
            return b"\x00"
        if t == 1:
            path = data[1:].decode("utf-8")
            if not os.path.exists(path):
                print(f"Cannot find {path}", file=log)
                return b"\x00"
            try:
                session.open_trial(path)
                return b"\x01"
            except Exception as e:  # Trial's parse errors: openTrial returns false
                print(f"load trial {path}: {e}", file=log)
                return b"\x00"
        if t in (2, 3):
            vol, mat, rows, commas, cm, rad, interp = struct.unpack_from("<7i", data, 1)
            path = data[29:].decode("utf-8")
            fn = session.load_tracking_results if t == 2 else session.save_tracking_results
            ok = fn(path, bool(mat), bool(rows), bool(commas), bool(cm), bool(rad), bool(interp), vol)
            return bytes([t if ok else 0])
        if t == 4:
            cam = _i(data, 1)
            path = data[5:].decode("utf-8")
            if not os.path.exists(path):
                print(f"Cannot find {path}", file=log)
                return b"\x00"
            session.load_filter_settings(cam, path)
            return b"\x04"
        if t == 5:
            session.set_frame(_i(data, 1))
            return b"\x05"
        if t == 6:
            pose = session.get_pose(_i(data, 1), _i(data, 5))
            return b"\x06" + struct.pack("<6d", *pose)
        if t == 7:
            session.set_pose(_i(data, 1), _i(data, 5), _d6(data, 9))
            return b"\x07"
        if t == 8:
            ncc = session.get_ncc(_i(data, 1), _d6(data, 5))
            return b"\x08" + bytes([len(ncc)]) + struct.pack(f"<{len(ncc)}d", *ncc)
        if t == 9:
            session.set_background(struct.unpack_from("<d", data, 1)[0])
            return b"\x09"
        if t == 10:
            w, h, img = session.get_image_data(_i(data, 1), _i(data, 5), _d6(data, 9))
            return b"\x0a" + struct.pack("<ii", w, h) + img
        if t == 11:
            vol, frame, repeats, max_iter = struct.unpack_from("<4i", data, 1)
            lo, hi = struct.unpack_from("<2d", data, 17)
            stall, dframe, method, cf, guess = struct.unpack_from("<5i", data, 33)
            session.optimize_frame(vol, frame, repeats, max_iter, lo, hi, stall, dframe, method, cf, guess)
            return b"\x0b"
        if t == 12:
            session.save_full_drr()
            return b"\x0c"
        if t == 13:
            return None
        if t == 14:
            return b"\x0e" + struct.pack("<i", session.num_volumes())
        if t == 15:
            return b"\x0f" + struct.pack("<i", session.num_frames_())
        if t == 16:
            return b"\x10" + struct.pack("<i", VERSION)
        if t == 17:
            session.set_volume_visibility(_i(data, 1), bool(_i(data, 5)))
            return b"\x11"
        print("Cannot handle message", file=log)
        return b"\x00"
    except (SessionError, L.AscError, struct.error, UnicodeDecodeError, ValueError, OSError, IndexError) as e:
        # a failed command answers 0 and the server keeps serving (the
        # reference's window would have shown the error)
        print(f"message {t}: {type(e).__name__}: {e}", file=log)
        return b"\x00"


def split_message(buf: bytes) -> Tuple[Optional[bytes], bytes]:
    """(one complete message, the rest) of what a connection has received;
    (None, buf) while a fixed-size message is incomplete.  A file command
    takes everything received (its path runs to the end)."""
    if not buf:
        return None, buf
    t = buf[0]
    n = FIXED.get(t)
    if n is None:
        if t in FILE_HEAD and len(buf) < FILE_HEAD[t]:
            return None, buf
        return buf, b""
    if len(buf) < n:
        return None, buf
    return buf[:n], buf[n:]


class _Handler(socketserver.BaseRequestHandler):
    def handle(self):
        srv: Server = self.server  # type: ignore[assignment]
        sock: socket.socket = self.request
        buf = b""
        while True:
            msg, buf = split_message(buf)
            if msg is None:
                chunk = sock.recv(1 << 20)
                if not chunk:
                    return
                buf += chunk
                continue
            if msg[0] in FILE_HEAD:  # the rest of a path still in flight
                while select.select([sock], [], [], 0.02)[0]:
                    more = sock.recv(1 << 20)
                    if not more:
                        break
                    msg += more
            with srv.lock:
                reply = handle_message(srv.session, msg, srv.log)
            if reply is None:
                return
            sock.sendall(reply)


class Server(socketserver.ThreadingTCPServer):
    """The reference's socket server on 127.0.0.1 (QTcpServer listening on
    QHostAddress::LocalHost); one Session, messages handled one at a time."""
    daemon_threads = True
    allow_reuse_address = True

    def __init__(self, session: Optional[Session] = None, port: int = PORT, log=sys.stderr):
        self.session = session or Session()
        self.lock = threading.Lock()
        self.log = log
        super().__init__(("127.0.0.1", port), _Handler)

    @property
    def port(self) -> int:
        return self.server_address[1]

    def start(self) -> threading.Thread:
        th = threading.Thread(target=self.serve_forever, daemon=True)
        th.start()
        return th


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--port", type=int, default=PORT)
    ap.add_argument("--storage", choices=["u16", "f16", "bf16", "f32"], default="u16")
    ap.add_argument("--drr-dir", default=None)
    a = ap.parse_args(argv)
    storage = {"u16": L.ASC_STORE_U16, "f16": L.ASC_STORE_F16, "bf16": L.ASC_STORE_BF16, "f32": L.ASC_STORE_F32}
    srv = Server(Session(storage[a.storage], drr_dir=a.drr_dir), a.port)
    print(f"listening on 127.0.0.1:{srv.port}", file=sys.stderr)
    srv.serve_forever()


if __name__ == "__main__":
    main()
