"""The socket server end to end on the GPU: a trial written to disk, loaded
through the reference's protocol over TCP on 127.0.0.1, scored (getNCC
against the oracle's trackFrame), exported (getImageCropped, saveFullDRR),
optimized (optimizeFrame under both cost models and initial guesses), its
poses saved and loaded as tracking files."""
import io
import socket
import struct

import numpy as np
import pytest

import trial_files
from autoscoper_gb300 import api, formats as F, geometry as G, scene as S, server as SV
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def pack(t, *args):
    b = bytearray([t])
    for a in args:
        if isinstance(a, int):
            b += int(a).to_bytes(4, "little", signed=a < 0)
        elif isinstance(a, float):
            b += struct.pack("<d", a)
        else:
            b += a.encode("utf-8")
    return bytes(b)


class Client:
    def __init__(self, port):
        self.s = socket.create_connection(("127.0.0.1", port), timeout=600)

    def call(self, t, *args, n=1):
        self.s.sendall(pack(t, *args))
        out = b""
        while len(out) < n:
            chunk = self.s.recv(n - len(out))
            assert chunk, "connection closed"
            out += chunk
        return out

    def ok(self, t, *args):
        r = self.call(t, *args)
        assert r == bytes([t]), (t, r)

    def pose(self, v, f):
        r = self.call(6, v, f, n=49)
        return np.array(struct.unpack("<6d", r[1:]))

    def ncc(self, v, pose):
        r = self.call(8, v, *[float(x) for x in pose], n=2)
        k = r[1]
        rest = self.s.recv(8 * k, socket.MSG_WAITALL)
        return list(struct.unpack(f"<{k}d", rest))


def _with_cf(sc, cf):
    import copy
    out = copy.copy(sc)
    out.cf_model = cf
    return out


@pytest.fixture(scope="module")
def trial(tmp_path_factory):
    tmp = tmp_path_factory.mktemp("trial")
    sc0 = S.make_scene([(24, 28, 32)], 1.0, (64, 64), 1.6, filters="sobel", seed=2)
    frames = [trial_files.render_targets(sc0)] * 3   # the same target in three frames
    sc, cfg = trial_files.synthetic_trial(tmp, frames=frames)
    return sc, cfg, tmp


def test_server_end_to_end(trial):
    sc, cfg, tmp = trial
    truth = np.asarray(sc.truth[0], np.float64)
    srv = SV.Server(SV.Session(drr_dir=str(tmp / "drr")), port=0, log=io.StringIO())
    srv.start()
    c = Client(srv.port)
    try:
        assert c.call(16, n=5) == b"\x10" + struct.pack("<i", 2)
        c.ok(1, cfg)
        assert c.call(14, n=5) == b"\x0e" + struct.pack("<i", 1)
        assert c.call(15, n=5) == b"\x0f" + struct.pack("<i", 3)
        # the key inserted at frame 0 on load: the volume matrix's pose
        pivot = S.pivot_matrix(F.load_trial(cfg).volumes[0])
        assert np.allclose(c.pose(0, 0), O.keycurve_store(G.to_xyzypr(pivot)))

        # getNCC against the oracle's trackFrame on the same trial
        loaded = F.load_trial(cfg, frame=0)
        tr = O.Tracker(loaded)
        for pose in (truth, truth + [0.8, -0.5, 0.3, 1.0, -0.5, 0.7]):
            got, want = c.ncc(0, pose), tr.track_frame(0, pose)
            for g, w in zip(got, want):  # the NCC bar per view
                assert abs(g - w) <= 1e-5 * max(abs(1.0 - w), 1e-2), (got, want)

        # getImageCropped: radiograph, DRR and mask bytes of the whole image
        r = c.call(10, 0, 1, *[float(x) for x in truth], n=9)
        w, h = struct.unpack("<ii", r[1:9])
        img = c.s.recv(3 * w * h, socket.MSG_WAITALL)
        assert (w, h) == (64, 64) and len(img) == 3 * w * h
        assert img[2 * w * h:].count(255) > 0   # the mask covers the bone

        # setPose / getPose through the key curves
        start = truth + [1.0, -0.8, 0.6, 1.2, -1.0, 0.8]
        c.ok(7, 0, 0, *[float(x) for x in start])
        assert np.array_equal(c.pose(0, 0), O.keycurve_store(start))
        # optimizeFrame at frame 0 (PSO + simplex, NCC, start from the curve)
        c.ok(11, 0, 0, 1, 40, -1.5, 1.5, 6, 1, 0, 0, 0)
        p0 = c.pose(0, 0)
        before = sum(c.ncc(0, O.keycurve_store(start)))
        after = sum(c.ncc(0, p0))
        assert after < before
        assert np.linalg.norm(p0[:3] - truth[:3]) < np.linalg.norm(start[:3] - truth[:3])
        # frame 1 from the previous frame's pose (guess 1), simplex only
        c.ok(11, 0, 1, 1, 40, -1.5, 1.5, 6, 1, 1, 0, 1)
        p1 = c.pose(0, 1)
        assert sum(c.ncc(0, p1)) <= after + 1e-4  # the simplex keeps its best vertex (rounded on storage)
        # a hidden volume renders zeros: the empty-mask cost in every view
        c.ok(17, 0, 0)
        assert c.ncc(0, truth) == [1.0 - 1e5, 1.0 - 1e5]
        c.ok(17, 0, 1)
        # frame 2 under the SAD cost model with a linear-extrapolation guess;
        # getNCC then scores SAD too (the tracker keeps the last cost model)
        c.ok(11, 0, 2, 1, 20, -1.0, 1.0, 4, 1, 0, 1, 2)
        assert np.all(np.isfinite(c.pose(0, 2)))
        assert np.allclose(c.ncc(0, truth), O.Tracker(_with_cf(loaded, 1)).track_frame(0, truth), rtol=1e-5)
        c.ok(17, 0, 0)
        assert c.ncc(0, truth) == [0.0, 0.0]
        c.ok(17, 0, 1)

        # tracking files: save, overwrite the curves, load back
        tra = str(tmp / "out" / "bone.tra")
        c.ok(3, 0, 1, 1, 1, 0, 0, 0, tra)
        saved = [c.pose(0, f) for f in range(3)]
        c.ok(7, 0, 1, *[0.0] * 6)
        c.ok(2, 0, 1, 1, 1, 0, 0, 0, tra)
        for f in range(3):
            assert np.allclose(c.pose(0, f), saved[f], atol=1e-4)
        assert c.call(2, 0, 1, 1, 1, 0, 0, 0, str(tmp / "missing.tra")) == b"\x00"

        # background images from the videos, then the full DRR export
        c.ok(9, 0.2)
        c.ok(12)
        for k in range(2):
            head = open(tmp / "drr" / f"image_cam{k:02d}.pgm").read().split("\n")[:3]
            assert head == ["P2", "64 64", "255"]
        c.ok(5, 1)
        c.s.sendall(pack(13))
        assert c.s.recv(1) == b""
    finally:
        c.s.close()
        srv.shutdown()
        srv.server_close()


def test_session_matches_engine_image_bytes(trial):
    """getImageData's bytes are the engine's images (asc_engine_image_data,
    checked against the oracle elsewhere) as the reference casts them,
    (unsigned char)(255 v)."""
    sc, cfg, tmp = trial
    ses = SV.Session()
    ses.open_trial(cfg)
    truth = np.asarray(sc.truth[0], np.float64)
    w, h, data = ses.get_image_data(0, 0, truth)
    rad, drr, mask = ses._engine(0).image_data(0, 0, truth)
    assert data == api.to_u8(rad).tobytes() + api.to_u8(drr).tobytes() + api.to_u8(mask).tobytes()
    assert (w, h) == (64, 64) and mask.max() == 1.0
