"""The socket protocol of the reference's server (Socket.cpp, version 2) and
the tracking files, on the CPU: messages packed as the reference's Python
client packs them (type byte, little-endian 4-byte ints, float64s, trailing
UTF-8 path), answered by a stub session over a real TCP connection on
127.0.0.1; .tra files written and read back through the library's
CoordFrame conversions."""
import math
import socket
import struct

import numpy as np
import pytest

from autoscoper_gb300 import server as SV
from autoscoper_gb300 import tracking as T


def pack(t, *args):
    b = bytearray([t])
    for a in args:
        if isinstance(a, bool) or isinstance(a, int):
            b += int(a).to_bytes(4, "little", signed=a < 0)
        elif isinstance(a, float):
            b += struct.pack("<d", a)
        else:
            b += a.encode("utf-8")
    return bytes(b)


class Stub:
    """Records the calls; answers with fixed values."""

    def __init__(self):
        self.calls = []
        self.frame = 0

    def __getattr__(self, name):
        def f(*a):
            self.calls.append((name, a))
            if name == "get_pose":
                return np.arange(6) + 0.5
            if name == "get_ncc":
                return [0.25, 1.5]
            if name == "get_image_data":
                return 3, 2, bytes(range(18))
            if name in ("load_tracking_results", "save_tracking_results"):
                return not a[0].endswith("missing.tra")
            if name == "num_volumes":
                return 3
            if name == "num_frames_":
                return 120
            if name == "open_trial" and a[0].endswith("bad.cfg"):
                raise ValueError("malformed")
            return None
        return f


POSE = [1.0, -2.0, 3.5, 10.0, -20.0, 30.0]


def test_split_message_sizes():
    assert SV.split_message(b"") == (None, b"")
    assert SV.split_message(pack(6, 1)) == (None, pack(6, 1))        # waits for the frame field
    msg = pack(6, 1, 2)
    assert SV.split_message(msg + b"\x10") == (msg, b"\x10")         # a second message stays buffered
    m11 = pack(11, 0, 4, 1, 1000, -3.0, 3.0, 25, 1, 0, 0, 1)
    assert len(m11) == SV.FIXED[11] and SV.split_message(m11) == (m11, b"")
    for t, args in ((7, (0, 3, *POSE)), (8, (1, *POSE)), (10, (0, 1, *POSE)), (17, (0, 1)), (9, (0.3,)), (5, (7,))):
        assert len(pack(t, *args)) == SV.FIXED[t], t
    f = pack(2, 0, 1, 1, 1, 0, 0, 0, "/x/y.tra")
    assert SV.split_message(f) == (f, b"")
    assert SV.split_message(f[:10]) == (None, f[:10])                # the head of a file command is fixed


def test_messages_reach_the_session(tmp_path):
    st = Stub()
    trial = tmp_path / "t.cfg"
    trial.write_text("")
    h = lambda m: SV.handle_message(st, m)  # noqa: E731
    assert h(pack(0)) == b"\x00"
    assert h(pack(16)) == b"\x10" + struct.pack("<i", 2)
    assert h(pack(1, str(trial))) == b"\x01" and st.calls[-1] == ("open_trial", (str(trial),))
    assert h(pack(1, str(tmp_path / "none.cfg"))) == b"\x00"
    bad = tmp_path / "bad.cfg"
    bad.write_text("")
    assert h(pack(1, str(bad))) == b"\x00"
    assert h(pack(2, 1, 1, 0, 1, 0, 1, 0, "/a/b.tra")) == b"\x02"
    assert st.calls[-1] == ("load_tracking_results", ("/a/b.tra", True, False, True, False, True, False, 1))
    assert h(pack(2, 1, 1, 0, 1, 0, 1, 0, "/a/missing.tra")) == b"\x00"
    assert h(pack(3, -1, 0, 0, 0, 1, 0, 1, "/a/c.tra")) == b"\x03"
    assert st.calls[-1] == ("save_tracking_results", ("/a/c.tra", False, False, False, True, False, True, -1))
    vie = tmp_path / "v.vie"
    vie.write_text("")
    assert h(pack(4, 1, str(vie))) == b"\x04" and st.calls[-1] == ("load_filter_settings", (1, str(vie)))
    assert h(pack(4, 1, str(tmp_path / "none.vie"))) == b"\x00"
    assert h(pack(5, 42)) == b"\x05" and st.calls[-1] == ("set_frame", (42,))
    r = h(pack(6, 2, 9))
    assert r[0] == 6 and struct.unpack("<6d", r[1:]) == tuple(np.arange(6) + 0.5)
    assert st.calls[-1] == ("get_pose", (2, 9))
    assert h(pack(7, 1, -1, *POSE)) == b"\x07"
    name, (v, f, p) = st.calls[-1]
    assert (name, v, f) == ("set_pose", 1, -1) and list(p) == POSE
    r = h(pack(8, 0, *POSE))
    assert r[:2] == b"\x08\x02" and struct.unpack("<2d", r[2:]) == (0.25, 1.5)
    assert h(pack(9, 0.35)) == b"\x09" and st.calls[-1] == ("set_background", (0.35,))
    r = h(pack(10, 0, 1, *POSE))
    assert r[0] == 10 and struct.unpack("<ii", r[1:9]) == (3, 2) and r[9:] == bytes(range(18))
    assert h(pack(11, 0, 4, 2, 1000, -3.0, 3.0, 25, -1, 1, 1, 2)) == b"\x0b"
    assert st.calls[-1] == ("optimize_frame", (0, 4, 2, 1000, -3.0, 3.0, 25, -1, 1, 1, 2))
    assert h(pack(12)) == b"\x0c" and st.calls[-1] == ("save_full_drr", ())
    assert h(pack(13)) is None
    assert h(pack(14)) == b"\x0e" + struct.pack("<i", 3)
    assert h(pack(15)) == b"\x0f" + struct.pack("<i", 120)
    assert h(pack(17, 2, 0)) == b"\x11" and st.calls[-1] == ("set_volume_visibility", (2, False))
    assert h(bytes([99])) == b"\x00"


def test_session_errors_answer_zero():
    class Failing(Stub):
        def __getattr__(self, name):
            def f(*a):
                raise SV.SessionError("no trial loaded")
            return f
    assert SV.handle_message(Failing(), pack(6, 0, 0)) == b"\x00"
    assert SV.handle_message(Failing(), pack(14)) == b"\x00"

    class LibFailing(Stub):
        def __getattr__(self, name):
            def f(*a):
                from autoscoper_gb300 import _lib as L
                raise L.AscError("asc_engine_eval_host", -3)
            return f
    import io
    log = io.StringIO()
    assert SV.handle_message(LibFailing(), pack(8, 0, *POSE), log) == b"\x00"
    assert "asc_engine_eval_host" in log.getvalue()


def _recv(sock, n):
    out = b""
    while len(out) < n:
        chunk = sock.recv(n - len(out))
        assert chunk
        out += chunk
    return out


def test_tcp_server_round_trip():
    import io
    srv = SV.Server(Stub(), port=0, log=io.StringIO())
    srv.start()
    try:
        with socket.create_connection(("127.0.0.1", srv.port), timeout=10) as c:
            c.sendall(pack(16))
            assert _recv(c, 5) == b"\x10" + struct.pack("<i", 2)
            # a message split across sends is put back together
            m = pack(7, 0, 5, *POSE)
            c.sendall(m[:20])
            c.sendall(m[20:])
            assert _recv(c, 1) == b"\x07"
            c.sendall(pack(6, 0, 5))
            r = _recv(c, 49)
            assert r[0] == 6
            c.sendall(pack(13))
            assert c.recv(1) == b""  # the server closes the connection
        assert [n for n, _ in srv.session.calls] == ["set_pose", "get_pose"]
    finally:
        srv.shutdown()
        srv.server_close()


# ---------------------------------------------------------------- tracking files

def _poses(rng, n):
    return [np.concatenate([rng.uniform(-50, 50, 3), rng.uniform(-80, 80, 3)]) for _ in range(n)]


@pytest.mark.parametrize("as_matrix,as_rows,commas,cm,rad", [
    (True, True, True, False, False), (True, False, False, True, False), (False, False, True, False, True),
    (False, False, False, True, True)])
def test_tracking_file_round_trip(tmp_path, as_matrix, as_rows, commas, cm, rad):
    rng = np.random.default_rng(3)
    frames = [[p, q] for p, q in zip(_poses(rng, 5), _poses(rng, 5))]
    frames[2][1] = None   # no key there
    path = str(tmp_path / "t.tra")
    T.write_tracking(path, frames, as_matrix, as_rows, commas, cm, rad)
    lines = open(path).read().split("\n")
    assert len(lines) == 6 and lines[-1] == ""
    assert lines[2].split("," if commas else " ")[-1] == "NaN"
    assert len(lines[0].split("," if commas else " ")) == 2 * (16 if as_matrix else 6)
    got = T.read_tracking(path, 10, 2, as_matrix, as_rows, commas, cm, rad)
    assert [(f, k) for f, k, _ in got] == [(f, k) for f in range(5) for k in range(2) if (f, k) != (2, 1)]
    for f, k, pose in got:
        want = frames[f][k]
        assert np.allclose(pose[:3], want[:3], atol=1e-12)
        d = (pose[3:] - want[3:] + 180.0) % 360.0 - 180.0
        assert np.allclose(d, 0, atol=1e-9)


def test_tracking_file_reading_rules(tmp_path):
    """Values are read as `istream >> double` reads them; at most n_frames
    lines; a short line keeps the previous line's values; a volume whose
    last value read is NaN inserts nothing."""
    path = tmp_path / "r.tra"
    path.write_text("1,2,3,4,5,6\r\n7,8\nNaN,NaN,NaN,NaN,NaN,NaN\n 9.5,x,1e1,,0,0\n1,1,1,1,1,1\n")
    got = T.read_tracking(str(path), 4, 1, as_matrix=False)
    assert [f for f, _, _ in got] == [0, 1, 3]
    assert list(got[0][2]) == [1, 2, 3, 4, 5, 6]
    assert list(got[1][2]) == [7, 8, 3, 4, 5, 6]
    assert list(got[2][2]) == [9.5, 0, 10, 0, 0, 0]


def test_tracking_matrix_is_the_coord_frame():
    p = np.array([10.0, -5.0, 2.5, 30.0, 0.0, 0.0])
    m = T.pose_to_matrix(p)
    c, s = math.cos(math.radians(30)), math.sin(math.radians(30))
    assert np.allclose(m, [c, s, 0, 0, -s, c, 0, 0, 0, 0, 1, 0, 10, -5, 2.5, 1], atol=1e-15)
    assert np.allclose(T.pose_from_matrix(m), p, atol=1e-12)
