"""CPU checks of the C ABI library: it loads, exports every entry point the
header declares, and its host-side optimizers reproduce the reference's
(oracle) trajectories exactly.  No GPU call is made."""
import ctypes
import os
import re

import numpy as np
import pytest

from autoscoper_gb300 import _lib
from autoscoper_gb300 import api
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    try:
        from autoscoper_gb300 import build
        build.build()
    except Exception as e:  # pragma: no cover
        pytest.skip(f"nvcc unavailable: {e}")
    return _lib.load()


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            src = open(os.path.join(inc, f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(asc_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


def test_exports_every_declared_symbol(lib):
    names = declared_symbols()
    assert len(names) > 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the ctypes table covers them all
    assert set(names) <= set(_lib.SIGNATURES), set(names) - set(_lib.SIGNATURES)


def test_status_strings(lib):
    assert lib.asc_status_string(0) == b"ok"
    assert lib.asc_status_string(-3) == b"empty volume"
    assert b"sm_103a" in lib.asc_version()


def test_bad_arguments_return_status_not_exit(lib):
    # argument checks run before any CUDA call
    h = ctypes.c_void_p()
    assert lib.asc_volume_create(None, 1, 1, 1, 16, None, None, 0, ctypes.byref(h)) == _lib.ASC_OK - 1
    assert lib.asc_raycast(None, None, None, 0.5, 1.0, 0.0, 1, None, 4, 4, None) == -7  # no volume: state error
    assert lib.asc_ncc(None, None, None, 10, 0, None, None) == -1
    assert lib.asc_engine_create(0, None, 0, None, 1, 1, 1, 0, 0, ctypes.byref(h)) == -1


def _quadratic(x):
    t = np.array([0.3, -0.2, 0.1, 1.0, -0.5, 0.25])
    return float(np.sum((np.asarray(x, dtype=np.float64) - t) ** 2) + 0.01)


def test_host_pso_matches_reference_sequential(lib):
    a_pos, a_val = api.pso_sequential(_quadratic, 100, -1.0, 1.0, 6, 25, 4321)
    b_pos, b_val = O.pso_reference(_quadratic, -1.0, 1.0, 6, 25, 4321)
    assert np.array_equal(a_pos, b_pos) and a_val == b_val


def test_host_amoeba_matches_reference(lib):
    P = np.zeros((7, 6))
    for i in range(1, 7):
        P[i, i - 1] = 0.1
    Y = np.array([_quadratic(p) for p in P])
    Pa, Ya, ita = api.amoeba(_quadratic, P, Y, 1e-3)
    Pb, Yb = P.copy(), Y.copy()
    itb = O.amoeba(_quadratic, Pb, Yb, 1e-3)
    assert ita == itb and np.array_equal(Pa, Pb) and np.array_equal(Ya, Yb)


def _quadratic_k(x, k):
    t = np.array([0.3, -0.2, 0.1, 1.0, -0.5, 0.25]) * (1 + 0.3 * k)
    return float(np.sum((np.asarray(x, dtype=np.float64) - t) ** 2 * (1 + 0.1 * np.arange(6))) + 0.01 * k)


def test_batched_speculative_amoeba_follows_sequential_trajectories(lib):
    """Lock-step speculative AMOEBA on 4 simplices = the reference AMOEBA on each."""
    ns = 4
    P = np.zeros((ns, 7, 6))
    for k in range(ns):
        for i in range(1, 7):
            P[k, i, i - 1] = 0.1 * (k + 1)
    Y = np.array([[_quadratic_k(p, k) for p in P[k]] for k in range(ns)])
    Pb, Yb, its = api.amoeba_batch(lambda who, X: [_quadratic_k(x, k) for k, x in zip(who, X)], P, Y, 1e-3)
    for k in range(ns):
        Pk, Yk = P[k].copy(), Y[k].copy()
        it = O.amoeba(lambda x, k=k: _quadratic_k(x, k), Pk, Yk, 1e-3)
        assert it == its[k]
        assert np.array_equal(Pk, Pb[k]) and np.array_equal(Yk, Yb[k])


def test_keycurve_store_matches_oracle(lib):
    """The pose storage of the trial's key curves (float translation, float
    quaternion rotation) is bit-identical to the oracle's restatement, which
    is pinned against the reference's Quaternion.hpp."""
    rng = np.random.default_rng(9)
    for _ in range(200):
        v = np.concatenate([rng.uniform(-80, 80, 3), rng.uniform(-179, 179, 3)])
        out = np.zeros(6)
        _lib.call("asc_keycurve_store", v.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                  out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        assert np.array_equal(out, O.keycurve_store(v)), (v, out, O.keycurve_store(v))


@pytest.mark.parametrize("seed", range(6))
def test_pose_curves_match_oracle(lib, seed):
    """asc_pose_curve (KeyCurve<float> x, y, z and KeyCurve<Quatf>, updated
    key by key as the reference does) against the oracle, which recomputes
    every tangent and segment from the final keys: bit-identical poses at
    every frame after every operation (NaN where both give NaN)."""
    import curve_cases
    from autoscoper_gb300 import api
    c, o = api.PoseCurve(), O.PoseCurves()
    for kind, f, mask, p in curve_cases.ops(seed):
        if kind == 0:
            c.insert(f, p, mask)
            o.insert(f, p, mask)
        elif kind == 1:
            c.erase(f, mask)
            o.erase(f, mask)
        else:
            c.clear()
            o.clear()
        for g in (f, f + 1, curve_cases.N_FRAMES - 1):
            km = sum(1 << k for k in range(4) if g in o.keys[k])
            assert c.keys(g) == km
        for g in curve_cases.eval_frames():
            a, b = c.eval(g), o.eval(g)
            assert np.array_equal(a, b, equal_nan=True), (seed, g, a, b)


def test_pose_curve_reads(lib):
    """Empty curves read the zero pose; one key is held at every frame; a
    stored key reads back as the key curves store it."""
    from autoscoper_gb300 import api
    c = api.PoseCurve()
    assert np.array_equal(c.eval(3), np.zeros(6))
    p = np.array([1.25, -3.5, 7.0, 20.0, -10.0, 5.0])
    c.insert(4, p)
    for f in (0, 4, 9):
        assert np.array_equal(c.eval(f), O.keycurve_store(p))
    assert c.keys(4) == 15 and c.keys(5) == 0
    c.erase(4, 8)
    assert c.keys(4) == 7 and np.array_equal(c.eval(4)[3:], np.zeros(3))


def test_tuning_table_parses(tmp_path):
    """asc_tuning_load reads the autotuner's table (host only) and rejects a
    malformed line; the committed table parses."""
    lib = _lib.load()
    good = tmp_path / "t.txt"
    good.write_text("# comment\n20 23 2 4 0 3  # headline\n\n18 21 2 3 2 2\n")
    assert lib.asc_tuning_load(str(good).encode()) == _lib.ASC_OK
    bad = tmp_path / "b.txt"
    bad.write_text("20 23 2 9 0 3\n")  # 9 ray blocks per SM: out of range
    assert lib.asc_tuning_load(str(bad).encode()) == -1
    assert lib.asc_tuning_load(str(tmp_path / "missing.txt").encode()) == -1
    if os.path.exists(_lib.TUNING):
        assert lib.asc_tuning_load(_lib.TUNING.encode()) == _lib.ASC_OK
