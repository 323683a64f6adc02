"""asc_ncc_noalloc: the NCC entry point for callers that cannot allocate
device memory (an application that keeps a fixed device-memory budget, or a
loop that cannot pay cudaMalloc's device-wide synchronisation).  Called
through the C ABI, it must return what asc_ncc returns for the same inputs,
on two calls in a row (the shared fixed array keeps the previous call's
contents), agree with the FP64 oracle's NCC within the NCC bar (1e-5
relative), and reject sizes above ASC_NOALLOC_MAX_N.

The file name makes pytest collect it after every other test file."""
import ctypes as C

import numpy as np
import pytest

from autoscoper_gb300 import _lib as L
from autoscoper_gb300 import api
from oracle import oracle as O

pytestmark = pytest.mark.gpu

ASC_NOALLOC_MAX_N = 1 << 24
TOL = 1e-12  # same kernel and same summation order as asc_ncc
TOL_ORACLE = 1e-5  # the NCC bar against the FP64 oracle, relative


def _inputs(n, seed):
    rng = np.random.default_rng(seed)
    f = rng.uniform(0, 1, n).astype(np.float32)
    g = (0.7 * f + 0.3 * rng.uniform(0, 1, n)).astype(np.float32)
    m = (rng.uniform(size=n) > 0.25).astype(np.float32)
    return f * m, g * m, m


def _result(lib, name, f, g, m, n, coverage):
    res = api.DeviceArray((1,), np.float64)
    st = getattr(lib, name)(f.ptr, g.ptr, m.ptr, n, coverage, res.ptr, None)
    assert st == L.ASC_OK, (name, st, lib.asc_last_error())
    L.call("asc_device_sync")
    return float(res.to_host()[0])


@pytest.mark.parametrize("coverage", [L.ASC_SUM_TREE, L.ASC_SUM_FULL])
def test_noalloc_matches_ncc_twice(coverage):
    lib = L.load()
    for call, (n, seed) in enumerate([(153600, 1), (70001, 2)]):
        f, g, m = _inputs(n, seed)
        df, dg, dm = (api.DeviceArray.from_host(x) for x in (f, g, m))
        want = _result(lib, "asc_ncc", df, dg, dm, n, coverage)
        got = _result(lib, "asc_ncc_noalloc", df, dg, dm, n, coverage)
        assert abs(got - want) <= TOL * max(1.0, abs(want)), (call, got, want)
        ref = O.ncc(f, g, m, tree=coverage == L.ASC_SUM_TREE)
        assert abs(got - ref) <= TOL_ORACLE * abs(ref), (call, got, ref)


def test_noalloc_rejects_oversize():
    lib = L.load()
    d = api.DeviceArray((4,), np.float32)
    res = api.DeviceArray((1,), np.float64)
    st = lib.asc_ncc_noalloc(d.ptr, d.ptr, d.ptr, ASC_NOALLOC_MAX_N + 1, L.ASC_SUM_FULL, res.ptr, None)
    assert st == -4  # ASC_ERR_RANGE
    assert b"ASC_NOALLOC_MAX_N" in lib.asc_last_error()
