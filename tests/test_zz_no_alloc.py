"""pl_residual_device_noalloc (static device scratch, no allocation) against pl_residual_host
(the handle's scratch pool) through the C ABI. Collected last so it also runs after every other
GPU test has used the library on the same device."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from panslbm2_gb300 import _capi as A
    from panslbm2_gb300.lattice import LatticePair
    lib = A.load()
    lp = LatticePair(15, 80, 64, 64, "fp32")     # pl_residual_host accepts n <= 15*N/6
    yield torch, A, lib, lp
    lp.close()


def _call(torch, A, lib, a, b, stream=None, expect=0):
    """Upload a and b on `stream` (a torch stream, or None for the legacy default stream) and
    reduce them there; returns the value and the status."""
    ctx = torch.cuda.stream(stream) if stream is not None else None
    if ctx:
        ctx.__enter__()
    try:
        da = [torch.from_numpy(x).to("cuda", non_blocking=False) for x in a]
        db = [torch.from_numpy(x).to("cuda", non_blocking=False) for x in b]
    finally:
        if ctx:
            ctx.__exit__(None, None, None)
    if stream is None:
        torch.cuda.synchronize()
    pa = (C.c_void_p * len(a))(*[t.data_ptr() for t in da])
    pb = (C.c_void_p * len(b))(*[t.data_ptr() for t in db])
    out = C.c_double()
    sp = C.c_void_p(stream.cuda_stream) if stream is not None else None
    rc = lib.pl_residual_device_noalloc(C.c_longlong(a[0].size), C.c_int(len(a)), pa, pb, sp, C.byref(out))
    del da, db
    return out.value, rc


def test_noalloc_residual_matches_host_entry_point(env):
    torch, A, lib, lp = env
    rng = np.random.default_rng(11)
    # two calls in a row: the second reuses the scratch the first left behind; sizes exercise the
    # capped 1024-block grid (300,000 values) and a small grid (1,000 values)
    for n, ncomp in ((300000, 3), (1000, 2)):
        a = [rng.standard_normal(n) for _ in range(ncomp)]
        b = [x + 1e-3 * rng.standard_normal(n) for x in a]
        ref = lp.residual_host(a, b)
        got, rc = _call(torch, A, lib, a, b)
        assert rc == A.PL_OK
        assert abs(got - ref) <= 1e-14 * abs(ref), (n, ncomp, got, ref)


def test_noalloc_residual_on_created_streams(env):
    """Inputs written on a created (non-default) stream and reduced on that stream; then the same
    data on a second created stream and on the legacy default stream: all equal the host entry
    point's value."""
    torch, A, lib, lp = env
    rng = np.random.default_rng(12)
    n = 200003
    a = [rng.standard_normal(n) for _ in range(3)]
    b = [x + 1e-2 * rng.standard_normal(n) for x in a]
    ref = lp.residual_host(a, b)
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    v1, r1 = _call(torch, A, lib, a, b, stream=s1)
    v2, r2 = _call(torch, A, lib, a, b, stream=s2)
    v3, r3 = _call(torch, A, lib, a, b)
    assert (r1, r2, r3) == (A.PL_OK, A.PL_OK, A.PL_OK)
    for v in (v1, v2, v3):
        assert abs(v - ref) <= 1e-14 * abs(ref), (v, ref)
    assert v1 == v2 == v3


def test_noalloc_residual_reports_nonfinite_input(env):
    torch, A, lib, lp = env
    rng = np.random.default_rng(13)
    a = [rng.standard_normal(5000)]
    b = [a[0] * 0.5]
    a[0][1234] = np.nan
    _, rc = _call(torch, A, lib, a, b)
    assert rc == A.PL_ERR_NONFINITE
    assert b"non-finite" in lib.pl_last_error()
    # the next call on clean data starts from a cleared flag
    a[0][1234] = 0.25
    got, rc = _call(torch, A, lib, a, b)
    assert rc == A.PL_OK
    assert abs(got - lp.residual_host(a, b)) <= 1e-14 * abs(got)


def test_noalloc_residual_rejects_bad_arguments(env):
    torch, A, lib, lp = env
    x = torch.zeros(16, dtype=torch.float64, device="cuda")
    p = (C.c_void_p * 4)(*([x.data_ptr()] * 4))
    out = C.c_double()
    assert lib.pl_residual_device_noalloc(C.c_longlong(16), C.c_int(4), p, p, None, C.byref(out)) == A.PL_ERR_ARG
    assert lib.pl_residual_device_noalloc(C.c_longlong(0), C.c_int(1), p, p, None, C.byref(out)) == A.PL_ERR_ARG
    host = np.zeros(16)
    ph = (C.c_void_p * 1)(host.ctypes.data)
    assert lib.pl_residual_device_noalloc(C.c_longlong(16), C.c_int(1), ph, ph, None, C.byref(out)) == A.PL_ERR_ARG
    assert b"device" in lib.pl_last_error()
    if torch.cuda.device_count() > 1:
        y = torch.zeros(16, dtype=torch.float64, device="cuda:1")
        py = (C.c_void_p * 1)(y.data_ptr())
        assert lib.pl_residual_device_noalloc(C.c_longlong(16), C.c_int(1), py, py, None,
                                              C.byref(out)) == A.PL_ERR_ARG
