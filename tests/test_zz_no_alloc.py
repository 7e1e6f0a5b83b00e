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


def _noalloc(torch, A, lib, a, b):
    da = [torch.from_numpy(x).cuda() for x in a]
    db = [torch.from_numpy(x).cuda() for x in b]
    pa = (C.c_void_p * len(a))(*[t.data_ptr() for t in da])
    pb = (C.c_void_p * len(b))(*[t.data_ptr() for t in db])
    torch.cuda.synchronize()
    out = C.c_double()
    A.check(lib.pl_residual_device_noalloc(C.c_longlong(a[0].size), C.c_int(len(a)), pa, pb, None, C.byref(out)))
    return out.value


def test_noalloc_residual_matches_host_entry_point(env):
    torch, A, lib, lp = env
    rng = np.random.default_rng(11)
    # two calls in a row: the second reuses the scratch the first left behind; sizes exercise the
    # capped 1024-block grid (300,000 values) and a small grid (1,000 values)
    for n, ncomp in ((300000, 3), (1000, 2)):
        a = [rng.standard_normal(n) for _ in range(ncomp)]
        b = [x + 1e-3 * rng.standard_normal(n) for x in a]
        ref = lp.residual_host(a, b)
        got = _noalloc(torch, A, lib, a, b)
        assert abs(got - ref) <= 1e-14 * abs(ref), (n, ncomp, got, ref)


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
