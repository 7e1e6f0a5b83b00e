"""Failure detection through the C ABI, with every failure made on the host (no GPU fault):
non-finite populations seen by the solve loop's residual check, invalid diffusivity, mismatched
sizes, an injected device-allocation failure and a snapshot slot that was never filled."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mods():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from panslbm2_gb300 import _capi as A
    from panslbm2_gb300 import heatsink as HS
    from panslbm2_gb300.lattice import LatticePair, phys
    return A, HS, LatticePair, phys


def _heatsink(mods, storage="fp64"):
    A, HS, LatticePair, phys = mods
    p = HS.Params(2, 24, 16)
    n = p.lx * p.ly
    ss = np.clip(HS.grf_design(2, p.lx, p.ly, seed=3, sigma=2.0), 0, 1)
    alpha, kappa, _, _ = p.design_fields(ss)
    lp = LatticePair(9, p.lx, p.ly, 1, storage)
    lp.set_field(A.ALPHA, alpha)
    lp.set_field(A.KAPPA, kappa)
    lp.init(0, np.ones(n), ux=np.zeros(n), uy=np.zeros(n), uz=np.zeros(n))
    lp.init(1, np.zeros(n), ux=np.zeros(n), uy=np.zeros(n), uz=np.zeros(n))
    prog = lp.program(HS.to_descs(HS.program_ops("forward", p)))
    ph = phys(nu=p.nu, gx=p.gx, gy=p.gy, gz=p.gz, tem0=p.tem0)
    return lp, prog, ph, n


@pytest.mark.parametrize("storage", ["fp64", "fp32"])
def test_nan_populations_end_the_solve_as_diverged(mods, storage):
    A = mods[0]
    lp, prog, ph, n = _heatsink(mods, storage)
    f = lp.get_populations(0)
    f[3, n // 2] = np.nan
    lp.set_populations(0, f)
    st, steps, res = lp.solve(A.AD_NATURAL, ph, prog, max_steps=10000, check_every=50, tol=1e-6)
    assert st == A.PL_DIVERGED
    assert steps <= 2 * 50 + 1          # at the first residual check that has two saved states
    lp.close()


def test_invalid_diffusivity_is_refused(mods):
    A, _, LatticePair, _ = mods
    lp = LatticePair(9, 8, 6, 1, "fp64")
    lib = lp.lib
    for bad in (0.0, -0.01, np.nan, np.inf):
        k = np.full(lp.n, 0.05)
        k[7] = bad
        rc = lib.pl_set_field(lp.h, A.KAPPA, k.ctypes.data_as(A.DP))
        assert rc == A.PL_ERR_ARG, bad
        assert b"diffusivity" in lib.pl_last_error()
    lp.set_field(A.KAPPA, np.full(lp.n, 0.05))     # a valid field is accepted afterwards
    lp.close()


def test_mismatched_sizes_are_refused(mods):
    A, _, LatticePair, _ = mods
    lp = LatticePair(9, 8, 6, 1, "fp64")
    lib = lp.lib
    big = np.zeros(lp.n * lp.q + 1)
    assert lib.pl_normalize(lp.h, big.ctypes.data_as(A.DP), big.size) == A.PL_ERR_ARG
    a = (A.DP * 1)(big.ctypes.data_as(A.DP))
    out = C.c_double()
    assert lib.pl_residual_host(lp.h, big.size, 1, a, a, C.byref(out)) == A.PL_ERR_ARG
    assert lib.pl_residual_host(lp.h, 16, 4, a, a, C.byref(out)) == A.PL_ERR_ARG
    h = C.c_void_p()
    assert lib.pl_create(9, 0, 6, 1, A.PL_FP64, C.byref(h)) == A.PL_ERR_ARG
    assert lib.pl_create(11, 8, 6, 1, A.PL_FP64, C.byref(h)) == A.PL_ERR_ARG
    lp.close()


def test_injected_allocation_failure(mods):
    A, HS, LatticePair, phys = mods
    lib = A.load()
    h = C.c_void_p()
    try:
        for after in (0, 1, 3):
            lib.pl_debug_fail_alloc(C.c_longlong(after))
            assert lib.pl_create(9, 32, 16, 1, A.PL_FP64, C.byref(h)) == A.PL_ERR_ALLOC
            assert b"injected" in lib.pl_last_error()
        # a handle that was created before the failure: a later allocation inside a call fails
        # cleanly and the handle stays usable once allocations succeed again
        lib.pl_debug_fail_alloc(C.c_longlong(-1))
        lp = LatticePair(9, 32, 16, 1, "fp64")
        lib.pl_debug_fail_alloc(C.c_longlong(0))
        v = np.ones(lp.n)
        assert lib.pl_set_field(lp.h, A.ALPHA, v.ctypes.data_as(A.DP)) == A.PL_ERR_ALLOC
        lib.pl_debug_fail_alloc(C.c_longlong(-1))
        lp.set_field(A.ALPHA, v)
        np.testing.assert_array_equal(lp.get_field(A.ALPHA), v)
        lp.close()
    finally:
        lib.pl_debug_fail_alloc(C.c_longlong(-1))


def test_snapshot_swap_tracks_empty_slots(mods):
    """A swap with a never-filled slot moves the snapshot out; the buffer it brings back holds no
    snapshot, so loading or sensitivities from it are refused instead of reading garbage."""
    A = mods[0]
    lp, prog, ph, n = _heatsink(mods)
    lp.collide(A.AD_NATURAL, ph)
    lp.step(A.AD_NATURAL, ph, prog, save=True)
    lp.snapshot(0, host=False)
    lib = lp.lib
    lp.swap_snapshot(5)           # the snapshot moves into slot 5; slot 0 now holds no snapshot
    assert lib.pl_store(lp.h, A.STORE_SNAP, 7) == A.PL_ERR_STATE
    assert lib.pl_load(lp.h, A.STORE_SNAP, 6) == A.PL_ERR_STATE
    lp.swap_snapshot(5)           # and back: slot 0 holds it again, slot 5 is empty
    lp.store(A.STORE_SNAP, 7)
    assert lib.pl_load(lp.h, A.STORE_SNAP, 5) == A.PL_ERR_STATE
    lp.load(A.STORE_SNAP, 7)
    lp.close()
