"""GPU parity: every CUDA path against the CPU oracle on the same seeded inputs.

FP64 storage runs the library's FP64 kernels, compiled without FMA contraction in the
reference's evaluation order, so populations / macros must agree to 1e-12 relative (stream and
wall BCs, pure data movement, must agree exactly). FP32 / FP16 / BF16 storage is checked with
the tolerances written beside each test.
"""
import zlib

import numpy as np
import pytest

from oracle.olib import Oracle
from panslbm2_gb300 import _capi as A
from panslbm2_gb300 import heatsink as HS
from panslbm2_gb300.lattice import LatticePair, phys
from tests._cases import field, pops
from tests._replay import replay

pytestmark = pytest.mark.gpu

SHAPES = [(9, 14, 11, 1), (15, 9, 10, 7)]
RTOL64 = 1e-12


@pytest.fixture(scope="module")
def o():
    return Oracle("oracle")


def close64(a, b, rtol=RTOL64):
    scale = max(1.0, float(np.max(np.abs(b))))
    err = float(np.max(np.abs(a - b))) / scale if a.size else 0.0
    assert err <= rtol, "max rel err %.3e" % err


def fresh(q, nx, ny, nz, storage="fp64"):
    return LatticePair(q, nx, ny, nz, storage)


# ---------------------------------------------------------------------------- streaming
@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("storage", ["fp64", "fp32"])
def test_stream_bit_exact(o, shape, mode, storage):
    q, nx, ny, nz = shape
    L = o.lat(q, nx, ny, nz)
    n = L.nx * L.ny * L.nz
    rng = np.random.default_rng(1)
    f, g = pops(rng, q, n), pops(rng, q, n, base=0.3)
    if storage == "fp32":
        f, g = f.astype(np.float32).astype(np.float64), g.astype(np.float32).astype(np.float64)
    lp = fresh(q, nx, ny, nz, storage)
    lp.set_populations(0, f)
    lp.set_populations(1, g)
    lp.stream(mode=mode, both=True)
    fa, ga = f.copy(), g.copy()
    o.stream(L, fa, inverse=bool(mode))
    o.stream(L, ga, inverse=bool(mode))
    assert np.array_equal(lp.get_populations(0), fa)
    assert np.array_equal(lp.get_populations(1), ga)


# ---------------------------------------------------------------------------- boundary ops
def _faces_with_interior(q, nx, ny, nz):
    lens = [nx, ny, nz]
    out = []
    for a in ([0, 1] if q == 9 else [0, 1, 2]):
        out += [(a, 0, -1), (a, lens[a] - 1, 1), (a, lens[a] // 2, 1), (a, lens[a] // 2, -1)]
    return out


BC_KINDS = ["WALL", "IWALL", "NS_U", "NS_RHO", "AD_T", "AD_Q", "AD_QC", "ANS_U", "ANS_RHO", "AAD_T", "AAD_Q",
            "AAD_RHO"]


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("kind", BC_KINDS)
def test_boundary_ops(o, shape, kind):
    """One boundary routine per edge/face (and interior line), program-only mode, FP64."""
    q, nx, ny, nz = shape
    L = o.lat(q, nx, ny, nz)
    n = L.nx * L.ny * L.nz
    k = getattr(A, "BC_" + kind)
    adjoint_inputs = kind in ("AAD_T", "AAD_Q", "AAD_RHO")
    rng = np.random.default_rng(zlib.crc32(("%d-%s" % (q, kind)).encode()))
    for (axis, pos, d) in _faces_with_interior(q, nx, ny, nz):
        f, g = pops(rng, q, n), pops(rng, q, n, base=0.5)
        ty = rng.integers(0, 3, n).astype(np.int32)
        if kind not in ("WALL", "IWALL", "AAD_RHO"):
            ty = (ty > 0).astype(np.int32)
        v0 = field(rng, n, 0.9, 1.1) if kind not in ("NS_U", "ANS_U") else field(rng, n, -0.05, 0.05)
        v1, v2 = field(rng, n, -0.05, 0.05), field(rng, n, -0.05, 0.05)
        ux, uy, uz = (field(rng, n, -0.05, 0.05) for _ in range(3))
        rho, tem, kap = field(rng, n, 0.95, 1.05), field(rng, n, 0, 1), field(rng, n, 0.01, 0.2)
        lat = int(rng.integers(0, 2)) if kind in ("WALL", "IWALL") else 0
        op = dict(kind=k, lat=lat, axis=axis, pos=pos, dir=d, type=ty, v0=v0, v1=v1, v2=v2, kappa=0.037, eps=0.7)
        lp = fresh(q, nx, ny, nz)
        lp.set_populations(0, f)
        lp.set_populations(1, g)
        lp.set_field(A.KAPPA, kap)
        if adjoint_inputs:
            for fid, v in ((A.FWD_RHO, rho), (A.FWD_UX, ux), (A.FWD_UY, uy), (A.FWD_UZ, uz), (A.FWD_TEM, tem)):
                lp.set_field(fid, v)
        else:
            for fid, v in ((A.UX, ux), (A.UY, uy), (A.UZ, uz)):
                lp.set_field(fid, v)
        prog = lp.program(HS.to_descs([op]))
        lp.stream(mode=3 if adjoint_inputs else 2, prog=prog, both=True)
        fa, ga = f.copy(), g.copy()
        replay(o, L, fa, ga, [op], n, ux=ux, uy=uy, uz=uz, rho=rho, tem=tem, kappa=kap)
        fg, gg = lp.get_populations(0), lp.get_populations(1)
        if kind in ("WALL", "IWALL"):
            assert np.array_equal(fg, fa) and np.array_equal(gg, ga)
        else:
            close64(fg, fa)
            close64(gg, ga)
        lp.close()


@pytest.mark.parametrize("shape", SHAPES)
def test_smoothing_program(o, shape):
    q, nx, ny, nz = shape
    L = o.lat(q, nx, ny, nz)
    n = L.nx * L.ny * L.nz
    rng = np.random.default_rng(9)
    f, g = pops(rng, q, n), pops(rng, q, n, base=0.5)
    ops = [dict(kind=A.BC_WALL, lat=0, axis=0, pos=0, dir=-1, type=np.full(n, 2, np.int32)),
           dict(kind=A.SMOOTH_CORNER, lat=0), dict(kind=A.SMOOTH_CORNER, lat=1),
           dict(kind=A.SMOOTH_AT, lat=1, i=3, j=4, k=2, di=-1, dj=1, dk=-1)]
    if q == 15:
        ops.append(dict(kind=A.SMOOTH_LINE, lat=0, axis=1, i=2, j=3, di=1, dj=-1))
    lp = fresh(q, nx, ny, nz)
    lp.set_populations(0, f)
    lp.set_populations(1, g)
    descs = HS.to_descs(ops)
    lp.stream(mode=2, prog=lp.program(descs), both=True)
    fa, ga = f.copy(), g.copy()
    replay(o, L, fa, ga, ops, n)
    assert np.array_equal(lp.get_populations(0), fa)
    assert np.array_equal(lp.get_populations(1), ga)


# ---------------------------------------------------------------------------- collides
FWD = ["NS_COLLIDE", "NS_BRINKMAN", "AD_NATURAL", "AD_FORCE", "AD_HEATEX", "AD_NATURAL_NOBRINK", "AD_FORCE_NOBRINK"]
ADJ = ["ANS_BRINKMAN", "AAD_NATURAL", "AAD_FORCE", "AAD_HEATEX", "AAD_MASSFLOW"]
FWD_NAMES = ["rho", "ux", "uy", "uz", "tem", "qx", "qy", "qz"]
ADJ_NAMES = ["ip", "iux", "iuy", "iuz", "imx", "imy", "imz", "item", "iqx", "iqy", "iqz"]


def _inputs(rng, n):
    d = dict(rho=field(rng, n, 0.95, 1.05), ux=field(rng, n, -0.05, 0.05), uy=field(rng, n, -0.05, 0.05),
             uz=field(rng, n, -0.05, 0.05), tem=field(rng, n, -0.5, 0.5), alpha=field(rng, n, 0.0, 0.2),
             diffusivity=field(rng, n, 0.01, 0.2), beta=field(rng, n, 0.0, 0.3), dirx=field(rng, n, -0.5, 0.5),
             diry=field(rng, n, -0.5, 0.5), dirz=field(rng, n, -0.5, 0.5))
    return d


def _load_design(lp, d):
    for fid, nm in ((A.ALPHA, "alpha"), (A.KAPPA, "diffusivity"), (A.BETA, "beta"), (A.DIRX, "dirx"),
                    (A.DIRY, "diry"), (A.DIRZ, "dirz")):
        lp.set_field(fid, d[nm])


PH = dict(nu=0.1, diff=0.02, gx=0.001, gy=-0.002, gz=0.0015, tem0=0.3)


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("kind", FWD + ADJ)
@pytest.mark.parametrize("storage", ["fp64", "fp32"])
def test_collide(o, shape, kind, storage):
    q, nx, ny, nz = shape
    L = o.lat(q, nx, ny, nz)
    n = L.nx * L.ny * L.nz
    rng = np.random.default_rng(21)
    d = _inputs(rng, n)
    k = getattr(A, kind)
    has_g = kind not in ("NS_COLLIDE", "NS_BRINKMAN", "ANS_BRINKMAN")
    f = pops(rng, q, n)
    g = pops(rng, q, n, base=0.5) if has_g else None
    if storage == "fp32":
        f = f.astype(np.float32).astype(np.float64)
        g = None if g is None else g.astype(np.float32).astype(np.float64)
    adj = k >= 10
    # oracle
    of = {nm: np.zeros(n) for nm in FWD_NAMES + ADJ_NAMES}
    if adj:
        for nm in ("rho", "ux", "uy", "uz", "tem"):
            of[nm] = d[nm].copy()
    snap = np.zeros(n * q)
    F = o.fields(gsnap=snap, alpha=d["alpha"], diffusivity=d["diffusivity"], beta=d["beta"], dirx=d["dirx"],
                 diry=d["diry"], dirz=d["dirz"], **of)
    fa = f.copy()
    ga = None if g is None else g.copy()
    o.collide(L, k, fa, ga, F, **PH, save=True)
    # GPU
    lp = fresh(q, nx, ny, nz, storage)
    lp.set_populations(0, f)
    if g is not None:
        lp.set_populations(1, g)
    _load_design(lp, d)
    if adj:
        for fid, nm in ((A.FWD_RHO, "rho"), (A.FWD_UX, "ux"), (A.FWD_UY, "uy"), (A.FWD_UZ, "uz"), (A.FWD_TEM, "tem")):
            lp.set_field(fid, d[nm])
    lp.collide(k, phys(**PH), save=True)
    tol = RTOL64 if storage == "fp64" else 2e-6
    close64(lp.get_populations(0), fa, tol)
    if g is not None:
        close64(lp.get_populations(1), ga, tol)
    names = ADJ_NAMES if adj else FWD_NAMES
    base = A.IP if adj else A.RHO
    for m, nm in enumerate(names):
        if q == 9 and nm.endswith("z"):
            continue
        if not has_g and nm in ("tem", "qx", "qy", "qz", "item", "iqx", "iqy", "iqz"):
            continue
        if kind == "AAD_FORCE" and nm == "iuz":
            continue
        close64(lp.get_field(base + m), of[nm], max(tol, 1e-11) if storage == "fp64" else 5e-5)
    if kind in ("AD_NATURAL", "AD_FORCE", "AAD_NATURAL", "AAD_FORCE", "AAD_MASSFLOW"):
        close64(lp.snapshot(1 if adj else 0).reshape(-1), snap, tol)
    lp.close()


# ---------------------------------------------------------------------------- heat-sink steps
def _heatsink_case(q):
    if q == 9:
        p = HS.Params(2, 24, 18)
    else:
        p = HS.Params(3, 12, 14, 10)
    return p


def _run_forward(o, p, storage, T, rng):
    nd = p.nd
    q = 9 if nd == 2 else 15
    L = o.lat(q, p.lx, p.ly, p.lz)
    n = L.nx * L.ny * L.nz
    ss = np.clip(HS.grf_design(nd, p.lx, p.ly, p.lz, seed=3, sigma=2.0), 0, 1)
    alpha, kappa, dads, dkds = p.design_fields(ss)
    rho0, ux0, uy0, uz0 = 1.0 + 0.01 * rng.standard_normal(n), 0.01 * rng.standard_normal(n), \
        0.01 * rng.standard_normal(n), (0.01 * rng.standard_normal(n) if nd == 3 else np.zeros(n))
    tem0 = 0.1 * rng.random(n)
    ops = HS.program_ops("forward", p)
    ph = dict(nu=p.nu, diff=0.0, gx=p.gx, gy=p.gy, gz=p.gz, tem0=p.tem0)
    # oracle: reference driver order (collide, stream, BCs, smoothing), heatsink.cpp:142-174
    f, g = np.zeros((q, n)), np.zeros((q, n))
    o.init(L, 0, f, o.fields(rho=rho0, ux=ux0, uy=uy0, uz=uz0))
    o.init(L, 1, g, o.fields(tem=tem0, ux=ux0, uy=uy0, uz=uz0))
    mac = {nm: np.zeros(n) for nm in FWD_NAMES}
    snap = np.zeros(n * q)
    for t in range(1, T + 1):
        o.collide(L, A.AD_NATURAL, f, g, o.fields(gsnap=snap, alpha=alpha, diffusivity=kappa, **mac), **ph, save=True)
        if t == T:
            break
        o.stream(L, f)
        o.stream(L, g)
        replay(o, L, f, g, ops, n, ux=mac["ux"], uy=mac["uy"], uz=mac["uz"], kappa=kappa)
    # GPU: collide, then fused steps
    lp = LatticePair(q, p.lx, p.ly, p.lz, storage)
    lp.set_field(A.ALPHA, alpha)
    lp.set_field(A.KAPPA, kappa)
    lp.init(0, rho0, ux=ux0, uy=uy0, uz=uz0)
    lp.init(1, tem0, ux=ux0, uy=uy0, uz=uz0)
    prog = lp.program(HS.to_descs(ops))
    lp.collide(A.AD_NATURAL, phys(**ph), save=True)
    for t in range(2, T + 1):
        lp.step(A.AD_NATURAL, phys(**ph), prog, save=(t == T))
    return lp, (f, g, mac, snap), (alpha, kappa, dads, dkds), ops, ph, L


@pytest.mark.parametrize("q", [9, 15])
@pytest.mark.parametrize("storage", ["fp64", "fp32"])
def test_heatsink_forward_steps(o, q, storage):
    rng = np.random.default_rng(5)
    p = _heatsink_case(q)
    T = 60
    lp, (f, g, mac, snap), _, _, _, _ = _run_forward(o, p, storage, T, rng)
    tol = 1e-11 if storage == "fp64" else 1e-4
    close64(lp.get_populations(0), f, tol)
    close64(lp.get_populations(1), g, tol)
    for m, nm in enumerate(FWD_NAMES):
        if q == 9 and nm.endswith("z"):
            continue
        close64(lp.get_field(A.RHO + m), mac[nm], tol if storage == "fp64" else 1e-4)
    close64(lp.snapshot(0).reshape(-1), snap, tol)
    lp.synchronize()


@pytest.mark.parametrize("q", [9, 15])
@pytest.mark.parametrize("storage", ["fp64", "fp32"])
def test_heatsink_adjoint_steps_and_sensitivity(o, q, storage):
    """Forward, snapshot, adjoint and sensitivity on one handle (the drivers' pf/pg reuse)."""
    rng = np.random.default_rng(6)
    p = _heatsink_case(q)
    T = 40
    lp, (f, g, mac, gsnap), (alpha, kappa, dads, dkds), _, _, L = _run_forward(o, p, storage, T, rng)
    n = lp.n
    tol = 1e-11 if storage == "fp64" else 5e-5
    close64(lp.snapshot(0).reshape(-1), gsnap, tol)   # kept on the device for the sensitivity
    lp.freeze_forward()
    ip0, iu0 = 0.01 * rng.standard_normal(n), [0.01 * rng.standard_normal(n) for _ in range(3)]
    it0, iq0 = 0.01 * rng.standard_normal(n), [0.01 * rng.standard_normal(n) for _ in range(3)]
    fu = [lp.get_field(A.FWD_UX), lp.get_field(A.FWD_UY), lp.get_field(A.FWD_UZ)]
    lp.init(2, ip0, iu0[0], iu0[1], iu0[2], ux=fu[0], uy=fu[1], uz=fu[2])
    lp.init(3, it0, iq0[0], iq0[1], iq0[2], ux=fu[0], uy=fu[1], uz=fu[2])
    ops = HS.program_ops("adjoint", p)
    ph = dict(nu=p.nu, diff=0.0, gx=p.gx, gy=p.gy, gz=p.gz, tem0=p.tem0)
    prog = lp.program(HS.to_descs(ops))
    lp.collide(A.AAD_NATURAL, phys(**ph), save=True)
    for t in range(2, T + 1):
        lp.step(A.AAD_NATURAL, phys(**ph), prog, save=(t == T))
    # oracle adjoint (adjointadvection.h:1111-1168, heatsink.cpp:181-212)
    fa, ga = np.zeros((q, n)), np.zeros((q, n))
    o.init(L, 2, fa, o.fields(ux=mac["ux"], uy=mac["uy"], uz=mac["uz"], ip=ip0, iux=iu0[0], iuy=iu0[1], iuz=iu0[2]))
    o.init(L, 3, ga, o.fields(ux=mac["ux"], uy=mac["uy"], uz=mac["uz"], item=it0, iqx=iq0[0], iqy=iq0[1], iqz=iq0[2]))
    am = {nm: np.zeros(n) for nm in ADJ_NAMES}
    igsnap = np.zeros(n * q)
    fwd = {nm: mac[nm] for nm in ("rho", "ux", "uy", "uz", "tem")}
    for t in range(1, T + 1):
        o.collide(L, A.AAD_NATURAL, fa, ga, o.fields(gsnap=igsnap, alpha=alpha, diffusivity=kappa, **fwd, **am), **ph,
                  save=True)
        if t == T:
            break
        o.stream(L, fa, inverse=True)
        o.stream(L, ga, inverse=True)
        replay(o, L, fa, ga, ops, n, ux=mac["ux"], uy=mac["uy"], uz=mac["uz"], rho=mac["rho"], tem=mac["tem"],
               kappa=kappa)
    tola = 1e-11 if storage == "fp64" else 2e-4
    close64(lp.get_populations(0), fa, tola)
    close64(lp.get_populations(1), ga, tola)
    for m, nm in enumerate(ADJ_NAMES):
        if q == 9 and nm.endswith("z"):
            continue
        close64(lp.get_field(A.IP + m), am[nm], tola)
    close64(lp.snapshot(1).reshape(-1), igsnap, tola)
    # AAD::SensitivityTemperatureAtHeatSource
    qn, mask = p.source()
    ref = np.zeros(n)
    Fo = o.fields(ux=mac["ux"], uy=mac["uy"], uz=mac["uz"], tem=mac["tem"], imx=am["imx"], imy=am["imy"],
                  imz=am["imz"], item=am["item"], iqx=am["iqx"], iqy=am["iqy"], iqz=am["iqz"], diffusivity=kappa)
    o.sensitivity(L, 0, ref, Fo, dads, dkds, gsnap, igsnap, qn, mask)
    got = lp.sensitivity(0, np.zeros(n), dads, dkds, qn, mask)
    close64(got, ref, 1e-10 if storage == "fp64" else 5e-3)
    for which in (1, 2, 3):
        r2 = np.zeros(n)
        o.sensitivity(L, which, r2, Fo, dads, dkds, gsnap, igsnap, qn, mask)
        close64(lp.sensitivity(which, np.zeros(n), dads, dkds, qn, mask), r2, 1e-10 if storage == "fp64" else 5e-3)
    lp.synchronize()


# ---------------------------------------------------------------------------- field utilities
@pytest.mark.parametrize("shape", [(9, 31, 23, 1), (15, 13, 11, 9)])
@pytest.mark.parametrize("R", [1.5, 2.4, 3.0])
@pytest.mark.parametrize("masked", [False, True])
def test_filters(o, shape, R, masked):
    q, nx, ny, nz = shape
    L = o.lat(q, nx, ny, nz)
    n = L.nx * L.ny * L.nz
    rng = np.random.default_rng(31)
    s, d = field(rng, n, 0, 1), field(rng, n, -1, 1)
    mask = None
    if masked:
        i, j, k = HS.grid(2 if q == 9 else 3, nx, ny, L.nz)
        mask = ((i < 3 * nx // 4) & (j < 3 * ny // 4)).astype(np.int32)
    lp = fresh(q, nx, ny, nz)
    # tanh differs between libm and CUDA by a few ulp: 1e-12 relative
    close64(lp.heaviside_var(R, 8.0, s, mask), o.heaviside_var(L, R, 8.0, s, mask), 1e-12)
    close64(lp.heaviside_sens(R, 8.0, s, d, mask), o.heaviside_sens(L, R, 8.0, s, d, mask), 1e-12)
    close64(lp.density_filter(R, s, mask), o.density_filter(L, R, s, mask), 1e-13)


def test_residual_and_normalize(o):
    lp = fresh(9, 64, 64, 1)
    rng = np.random.default_rng(4)
    for ncomp in (1, 2, 3):
        a = [field(rng, 3000, -1, 1) for _ in range(ncomp)]
        b = [field(rng, 3000, -1, 1) for _ in range(ncomp)]
        assert abs(lp.residual_host(a, b) - o.residual(a, b)) <= 1e-14 * o.residual(a, b)
    v = field(rng, 4000, -3, 2)
    w = v.copy()
    o.normalize(w)
    assert np.array_equal(lp.normalize(v), w)


def test_solve_matches_driver_loop(o):
    """pl_solve (collide + fused steps, residual every 10 steps) against the oracle's driver loop."""
    p = HS.Params(2, 20, 16)
    q, n = 9, 20 * 16
    L = o.lat(q, p.lx, p.ly)
    ss = np.clip(HS.grf_design(2, p.lx, p.ly, seed=7, sigma=2.0), 0, 1)
    alpha, kappa, _, _ = p.design_fields(ss)
    ops = HS.program_ops("forward", p)
    ph = dict(nu=p.nu, diff=0.0, gx=p.gx, gy=p.gy, gz=p.gz, tem0=p.tem0)
    one, zero = np.ones(n), np.zeros(n)
    lp = fresh(q, p.lx, p.ly, 1)
    lp.set_field(A.ALPHA, alpha)
    lp.set_field(A.KAPPA, kappa)
    lp.init(0, one, ux=zero, uy=zero, uz=zero)
    lp.init(1, zero, ux=zero, uy=zero, uz=zero)
    prog = lp.program(HS.to_descs(ops))
    tol = 2e-3
    st, steps, res = lp.solve(A.AD_NATURAL, phys(**ph), prog, max_steps=400, check_every=10, tol=tol)
    # oracle driver loop with the same check cadence
    f, g = np.zeros((q, n)), np.zeros((q, n))
    o.init(L, 0, f, o.fields(rho=one, ux=zero, uy=zero, uz=zero))
    o.init(L, 1, g, o.fields(tem=zero, ux=zero, uy=zero, uz=zero))
    cur = {nm: np.zeros(n) for nm in FWD_NAMES}
    prev = {nm: np.zeros(n) for nm in FWD_NAMES}
    ost, osteps, ores = A.PL_MAX_STEPS, 400, None
    for t in range(1, 401):
        o.collide(L, A.AD_NATURAL, f, g, o.fields(alpha=alpha, diffusivity=kappa, **cur), **ph, save=True)
        if t % 10 == 0:
            r0 = o.residual([cur["ux"], cur["uy"]], [prev["ux"], prev["uy"]])
            r1 = o.residual([cur["qx"], cur["qy"]], [prev["qx"], prev["qy"]])
            ores = (r0, r1)
            if r0 < tol and r1 < tol:
                ost, osteps = A.PL_CONVERGED, t
                break
        o.stream(L, f)
        o.stream(L, g)
        replay(o, L, f, g, ops, n, ux=cur["ux"], uy=cur["uy"], kappa=kappa)
        cur, prev = prev, cur
    assert (st, steps) == (ost, osteps)
    assert abs(res[0] - ores[0]) <= 1e-9 * ores[0] and abs(res[1] - ores[1]) <= 1e-9 * ores[1]


@pytest.mark.parametrize("q", [9, 15])
@pytest.mark.parametrize("n", [4, 7, 12])
def test_graph_steps_equal_eager_steps(o, q, n):
    """pl_steps replays a captured two-step CUDA graph; it must equal n eager pl_step calls."""
    p = _heatsink_case(q)
    ss = np.clip(HS.grf_design(p.nd, p.lx, p.ly, p.lz, seed=5, sigma=2.0), 0, 1)
    alpha, kappa, _, _ = p.design_fields(ss)
    nn = p.lx * p.ly * p.lz
    one, zero = np.ones(nn), np.zeros(nn)
    ph = phys(nu=p.nu, diff=0.0, gx=p.gx, gy=p.gy, gz=p.gz, tem0=p.tem0)
    out = []
    for graph in (True, False):
        lp = LatticePair(q, p.lx, p.ly, p.lz, "fp32")
        lp.set_option(A.OPT_GRAPHS, graph)
        lp.set_field(A.ALPHA, alpha)
        lp.set_field(A.KAPPA, kappa)
        lp.init(0, one, ux=zero, uy=zero, uz=zero)
        lp.init(1, 0.1 * one, ux=zero, uy=zero, uz=zero)
        prog = lp.program(HS.to_descs(HS.program_ops("forward", p)))
        lp.collide(A.AD_NATURAL, ph)
        if graph:
            lp.steps(A.AD_NATURAL, ph, prog, n)
            lp.steps(A.AD_NATURAL, ph, prog, n)      # replays the cached graph
        else:
            for _ in range(2 * n):
                lp.step(A.AD_NATURAL, ph, prog, save=False)
        out.append((lp.get_populations(0), lp.get_populations(1)))
        lp.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("q", [9, 15])
@pytest.mark.parametrize("storage", ["fp16", "bf16"])
def test_heatsink_forward_16bit_storage(o, q, storage):
    """Shifted 16-bit population storage (f - w_c * shift, FP32 compute) against the FP64 oracle
    after 60 heat-sink steps. Tolerance, relative to max(1, max |field|): 5e-4 for FP16, 5e-3 for
    BF16 (measured on GB300: FP16 g / T within 3e-4 / 2e-4 of their maxima, BF16 within
    2.2e-3 / 2.7e-3)."""
    rng = np.random.default_rng(5)
    p = _heatsink_case(q)
    lp, (f, g, mac, snap), _, _, _, _ = _run_forward(o, p, storage, 60, rng)
    tol = 5e-4 if storage == "fp16" else 5e-3
    close64(lp.get_populations(0), f, tol)
    close64(lp.get_populations(1), g, tol)
    for m, nm in enumerate(FWD_NAMES):
        if q == 9 and nm.endswith("z"):
            continue
        close64(lp.get_field(A.RHO + m), mac[nm], tol)
    lp.close()
