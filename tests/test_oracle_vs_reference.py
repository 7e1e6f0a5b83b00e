"""Pin the oracle (plain-C restatement) against the PANSLBM2 reference itself.

Runs only where the reference sources are present (the reference-backed library is compiled
from them by oracle/build.py); both sides use -ffp-contract=off, so results must agree
bit-for-bit except where noted.
"""
import itertools

import numpy as np
import pytest

from oracle import build as obuild
from tests._cases import field, pops

pytestmark = pytest.mark.skipif(obuild.reference_root() is None, reason="reference sources not present")


@pytest.fixture(scope="module")
def libs():
    from oracle.olib import Oracle
    obuild.build_oracle()
    obuild.build_ref()
    return Oracle("oracle"), Oracle("ref")


SHAPES = [(9, 7, 6, 1), (15, 5, 6, 4)]


def _lat(o, q, nx, ny, nz):
    return o.lat(q, nx, ny, nz)


def _eq(a, b, exact=True, tol=0.0):
    if exact:
        assert np.array_equal(a, b), f"max abs diff {np.max(np.abs(a - b))}"
    else:
        np.testing.assert_allclose(a, b, rtol=tol, atol=tol)


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("inverse", [False, True])
def test_stream(libs, shape, inverse):
    o, r = libs
    q, nx, ny, nz = shape
    L = o.lat(q, nx, ny, nz)
    n = nx * ny * nz
    f = np.ascontiguousarray(np.arange(q * n, dtype=np.float64).reshape(q, n))
    a, b = f.copy(), f.copy()
    o.stream(L, a, inverse)
    r.stream(L, b, inverse)
    _eq(a, b)


def _faces(q, nx, ny, nz):
    axes = [0, 1] if q == 9 else [0, 1, 2]
    lens = [nx, ny, nz]
    out = []
    for a in axes:
        for d in (-1, 1):
            out.append((a, 0 if d < 0 else lens[a] - 1, d))
        out.append((a, lens[a] // 2, 1))      # interior line, +1 side
        out.append((a, lens[a] // 2, -1))     # interior line, -1 side
    return out


BC_KINDS = ["WALL", "IWALL", "NS_U", "NS_RHO", "AD_T", "AD_Q", "AD_QC", "ANS_U", "ANS_RHO", "AAD_T", "AAD_Q",
            "AAD_RHO"]


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("kind", BC_KINDS)
def test_boundary_conditions(libs, shape, kind):
    from oracle import olib
    o, r = libs
    q, nx, ny, nz = shape
    if kind == "AAD_RHO" and q == 15:
        pytest.skip("reference D3Q15 iBoundaryConditionSetRho overloads do not compile (adjointadvection.h:583)")
    L = o.lat(q, nx, ny, nz)
    n = nx * ny * nz
    rng = np.random.default_rng(hash((q, kind)) % 2**32)
    k = getattr(olib, "BC_" + kind)
    for (axis, pos, d) in _faces(q, nx, ny, nz):
        f = pops(rng, q, n)
        g = pops(rng, q, n, base=0.5)
        if kind in ("WALL", "IWALL"):
            ty = rng.integers(0, 3, n).astype(np.int32)
        elif kind == "AAD_RHO":
            ty = rng.integers(0, 3, n).astype(np.int32)
        else:
            ty = rng.integers(0, 2, n).astype(np.int32)
        kw = dict(v0=field(rng, n, 0.9, 1.1), v1=field(rng, n, -0.05, 0.05), v2=field(rng, n, -0.05, 0.05),
                  ux=field(rng, n, -0.05, 0.05), uy=field(rng, n, -0.05, 0.05), uz=field(rng, n, -0.05, 0.05),
                  rho=field(rng, n, 0.95, 1.05), tem=field(rng, n, 0.0, 1.0), diffusivity=field(rng, n, 0.01, 0.2),
                  kappa=0.037, eps=0.7)
        if kind in ("NS_U", "ANS_U"):
            kw["v0"] = field(rng, n, -0.05, 0.05)
        fa, ga, fb, gb = f.copy(), g.copy(), f.copy(), g.copy()
        o.apply_bc(L, fa, k, axis, pos, d, ty, g=ga, **kw)
        r.apply_bc(L, fb, k, axis, pos, d, ty, g=gb, **kw)
        _eq(fa, fb)
        _eq(ga, gb)


@pytest.mark.parametrize("shape", SHAPES)
def test_smoothing(libs, shape):
    o, r = libs
    q, nx, ny, nz = shape
    L = o.lat(q, nx, ny, nz)
    n = nx * ny * nz
    rng = np.random.default_rng(5)
    f = pops(rng, q, n)
    a, b = f.copy(), f.copy()
    o.smooth_corner(L, a)
    r.smooth_corner(L, b)
    _eq(a, b)
    a, b = f.copy(), f.copy()
    o.smooth_at(L, a, 2, 3, 1, -1, 1, -1)
    r.smooth_at(L, b, 2, 3, 1, -1, 1, -1)
    _eq(a, b)
    if q == 15:
        for plane in range(3):
            a, b = f.copy(), f.copy()
            o.smooth_line(L, a, plane, 2, 1, 1, -1)
            r.smooth_line(L, b, plane, 2, 1, 1, -1)
            _eq(a, b)


FWD = ["NS_COLLIDE", "NS_BRINKMAN", "AD_NATURAL", "AD_FORCE", "AD_HEATEX", "AD_NATURAL_NOBRINK", "AD_FORCE_NOBRINK"]
ADJ = ["ANS_BRINKMAN", "AAD_NATURAL", "AAD_FORCE", "AAD_HEATEX", "AAD_MASSFLOW"]


def _all_fields(rng, n):
    d = {}
    for name in ("rho",):
        d[name] = field(rng, n, 0.95, 1.05)
    for name in ("ux", "uy", "uz"):
        d[name] = field(rng, n, -0.05, 0.05)
    for name in ("tem", "qx", "qy", "qz", "ip", "iux", "iuy", "iuz", "imx", "imy", "imz", "item", "iqx", "iqy",
                 "iqz", "dirx", "diry", "dirz"):
        d[name] = field(rng, n, -0.5, 0.5)
    d["alpha"] = field(rng, n, 0.0, 0.2)
    d["diffusivity"] = field(rng, n, 0.01, 0.2)
    d["beta"] = field(rng, n, 0.0, 0.3)
    return d


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("kind", FWD + ADJ)
def test_collide(libs, shape, kind):
    from oracle import olib
    o, r = libs
    q, nx, ny, nz = shape
    L = o.lat(q, nx, ny, nz)
    n = nx * ny * nz
    rng = np.random.default_rng(11)
    k = getattr(olib, kind)
    base = _all_fields(rng, n)
    f = pops(rng, q, n)
    g = None if kind in ("NS_COLLIDE", "NS_BRINKMAN", "ANS_BRINKMAN") else pops(rng, q, n, base=0.5)
    outs = []
    for lib in (o, r):
        d = {kk: v.copy() for kk, v in base.items()}
        snap = np.zeros(n * q)
        F = lib.fields(gsnap=snap, **d)
        fa = f.copy()
        ga = None if g is None else g.copy()
        lib.collide(L, k, fa, ga, F, nu=0.1, diff=0.02, gx=0.001, gy=-0.002, gz=0.0015, tem0=0.3, save=True)
        outs.append((fa, ga, d, snap))
    (fa, ga, da, sa), (fb, gb, db, sb) = outs
    _eq(fa, fb)
    if ga is not None:
        _eq(ga, gb)
    for kk in da:
        _eq(da[kk], db[kk])
    _eq(sa, sb)


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("which", [0, 1, 2, 3])
def test_init(libs, shape, which):
    o, r = libs
    q, nx, ny, nz = shape
    L = o.lat(q, nx, ny, nz)
    n = nx * ny * nz
    base = _all_fields(np.random.default_rng(3), n)
    a, b = np.zeros((q, n)), np.zeros((q, n))
    o.init(L, which, a, o.fields(**base))
    r.init(L, which, b, r.fields(**base))
    _eq(a, b)


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("which", [0, 1, 2, 3])
def test_sensitivity(libs, shape, which):
    o, r = libs
    q, nx, ny, nz = shape
    L = o.lat(q, nx, ny, nz)
    n = nx * ny * nz
    rng = np.random.default_rng(7)
    base = _all_fields(rng, n)
    dads, dkds = field(rng, n, -1, 1), field(rng, n, -0.1, 0.1)
    g, ig = field(rng, n * q, 0, 0.2), field(rng, n * q, -1, 1)
    qn = field(rng, n, 0.0, 0.02)
    mask = rng.integers(0, 2, n).astype(np.int32)
    a, b = field(rng, n, -1, 1), None
    b = a.copy()
    o.sensitivity(L, which, a, o.fields(**base), dads, dkds, g, ig, qn, mask)
    r.sensitivity(L, which, b, r.fields(**base), dads, dkds, g, ig, qn, mask)
    _eq(a, b)


@pytest.mark.parametrize("shape", [(9, 13, 11, 1), (15, 7, 8, 6)])
@pytest.mark.parametrize("R", [1.5, 2.4, 3.0])
@pytest.mark.parametrize("masked", [False, True])
def test_filters(libs, shape, R, masked):
    o, r = libs
    q, nx, ny, nz = shape
    L = o.lat(q, nx, ny, nz)
    n = nx * ny * nz
    rng = np.random.default_rng(13)
    s = field(rng, n, 0, 1)
    dfd = field(rng, n, -1, 1)
    mask = None
    if masked:
        ii, jj, kk = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(L.nz), indexing="ij")
        mask = np.ascontiguousarray(((ii < 3 * nx // 4) & (jj < 3 * ny // 4)).transpose(2, 1, 0).reshape(-1).astype(np.int32))
    _eq(o.heaviside_var(L, R, 8.0, s, mask), r.heaviside_var(L, R, 8.0, s, mask))
    _eq(o.heaviside_sens(L, R, 8.0, s, dfd, mask), r.heaviside_sens(L, R, 8.0, s, dfd, mask))
    _eq(o.density_filter(L, R, s, mask), r.density_filter(L, R, s, mask))


@pytest.mark.parametrize("shape", [(9, 13, 11, 1), (15, 7, 8, 6)])
@pytest.mark.parametrize("R", [1.5, 2.4, 3.0])
def test_filters_general_weight(libs, shape, R):
    """a weight functor of no special form (here a random positive table per node and tap):
    the oracle's table restatement equals the reference's routines called with that functor"""
    o, r = libs
    q, nx, ny, nz = shape
    L = o.lat(q, nx, ny, nz)
    n = L.nx * L.ny * L.nz
    nt = o.filter_ntaps(L, R)
    assert nt == r.filter_ntaps(L, R)
    rng = np.random.default_rng(17)
    s, dfd = field(rng, n, 0, 1), field(rng, n, -1, 1)
    w = 0.1 + rng.random((n, nt))
    for op in (0, 1, 2):
        _eq(o.filter_table(L, op, R, s, w, b=dfd, beta=8.0), r.filter_table(L, op, R, s, w, b=dfd, beta=8.0))


@pytest.mark.parametrize("ncomp", [1, 2, 3])
def test_residual_normalize(libs, ncomp):
    o, r = libs
    rng = np.random.default_rng(ncomp)
    a = [field(rng, 1000, -1, 1) for _ in range(ncomp)]
    b = [field(rng, 1000, -1, 1) for _ in range(ncomp)]
    assert o.residual(a, b) == r.residual(a, b)
    v1, v2 = a[0].copy(), a[0].copy()
    o.normalize(v1)
    r.normalize(v2)
    _eq(v1, v2)
