"""Golden cases: seeded inputs plus a runner that applies one PANSLBM2 operation (or a short
driver loop) through an oracle-like library.

A runner takes an `oracle.olib.Oracle` (over the C restatement, or over the build that compiles
the reference's own headers) and the case's inputs, and returns the outputs. make_golden.py runs
every case through the reference build and stores inputs and outputs in tests/golden/<case>.npz;
test_golden.py reruns the C restatement on the stored inputs, test_gpu_golden.py the CUDA
library. Reference routines per case:

  stream   D2Q9::Stream / iStream (d2q9.h:165-427), D3Q15::Stream / iStream (d3q15.h:256-980)
  bc       every edge/face routine of one kind on all edges/faces and two interior lines
           (d2q9.h:429-575, d3q15.h:982-1239, navierstokes.h:91-426, advection.h:98-524,
           adjointnavierstokes.h:97-392, adjointadvection.h:154-751; on D2Q9 also
           nsincompressible.h:46-140, adjointnsincompressible.h:49-92)
  smooth   SmoothCorner, SmoothCornerAt, SmoothCornerAlong{YZ,ZX,XY} (d2q9.h:577-587,
           d3q15.h:1241-1303)
  collide  the twelve Macro*Collide* routines with save (navierstokes.h:430-546,
           advection.h:528-1044, adjointnavierstokes.h:396-470, adjointadvection.h:892-1355)
           and, on D2Q9, the three incompressible ones (nsincompressible.h:144-200,
           adjointnsincompressible.h:143-178)
  init     NS / AD / ANS / AAD InitialCondition; NSin / ANSin on D2Q9
  sens     the four sensitivity routines (adjointadvection.h:1443-1543,
           adjointnavierstokes.h:540-554)
  filter   HeavisideFilter::GetFilteredVariable / GetFilteredSensitivity, DensityFilter
  resid    Residual (residual.h:8-51), Normalize (normalize.h:8-23)
  hsfwd    heat-sink forward driver loop (heatsink.cpp:142-174): collide, Stream, boundary
           calls, SmoothCorner; T steps from a perturbed equilibrium
  hsadj    the adjoint driver loop (heatsink.cpp:181-212) from the hsfwd state, then the
           four sensitivities
  nsinch   an incompressible Brinkman channel on D2Q9: NSin forward steps (walls, NSin velocity
           inlet and pressure outlet), ANSin adjoint steps, the Brinkman sensitivity
  el       the elastic routines on D2Q9: EL::MacroCollide / MacroExtendedCollide, AEL::MacroCollide
           (elastic.h:109-166, adjointelastic.h:96-125), the stress boundary routines on every edge
           and two interior lines (elastic.h:60-104, adjointelastic.h:48-92), the two initial
           conditions and AEL::SensitivityCompliance (adjointelastic.h:149-155)
  hst      the transient heat-sink loops of production/heatsink_transient.cpp:135-205 on a small
           lattice: forward from rest keeping every time level's macros and g snapshot, the adjoint
           swept backward with one SensitivityTemperatureAtHeatSource term per step, and the
           time-averaged source temperature
  elsens   the compliance-sensitivity driver loop of test/elsens.cpp on a small plate: EL forward
           steps (wall on x = 0, traction on x = lx-1, SmoothCorner) accumulating the displacement,
           AEL adjoint steps, the compliance sensitivity, Normalize
"""
import zlib

import numpy as np

from panslbm2_gb300 import _capi as A
from panslbm2_gb300 import heatsink as HS
from tests._cases import field, pops
from tests._replay import replay

SHAPES = {"q9": (9, 7, 6, 1), "q15": (15, 5, 6, 4)}
FILTER_SHAPES = {"q9": (9, 13, 11, 1), "q15": (15, 7, 8, 6)}
HS_SHAPES = {"q9": (2, 16, 12, 1), "q15": (3, 8, 9, 7)}
FWD = ["NS_COLLIDE", "NS_BRINKMAN", "AD_NATURAL", "AD_FORCE", "AD_HEATEX", "AD_NATURAL_NOBRINK", "AD_FORCE_NOBRINK"]
ADJ = ["ANS_BRINKMAN", "AAD_NATURAL", "AAD_FORCE", "AAD_HEATEX", "AAD_MASSFLOW"]
# the incompressible variants exist for D2Q9 only
FWD_IN, ADJ_IN = ["NSIN_COLLIDE", "NSIN_BRINKMAN"], ["ANSIN_BRINKMAN"]
NO_G = ("NS_COLLIDE", "NS_BRINKMAN", "ANS_BRINKMAN", "NSIN_COLLIDE", "NSIN_BRINKMAN", "ANSIN_BRINKMAN")
FWD_NAMES = ["rho", "ux", "uy", "uz", "tem", "qx", "qy", "qz"]
ADJ_NAMES = ["ip", "iux", "iuy", "iuz", "imx", "imy", "imz", "item", "iqx", "iqy", "iqz"]
BC_KINDS = ["WALL", "IWALL", "NS_U", "NS_RHO", "AD_T", "AD_Q", "AD_QC", "ANS_U", "ANS_RHO", "AAD_T", "AAD_Q",
            "AAD_RHO", "NSIN_U", "NSIN_RHO", "ANSIN_U"]
BC_2D_ONLY = ("NSIN_U", "NSIN_RHO", "ANSIN_U")
PH = dict(nu=0.1, diff=0.02, gx=0.001, gy=-0.002, gz=0.0015, tem0=0.3)
HS_FWD_STEPS, HS_ADJ_STEPS = 25, 20


def _rng(name):
    return np.random.default_rng(zlib.crc32(name.encode()))


def _shape(inp):
    return tuple(int(x) for x in inp["shape"])


def faces_with_interior(q, nx, ny, nz):
    lens = [nx, ny, nz]
    out = []
    for a in ([0, 1] if q == 9 else [0, 1, 2]):
        out += [(a, 0, -1), (a, lens[a] - 1, 1), (a, lens[a] // 2, 1), (a, lens[a] // 2, -1)]
    return out


# ---------------------------------------------------------------------------- stream
def stream_inputs(name, sk, inverse):
    q, nx, ny, nz = SHAPES[sk]
    n = nx * ny * nz
    f = np.arange(q * n, dtype=np.float64).reshape(q, n) * 0.25 + 1.0   # index-coded populations
    return dict(shape=np.array([q, nx, ny, nz]), inverse=np.array(int(inverse)), f=f)


def stream_run(lib, inp):
    q, nx, ny, nz = _shape(inp)
    L = lib.lat(q, nx, ny, nz)
    f = inp["f"].copy()
    lib.stream(L, f, bool(inp["inverse"]))
    return dict(f=f)


# ---------------------------------------------------------------------------- boundary kinds
def bc_op(kind, axis, pos, d, inp):
    return dict(kind=getattr(A, "BC_" + kind), lat=int(inp["lat"]), axis=axis, pos=pos, dir=d, type=inp["type"],
                v0=inp["v0"], v1=inp["v1"], v2=inp["v2"], kappa=0.037, eps=0.7)


def bc_inputs(name, sk, kind):
    q, nx, ny, nz = SHAPES[sk]
    n = nx * ny * nz
    rng = _rng(name)
    ty = rng.integers(0, 3, n).astype(np.int32)
    if kind not in ("WALL", "IWALL", "AAD_RHO"):
        ty = (ty > 0).astype(np.int32)
    return dict(shape=np.array([q, nx, ny, nz]), kind=np.array(BC_KINDS.index(kind)),
                lat=np.array(int(rng.integers(0, 2)) if kind in ("WALL", "IWALL") else 0),
                f=pops(rng, q, n), g=pops(rng, q, n, base=0.5), type=ty,
                v0=field(rng, n, 0.9, 1.1) if kind not in ("NS_U", "ANS_U", "NSIN_U") else field(rng, n, -0.05, 0.05),
                v1=field(rng, n, -0.05, 0.05), v2=field(rng, n, -0.05, 0.05), ux=field(rng, n, -0.05, 0.05),
                uy=field(rng, n, -0.05, 0.05), uz=field(rng, n, -0.05, 0.05), rho=field(rng, n, 0.95, 1.05),
                tem=field(rng, n, 0, 1), kap=field(rng, n, 0.01, 0.2))


def bc_ops(inp):
    q, nx, ny, nz = _shape(inp)
    kind = BC_KINDS[int(inp["kind"])]
    return [bc_op(kind, a, p, d, inp) for (a, p, d) in faces_with_interior(q, nx, ny, nz)]


def bc_run(lib, inp):
    q, nx, ny, nz = _shape(inp)
    L = lib.lat(q, nx, ny, nz)
    n = nx * ny * nz
    f, g = inp["f"].copy(), inp["g"].copy()
    replay(lib, L, f, g, bc_ops(inp), n, ux=inp["ux"], uy=inp["uy"], uz=inp["uz"], rho=inp["rho"], tem=inp["tem"],
           kappa=inp["kap"])
    return dict(f=f, g=g)


# ---------------------------------------------------------------------------- smoothing
def smooth_ops(q):
    ops = [dict(kind=A.SMOOTH_CORNER, lat=0), dict(kind=A.SMOOTH_CORNER, lat=1),
           dict(kind=A.SMOOTH_AT, lat=0, i=2, j=3, k=1, di=-1, dj=1, dk=-1)]
    if q == 15:
        for plane in range(3):
            ops.append(dict(kind=A.SMOOTH_LINE, lat=1, axis=plane, i=2, j=1, di=1, dj=-1))
    return ops


def smooth_inputs(name, sk):
    q, nx, ny, nz = SHAPES[sk]
    n = nx * ny * nz
    rng = _rng(name)
    return dict(shape=np.array([q, nx, ny, nz]), f=pops(rng, q, n), g=pops(rng, q, n, base=0.5))


def smooth_run(lib, inp):
    q, nx, ny, nz = _shape(inp)
    L = lib.lat(q, nx, ny, nz)
    f, g = inp["f"].copy(), inp["g"].copy()
    replay(lib, L, f, g, smooth_ops(q), nx * ny * nz)
    return dict(f=f, g=g)


# ---------------------------------------------------------------------------- collides
def design_inputs(rng, n):
    return dict(rho=field(rng, n, 0.95, 1.05), ux=field(rng, n, -0.05, 0.05), uy=field(rng, n, -0.05, 0.05),
                uz=field(rng, n, -0.05, 0.05), tem=field(rng, n, -0.5, 0.5), alpha=field(rng, n, 0.0, 0.2),
                diffusivity=field(rng, n, 0.01, 0.2), beta=field(rng, n, 0.0, 0.3), dirx=field(rng, n, -0.5, 0.5),
                diry=field(rng, n, -0.5, 0.5), dirz=field(rng, n, -0.5, 0.5))


def collide_inputs(name, sk, kind):
    q, nx, ny, nz = SHAPES[sk]
    n = nx * ny * nz
    rng = _rng(name)
    d = design_inputs(rng, n)
    has_g = kind not in NO_G
    d.update(shape=np.array([q, nx, ny, nz]), kind=np.array(getattr(A, kind)), f=pops(rng, q, n),
             g=pops(rng, q, n, base=0.5) if has_g else np.zeros((0,)))
    return d


def collide_run(lib, inp):
    q, nx, ny, nz = _shape(inp)
    L = lib.lat(q, nx, ny, nz)
    n = nx * ny * nz
    k = int(inp["kind"])
    of = {nm: np.zeros(n) for nm in FWD_NAMES + ADJ_NAMES}
    if k >= 10:
        for nm in ("rho", "ux", "uy", "uz", "tem"):
            of[nm] = inp[nm].copy()
    snap = np.zeros(n * q)
    F = lib.fields(gsnap=snap, alpha=inp["alpha"], diffusivity=inp["diffusivity"], beta=inp["beta"],
                   dirx=inp["dirx"], diry=inp["diry"], dirz=inp["dirz"], **of)
    f = inp["f"].copy()
    g = inp["g"].copy() if inp["g"].size else None
    lib.collide(L, k, f, g, F, **PH, save=True)
    out = dict(f=f, snap=snap)
    if g is not None:
        out["g"] = g
    for nm in (ADJ_NAMES if k >= 10 else FWD_NAMES):
        out["m_" + nm] = of[nm]
    return out


# ---------------------------------------------------------------------------- initial conditions
def init_inputs(name, sk, which):
    q, nx, ny, nz = SHAPES[sk]
    n = nx * ny * nz
    rng = _rng(name)
    d = {nm: field(rng, n, -0.5, 0.5) for nm in ("ux", "uy", "uz", "tem", "ip", "iux", "iuy", "iuz", "item", "iqx",
                                                 "iqy", "iqz")}
    d["rho"] = field(rng, n, 0.95, 1.05)
    d.update(shape=np.array([q, nx, ny, nz]), which=np.array(which))
    return d


INIT_KEYS = ("rho", "ux", "uy", "uz", "tem", "ip", "iux", "iuy", "iuz", "item", "iqx", "iqy", "iqz")


def init_run(lib, inp):
    q, nx, ny, nz = _shape(inp)
    L = lib.lat(q, nx, ny, nz)
    f = np.zeros((q, nx * ny * nz))
    lib.init(L, int(inp["which"]), f, lib.fields(**{k: inp[k] for k in INIT_KEYS}))
    return dict(f=f)


# ---------------------------------------------------------------------------- sensitivities
SENS_KEYS = ("ux", "uy", "uz", "tem", "imx", "imy", "imz", "item", "iqx", "iqy", "iqz", "diffusivity")


def sens_inputs(name, sk, which):
    q, nx, ny, nz = SHAPES[sk]
    n = nx * ny * nz
    rng = _rng(name)
    d = {nm: field(rng, n, -0.5, 0.5) for nm in SENS_KEYS}
    d["diffusivity"] = field(rng, n, 0.01, 0.2)
    d.update(shape=np.array([q, nx, ny, nz]), which=np.array(which), dads=field(rng, n, -1, 1),
             dkds=field(rng, n, -0.1, 0.1), gsnap=field(rng, n * q, 0, 0.2), igsnap=field(rng, n * q, -1, 1),
             qn=field(rng, n, 0.0, 0.02), mask=rng.integers(0, 2, n).astype(np.int32), dfds=field(rng, n, -1, 1))
    return d


def sens_run(lib, inp):
    q, nx, ny, nz = _shape(inp)
    L = lib.lat(q, nx, ny, nz)
    a = inp["dfds"].copy()
    lib.sensitivity(L, int(inp["which"]), a, lib.fields(**{k: inp[k] for k in SENS_KEYS}), inp["dads"], inp["dkds"],
                    inp["gsnap"], inp["igsnap"], inp["qn"], inp["mask"])
    return dict(dfds=a)


# ---------------------------------------------------------------------------- filters
def filter_mask(q, nx, ny, nz):
    ii, jj, kk = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    return np.ascontiguousarray(((ii < 3 * nx // 4) & (jj < 3 * ny // 4)).transpose(2, 1, 0).reshape(-1)
                                .astype(np.int32))


def filter_inputs(name, sk, R, masked):
    q, nx, ny, nz = FILTER_SHAPES[sk]
    n = nx * ny * nz
    rng = _rng(name)
    return dict(shape=np.array([q, nx, ny, nz]), R=np.array(R), beta=np.array(8.0), s=field(rng, n, 0, 1),
                dfd=field(rng, n, -1, 1),
                mask=filter_mask(q, nx, ny, nz) if masked else np.zeros((0,), np.int32))


def filter_run(lib, inp):
    q, nx, ny, nz = _shape(inp)
    L = lib.lat(q, nx, ny, nz)
    R, beta = float(inp["R"]), float(inp["beta"])
    mask = inp["mask"] if inp["mask"].size else None
    return dict(var=lib.heaviside_var(L, R, beta, inp["s"], mask),
                sens=lib.heaviside_sens(L, R, beta, inp["s"], inp["dfd"], mask),
                dens=lib.density_filter(L, R, inp["s"], mask))


# ---------------------------------------------------------------------------- residual / normalize
def resid_inputs(name, ncomp):
    rng = _rng(name)
    d = {"a%d" % m: field(rng, 1000, -1, 1) for m in range(ncomp)}
    d.update({"b%d" % m: field(rng, 1000, -1, 1) for m in range(ncomp)})
    d["ncomp"] = np.array(ncomp)
    return d


def resid_run(lib, inp):
    nc = int(inp["ncomp"])
    a = [inp["a%d" % m] for m in range(nc)]
    b = [inp["b%d" % m] for m in range(nc)]
    v = a[0].copy()
    lib.normalize(v)
    return dict(residual=np.array(lib.residual(a, b)), normalized=v)


# ---------------------------------------------------------------------------- heat-sink driver loops
def hs_params(sk):
    nd, lx, ly, lz = HS_SHAPES[sk]
    return HS.Params(nd, lx, ly, lz)


def hs_inputs(name, sk):
    p = hs_params(sk)
    n = p.lx * p.ly * p.lz
    rng = _rng(name)
    ss = np.clip(HS.grf_design(p.nd, p.lx, p.ly, p.lz, seed=3, sigma=2.0), 0, 1)
    alpha, kappa, dads, dkds = p.design_fields(ss)
    return dict(sk=np.array(0 if sk == "q9" else 1), alpha=alpha, kappa=kappa, dads=dads, dkds=dkds,
                rho0=1.0 + 0.01 * rng.standard_normal(n), ux0=0.01 * rng.standard_normal(n),
                uy0=0.01 * rng.standard_normal(n),
                uz0=0.01 * rng.standard_normal(n) if p.nd == 3 else np.zeros(n), tem0=0.1 * rng.random(n),
                ip0=0.01 * rng.standard_normal(n), iux0=0.01 * rng.standard_normal(n),
                iuy0=0.01 * rng.standard_normal(n), iuz0=0.01 * rng.standard_normal(n),
                it0=0.01 * rng.standard_normal(n), iqx0=0.01 * rng.standard_normal(n),
                iqy0=0.01 * rng.standard_normal(n), iqz0=0.01 * rng.standard_normal(n))


def hs_phys(p):
    return dict(nu=p.nu, diff=0.0, gx=p.gx, gy=p.gy, gz=p.gz, tem0=p.tem0)


def hs_forward(lib, inp, p):
    q = 9 if p.nd == 2 else 15
    L = lib.lat(q, p.lx, p.ly, p.lz)
    n = p.lx * p.ly * p.lz
    ops = HS.program_ops("forward", p)
    ph = hs_phys(p)
    f, g = np.zeros((q, n)), np.zeros((q, n))
    lib.init(L, 0, f, lib.fields(rho=inp["rho0"], ux=inp["ux0"], uy=inp["uy0"], uz=inp["uz0"]))
    lib.init(L, 1, g, lib.fields(tem=inp["tem0"], ux=inp["ux0"], uy=inp["uy0"], uz=inp["uz0"]))
    mac = {nm: np.zeros(n) for nm in FWD_NAMES}
    snap = np.zeros(n * q)
    for t in range(1, HS_FWD_STEPS + 1):
        lib.collide(L, A.AD_NATURAL, f, g, lib.fields(gsnap=snap, alpha=inp["alpha"], diffusivity=inp["kappa"], **mac),
                    **ph, save=True)
        if t == HS_FWD_STEPS:
            break
        lib.stream(L, f)
        lib.stream(L, g)
        replay(lib, L, f, g, ops, n, ux=mac["ux"], uy=mac["uy"], uz=mac["uz"], kappa=inp["kappa"])
    return L, f, g, mac, snap


def hsfwd_run(lib, inp):
    p = hs_params("q9" if int(inp["sk"]) == 0 else "q15")
    _, f, g, mac, snap = hs_forward(lib, inp, p)
    out = dict(f=f, g=g, snap=snap)
    out.update({"m_" + k: v for k, v in mac.items()})
    return out


def hsadj_run(lib, inp):
    p = hs_params("q9" if int(inp["sk"]) == 0 else "q15")
    L, _, _, mac, gsnap = hs_forward(lib, inp, p)
    q = 9 if p.nd == 2 else 15
    n = p.lx * p.ly * p.lz
    ops = HS.program_ops("adjoint", p)
    ph = hs_phys(p)
    fa, ga = np.zeros((q, n)), np.zeros((q, n))
    lib.init(L, 2, fa, lib.fields(ux=mac["ux"], uy=mac["uy"], uz=mac["uz"], ip=inp["ip0"], iux=inp["iux0"],
                                  iuy=inp["iuy0"], iuz=inp["iuz0"]))
    lib.init(L, 3, ga, lib.fields(ux=mac["ux"], uy=mac["uy"], uz=mac["uz"], item=inp["it0"], iqx=inp["iqx0"],
                                  iqy=inp["iqy0"], iqz=inp["iqz0"]))
    am = {nm: np.zeros(n) for nm in ADJ_NAMES}
    igsnap = np.zeros(n * q)
    fwd = {nm: mac[nm] for nm in ("rho", "ux", "uy", "uz", "tem")}
    for t in range(1, HS_ADJ_STEPS + 1):
        lib.collide(L, A.AAD_NATURAL, fa, ga, lib.fields(gsnap=igsnap, alpha=inp["alpha"], diffusivity=inp["kappa"],
                                                         **fwd, **am), **ph, save=True)
        if t == HS_ADJ_STEPS:
            break
        lib.stream(L, fa, True)
        lib.stream(L, ga, True)
        replay(lib, L, fa, ga, ops, n, ux=mac["ux"], uy=mac["uy"], uz=mac["uz"], rho=mac["rho"], tem=mac["tem"],
               kappa=inp["kappa"])
    out = dict(f=fa, g=ga, snap=igsnap)
    out.update({"m_" + k: v for k, v in am.items()})
    qn, mask = p.source()
    Fo = lib.fields(ux=mac["ux"], uy=mac["uy"], uz=mac["uz"], tem=mac["tem"], imx=am["imx"], imy=am["imy"],
                    imz=am["imz"], item=am["item"], iqx=am["iqx"], iqy=am["iqy"], iqz=am["iqz"],
                    diffusivity=inp["kappa"])
    for which in range(4):
        s = np.zeros(n)
        lib.sensitivity(L, which, s, Fo, inp["dads"], inp["dkds"], gsnap, igsnap, qn, mask)
        out["sens%d" % which] = s
    return out


# ---------------------------------------------------------------------------- incompressible channel
NSIN_SHAPE = (9, 20, 12, 1)
NSIN_FWD_STEPS, NSIN_ADJ_STEPS = 30, 25


def nsin_program(kind, nx, ny, uin):
    """Walls on the y edges, velocity inlet on x = 0, pressure outlet on x = nx-1 (forward); the
    matching adjoint calls (iBoundaryCondition walls, ANSin::iBoundaryConditionSetU,
    ANS::iBoundaryConditionSetRho, which ANSin reuses)."""
    n = nx * ny
    if kind == "forward":
        return [dict(kind=A.BC_WALL, lat=0, axis=1, pos=0, dir=-1), dict(kind=A.BC_WALL, lat=0, axis=1, pos=ny - 1, dir=1),
                dict(kind=A.BC_NSIN_U, axis=0, pos=0, dir=-1, v0=uin, v1=np.zeros(n)),
                dict(kind=A.BC_NSIN_RHO, axis=0, pos=nx - 1, dir=1, c0=1.0, c1=0.0)]
    return [dict(kind=A.BC_IWALL, lat=0, axis=1, pos=0, dir=-1), dict(kind=A.BC_IWALL, lat=0, axis=1, pos=ny - 1, dir=1),
            dict(kind=A.BC_ANSIN_U, axis=0, pos=0, dir=-1, eps=0.3),
            dict(kind=A.BC_ANS_RHO, axis=0, pos=nx - 1, dir=1)]


def nsin_inputs(name):
    q, nx, ny, nz = NSIN_SHAPE
    n = nx * ny
    rng = _rng(name)
    jj = np.repeat(np.arange(ny), nx).astype(np.float64)
    uin = 0.02 * 4.0 * jj * (ny - 1 - jj) / (ny - 1) ** 2
    return dict(alpha=field(rng, n, 0.0, 0.1), dads=field(rng, n, -1, 1), uin=uin,
                rho0=1.0 + 0.01 * rng.standard_normal(n), ux0=0.01 * rng.standard_normal(n),
                uy0=0.01 * rng.standard_normal(n), ip0=0.01 * rng.standard_normal(n),
                iux0=0.01 * rng.standard_normal(n), iuy0=0.01 * rng.standard_normal(n))


def nsin_run(lib, inp):
    """NSin::MacroBrinkmanCollide, Stream and the forward boundary calls for NSIN_FWD_STEPS, then
    ANSin::MacroBrinkmanCollide, iStream and the adjoint calls for NSIN_ADJ_STEPS, then
    ANSin::SensitivityBrinkman (the ANS routine)."""
    q, nx, ny, nz = NSIN_SHAPE
    n = nx * ny
    L = lib.lat(q, nx, ny, 1)
    ph = dict(nu=0.1, diff=0.0, gx=0.0, gy=0.0, gz=0.0, tem0=0.0)
    f = np.zeros((q, n))
    lib.init(L, 4, f, lib.fields(rho=inp["rho0"], ux=inp["ux0"], uy=inp["uy0"]))
    mac = {nm: np.zeros(n) for nm in ("rho", "ux", "uy")}
    ops = nsin_program("forward", nx, ny, inp["uin"])
    for t in range(1, NSIN_FWD_STEPS + 1):
        lib.collide(L, A.NSIN_BRINKMAN, f, None, lib.fields(alpha=inp["alpha"], **mac), **ph, save=True)
        if t == NSIN_FWD_STEPS:
            break
        lib.stream(L, f)
        replay(lib, L, f, None, ops, n)
    fa = np.zeros((q, n))
    lib.init(L, 5, fa, lib.fields(ux=mac["ux"], uy=mac["uy"], ip=inp["ip0"], iux=inp["iux0"], iuy=inp["iuy0"]))
    am = {nm: np.zeros(n) for nm in ("ip", "iux", "iuy", "imx", "imy")}
    ops = nsin_program("adjoint", nx, ny, inp["uin"])
    for t in range(1, NSIN_ADJ_STEPS + 1):
        lib.collide(L, A.ANSIN_BRINKMAN, fa, None, lib.fields(alpha=inp["alpha"], **mac, **am), **ph, save=True)
        if t == NSIN_ADJ_STEPS:
            break
        lib.stream(L, fa, True)
        replay(lib, L, fa, None, ops, n)
    s = np.zeros(n)
    lib.sensitivity(L, 3, s, lib.fields(ux=mac["ux"], uy=mac["uy"], imx=am["imx"], imy=am["imy"]), inp["dads"])
    out = dict(f=f, fa=fa, sens=s)
    out.update({"m_" + k: v for k, v in mac.items()})
    out.update({"m_" + k: v for k, v in am.items()})
    return out


# ---------------------------------------------------------------------------- elastic (D2Q9)
EL_SHAPE = (9, 9, 7, 1)
EL_TAU = 0.8
EL_FWD_NAMES = ("ux", "uy", "sxx", "sxy", "syx", "syy")
EL_ADJ_NAMES = ("irho", "imx", "imy", "isxx", "isxy", "isyx", "isyy")
EL_KINDS = ("EL_COLLIDE", "EL_EXTENDED", "AEL_COLLIDE")
EL_BC_KINDS = ("EL_STRESS", "AEL_STRESS")
# oracle field names of the elastic macros (AEL irho travels in ip)
EL_FIELD = dict(ux="ux", uy="uy", sxx="sxx", sxy="sxy", syx="syx", syy="syy", irho="ip", imx="imx", imy="imy",
                isxx="isxx", isxy="isxy", isyx="isyx", isyy="isyy")


def el_inputs(name, what, kind=""):
    """what: collide / bc / init6 / init7 / sens"""
    q, nx, ny, nz = EL_SHAPE
    n = nx * ny
    rng = _rng(name)
    d = dict(shape=np.array([q, nx, ny, nz]), what=np.array(what), kind=np.array(kind), f=pops(rng, q, n),
             rho=field(rng, n, 0.9, 1.1), gamma=field(rng, n, 0.1, 1.0),
             type=(rng.integers(0, 3, n) > 0).astype(np.int32), v0=field(rng, n, -0.5, 0.5),
             v1=field(rng, n, -0.5, 0.5), dfds=field(rng, n, -1, 1))
    for nm in EL_FWD_NAMES + EL_ADJ_NAMES:
        d["in_" + nm] = field(rng, n, -0.5, 0.5)
    return d


def el_fields(lib, inp, prefix):
    kw = {EL_FIELD[nm]: inp[prefix + nm] for nm in EL_FWD_NAMES + EL_ADJ_NAMES}
    return lib.fields(rho=inp["rho"], gamma=inp["gamma"], **kw)


def el_bc_ops(inp):
    q, nx, ny, nz = _shape(inp)
    kind = str(inp["kind"])
    return [dict(kind=getattr(A, "BC_" + kind), lat=0, axis=a, pos=p, dir=d, type=inp["type"], v0=inp["v0"],
                 v1=inp["v1"], v2=inp["rho"]) for (a, p, d) in faces_with_interior(q, nx, ny, nz)]


def el_run(lib, inp):
    q, nx, ny, nz = _shape(inp)
    L = lib.lat(q, nx, ny, 1)
    n = nx * ny
    what = str(inp["what"])
    f = inp["f"].copy()
    if what == "collide":
        kind = getattr(A, str(inp["kind"]))
        out = {nm: np.zeros(n) for nm in EL_FWD_NAMES + EL_ADJ_NAMES}
        F = lib.fields(rho=inp["rho"], gamma=inp["gamma"], **{EL_FIELD[k]: v for k, v in out.items()})
        lib.collide(L, kind, f, None, F, tau=EL_TAU, save=True)
        names = EL_ADJ_NAMES if kind == A.AEL_COLLIDE else EL_FWD_NAMES
        res = dict(f=f)
        res.update({"m_" + nm: out[nm] for nm in names})
        return res
    if what == "bc":
        replay(lib, L, f, None, el_bc_ops(inp), n)
        return dict(f=f)
    if what in ("init6", "init7"):
        g = np.zeros((q, n))
        lib.init(L, int(what[-1]), g, el_fields(lib, inp, "in_"))
        return dict(f=g)
    dfds = inp["dfds"].copy()
    lib.sensitivity(L, 4, dfds, el_fields(lib, inp, "in_"), None)
    return dict(dfds=dfds)


ELS_SHAPE = (9, 21, 15, 1)
ELS_FWD_STEPS, ELS_ADJ_STEPS = 40, 30
ELS_STRESS0 = -0.01


def elsens_program(kind, nx, ny, rho):
    """test/elsens.cpp:61-66 (forward) and 75-84 (adjoint): BARRIER where i == 0 on the whole
    boundary, the traction ty = STRESS0 on the middle of x = nx-1 (zero elsewhere) on every node
    with i != 0, then SmoothCorner."""
    n = nx * ny
    ii = np.tile(np.arange(nx), ny)
    jj = np.repeat(np.arange(ny), nx)
    wall = (ii == 0).astype(np.int32)
    sel = (ii != 0).astype(np.int32)
    ty = np.where((ii == nx - 1) & (np.abs(jj - 0.5 * ny) < 0.2 * ny), ELS_STRESS0, 0.0)
    edges = [(0, 0, -1), (0, nx - 1, 1), (1, 0, -1), (1, ny - 1, 1)]
    wk, sk = (A.BC_WALL, A.BC_EL_STRESS) if kind == "forward" else (A.BC_IWALL, A.BC_AEL_STRESS)
    ops = [dict(kind=wk, lat=0, axis=a, pos=p, dir=d, type=wall) for (a, p, d) in edges]
    ops += [dict(kind=sk, lat=0, axis=a, pos=p, dir=d, type=sel, v0=np.zeros(n), v1=ty, v2=rho) for (a, p, d) in edges]
    ops.append(dict(kind=A.SMOOTH_CORNER, lat=0))
    return ops


def elsens_inputs(name):
    q, nx, ny, nz = ELS_SHAPE
    n = nx * ny
    rng = _rng(name)
    ii = np.tile(np.arange(nx), ny).astype(np.float64)
    jj = np.repeat(np.arange(ny), nx).astype(np.float64)
    s = np.where((ii - 0.5 * nx) ** 2 + jj ** 2 < (0.3 * nx) ** 2, 0.1, 0.9)
    return dict(rho=1.0 + 0.05 * rng.uniform(-1, 1, n), gamma=s ** 0.25)


def elsens_run(lib, inp):
    """EL::MacroExtendedCollide, Stream and the forward calls for ELS_FWD_STEPS (accumulating
    rx += ux, ry += uy after each step), AEL::MacroCollide, iStream and the adjoint calls for
    ELS_ADJ_STEPS, AEL::SensitivityCompliance and Normalize (test/elsens.cpp:52-92)."""
    q, nx, ny, nz = ELS_SHAPE
    n = nx * ny
    L = lib.lat(q, nx, ny, 1)
    z = np.zeros(n)
    f = np.zeros((q, n))
    mac = {nm: np.zeros(n) for nm in EL_FWD_NAMES + EL_ADJ_NAMES}
    F = lib.fields(rho=inp["rho"], gamma=inp["gamma"], **{EL_FIELD[k]: v for k, v in mac.items()})
    lib.init(L, 6, f, lib.fields(rho=inp["rho"], ux=z, uy=z, sxx=z, sxy=z, syx=z, syy=z))
    rx, ry = np.zeros(n), np.zeros(n)
    ops = elsens_program("forward", nx, ny, inp["rho"])
    for _ in range(ELS_FWD_STEPS):
        lib.collide(L, A.EL_EXTENDED, f, None, F, tau=EL_TAU, save=True)
        lib.stream(L, f)
        replay(lib, L, f, None, ops, n)
        rx += mac["ux"]
        ry += mac["uy"]
    fa = np.zeros((q, n))
    lib.init(L, 7, fa, lib.fields(ip=z, imx=z, imy=z, isxx=z, isxy=z, isyx=z, isyy=z, gamma=inp["gamma"]))
    ops = elsens_program("adjoint", nx, ny, inp["rho"])
    for _ in range(ELS_ADJ_STEPS):
        lib.collide(L, A.AEL_COLLIDE, fa, None, F, tau=EL_TAU, save=True)
        lib.stream(L, fa, True)
        replay(lib, L, fa, None, ops, n)
    dfds = np.zeros(n)
    lib.sensitivity(L, 4, dfds, F, None)
    lib.normalize(dfds)
    out = dict(f=f, fa=fa, rx=rx, ry=ry, dfds=dfds)
    out.update({"m_" + k: v for k, v in mac.items()})
    return out


# ---------------------------------------------------------------------------- transient heat sink
HST_SHAPE = (2, 16, 12, 1)
HST_LEVELS = 25   # time levels 0..nt-1 (the driver's nt)


def hst_params():
    nd, lx, ly, lz = HST_SHAPE
    return HS.Params(nd, lx, ly, lz)


def hst_inputs(name):
    p = hst_params()
    ss = np.clip(HS.grf_design(p.nd, p.lx, p.ly, p.lz, seed=5, sigma=2.0), 0, 1)
    alpha, kappa, dads, dkds = p.design_fields(ss)
    return dict(alpha=alpha, kappa=kappa, dads=dads, dkds=dkds)


def hst_run(lib, inp):
    """production/heatsink_transient.cpp:135-205 with every time level kept: rho, u, T and the g
    snapshot gi[t] of t = 1..nt-1 from the forward loop (t = 0: rest, gi[0] zero), then the adjoint
    from t = nt-2 down to 0 with the sensitivity term of each step; objective sum_t sum_{i<L} T / (L nt)."""
    p = hst_params()
    q, n, nt = 9, p.lx * p.ly, HST_LEVELS
    L = lib.lat(q, p.lx, p.ly, 1)
    ph = hs_phys(p)
    ops_f, ops_a = HS.program_ops("forward", p), HS.program_ops("adjoint", p)
    z = np.zeros(n)
    f, g = np.zeros((q, n)), np.zeros((q, n))
    lv = {0: dict(rho=np.ones(n), ux=z.copy(), uy=z.copy(), uz=z.copy(), tem=z.copy(), gi=np.zeros(n * q))}
    lib.init(L, 0, f, lib.fields(rho=lv[0]["rho"], ux=z, uy=z, uz=z))
    lib.init(L, 1, g, lib.fields(tem=z, ux=z, uy=z, uz=z))
    for t in range(1, nt):
        mac = {nm: np.zeros(n) for nm in FWD_NAMES}
        snap = np.zeros(n * q)
        lib.collide(L, A.AD_NATURAL, f, g, lib.fields(gsnap=snap, alpha=inp["alpha"], diffusivity=inp["kappa"], **mac),
                    **ph, save=True)
        lv[t] = dict(rho=mac["rho"], ux=mac["ux"], uy=mac["uy"], uz=mac["uz"], tem=mac["tem"], gi=snap)
        lib.stream(L, f)
        lib.stream(L, g)
        replay(lib, L, f, g, ops_f, n, ux=mac["ux"], uy=mac["uy"], kappa=inp["kappa"])
    fa, ga = np.zeros((q, n)), np.zeros((q, n))
    last = lv[nt - 1]
    lib.init(L, 2, fa, lib.fields(ux=last["ux"], uy=last["uy"], uz=z, ip=z, iux=z, iuy=z, iuz=z))
    lib.init(L, 3, ga, lib.fields(ux=last["ux"], uy=last["uy"], uz=z, item=z, iqx=z, iqy=z, iqz=z))
    am = {nm: np.zeros(n) for nm in ADJ_NAMES}
    dfdss = np.zeros(n)
    qn, mask = p.source()
    for t in range(nt - 2, -1, -1):
        s = lv[t]
        igi = np.zeros(n * q)
        lib.collide(L, A.AAD_NATURAL, fa, ga, lib.fields(gsnap=igi, alpha=inp["alpha"], diffusivity=inp["kappa"],
                                                         rho=s["rho"], ux=s["ux"], uy=s["uy"], uz=s["uz"],
                                                         tem=s["tem"], **am), **ph, save=True)
        Fo = lib.fields(ux=s["ux"], uy=s["uy"], uz=s["uz"], tem=s["tem"], imx=am["imx"], imy=am["imy"], imz=am["imz"],
                        item=am["item"], iqx=am["iqx"], iqy=am["iqy"], iqz=am["iqz"], diffusivity=inp["kappa"])
        lib.sensitivity(L, 0, dfdss, Fo, inp["dads"], inp["dkds"], s["gi"], igi, qn, mask)
        lib.stream(L, fa, True)
        lib.stream(L, ga, True)
        replay(lib, L, fa, ga, ops_a, n, ux=s["ux"], uy=s["uy"], rho=s["rho"], tem=s["tem"], kappa=inp["kappa"])
    obj = 0.0
    for t in range(nt):
        for i in range(p.lx):
            if i < p.L:
                obj += lv[t]["tem"][i]
    obj /= p.L * nt
    return dict(dfdss=dfdss, objective=np.array(obj), fa=fa, ga=ga, tem_last=last["tem"])


# ---------------------------------------------------------------------------- registry
def all_cases():
    """name -> (make_inputs, run)."""
    cases = {}
    for sk in SHAPES:
        for inv in (0, 1):
            nm = "stream_%s_%s" % (sk, "inv" if inv else "fwd")
            cases[nm] = (lambda nm=nm, sk=sk, inv=inv: stream_inputs(nm, sk, inv), stream_run)
        for kind in BC_KINDS:
            if kind == "AAD_RHO" and sk == "q15":
                continue   # the reference's D3Q15 iBoundaryConditionSetRho overloads do not compile
            if kind in BC_2D_ONLY and sk == "q15":
                continue
            nm = "bc_%s_%s" % (sk, kind)
            cases[nm] = (lambda nm=nm, sk=sk, kind=kind: bc_inputs(nm, sk, kind), bc_run)
        nm = "smooth_%s" % sk
        cases[nm] = (lambda nm=nm, sk=sk: smooth_inputs(nm, sk), smooth_run)
        for kind in FWD + ADJ + (FWD_IN + ADJ_IN if sk == "q9" else []):
            nm = "collide_%s_%s" % (sk, kind)
            cases[nm] = (lambda nm=nm, sk=sk, kind=kind: collide_inputs(nm, sk, kind), collide_run)
        for which in range(6 if sk == "q9" else 4):
            nm = "init_%s_%d" % (sk, which)
            cases[nm] = (lambda nm=nm, sk=sk, w=which: init_inputs(nm, sk, w), init_run)
        for which in range(4):
            nm = "sens_%s_%d" % (sk, which)
            cases[nm] = (lambda nm=nm, sk=sk, w=which: sens_inputs(nm, sk, w), sens_run)
        for R in (1.5, 3.0):
            for masked in (0, 1):
                nm = "filter_%s_R%s_%s" % (sk, str(R).replace(".", "p"), "masked" if masked else "full")
                cases[nm] = (lambda nm=nm, sk=sk, R=R, m=masked: filter_inputs(nm, sk, R, m), filter_run)
        nm = "hsfwd_%s" % sk
        cases[nm] = (lambda nm=nm, sk=sk: hs_inputs(nm, sk), hsfwd_run)
        nm = "hsadj_%s" % sk
        cases[nm] = (lambda nm=nm, sk=sk: hs_inputs(nm, sk), hsadj_run)
    cases["nsinch_q9"] = (lambda: nsin_inputs("nsinch_q9"), nsin_run)
    for kind in EL_KINDS:
        nm = "el_collide_" + kind
        cases[nm] = (lambda nm=nm, kind=kind: el_inputs(nm, "collide", kind), el_run)
    for kind in EL_BC_KINDS:
        nm = "el_bc_" + kind
        cases[nm] = (lambda nm=nm, kind=kind: el_inputs(nm, "bc", kind), el_run)
    for what in ("init6", "init7", "sens"):
        nm = "el_" + what
        cases[nm] = (lambda nm=nm, what=what: el_inputs(nm, what), el_run)
    cases["elsens_q9"] = (lambda: elsens_inputs("elsens_q9"), elsens_run)
    cases["hst_q9"] = (lambda: hst_inputs("hst_q9"), hst_run)
    for nc in (1, 2, 3):
        nm = "resid_%d" % nc
        cases[nm] = (lambda nm=nm, nc=nc: resid_inputs(nm, nc), resid_run)
    return cases


def load(path):
    """(inputs, outputs) of a stored case."""
    z = np.load(path)
    inp = {k[3:]: z[k] for k in z.files if k.startswith("in_")}
    out = {k[4:]: z[k] for k in z.files if k.startswith("out_")}
    return inp, out
