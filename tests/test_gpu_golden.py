"""The CUDA library (FP64 storage and compute, through the C ABI) against the golden fixtures
the reference itself produced (tests/golden/*.npz). Stream, walls and smoothing move data
only and must agree bit for bit; every other output agrees to 1e-12 relative to the field's
largest magnitude (FP64 kernels compiled without FMA contraction, same evaluation order;
reductions in the filters and residual use a fixed tree whose summation order differs).

The standalone sensitivity cases feed arbitrary snapshots, which the library only takes from its
own collides; the sensitivities are checked through hsadj_* (forward, adjoint, snapshots and
the four sensitivity routines on one handle)."""
import glob
import os

import numpy as np
import pytest

from panslbm2_gb300 import _capi as A
from panslbm2_gb300 import heatsink as HS
from panslbm2_gb300.lattice import LatticePair, phys
from tests.golden import cases as C

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
RTOL = 1e-12


def _files(prefix):
    fs = sorted(glob.glob(os.path.join(HERE, "golden", prefix + "_*.npz")))
    return pytest.mark.parametrize("path", fs, ids=[os.path.basename(f)[:-4] for f in fs])


def close(a, b, rtol=RTOL):
    a, b = np.asarray(a, np.float64).reshape(-1), np.asarray(b, np.float64).reshape(-1)
    scale = max(1.0, float(np.max(np.abs(b)))) if b.size else 1.0
    err = float(np.max(np.abs(a - b))) / scale if b.size else 0.0
    assert err <= rtol, "max rel err %.3e" % err


def lattice(inp):
    q, nx, ny, nz = C._shape(inp)
    return LatticePair(q, nx, ny, nz, "fp64"), q, nx * ny * nz


@_files("stream")
def test_stream(path):
    inp, out = C.load(path)
    lp, q, n = lattice(inp)
    lp.set_populations(0, inp["f"])
    lp.set_populations(1, inp["f"])
    lp.stream(mode=int(inp["inverse"]), both=False)
    assert np.array_equal(lp.get_populations(0), out["f"])
    lp.close()


@_files("bc")
def test_boundary_kind(path):
    inp, out = C.load(path)
    lp, q, n = lattice(inp)
    kind = C.BC_KINDS[int(inp["kind"])]
    adjoint_inputs = kind in ("AAD_T", "AAD_Q", "AAD_RHO")
    lp.set_populations(0, inp["f"])
    lp.set_populations(1, inp["g"])
    lp.set_field(A.KAPPA, inp["kap"])
    if adjoint_inputs:
        for fid, nm in ((A.FWD_RHO, "rho"), (A.FWD_UX, "ux"), (A.FWD_UY, "uy"), (A.FWD_UZ, "uz"), (A.FWD_TEM, "tem")):
            lp.set_field(fid, inp[nm])
    else:
        for fid, nm in ((A.UX, "ux"), (A.UY, "uy"), (A.UZ, "uz")):
            lp.set_field(fid, inp[nm])
    prog = lp.program(HS.to_descs(C.bc_ops(inp)))
    lp.stream(mode=3 if adjoint_inputs else 2, prog=prog, both=True)
    f, g = lp.get_populations(0), lp.get_populations(1)
    if kind in ("WALL", "IWALL"):
        assert np.array_equal(f, out["f"]) and np.array_equal(g, out["g"])
    else:
        close(f, out["f"])
        close(g, out["g"])
    lp.close()


@_files("smooth")
def test_smoothing(path):
    inp, out = C.load(path)
    lp, q, n = lattice(inp)
    lp.set_populations(0, inp["f"])
    lp.set_populations(1, inp["g"])
    lp.stream(mode=2, prog=lp.program(HS.to_descs(C.smooth_ops(q))), both=True)
    assert np.array_equal(lp.get_populations(0), out["f"])
    assert np.array_equal(lp.get_populations(1), out["g"])
    lp.close()


@_files("collide")
def test_collide(path):
    inp, out = C.load(path)
    lp, q, n = lattice(inp)
    k = int(inp["kind"])
    lp.set_populations(0, inp["f"])
    if inp["g"].size:
        lp.set_populations(1, inp["g"])
    for fid, nm in ((A.ALPHA, "alpha"), (A.KAPPA, "diffusivity"), (A.BETA, "beta"), (A.DIRX, "dirx"),
                    (A.DIRY, "diry"), (A.DIRZ, "dirz")):
        lp.set_field(fid, inp[nm])
    if k >= 10:
        for fid, nm in ((A.FWD_RHO, "rho"), (A.FWD_UX, "ux"), (A.FWD_UY, "uy"), (A.FWD_UZ, "uz"), (A.FWD_TEM, "tem")):
            lp.set_field(fid, inp[nm])
    lp.collide(k, phys(**C.PH), save=True)
    close(lp.get_populations(0), out["f"])
    if inp["g"].size:
        close(lp.get_populations(1), out["g"])
    names, base = (C.ADJ_NAMES, A.IP) if k >= 10 else (C.FWD_NAMES, A.RHO)
    for m, nm in enumerate(names):
        if q == 9 and nm.endswith("z"):
            continue
        if not inp["g"].size and nm in ("tem", "qx", "qy", "qz", "item", "iqx", "iqy", "iqz"):
            continue
        if k == A.AAD_FORCE and nm == "iuz":
            continue     # not saved by the reference's 3D routine (its output array stays as it was)
        close(lp.get_field(base + m), out["m_" + nm], 1e-11)
    if k in (A.AD_NATURAL, A.AD_FORCE, A.AAD_NATURAL, A.AAD_FORCE, A.AAD_MASSFLOW):
        close(lp.snapshot(1 if k >= 10 else 0), out["snap"])
    lp.close()


@_files("init")
def test_initial_condition(path):
    inp, out = C.load(path)
    lp, q, n = lattice(inp)
    w = int(inp["which"])
    a = {0: ("rho",), 1: ("tem",), 2: ("ip", "iux", "iuy", "iuz"), 3: ("item", "iqx", "iqy", "iqz"), 4: ("rho",),
         5: ("ip", "iux", "iuy", "iuz")}[w]
    args = [inp[nm] for nm in a]
    if w == 5:   # ANSin::InitialCondition takes the velocity but does not read it
        lp.init(w, *args)
    else:
        lp.init(w, *args, ux=inp["ux"], uy=inp["uy"], uz=inp["uz"])
    close(lp.get_populations(0 if w in (0, 2, 4, 5) else 1), out["f"])
    lp.close()


@_files("filter")
def test_filters(path):
    inp, out = C.load(path)
    lp, q, n = lattice(inp)
    R, beta = float(inp["R"]), float(inp["beta"])
    mask = inp["mask"] if inp["mask"].size else None
    close(lp.heaviside_var(R, beta, inp["s"], mask), out["var"])
    close(lp.heaviside_sens(R, beta, inp["s"], inp["dfd"], mask), out["sens"])
    close(lp.density_filter(R, inp["s"], mask), out["dens"])
    lp.close()


@_files("resid")
def test_residual_normalize(path):
    inp, out = C.load(path)
    lp = LatticePair(9, 40, 40, 1, "fp64")
    nc = int(inp["ncomp"])
    r = lp.residual_host([inp["a%d" % m] for m in range(nc)], [inp["b%d" % m] for m in range(nc)])
    assert abs(r - float(out["residual"])) <= RTOL * abs(float(out["residual"]))
    assert np.array_equal(lp.normalize(inp["a0"].copy()), out["normalized"])
    lp.close()


def _forward(inp):
    p = C.hs_params("q9" if int(inp["sk"]) == 0 else "q15")
    q = 9 if p.nd == 2 else 15
    lp = LatticePair(q, p.lx, p.ly, p.lz, "fp64")
    lp.set_field(A.ALPHA, inp["alpha"])
    lp.set_field(A.KAPPA, inp["kappa"])
    lp.init(0, inp["rho0"], ux=inp["ux0"], uy=inp["uy0"], uz=inp["uz0"])
    lp.init(1, inp["tem0"], ux=inp["ux0"], uy=inp["uy0"], uz=inp["uz0"])
    ph = phys(**C.hs_phys(p))
    prog = lp.program(HS.to_descs(HS.program_ops("forward", p)))
    lp.collide(A.AD_NATURAL, ph, save=True)
    for t in range(2, C.HS_FWD_STEPS + 1):
        lp.step(A.AD_NATURAL, ph, prog, save=(t == C.HS_FWD_STEPS))
    return lp, p, q, ph


@_files("hsfwd")
def test_heatsink_forward(path):
    inp, out = C.load(path)
    lp, p, q, _ = _forward(inp)
    close(lp.get_populations(0), out["f"], 1e-11)
    close(lp.get_populations(1), out["g"], 1e-11)
    for m, nm in enumerate(C.FWD_NAMES):
        if q == 9 and nm.endswith("z"):
            continue
        close(lp.get_field(A.RHO + m), out["m_" + nm], 1e-11)
    close(lp.snapshot(0), out["snap"], 1e-11)
    lp.close()


@_files("hsadj")
def test_heatsink_adjoint_and_sensitivities(path):
    inp, out = C.load(path)
    lp, p, q, ph = _forward(inp)
    g0 = lp.snapshot(0)                 # also kept on the device for the sensitivity
    lp.freeze_forward()
    fu = [lp.get_field(A.FWD_UX), lp.get_field(A.FWD_UY), lp.get_field(A.FWD_UZ)]
    lp.init(2, inp["ip0"], inp["iux0"], inp["iuy0"], inp["iuz0"], ux=fu[0], uy=fu[1], uz=fu[2])
    lp.init(3, inp["it0"], inp["iqx0"], inp["iqy0"], inp["iqz0"], ux=fu[0], uy=fu[1], uz=fu[2])
    prog = lp.program(HS.to_descs(HS.program_ops("adjoint", p)))
    lp.collide(A.AAD_NATURAL, ph, save=True)
    for t in range(2, C.HS_ADJ_STEPS + 1):
        lp.step(A.AAD_NATURAL, ph, prog, save=(t == C.HS_ADJ_STEPS))
    close(lp.get_populations(0), out["f"], 1e-11)
    close(lp.get_populations(1), out["g"], 1e-11)
    for m, nm in enumerate(C.ADJ_NAMES):
        if q == 9 and nm.endswith("z"):
            continue
        close(lp.get_field(A.IP + m), out["m_" + nm], 1e-11)
    g1 = lp.snapshot(1)
    close(g1, out["snap"], 1e-11)
    qn, mask = p.source()
    n = lp.n
    got = []
    for which in range(4):
        got.append(lp.sensitivity(which, np.zeros(n), inp["dads"], inp["dkds"], qn, mask))
        close(got[-1], out["sens%d" % which], 1e-10)
    # the same sensitivities from snapshots loaded back from host copies (pl_set_snapshot)
    lp.set_snapshot(0, g0)
    lp.set_snapshot(1, g1)
    for which in range(2):
        assert np.array_equal(lp.sensitivity(which, np.zeros(n), inp["dads"], inp["dkds"], qn, mask), got[which])
    lp.close()


@_files("nsinch")
def test_incompressible_channel(path):
    """NSin forward and ANSin adjoint through fused steps (pull + boundary program + collide),
    then the Brinkman sensitivity, against the reference's own loop."""
    inp, out = C.load(path)
    q, nx, ny, _ = C.NSIN_SHAPE
    lp = LatticePair(q, nx, ny, 1, "fp64")
    n = nx * ny
    ph = phys(nu=0.1, diff=0.0)
    lp.set_field(A.ALPHA, inp["alpha"])
    lp.init(4, inp["rho0"], ux=inp["ux0"], uy=inp["uy0"])
    prog = lp.program(HS.to_descs(C.nsin_program("forward", nx, ny, inp["uin"])))
    lp.collide(A.NSIN_BRINKMAN, ph, save=True)
    for t in range(2, C.NSIN_FWD_STEPS + 1):
        lp.step(A.NSIN_BRINKMAN, ph, prog, save=(t == C.NSIN_FWD_STEPS))
    close(lp.get_populations(0), out["f"], 1e-11)
    for fid, nm in ((A.RHO, "rho"), (A.UX, "ux"), (A.UY, "uy")):
        close(lp.get_field(fid), out["m_" + nm], 1e-11)
    lp.freeze_forward()
    lp.init(5, inp["ip0"], inp["iux0"], inp["iuy0"], np.zeros(n))
    prog = lp.program(HS.to_descs(C.nsin_program("adjoint", nx, ny, inp["uin"])))
    lp.collide(A.ANSIN_BRINKMAN, ph, save=True)
    for t in range(2, C.NSIN_ADJ_STEPS + 1):
        lp.step(A.ANSIN_BRINKMAN, ph, prog, save=(t == C.NSIN_ADJ_STEPS))
    close(lp.get_populations(0), out["fa"], 1e-11)
    for fid, nm in ((A.IP, "ip"), (A.IUX, "iux"), (A.IUY, "iuy"), (A.IMX, "imx"), (A.IMY, "imy")):
        close(lp.get_field(fid), out["m_" + nm], 1e-11)
    close(lp.sensitivity(3, np.zeros(n), inp["dads"]), out["sens"], 1e-10)
    lp.close()


def test_incompressible_kinds_are_d2q9_only():
    lp = LatticePair(15, 6, 5, 4, "fp64")
    with pytest.raises(A.PanslbmError, match="D2Q9 only"):
        lp.collide(A.NSIN_COLLIDE, phys(nu=0.1, diff=0.0))
    with pytest.raises(A.PanslbmError, match="D2Q9 only"):
        lp.program(HS.to_descs([dict(kind=A.BC_NSIN_U, axis=0, pos=0, dir=-1)]))
    lp.close()


def _el_lattice(inp, storage="fp64"):
    q, nx, ny, _ = C._shape(inp)
    return LatticePair(q, nx, ny, 1, storage), nx * ny


@_files("el")
@pytest.mark.parametrize("storage", ["fp64", "fp32"])
def test_elastic_routines(path, storage):
    """EL / AEL collides, stress boundary routines, initial conditions and the compliance
    sensitivity against the reference's outputs: FP64 to 1e-12 (bit-exact arithmetic order, the
    stress routines divide), FP32 compute to 2e-6 of the field's largest magnitude."""
    inp, out = C.load(path)
    lp, n = _el_lattice(inp, storage)
    tol = RTOL if storage == "fp64" else 2e-6
    what = str(inp["what"])
    lp.set_field(A.DENSITY, inp["rho"])
    lp.set_field(A.GAMMA, inp["gamma"])
    if what == "collide":
        kind = getattr(A, str(inp["kind"]))
        lp.set_populations(0, inp["f"])
        lp.collide(kind, phys(tau=C.EL_TAU), save=True)
        close(lp.get_populations(0), out["f"], tol)
        fids = dict(ux=A.UX, uy=A.UY, sxx=A.SXX, sxy=A.SXY, syx=A.SYX, syy=A.SYY, irho=A.IRHO, imx=A.IMX, imy=A.IMY,
                    isxx=A.ISXX, isxy=A.ISXY, isyx=A.ISYX, isyy=A.ISYY)
        for nm in (C.EL_ADJ_NAMES if kind == A.AEL_COLLIDE else C.EL_FWD_NAMES):
            close(lp.get_field(fids[nm]), out["m_" + nm], tol * 10)
    elif what == "bc":
        lp.set_populations(0, inp["f"])
        prog = lp.program(HS.to_descs(C.el_bc_ops(inp)))
        lp.stream(mode=3 if str(inp["kind"]) == "AEL_STRESS" else 2, prog=prog, both=False)
        close(lp.get_populations(0), out["f"], tol)
    elif what in ("init6", "init7"):
        names = C.EL_FWD_NAMES if what == "init6" else C.EL_ADJ_NAMES
        arrays = [inp["rho"]] + [inp["in_" + nm] for nm in names] if what == "init6" else \
            [inp["in_" + nm] for nm in names]
        lp.init_elastic(0 if what == "init6" else 1, arrays)
        close(lp.get_populations(0), out["f"], tol)
    else:
        arrays = [inp["in_" + nm] for nm in ("sxx", "sxy", "syx", "syy", "irho", "isxx", "isxy", "isyx", "isyy")]
        got = lp.sensitivity_compliance(inp["dfds"], arrays)
        if storage == "fp64":
            assert np.array_equal(got, out["dfds"])   # rounded term by term, like the reference
        else:
            close(got, out["dfds"], tol)
    lp.close()


@_files("elsens")
@pytest.mark.parametrize("fused", [True, False])
def test_elastic_compliance_driver(path, fused):
    """test/elsens.cpp on a small plate: EL forward steps (fused pull + boundary program +
    MacroExtendedCollide, or collide and stream calls separately) with the displacement summed
    over the steps, AEL adjoint steps, the compliance sensitivity from the saved macros on the
    device and Normalize, against the reference's own loop."""
    inp, out = C.load(path)
    q, nx, ny, _ = C.ELS_SHAPE
    n = nx * ny
    lp = LatticePair(q, nx, ny, 1, "fp64")
    ph = phys(tau=C.EL_TAU)
    z = np.zeros(n)
    lp.set_field(A.DENSITY, inp["rho"])
    lp.set_field(A.GAMMA, inp["gamma"])
    lp.init_elastic(0, [inp["rho"], z, z, z, z, z, z])
    prog = lp.program(HS.to_descs(C.elsens_program("forward", nx, ny, inp["rho"])))
    rx, ry = np.zeros(n), np.zeros(n)
    for t in range(C.ELS_FWD_STEPS):
        if t == 0 or not fused:
            lp.collide(A.EL_EXTENDED, ph, save=True)
        else:
            lp.step(A.EL_EXTENDED, ph, prog, save=True)
        rx += lp.get_field(A.UX)
        ry += lp.get_field(A.UY)
        if not fused or t == C.ELS_FWD_STEPS - 1:
            lp.stream(mode=0, prog=prog, both=False)
    close(lp.get_populations(0), out["f"], 1e-11)
    close(rx, out["rx"], 1e-11)
    close(ry, out["ry"], 1e-11)
    for fid, nm in ((A.UX, "ux"), (A.UY, "uy"), (A.SXX, "sxx"), (A.SXY, "sxy"), (A.SYX, "syx"), (A.SYY, "syy")):
        close(lp.get_field(fid), out["m_" + nm], 1e-11)
    lp.init_elastic(1, [z] * 7)
    prog = lp.program(HS.to_descs(C.elsens_program("adjoint", nx, ny, inp["rho"])))
    for t in range(C.ELS_ADJ_STEPS):
        if t == 0 or not fused:
            lp.collide(A.AEL_COLLIDE, ph, save=True)
        else:
            lp.step(A.AEL_COLLIDE, ph, prog, save=True)
        if not fused or t == C.ELS_ADJ_STEPS - 1:
            lp.stream(mode=1, prog=prog, both=False)
    close(lp.get_populations(0), out["fa"], 1e-11)
    for fid, nm in ((A.IRHO, "irho"), (A.IMX, "imx"), (A.IMY, "imy"), (A.ISXX, "isxx"), (A.ISXY, "isxy"),
                    (A.ISYX, "isyx"), (A.ISYY, "isyy")):
        close(lp.get_field(fid), out["m_" + nm], 1e-11)
    close(lp.normalize(lp.sensitivity_compliance(np.zeros(n))), out["dfds"], 1e-10)
    lp.close()


def test_elastic_kinds_are_d2q9_only():
    lp = LatticePair(15, 6, 5, 4, "fp64")
    with pytest.raises(A.PanslbmError, match="D2Q9 only"):
        lp.collide(A.EL_COLLIDE, phys(tau=0.8))
    with pytest.raises(A.PanslbmError, match="D2Q9 only"):
        lp.program(HS.to_descs([dict(kind=A.BC_EL_STRESS, axis=0, pos=0, dir=-1)]))
    lp.close()
