"""The drop-in template API on the GPU: tests/dropin/heatsink_driver.cpp, written against
PANSLBM2's API and built on dropin/src + the CUDA library, runs the golden heat-sink cases
(forward loop; forward + adjoint loops + the four sensitivities) and must reproduce the
reference's own outputs (tests/golden/hs*_*.npz) to 1e-11 relative (FP64 storage and compute;
1e-10 for the sensitivities)."""
import glob
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from tests.golden import cases as C

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "panslbm2_gb300")


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    out = str(tmp_path_factory.mktemp("dropin") / "heatsink_driver")
    cmd = [cxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "dropin", "heatsink_driver.cpp"), "-L", LIBDIR, "-lpanslbm_gb300",
           "-Wl,-rpath," + LIBDIR, "-o", out]
    subprocess.check_call(cmd)
    return out


def close(a, b, rtol):
    a, b = np.asarray(a, np.float64).reshape(-1), np.asarray(b, np.float64).reshape(-1)
    scale = max(1.0, float(np.max(np.abs(b))))
    err = float(np.max(np.abs(a - b))) / scale
    assert err <= rtol, "max rel err %.3e" % err


def run(driver, tmp_path, mode, inp):
    p = C.hs_params("q9" if int(inp["sk"]) == 0 else "q15")
    fin, fout = tmp_path / "in.bin", tmp_path / "out.bin"
    names = ["alpha", "kappa", "dads", "dkds", "rho0", "ux0", "uy0", "uz0", "tem0", "ip0", "iux0", "iuy0", "iuz0", "it0",
             "iqx0", "iqy0", "iqz0"]
    with open(fin, "wb") as fh:
        fh.write(struct.pack("6i", p.nd, p.lx, p.ly, p.lz, C.HS_FWD_STEPS, C.HS_ADJ_STEPS))
        fh.write(struct.pack("7d", p.nu, p.gx, p.gy, p.gz, p.tem0, p.qn, p.L))
        for nm in names:
            fh.write(np.ascontiguousarray(inp[nm], np.float64).tobytes())
    subprocess.check_call([driver, mode, str(fin), str(fout)])
    return p, np.fromfile(fout, np.float64)


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "hsfwd_*.npz"))),
                         ids=lambda s: os.path.basename(s)[:-4])
def test_dropin_forward_loop(driver, tmp_path, path):
    inp, out = C.load(path)
    p, got = run(driver, tmp_path, "fwd", inp)
    q, n = (9 if p.nd == 2 else 15), p.lx * p.ly * p.lz
    close(got[:q * n], out["f"], 1e-11)
    close(got[q * n:2 * q * n], out["g"], 1e-11)
    mac = got[2 * q * n:].reshape(8, n)
    for m, nm in enumerate(C.FWD_NAMES):
        if p.nd == 2 and nm.endswith("z"):
            continue
        close(mac[m], out["m_" + nm], 1e-11)


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "hsadj_*.npz"))),
                         ids=lambda s: os.path.basename(s)[:-4])
def test_dropin_adjoint_loop_and_sensitivities(driver, tmp_path, path):
    inp, out = C.load(path)
    p, got = run(driver, tmp_path, "adj", inp)
    q, n = (9 if p.nd == 2 else 15), p.lx * p.ly * p.lz
    close(got[:q * n], out["f"], 1e-11)
    close(got[q * n:2 * q * n], out["g"], 1e-11)
    rest = got[2 * q * n:]
    mac = rest[:11 * n].reshape(11, n)
    for m, nm in enumerate(C.ADJ_NAMES):
        if p.nd == 2 and nm.endswith("z"):
            continue
        close(mac[m], out["m_" + nm], 1e-11)
    sens = rest[11 * n:].reshape(4, n)
    for w in range(4):
        close(sens[w], out["sens%d" % w], 1e-10)


@pytest.fixture(scope="module")
def nsin_driver(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    out = str(tmp_path_factory.mktemp("dropin") / "nsin_channel_driver")
    cmd = [cxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "dropin", "nsin_channel_driver.cpp"), "-L", LIBDIR, "-lpanslbm_gb300",
           "-Wl,-rpath," + LIBDIR, "-o", out]
    subprocess.check_call(cmd)
    return out


def test_dropin_incompressible_channel(nsin_driver, tmp_path):
    """NSin forward + ANSin adjoint + the Brinkman sensitivity written against the template API
    reproduce the reference's own loop (tests/golden/nsinch_q9.npz)."""
    inp, out = C.load(os.path.join(ROOT, "tests", "golden", "nsinch_q9.npz"))
    q, nx, ny, _ = C.NSIN_SHAPE
    n = nx * ny
    fin, fout = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(fin, "wb") as fh:
        fh.write(struct.pack("4i", nx, ny, C.NSIN_FWD_STEPS, C.NSIN_ADJ_STEPS))
        fh.write(struct.pack("2d", 0.1, 0.3))
        for nm in ("alpha", "dads", "uin", "rho0", "ux0", "uy0", "ip0", "iux0", "iuy0"):
            fh.write(np.ascontiguousarray(inp[nm], np.float64).tobytes())
    subprocess.check_call([nsin_driver, str(fin), str(fout)])
    got = np.fromfile(fout, np.float64)
    close(got[:q * n], out["f"], 1e-11)
    o = q * n
    for nm in ("rho", "ux", "uy"):
        close(got[o:o + n], out["m_" + nm], 1e-11)
        o += n
    close(got[o:o + q * n], out["fa"], 1e-11)
    o += q * n
    for nm in ("ip", "iux", "iuy", "imx", "imy"):
        close(got[o:o + n], out["m_" + nm], 1e-11)
        o += n
    close(got[o:o + n], out["sens"], 1e-10)


@pytest.fixture(scope="module")
def elastic_driver(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    out = str(tmp_path_factory.mktemp("dropin") / "elastic_driver")
    cmd = [cxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "dropin", "elastic_driver.cpp"), "-L", LIBDIR, "-lpanslbm_gb300",
           "-Wl,-rpath," + LIBDIR, "-o", out]
    subprocess.check_call(cmd)
    return out


def test_dropin_elastic_compliance(elastic_driver, tmp_path):
    """The loops of the reference's test/elsens.cpp (EL forward with the displacement summed on
    the host, AEL adjoint, the compliance sensitivity, Normalize) written against the template API
    reproduce the reference's own loop (tests/golden/elsens_q9.npz)."""
    inp, out = C.load(os.path.join(ROOT, "tests", "golden", "elsens_q9.npz"))
    q, nx, ny, _ = C.ELS_SHAPE
    n = nx * ny
    fin, fout = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(fin, "wb") as fh:
        fh.write(struct.pack("4i", nx, ny, C.ELS_FWD_STEPS, C.ELS_ADJ_STEPS))
        fh.write(struct.pack("2d", C.EL_TAU, C.ELS_STRESS0))
        for nm in ("rho", "gamma"):
            fh.write(np.ascontiguousarray(inp[nm], np.float64).tobytes())
    subprocess.check_call([elastic_driver, str(fin), str(fout)])
    got = np.fromfile(fout, np.float64)
    close(got[:q * n], out["f"], 1e-11)
    o = q * n
    for nm in ("rx", "ry", "m_ux", "m_uy", "m_sxx", "m_sxy", "m_syx", "m_syy"):
        close(got[o:o + n], out[nm], 1e-11)
        o += n
    close(got[o:o + q * n], out["fa"], 1e-11)
    o += q * n
    for nm in ("irho", "imx", "imy", "isxx", "isxy", "isyx", "isyy"):
        close(got[o:o + n], out["m_" + nm], 1e-11)
        o += n
    close(got[o:o + n], out["dfds"], 1e-10)
