"""The drop-in headers (dropin/src) compile as PANSLBM2's template API: the heat-sink test
driver written against that API, and, where the reference sources are present, the reference's
own production drivers unchanged (copied to a scratch directory whose ../src is dropin/src).
The drop-in tree is self-contained: no header of the reference is on the include path.
No GPU needed: compile and link only."""
import os
import shutil
import subprocess

import pytest

from oracle import build as obuild

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "panslbm2_gb300")
LIB = os.path.join(LIBDIR, "libpanslbm_gb300.so")
CXX = shutil.which("g++")

pytestmark = pytest.mark.skipif(CXX is None, reason="g++ not found")


def _compile(src, out, extra=()):
    cmd = [CXX, "-std=c++17", "-O1", "-Wall", "-Wextra", "-Wno-unused-parameter", "-I", os.path.join(ROOT, "include")]
    cmd += list(extra)
    if os.path.exists(LIB):
        cmd += [src, "-L", LIBDIR, "-lpanslbm_gb300", "-o", out]
    else:
        cmd += ["-c", src, "-o", out]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr[-4000:]


@pytest.mark.parametrize("driver", ["heatsink_driver", "nsin_channel_driver", "elastic_driver", "filter_driver"])
def test_test_driver_builds(tmp_path, driver):
    _compile(os.path.join(ROOT, "tests", "dropin", driver + ".cpp"), str(tmp_path / driver))


@pytest.mark.skipif(obuild.reference_root() is None, reason="reference sources not present")
@pytest.mark.parametrize("driver", ["heatsink", "heatsink3D", "ncpump", "ncpump_periodic", "heatsink_transient", "nsopt"])
def test_reference_production_driver_builds_unchanged(tmp_path, driver):
    ref = obuild.reference_root()
    (tmp_path / "production").mkdir()
    shutil.copy(os.path.join(ref, "production", driver + ".cpp"), tmp_path / "production")
    os.symlink(os.path.join(ROOT, "dropin", "src"), tmp_path / "src")
    # the reference's own code trips -Wall here and there: build it as the reference does, quietly
    cmd = [CXX, "-std=c++17", "-O1", "-w", "-I", os.path.join(ROOT, "include")]
    src, out = str(tmp_path / "production" / (driver + ".cpp")), str(tmp_path / driver)
    if os.path.exists(LIB):
        cmd += [src, "-L", LIBDIR, "-lpanslbm_gb300", "-o", out]
    else:
        cmd += ["-c", src, "-o", out]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr[-4000:]


@pytest.mark.skipif(obuild.reference_root() is None, reason="reference sources not present")
@pytest.mark.parametrize("driver", ["elsens"])
def test_reference_test_driver_builds_unchanged(tmp_path, driver):
    """The reference's own elastic sensitivity driver (test/elsens.cpp: EL, AEL, Normalize and the
    XML exporter) compiles against the drop-in headers unchanged."""
    ref = obuild.reference_root()
    (tmp_path / "test").mkdir()
    shutil.copy(os.path.join(ref, "test", driver + ".cpp"), tmp_path / "test")
    os.symlink(os.path.join(ROOT, "dropin", "src"), tmp_path / "src")
    cmd = [CXX, "-std=c++17", "-O1", "-w", "-I", os.path.join(ROOT, "include")]
    src, out = str(tmp_path / "test" / (driver + ".cpp")), str(tmp_path / driver)
    if os.path.exists(LIB):
        cmd += [src, "-L", LIBDIR, "-lpanslbm_gb300", "-o", out]
    else:
        cmd += ["-c", src, "-o", out]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr[-4000:]
