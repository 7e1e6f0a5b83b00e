"""The drop-in VTK writers and readers (dropin/src/utility/vtk*.h) against the reference's own
headers: tests/dropin/vtk_roundtrip.cpp writes a legacy file and a .pvts/.vts pair, reads them
back, and dumps what it read. Every file must equal, byte for byte, the one the reference's
headers produce (tests/golden/vtk/, written by running this module as a script where the
reference sources are). Host code only; no GPU.

    python -m tests.test_vtk_dropin   # regenerate tests/golden/vtk from the reference build
"""
import os
import shutil
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
from oracle import build as obuild  # noqa: E402

SRC = os.path.join(ROOT, "tests", "dropin", "vtk_roundtrip.cpp")
GOLDEN = os.path.join(ROOT, "tests", "golden", "vtk")
SHAPE = ("7", "5", "3")
FILES = ("legacy.vtk", "xml.pvts", "xml_0.vts", "read.bin")
CXX = shutil.which("g++")


def run(workdir, ref=None):
    """Build the round trip (against the reference's headers when `ref` is its root) and run it in
    workdir; returns its stdout with the directory name taken out."""
    exe = os.path.join(workdir, "roundtrip")
    cmd = [CXX, "-std=c++17", "-O2", "-pthread", SRC, "-o", exe]
    if ref:
        cmd += ["-DUSE_REF", "-I", ref, "-w"]
    subprocess.check_call(cmd)
    out = os.path.join(workdir, "out")
    os.makedirs(out, exist_ok=True)
    p = subprocess.run([exe, out, *SHAPE], capture_output=True, text=True, check=True)
    return out, p.stdout.replace(out, "<dir>")


@pytest.mark.skipif(CXX is None, reason="g++ not found")
def test_dropin_vtk_matches_reference_bytes(tmp_path):
    out, stdout = run(str(tmp_path))
    for f in FILES:
        with open(os.path.join(out, f), "rb") as a, open(os.path.join(GOLDEN, f), "rb") as b:
            assert a.read() == b.read(), f
    with open(os.path.join(GOLDEN, "stdout.txt")) as fh:
        assert stdout == fh.read()


@pytest.mark.skipif(CXX is None or obuild.reference_root() is None, reason="reference sources not present")
def test_vtk_fixtures_are_the_reference_output(tmp_path):
    out, stdout = run(str(tmp_path), obuild.reference_root())
    for f in FILES:
        with open(os.path.join(out, f), "rb") as a, open(os.path.join(GOLDEN, f), "rb") as b:
            assert a.read() == b.read(), f
    with open(os.path.join(GOLDEN, "stdout.txt")) as fh:
        assert stdout == fh.read()


if __name__ == "__main__":
    import tempfile
    if obuild.reference_root() is None:
        raise SystemExit("reference sources not found: the VTK fixtures come from the reference build")
    with tempfile.TemporaryDirectory() as d:
        out, stdout = run(d, obuild.reference_root())
        os.makedirs(GOLDEN, exist_ok=True)
        for f in FILES:
            shutil.copy(os.path.join(out, f), os.path.join(GOLDEN, f))
        with open(os.path.join(GOLDEN, "stdout.txt"), "w") as fh:
            fh.write(stdout)
    print("wrote", GOLDEN)
