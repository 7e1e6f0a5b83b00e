"""Build recipe for the oracle (test infrastructure only).

* ``liboracle.so``  -- the plain-C restatement (oracle.c), built with gcc on any host;
* ``_ref/libref.so`` -- the same API bound to the PANSLBM2 reference's own header templates,
  compiled from the reference sources where they lie: the tree named by PANSLBM2_REF, or the
  one a build step passed to ``build_ref(root=...)`` (recorded in ``_ref/REFERENCE_ROOT``).
  Built only where those sources exist; nothing is copied from them. With neither set, the
  reference-backed checks are skipped and say so.

Both use ``-O2 -ffp-contract=off`` so that the two agree bit-for-bit on the scalar path.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
MARKER = os.path.join(HERE, "_ref", "REFERENCE_ROOT")
FLAGS = ["-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-fno-fast-math"]


def _newer(out, srcs):
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    return all(os.path.getmtime(s) <= t for s in srcs)


def build_oracle(force=False):
    out = os.path.join(HERE, "liboracle.so")
    srcs = [os.path.join(HERE, "oracle.c"), os.path.join(HERE, "oracle.h")]
    if force or not _newer(out, srcs):
        cmd = ["gcc", "-std=c11"] + FLAGS + ["-o", out, srcs[0], "-lm"]
        subprocess.check_call(cmd)
    return out


def _is_reference(root):
    return bool(root) and os.path.isfile(os.path.join(root, "src", "particle", "d2q9.h"))


def reference_root():
    """The reference tree: PANSLBM2_REF if it names one, else the tree the last build_ref(root=...)
    recorded; None when neither exists on this machine (PANSLBM2_REF not set: the
    reference-backed checks skip)."""
    env = os.environ.get("PANSLBM2_REF")
    if _is_reference(env):
        return env
    try:
        with open(MARKER) as fh:
            rec = fh.read().strip()
    except OSError:
        rec = None
    return rec if _is_reference(rec) else None


def build_ref(force=False, root=None):
    """Compile the reference-backed library from the tree `root` (default: reference_root());
    returns its path or None when the sources are absent."""
    root = root if _is_reference(root) else reference_root()
    if root is None:
        return None
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    with open(MARKER, "w") as fh:
        fh.write(root + "\n")
    out = os.path.join(outdir, "libref.so")
    srcs = [os.path.join(HERE, f) for f in ("ref_harness.cpp", "ref_api.cpp", "oracle.h")]
    if not force and _newer(out, srcs):
        return out
    objs = []
    for dim in (2, 3):
        o = os.path.join(outdir, "ref%d.o" % dim)
        subprocess.check_call(["g++", "-std=c++17", "-DREF_DIM=%d" % dim, "-I", root, "-I", HERE, "-c",
                               "-o", o, os.path.join(HERE, "ref_harness.cpp"), "-w"] + FLAGS[:-1])
        objs.append(o)
    subprocess.check_call(["g++", "-std=c++17", "-I", HERE] + FLAGS + ["-o", out, os.path.join(HERE, "ref_api.cpp")]
                          + objs)
    return out


def build_ref_mma(force=False, root=None):
    """The reference's own MMA<double> behind a C entry point (golden vectors of the MMA update);
    None when the reference sources are absent."""
    root = root if _is_reference(root) else reference_root()
    if root is None:
        return None
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    out = os.path.join(outdir, "libref_mma.so")
    src = os.path.join(HERE, "ref_mma.cpp")
    if force or not _newer(out, [src]):
        subprocess.check_call(["g++", "-std=c++17", "-I", root, "-w"] + FLAGS + ["-o", out, src])
    return out


if __name__ == "__main__":
    print(build_oracle(force="-f" in sys.argv))
    print(build_ref(force="-f" in sys.argv, root=sys.argv[-1] if len(sys.argv) > 1 else None))
