"""Regenerate the golden fixtures of tests/golden from the reference itself.

Builds the library that compiles PANSLBM2's own headers (oracle/build.py: build_ref, which needs
the reference sources) and runs every case of cases.py through it; writes one compressed
<case>.npz per case holding the inputs (in_*) and the reference's outputs (out_*).

    python -m tests.golden.make_golden [--check]

--check only verifies that the stored outputs still equal the reference's (bit for bit).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from oracle import build as obuild  # noqa: E402
from oracle.olib import Oracle  # noqa: E402
from tests.golden import cases as C  # noqa: E402


MMA_CASES = {"mma_m1": dict(n=600, m=1, seed=21), "mma_m2": dict(n=400, m=2, seed=22)}
MMA_ITERS = 5


def mma_inputs(n, m, seed):
    """The drivers' MMA settings (production/heatsink.cpp:74-81: a0 = 1, a = 0, c = 1e4, d = 0,
    bounds [0, 1], move 0.2) with seeded objective gradients and volume-type constraints."""
    rng = np.random.default_rng(seed)
    x0 = rng.uniform(0.2, 0.8, n)
    dfdx = rng.standard_normal((MMA_ITERS, n)) * 0.1
    g = rng.uniform(-0.2, 0.1, (MMA_ITERS, m))
    dgdx = -np.abs(1.0 / n + 0.2 / n * rng.standard_normal((MMA_ITERS, m, n)))
    return dict(n=np.array(n), m=np.array(m), a0=np.array(1.0), a=np.zeros(m), c=np.full(m, 1.0e4), d=np.zeros(m),
                xmin=np.zeros(n), xmax=np.ones(n), move=np.array(0.2), x0=x0, f=rng.uniform(1.0, 2.0, MMA_ITERS),
                dfdx=dfdx, g=g, dgdx=dgdx)


def mma_reference(inp):
    """x after each of the MMA_ITERS updates of the reference's MMA<double>."""
    import ctypes as C
    lib = C.CDLL(obuild.build_ref_mma())
    n, m = int(inp["n"]), int(inp["m"])
    dp = lambda v: np.ascontiguousarray(v, np.float64).ctypes.data_as(C.POINTER(C.c_double))
    x = inp["x0"].copy()
    hist = np.zeros((MMA_ITERS, n))
    arrays = [np.ascontiguousarray(inp[k], np.float64) for k in ("a", "c", "d", "xmin", "xmax", "f", "dfdx", "g", "dgdx")]
    lib.ref_mma_run(n, m, C.c_double(float(inp["a0"])), *[dp(v) for v in arrays[:5]], C.c_double(float(inp["move"])),
                    MMA_ITERS, dp(x), *[dp(v) for v in arrays[5:]], dp(hist))
    return dict(xhist=hist)


def main():
    check = "--check" in sys.argv
    if obuild.reference_root() is None:
        raise SystemExit("reference sources not found: the golden fixtures come from the reference build")
    obuild.build_ref()
    ref = Oracle("ref")
    bad = 0
    for name, (make, run) in sorted(C.all_cases().items()):
        path = os.path.join(HERE, name + ".npz")
        if check:
            inp, out = C.load(path)
            got = run(ref, inp)
            ok = all(np.array_equal(got[k], out[k]) for k in out) and set(got) == set(out)
            bad += not ok
            print(("ok   " if ok else "DIFF ") + name)
            continue
        inp = make()
        out = run(ref, inp)
        np.savez_compressed(path, **{"in_" + k: v for k, v in inp.items()}, **{"out_" + k: v for k, v in out.items()})
    for name, kw in MMA_CASES.items():
        path = os.path.join(HERE, name + ".npz")
        if check:
            inp, out = C.load(path)
            ok = np.array_equal(mma_reference(inp)["xhist"], out["xhist"])
            bad += not ok
            print(("ok   " if ok else "DIFF ") + name)
            continue
        inp = mma_inputs(**kw)
        out = mma_reference(inp)
        np.savez_compressed(path, **{"in_" + k: v for k, v in inp.items()}, **{"out_" + k: v for k, v in out.items()})
    if check and bad:
        raise SystemExit("%d golden cases differ from the reference" % bad)
    print("%d cases" % len(C.all_cases()))


if __name__ == "__main__":
    main()
