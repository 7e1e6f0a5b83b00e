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
    if check and bad:
        raise SystemExit("%d golden cases differ from the reference" % bad)
    print("%d cases" % len(C.all_cases()))


if __name__ == "__main__":
    main()
