"""The oracle (C restatement) against the golden fixtures the reference produced
(tests/golden/*.npz, written by tests/golden/make_golden.py from the build of the reference's
own headers). Both sides evaluate in FP64 without FMA contraction, so every output must agree
bit for bit. Runs without the reference sources and without a GPU."""
import glob
import os

import numpy as np
import pytest

from oracle import build as obuild
from tests.golden import cases as C

HERE = os.path.dirname(os.path.abspath(__file__))
FILES = sorted(f for f in glob.glob(os.path.join(HERE, "golden", "*.npz")) if not os.path.basename(f).startswith("mma_"))


@pytest.fixture(scope="module")
def oracle():
    from oracle.olib import Oracle
    obuild.build_oracle()
    return Oracle("oracle")


def test_every_case_has_a_fixture():
    have = {os.path.basename(f)[:-4] for f in FILES}
    assert set(C.all_cases()) == have


@pytest.mark.parametrize("path", FILES, ids=[os.path.basename(f)[:-4] for f in FILES])
def test_oracle_matches_reference_golden(oracle, path):
    name = os.path.basename(path)[:-4]
    inp, out = C.load(path)
    got = C.all_cases()[name][1](oracle, inp)
    assert set(got) == set(out)
    for k in out:
        assert np.array_equal(got[k], out[k]), "%s: %s differs, max abs %.3e" % (
            name, k, float(np.max(np.abs(got[k] - out[k]))) if out[k].size else 0.0)


@pytest.mark.skipif(obuild.reference_root() is None, reason="reference sources not present")
def test_mma_fixtures_are_the_reference_output():
    """The MMA fixtures (tests/golden/mma_*.npz) are what the reference's MMA<double> produces."""
    from tests.golden import make_golden as MG
    for name in MG.MMA_CASES:
        inp, out = C.load(os.path.join(HERE, "golden", name + ".npz"))
        assert np.array_equal(MG.mma_reference(inp)["xhist"], out["xhist"]), name


def test_fixture_inputs_regenerate(oracle):
    """The stored inputs are the seeded generators' (so the fixtures can be rebuilt)."""
    for name in ("stream_q9_fwd", "bc_q15_AD_Q", "collide_q9_AAD_NATURAL", "hsfwd_q9"):
        inp, _ = C.load(os.path.join(HERE, "golden", name + ".npz"))
        again = C.all_cases()[name][0]()
        for k in inp:
            assert np.array_equal(inp[k], again[k]), (name, k)
