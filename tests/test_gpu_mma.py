"""The device MMA (pl_mma_*) against the reference's own MMA<double> (golden fixtures
tests/golden/mma_*.npz, written by tests/golden/make_golden.py): five consecutive updates (the
k < 2 and k >= 2 asymptote rules) with the drivers' settings, m = 1 and m = 2. The device sums
over the n variables in a fixed tree instead of serially, so the designs agree to 1e-9 rather
than bit for bit."""
import glob
import os

import numpy as np
import pytest

from tests.golden import cases as C

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(HERE, "golden", "mma_*.npz"))),
                         ids=lambda s: os.path.basename(s)[:-4])
def test_mma_matches_reference(path):
    from panslbm2_gb300.mma import MMA
    inp, out = C.load(path)
    n, m = int(inp["n"]), int(inp["m"])
    opt = MMA(n, m, float(inp["a0"]), inp["a"], inp["c"], inp["d"], inp["xmin"], inp["xmax"], move=float(inp["move"]))
    x = inp["x0"].copy()
    for it in range(out["xhist"].shape[0]):
        x = opt.update(x, float(inp["f"][it]), inp["dfdx"][it], inp["g"][it], inp["dgdx"][it])
        err = float(np.max(np.abs(x - out["xhist"][it])))
        assert err <= 1e-9, (it, err)
        assert np.all(x >= inp["xmin"]) and np.all(x <= inp["xmax"])
    opt.close()


def test_mma_rejects_bad_arguments():
    from panslbm2_gb300 import _capi as A
    from panslbm2_gb300.mma import MMA
    with pytest.raises(A.PanslbmError):
        MMA(10, 5, 1.0, np.zeros(5), np.ones(5), np.zeros(5), np.zeros(10), np.ones(10))
