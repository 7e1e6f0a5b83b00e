"""Transient heat-sink evaluation on the device with checkpointed forward states
(panslbm2_gb300/transient.py) against the reference's own transient loops, which keep every time
level in memory (tests/golden/hst_q9.npz from production/heatsink_transient.cpp:135-205): the
time-averaged source temperature, the accumulated sensitivity and the final adjoint populations,
FP64, with checkpoints every 7 steps (four segments recomputed) and with one segment."""
import os

import numpy as np
import pytest

from panslbm2_gb300.transient import TransientHeatSink
from tests.golden import cases as C

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def close(a, b, rtol):
    a, b = np.asarray(a, np.float64).reshape(-1), np.asarray(b, np.float64).reshape(-1)
    scale = max(1e-300, float(np.max(np.abs(b))))
    err = float(np.max(np.abs(a - b))) / scale
    assert err <= rtol, "max rel err %.3e" % err


@pytest.mark.parametrize("every", [7, 100])
def test_transient_checkpointed_adjoint(every):
    inp, out = C.load(os.path.join(HERE, "golden", "hst_q9.npz"))
    tr = TransientHeatSink(C.hst_params(), "fp64", checkpoint_every=every)
    r = tr.evaluate(inp["alpha"], inp["kappa"], inp["dads"], inp["dkds"], C.HST_LEVELS)
    assert r["segments"] == (C.HST_LEVELS - 2) // every + 1
    assert abs(r["objective"] - float(out["objective"])) <= 1e-12 * abs(float(out["objective"]))
    close(r["dfdss"], out["dfdss"], 1e-10)
    close(tr.lp.get_populations(0), out["fa"], 1e-11)
    close(tr.lp.get_populations(1), out["ga"], 1e-11)
    tr.close()


def test_transient_checkpoints_leave_the_result_unchanged_3d():
    """D3Q15, FP32: recomputing the forward states from checkpoints every 3 steps gives the same
    objective and sensitivity, bit for bit, as one segment (the recomputation is deterministic)."""
    from panslbm2_gb300 import heatsink as HS
    p = HS.Params(3, 8, 9, 7)
    ss = np.clip(HS.grf_design(3, 8, 9, 7, seed=2, sigma=2.0), 0, 1)
    alpha, kappa, dads, dkds = p.design_fields(ss)
    res = []
    for every in (3, 100):
        tr = TransientHeatSink(p, "fp32", checkpoint_every=every)
        res.append(tr.evaluate(alpha, kappa, dads, dkds, 12))
        tr.close()
    assert res[0]["segments"] == 4 and res[1]["segments"] == 1
    assert res[0]["objective"] == res[1]["objective"]
    assert np.array_equal(res[0]["dfdss"], res[1]["dfdss"])
    assert np.all(np.isfinite(res[0]["dfdss"])) and np.any(res[0]["dfdss"] != 0)
