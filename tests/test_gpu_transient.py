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


def test_forced_transient_with_time_varying_inflow_matches_oracle():
    """The forced-convection transient (volumetric source, objective weight, u(t) inflow on NS SetU
    and ANS iSetU) on D2Q9, FP64, checkpoints every 4 levels, against the oracle's run keeping
    every level; tau_in = 20 so the inflow ramps within the 30 levels."""
    from oracle.olib import Oracle
    from panslbm2_gb300 import forced as FC
    from tests import _forced_oracle as FO
    p = FC.ForcedParams(2, 24, 12)
    ss = p.project(np.clip(p.design(seed=6, sigma=3.0), 0, 1))
    tr = TransientHeatSink(p, "fp64", checkpoint_every=4, tau_in=20.0)
    r = tr.evaluate_design(ss, 30)
    tr.close()
    o = Oracle("oracle")
    o.set_threads(1)
    ref = FO.forced_transient(o, p, ss, 30, tau_in=20.0)
    assert abs(r["objective"] - ref["objective"]) <= 1e-12 * abs(ref["objective"])
    close(r["dfdss"], ref["dfdss"], 1e-10)


def test_forced_transient_fp32_objective_against_fp64_3d():
    """The transient configuration's physics in 3D (base-plate source, u(t) inflow) on a small
    D3Q15 lattice over 300 levels: the FP32 objective within 1e-4 relative of FP64 and the FP32
    sensitivity close to FP64. Checkpointing is bit-neutral in FP64. In FP32 a segment start
    runs its stream and its collide as two kernels where the other levels run the fused step, in
    which the compiler may contract a boundary op's products into the collide's sums; the two
    checkpoint schedules then differ in the last FP32 bits (measured on GB300: objective 4.7e-9
    relative), so FP32 is compared within 1e-6."""
    from panslbm2_gb300 import forced as FC
    p = FC.ForcedParams(3, 40, 24, 24, plate=(12, 2, 12))
    ss = p.project(np.clip(p.design(seed=7, sigma=4.0), 0, 1))
    out = {}
    for st, every in (("fp64", 100), ("fp64", 7), ("fp32", 100), ("fp32", 7)):
        tr = TransientHeatSink(p, st, checkpoint_every=every, tau_in=100.0)
        out[(st, every)] = tr.evaluate_design(ss, 300)
        tr.close()
    a, b = out[("fp32", 100)], out[("fp64", 100)]
    assert abs(a["objective"] - b["objective"]) <= 1e-4 * abs(b["objective"])
    assert np.linalg.norm(a["dfdss"] - b["dfdss"]) <= 1e-2 * np.linalg.norm(b["dfdss"])
    assert b["objective"] == out[("fp64", 7)]["objective"]
    assert np.array_equal(b["dfdss"], out[("fp64", 7)]["dfdss"])
    c = out[("fp32", 7)]
    assert abs(a["objective"] - c["objective"]) <= 1e-6 * abs(a["objective"])
    assert np.max(np.abs(a["dfdss"] - c["dfdss"])) <= 1e-6 * np.max(np.abs(a["dfdss"]))
