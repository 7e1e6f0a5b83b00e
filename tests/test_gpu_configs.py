"""The benchmark configurations' own physics on the device against the CPU oracle.

* lid-driven cavity, D2Q9 NS, 100 x 100, 20,000 steps, FP64 (test/cavityflow.cpp:43-67);
* forced-convection heat sink (parabolic inflow, pressure outlet with zero temperature gradient,
  volumetric heat source, mean-solid-temperature objective): forward, adjoint and the sensitivity
  terms on the 200 x 100 lattice (D2Q9, FP64) and on a small D3Q15 lattice with a base-plate
  source, against the oracle's run of the same steps;
* the time-varying inflow scale on NS SetU / ANS iSetU.
The volumetric source, the objective source and the inflow scale have no reference routine: for
those terms the oracle (the CPU restatement) is the reference.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle.olib import Oracle
    o = Oracle("oracle")
    import os
    o.set_threads(os.cpu_count() or 1)
    return o


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_cavity_100x100_20000_steps_fp64(env):
    from panslbm2_gb300 import forced as FC
    from tests import _forced_oracle as FO
    rho, ux, uy, _ = FC.run_cavity(100, 100, 20000, storage="fp64")
    mac = FO.cavity(env, 100, 100, 20000)
    assert rel(rho, mac["rho"]) <= 1e-12
    assert rel(ux, mac["ux"]) <= 1e-12
    assert rel(uy, mac["uy"]) <= 1e-12
    # the lid drives a primary vortex: the top row moves with the lid, the centre line reverses
    assert np.all(ux.reshape(100, 100)[98, 2:-2] > 0) and ux.reshape(100, 100)[40, 50] < 0


def _compare(res, ref, tol_f, tol_a, tol_s):
    for k in ("rho", "ux", "uy", "tem"):
        assert rel(res["fwd"][k], ref["fwd"][k]) <= tol_f, k
    for k in ("ip", "iux", "iuy", "item", "iqx", "iqy"):
        assert rel(res["adj"][k], ref["adj"][k]) <= tol_a, k
    assert abs(res["objective"] - ref["objective"]) <= tol_f * abs(ref["objective"])
    assert rel(res["dJdss"], ref["dJdss"]) <= tol_s


def test_forced_heatsink_2d_200x100_fp64(env):
    from panslbm2_gb300 import forced as FC
    from tests import _forced_oracle as FO
    p = FC.ForcedParams(2, 200, 100)
    hs = FC.ForcedHeatSink(p, "fp64")
    try:
        s = p.design(seed=0)
        ss = hs.filtered(s)
        res = hs.iterate(s, filtered=ss, fixed_steps=(600, 400))
    finally:
        hs.close()
    ref = FO.forced_iteration(env, p, ss, 600, 400)
    _compare(res, ref, 1e-12, 1e-11, 1e-10)
    assert np.all(np.isfinite(res["dJds"]))
    # heat reaches the solid and the flow leaves through the outlet
    assert res["objective"] > 0 and np.mean(res["fwd"]["ux"].reshape(100, 200)[1:-1, -1]) > 0


def test_forced_heatsink_3d_base_plate_fp64(env):
    from panslbm2_gb300 import forced as FC
    from tests import _forced_oracle as FO
    p = FC.ForcedParams(3, 24, 20, 16, plate=(8, 2, 8))
    hs = FC.ForcedHeatSink(p, "fp64")
    try:
        s = p.design(seed=1, sigma=3.0)
        ss = hs.filtered(s)
        res = hs.iterate(s, filtered=ss, fixed_steps=(150, 120))
    finally:
        hs.close()
    ref = FO.forced_iteration(env, p, ss, 150, 120)
    _compare(res, ref, 1e-12, 1e-11, 1e-10)
    assert np.all(res["ss"][p.plate] == 0.0)


def test_forced_heatsink_fp32_close_to_fp64(env):
    from panslbm2_gb300 import forced as FC
    p = FC.ForcedParams(2, 64, 32)
    s = p.design(seed=4, sigma=4.0)
    out = {}
    for st in ("fp64", "fp32"):
        hs = FC.ForcedHeatSink(p, st)
        try:
            out[st] = hs.iterate(s, fixed_steps=(3000, 3000))
        finally:
            hs.close()
    a, b = out["fp32"], out["fp64"]
    assert abs(a["objective"] - b["objective"]) <= 1e-4 * abs(b["objective"])
    assert rel(a["dJdss"], b["dJdss"]) <= 1e-2


def test_inflow_scale(env):
    """u(t) = s u on the inflow: the device's scaled SetU / iSetU equal the oracle's."""
    from panslbm2_gb300 import forced as FC
    from tests import _forced_oracle as FO
    p = FC.ForcedParams(2, 40, 20)
    hs = FC.ForcedHeatSink(p, "fp64")
    try:
        hs.lp.set_inflow_scale(0.37)
        s = p.design(seed=2, sigma=3.0)
        ss = hs.filtered(s)
        res = hs.iterate(s, filtered=ss, fixed_steps=(80, 60))
    finally:
        hs.close()
    ref = FO.forced_iteration(env, p, ss, 80, 60, uscale=0.37)
    _compare(res, ref, 1e-12, 1e-11, 1e-10)
    ref1 = FO.forced_iteration(env, p, ss, 80, 60, uscale=1.0)
    assert rel(res["fwd"]["ux"], ref1["fwd"]["ux"]) > 1e-3     # the scale took effect
