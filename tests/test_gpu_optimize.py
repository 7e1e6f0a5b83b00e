"""The forced heat-sink optimisation loop (panslbm2_gb300.optimize: the steps of
production/heatsink.cpp:93-280 on the device, MMA on the device) on a small lattice: three design
iterations to residual 1e-6 from the seeded design. The design stays in [0, 1], each update stays
within the move limit 0.2, the base plate stays solid, and the volume constraint and the
objective are finite."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_three_design_iterations():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from panslbm2_gb300.forced import ForcedParams
    from panslbm2_gb300.optimize import ForcedOptimisation
    p = ForcedParams(2, 60, 30)
    opt = ForcedOptimisation(p, "fp64")
    try:
        s = p.design(seed=3, sigma=4.0)
        s[~p.design_mask] = 0.0
        recs = []
        for _ in range(3):
            s_new, rec = opt.iteration(s, tol=1e-6, max_steps=60000)
            assert np.all(s_new >= 0.0) and np.all(s_new <= 1.0)
            assert np.max(np.abs(s_new - s)) <= 0.2 + 1e-12
            assert np.all(s_new[~p.design_mask] == 0.0)
            assert np.isfinite(rec["objective"]) and np.isfinite(rec["g"])
            recs.append(rec)
            s = s_new
        print([(r["objective"], r["g"], r["dsmax"], r["forward_steps"], r["adjoint_steps"]) for r in recs])
        assert all(all(r["converged"]) for r in recs)
    finally:
        opt.close()
