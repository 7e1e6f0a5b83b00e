"""One design iteration of the heat-sink topology optimisation on the device.

The steps of one outer iteration of production/heatsink.cpp:94-260, minus the MMA update:

1. Heaviside-filter the design s into ss (HeavisideFilter::GetFilteredVariable);
2. map ss to alpha, kappa and their derivatives (heatsink.cpp:107-113);
3. run the forward loop to the residual tolerance (heatsink.cpp:142-174);
4. run the adjoint loop to the residual tolerance (heatsink.cpp:181-212);
5. compute the heat-source objective (mean T on the source) and its sensitivity
   (AAD::SensitivityTemperatureAtHeatSource);
6. filter the sensitivity (HeavisideFilter::GetFilteredSensitivity) and normalise it.

All of it runs through the C ABI on one lattice handle. The forward solution stays on the device
for the adjoint (pl_freeze_forward), and the g snapshots stay there for the sensitivity.
"""
import time

import numpy as np

from . import _capi as A
from . import heatsink as HS
from .lattice import LatticePair, phys


class HeatSinkDesign:
    """A heat-sink design problem on one device lattice (natural convection, the heatsink.cpp /
    heatsink3D.cpp boundary programs)."""

    def __init__(self, p, storage="fp64", R=2.4, beta=8.0):
        self.p, self.R, self.beta = p, R, beta
        self.q = 9 if p.nd == 2 else 15
        self.n = p.lx * p.ly * p.lz
        self.lp = LatticePair(self.q, p.lx, p.ly, p.lz, storage)
        self.prog_f = self.lp.program(HS.to_descs(HS.program_ops("forward", p)))
        self.prog_a = self.lp.program(HS.to_descs(HS.program_ops("adjoint", p)))
        self.ph = phys(nu=p.nu, diff=0.0, gx=p.gx, gy=p.gy, gz=p.gz, tem0=p.tem0)
        self.qn, self.mask = p.source()

    def close(self):
        self.lp.close()

    def iterate(self, s, tol=1e-6, max_steps=100000, check_every=100, filtered=None):
        """One design iteration from rest; returns a dict with the objective, its sensitivity to
        the filtered design (dfdss), the normalised filtered sensitivity (dfds), the step counts
        and the wall time of each phase. `filtered` replaces the Heaviside-filtered design."""
        lp, n, t = self.lp, self.n, {}
        zero, one = np.zeros(n), np.ones(n)
        t0 = time.perf_counter()
        ss = lp.heaviside_var(self.R, self.beta, s) if filtered is None else np.asarray(filtered, np.float64)
        alpha, kappa, dads, dkds = self.p.design_fields(ss)
        lp.set_field(A.ALPHA, alpha)
        lp.set_field(A.KAPPA, kappa)
        lp.init(0, one, ux=zero, uy=zero, uz=zero)
        lp.init(1, zero, ux=zero, uy=zero, uz=zero)
        t["setup"] = time.perf_counter() - t0
        t1 = time.perf_counter()
        st_f, steps_f, res_f = lp.solve(A.AD_NATURAL, self.ph, self.prog_f, max_steps, check_every, tol)
        lp.snapshot(0, host=False)
        lp.freeze_forward()
        t["forward"] = time.perf_counter() - t1
        t2 = time.perf_counter()
        fu = [lp.get_field(A.FWD_UX), lp.get_field(A.FWD_UY), lp.get_field(A.FWD_UZ)]
        tem = lp.get_field(A.FWD_TEM)
        lp.init(2, zero, zero, zero, zero, ux=fu[0], uy=fu[1], uz=fu[2])
        lp.init(3, zero, zero, zero, zero, ux=fu[0], uy=fu[1], uz=fu[2])
        st_a, steps_a, res_a = lp.solve(A.AAD_NATURAL, self.ph, self.prog_a, max_steps, check_every, tol)
        lp.snapshot(1, host=False)
        t["adjoint"] = time.perf_counter() - t2
        t3 = time.perf_counter()
        obj = float(np.sum(tem[self.mask.astype(bool)]) / self.p.L)
        dfdss = lp.sensitivity(0, np.zeros(n), dads, dkds, self.qn, self.mask)
        dfds = lp.normalize(lp.heaviside_sens(self.R, self.beta, s, dfdss))
        t["sensitivity"] = time.perf_counter() - t3
        t["total"] = time.perf_counter() - t0
        return dict(objective=obj, dfdss=dfdss, dfds=dfds, forward=(st_f, steps_f, res_f),
                    adjoint=(st_a, steps_a, res_a), seconds=t)
