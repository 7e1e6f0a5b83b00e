"""One transient heat-sink design evaluation on the device, with checkpointed forward states.

The loops of production/heatsink_transient.cpp:135-205 (2D) and heatsink3D_transient.cpp (3D):
a forward run of nt-1 time steps from rest (NS + AD, natural convection, Brinkman), then the
adjoint swept backward over the same steps, each adjoint step adding its term of
AAD::SensitivityTemperatureAtHeatSource, and the time-averaged source temperature as objective.

The reference keeps every time step's rho, u, T and g snapshot in host memory (nt arrays of each,
heatsink_transient.cpp:45-52). Here the forward run keeps only a checkpoint of the populations
every `checkpoint_every` steps, on the device (pl_store). The adjoint sweep walks the segments
backward: it parks the adjoint populations, restores the segment's checkpoint, recomputes the
segment's forward steps storing their macros and snapshots on the device, brings the adjoint
populations back and runs the segment's adjoint steps, each reading its step's forward state
(pl_load). The sensitivity accumulates on the device (pl_sensitivity_device) and the objective's
time sum too (pl_accumulate); the host sees two arrays at the end.

Step order per adjoint time step t (heatsink_transient.cpp:181-204): AAD collide with the forward
state of step t, the sensitivity term of step t (forward snapshot gi[t], adjoint snapshot igi),
then iStream and the adjoint boundary calls with the velocity of step t. The reference's forward
loop never writes gi[0], which its adjoint reads at t = 0 (allocated but not initialised); here
that snapshot is zero.

The same sweep runs the forced-convection heat sink of panslbm2_gb300.forced (the transient
benchmark configuration): AD / AAD ForceConvection kinds with the volumetric heat source, the
time-varying inflow u(t) = u_max (1 - exp(-t / tau_in)) through pl_set_inflow_scale (NS SetU of
forward step t and ANS iSetU of adjoint step t use u(t)), the time-averaged objective
J = (1 / nt) sum_t sum_x w(x) T_t(x) entering each adjoint collide as the objective weight w / nt,
and per step the Brinkman and diffusivity terms (AAD::SensitivityBrinkmanDiffusivity) plus, in 2D,
the heat-source term.
"""
import math
import time

import numpy as np

from . import _capi as A
from . import heatsink as HS
from .lattice import LatticePair, phys


class TransientHeatSink:
    """p: heatsink.Params (natural convection, the reference's transient driver) or
    forced.ForcedParams (forced convection with the time-varying inflow, time constant tau_in)"""

    def __init__(self, p, storage="fp64", checkpoint_every=100, tau_in=500.0):
        from .forced import ForcedParams
        self.p, self.K = p, int(checkpoint_every)
        self.forced = isinstance(p, ForcedParams)
        self.q = 9 if p.nd == 2 else 15
        self.n = p.lx * p.ly * p.lz
        self.lp = LatticePair(self.q, p.lx, p.ly, p.lz, storage)
        # every step of the sweep takes its snapshot: write it in the step's own pass
        self.lp.set_option(A.OPT_SNAPSHOT_IN_STEP, 1)
        if self.forced:
            self.kf, self.ka = A.AD_FORCE, A.AAD_FORCE
            self.prog_f = self.lp.program(HS.to_descs(p.program_ops("forward")))
            self.prog_a = self.lp.program(HS.to_descs(p.program_ops("adjoint")))
            self.ph = phys(nu=p.nu)
            self.tau_in = float(tau_in)
        else:
            self.kf, self.ka = A.AD_NATURAL, A.AAD_NATURAL
            self.prog_f = self.lp.program(HS.to_descs(HS.program_ops("forward", p)))
            self.prog_a = self.lp.program(HS.to_descs(HS.program_ops("adjoint", p)))
            self.ph = phys(nu=p.nu, diff=0.0, gx=p.gx, gy=p.gy, gz=p.gz, tem0=p.tem0)
            self.qn, self.mask = p.source()

    def inflow(self, t):
        """u(t) / u_max of forward time level t (forced convection; 1 otherwise)"""
        if not self.forced:
            return 1.0
        return 1.0 - math.exp(-t / self.tau_in)

    def _bc_scale(self, t):
        if self.forced:
            self.lp.set_inflow_scale(self.inflow(t))

    def close(self):
        self.lp.close()

    def _recompute(self, seg, t_last):
        """forward steps of segment `seg` (t0 = seg*K + 1 .. t_last) from its checkpoint; their
        macros and forward snapshots go to device slots t - t0"""
        lp, ph = self.lp, self.ph
        lp.load(A.STORE_POPS, seg)
        t0 = seg * self.K + 1
        for t in range(t0, t_last + 1):
            if t == t0:
                lp.collide(self.kf, ph, save=True)
            else:
                self._bc_scale(t - 1)   # the boundary calls in this step close forward step t - 1
                lp.step(self.kf, ph, self.prog_f, save=True)
            lp.snapshot(0, host=False)
            lp.store(A.STORE_FWD, t - t0)
            lp.swap_snapshot(t - t0)   # moved, not copied: each snapshot is read back once

    def evaluate_design(self, ss, nt, release=True):
        """forced convection: the sweep for the filtered design ss (design maps, heat source and
        objective weight of forced.ForcedParams)"""
        p = self.p
        alpha, kappa, dads, dkds = p.design_fields(ss)
        Q, dQ = p.heat_source(ss)
        self.lp.set_field(A.HEAT_SOURCE, Q)
        self.w = p.objective_weight(ss)
        self.lp.set_field(A.OBJ_WEIGHT, self.w / nt)
        self.dQ = dQ
        return self.evaluate(alpha, kappa, dads, dkds, nt, release)

    def evaluate(self, alpha, kappa, dads, dkds, nt, release=True):
        """objective (time-averaged temperature on the heat source; forced convection: time
        average of sum w T), its sensitivity dfdss (the reference's sign convention) and the phase
        times; nt counts the time levels 0..nt-1 as the reference's loops do. With release=False
        the device stores stay allocated for the next evaluation."""
        lp, n, K, nd = self.lp, self.n, self.K, self.p.nd
        zero, one = np.zeros(n), np.ones(n)
        times = {}
        t0 = time.perf_counter()
        lp.set_field(A.ALPHA, alpha)
        lp.set_field(A.KAPPA, kappa)
        lp.set_field(A.ACC, zero)
        lp.set_field(A.DFDS, zero)
        # forward (heatsink_transient.cpp:135-170): checkpoints at the segment starts t = 1, K+1, ...
        lp.init(0, one, ux=zero, uy=zero, uz=zero)
        lp.init(1, zero, ux=zero, uy=zero, uz=zero)
        nseg = 0
        for t in range(1, nt):
            if (t - 1) % K == 0:
                if t > 1:
                    self._bc_scale(t - 1)
                    lp.stream(mode=0, prog=self.prog_f, both=True)
                lp.store(A.STORE_POPS, (t - 1) // K)
                nseg += 1
                lp.collide(self.kf, self.ph, save=True)
            else:
                self._bc_scale(t - 1)
                lp.step(self.kf, self.ph, self.prog_f, save=True)
            lp.accumulate(A.ACC, A.TEM)
        ul = [lp.get_field(A.UX), lp.get_field(A.UY), lp.get_field(A.UZ) if nd == 3 else zero]
        times["forward"] = time.perf_counter() - t0
        # adjoint (heatsink_transient.cpp:172-205), segment by segment from the last
        t1 = time.perf_counter()
        lp.init(2, zero, zero, zero, zero, ux=ul[0], uy=ul[1], uz=ul[2])
        lp.init(3, zero, zero, zero, zero, ux=ul[0], uy=ul[1], uz=ul[2])
        park = nseg   # store slot of the adjoint populations while a segment is recomputed
        first = True
        loaded_seg = -1
        for t in range(nt - 2, -1, -1):
            if t >= 1:
                seg = (t - 1) // K
                if seg != loaded_seg:
                    lp.store(A.STORE_POPS, park)
                    self._recompute(seg, min(seg * K + K, nt - 2))
                    lp.load(A.STORE_POPS, park)
                    loaded_seg = seg
                lp.load(A.STORE_FWD, t - (seg * K + 1))
                lp.swap_snapshot(t - (seg * K + 1))
            else:
                # time level 0: the state at rest, and no forward snapshot
                for fid, v in ((A.FWD_RHO, one), (A.FWD_UX, zero), (A.FWD_UY, zero), (A.FWD_UZ, zero),
                               (A.FWD_TEM, zero)):
                    lp.set_field(fid, v)
                lp.set_snapshot(0, np.zeros(n * self.q))
            lp.collide(self.ka, self.ph, save=True)
            lp.snapshot(1, host=False)
            if self.forced:
                # AAD::SensitivityBrinkmanDiffusivity; in 2D the design-dependent heat source adds
                # -item dQ/dss per step (dQ/dss = -q_h, uniform), in the reference's sign
                lp.sensitivity_device(1, dads if first else None, dkds if first else None)
                if nd == 2:
                    lp.accumulate(A.DFDS, A.ITEM, -float(self.dQ[0]))
            elif first:
                lp.sensitivity_device(0, dads, dkds, self.qn, self.mask)
            else:
                lp.sensitivity_device(0)
            first = False
            self._bc_scale(t)
            lp.stream(mode=1, prog=self.prog_a, both=True)
        dfdss = lp.get_field(A.DFDS)
        acc = lp.get_field(A.ACC)
        times["adjoint"] = time.perf_counter() - t1
        if release:
            lp.store_release()
        if self.forced:
            lp.set_inflow_scale(1.0)
            objective = float(np.sum(self.w * acc)) / nt
        else:
            objective = float(np.sum(acc[self.mask != 0])) / (self.p.L * nt)
        return dict(objective=objective, dfdss=dfdss, times=times, segments=nseg)


def main(argv=None):
    """python -m panslbm2_gb300.transient [--shape X,Y,Z] [--levels N] [--every K] [--physics forced|natural]:
    one timed transient evaluation (after a short warm-up), FP32, seeded design 0"""
    import argparse
    import json
    from . import forced as FC
    ap = argparse.ArgumentParser()
    ap.add_argument("--shape", default="96,96,48")
    ap.add_argument("--levels", type=int, default=202)
    ap.add_argument("--every", type=int, default=100)
    ap.add_argument("--physics", default="forced", choices=["forced", "natural"])
    ap.add_argument("--storage", default="fp32")
    a = ap.parse_args(argv)
    nx, ny, nz = (int(v) for v in a.shape.split(","))
    if a.physics == "forced":
        p = FC.ForcedParams(3, nx, ny, nz)
        ss = p.project(p.design(seed=0))
        tr = TransientHeatSink(p, a.storage, checkpoint_every=a.every)
        run = lambda nt: tr.evaluate_design(ss, nt)  # noqa: E731
    else:
        p = HS.Params(3, nx, ny, nz)
        ss = HS.grf_design(3, nx, ny, nz, seed=0, sigma=8.0)
        alpha, kappa, dads, dkds = p.design_fields(ss)
        tr = TransientHeatSink(p, a.storage, checkpoint_every=a.every)
        run = lambda nt: tr.evaluate(alpha, kappa, dads, dkds, nt)  # noqa: E731
    run(min(a.levels, 2 * a.every + 2))
    t0 = time.perf_counter()
    r = run(a.levels)
    print(json.dumps(dict(shape=[nx, ny, nz], levels=a.levels, every=a.every, physics=a.physics,
                          seconds=round(time.perf_counter() - t0, 4), phases=r["times"], objective=r["objective"])))
    tr.close()


if __name__ == "__main__":
    main()
