"""Forced-convection heat-sink workloads and the lid-driven cavity.

Cavity (test/cavityflow.cpp:43-67): D2Q9 NS::MacroCollide, bounce-back on the left, right and
bottom walls, the Zou-He velocity lid on the top row, SmoothCorner, every step.

Forced-convection heat sink (2D on D2Q9, 3D on D3Q15): the coupled NS + AD forced-convection
collide with Brinkman drag (AD::MacroBrinkmanCollideForceConvection, advection.h:812-926) and
its adjoint (AAD::MacroBrinkmanCollideForceConvection, adjointadvection.h:995-1109), with the
boundary set of the reference's forced-convection test driver (test/nsadsens.cpp:77-133):

  * inflow on x = 0: parabolic velocity through NS::BoundaryConditionSetU (Zou-He), T = 0 through
    AD::BoundaryConditionSetT; adjoints ANS::iBoundaryConditionSetU, AAD::iBoundaryConditionSetT;
  * outflow on x = lx - 1: the pressure outlet NS::BoundaryConditionSetRho (rho = 1, no
    tangential velocity) and a zero normal temperature gradient through
    AD::BoundaryConditionSetQ with q = 0; adjoints AAD::iBoundaryConditionSetRho (2D, the coupled
    routine with the SetQ branch) / ANS::iBoundaryConditionSetRho (3D, where the reference's
    coupled routine does not exist) and AAD::iBoundaryConditionSetQ;
  * channel walls: bounce-back for the flow, adiabatic (SetQ, q = 0) for heat;
  * SmoothCorner on both sets.

Three terms have no reference routine (the reference heat sinks take their heat through a
boundary flux): the volumetric heat source Q(x) (PL_HEAT_SOURCE), the volumetric objective and
its adjoint source (PL_OBJ_WEIGHT), and the time-varying inflow scale (pl_set_inflow_scale).
Their oracle is the CPU restatement in oracle/; parity against the reference is unpinned for
those terms only.

Physics constants follow the forced-convection configurations: nu = 0.1, Pr = 6 (kappa_f =
nu / Pr), kappa_s = 10 kappa_f, u_max = 0.02, q_h = 1e-3, alpha(g) = a_max q (1 - g) / (q + g)
with a_max = 0.1, q = 0.01 (g = 1 fluid, g = 0 solid), Heaviside filter R = 3, beta = 8.
2D: Q = q_h (1 - g) in the solid, objective = mean solid temperature sum (1-g) T / sum (1-g).
3D: Q = q_h in a 40 x 4 x 40 base plate (x, y, z) on the bottom wall, centred in x and z, kept
solid; objective = mean base-plate temperature.
"""
import math
import time

import numpy as np

from . import _capi as A
from .heatsink import faces, grid, grf_design, to_descs
from .lattice import LatticePair, phys


# ------------------------------------------------------------------------------- cavity
def cavity_ops(lx, ly, u0=0.1):
    """Boundary calls of one cavity time step (test/cavityflow.cpp:58-64), reference order."""
    i, j, _ = grid(2, lx, ly)
    F = faces(2, lx, ly)
    wall = ((i == 0) | (i == lx - 1) | (j == 0)).astype(np.int32)
    lid = (j == ly - 1).astype(np.int32)
    ops = [dict(kind=A.BC_WALL, lat=0, axis=a, pos=pos, dir=d, type=wall) for (a, pos, d) in F]
    ops += [dict(kind=A.BC_NS_U, lat=0, axis=a, pos=pos, dir=d, type=lid, c0=u0, c1=0.0) for (a, pos, d) in F]
    ops.append(dict(kind=A.SMOOTH_CORNER, lat=0))
    return ops


def run_cavity(lx=100, ly=100, steps=20000, nu=0.1, u0=0.1, storage="fp64"):
    """The cavity from rest (rho = 1, u = 0) for `steps` time steps on the device; returns rho,
    ux, uy of the last collide and the device seconds."""
    n = lx * ly
    lp = LatticePair(9, lx, ly, 1, storage)
    try:
        zero = np.zeros(n)
        lp.init(0, np.ones(n), ux=zero, uy=zero, uz=zero)
        prog = lp.program(to_descs(cavity_ops(lx, ly, u0)))
        ph = phys(nu=nu)
        t0 = time.perf_counter()
        lp.collide(A.NS_COLLIDE, ph)
        if steps > 2:
            lp.steps(A.NS_COLLIDE, ph, prog, steps - 2)
        if steps > 1:
            lp.step(A.NS_COLLIDE, ph, prog, save=True)
        lp.synchronize()
        sec = time.perf_counter() - t0
        return lp.get_field(A.RHO), lp.get_field(A.UX), lp.get_field(A.UY), sec
    finally:
        lp.close()


# --------------------------------------------------------------- forced-convection heat sink
class ForcedParams:
    """Constants, design maps and boundary programs of the forced-convection heat sink."""

    def __init__(self, nd, lx, ly, lz=1, umax=0.02, nu=0.1, Pr=6.0, kratio=10.0, qh=1e-3, amax=0.1, qa=0.01,
                 qg=1.0, R=3.0, beta=8.0, plate=(40, 4, 40)):
        self.nd, self.lx, self.ly, self.lz = nd, lx, ly, (lz if nd == 3 else 1)
        self.umax, self.nu, self.Pr = umax, nu, Pr
        self.diff_fluid = nu / Pr
        self.diff_solid = kratio * self.diff_fluid
        self.qh, self.amax, self.qa, self.qg, self.R, self.beta = qh, amax, qa, qg, R, beta
        self.n = lx * ly * self.lz
        self.i, self.j, self.k = grid(nd, lx, ly, self.lz)
        if nd == 3:
            px, py, pz = plate
            x0, z0 = (lx - px) // 2, (self.lz - pz) // 2
            i, j, k = self.i, self.j, self.k
            self.plate = (i >= x0) & (i < x0 + px) & (j >= 1) & (j < 1 + py) & (k >= z0) & (k < z0 + pz)
        else:
            self.plate = np.zeros(self.n, dtype=bool)
        self.design_mask = ~self.plate

    # design maps --------------------------------------------------------------------------
    def project(self, ss):
        """the filtered design with the base plate held solid"""
        ss = np.array(ss, dtype=np.float64)
        ss[self.plate] = 0.0
        return ss

    def design_fields(self, ss):
        """alpha, kappa and their derivatives from the filtered design (1 fluid, 0 solid)."""
        df, ds, qa, qg = self.diff_fluid, self.diff_solid, self.qa, self.qg
        alpha = self.amax * qa * (1.0 - ss) / (qa + ss)
        dads = -self.amax * qa * (1.0 + qa) / (qa + ss) ** 2
        kappa = ds + (df - ds) * ss * (1.0 + qg) / (ss + qg)
        dkds = (df - ds) * qg * (1.0 + qg) / (ss + qg) ** 2
        return alpha, kappa, dads, dkds

    def heat_source(self, ss):
        """volumetric source Q and dQ/dss"""
        if self.nd == 2:
            return self.qh * (1.0 - ss), np.full(self.n, -self.qh)
        return np.where(self.plate, self.qh, 0.0), np.zeros(self.n)

    def objective_weight(self, ss):
        """w = dJ/dT of the objective J = sum w T"""
        if self.nd == 2:
            return (1.0 - ss) / np.sum(1.0 - ss)
        return self.plate / float(np.count_nonzero(self.plate))

    def objective(self, ss, tem):
        """J and its explicit design derivative dJ/dss at fixed T"""
        if self.nd == 2:
            S = np.sum(1.0 - ss)
            J = float(np.sum((1.0 - ss) * tem) / S)
            return J, (J - tem) / S
        J = float(np.mean(tem[self.plate]))
        return J, np.zeros(self.n)

    def inflow(self):
        """parabolic inflow velocity on every node (zero on the channel walls)"""
        H = self.ly - 1
        u = 4.0 * self.umax * self.j * (H - self.j) / (H * H)
        if self.nd == 3:
            W = self.lz - 1
            u = u * 4.0 * self.k * (W - self.k) / (W * W)
        return np.ascontiguousarray(u, dtype=np.float64)

    # boundary programs --------------------------------------------------------------------
    def masks(self):
        i, j, k = self.i, self.j, self.k
        lx, ly, lz = self.lx, self.ly, self.lz
        side = (j == 0) | (j == ly - 1)
        if self.nd == 3:
            side = side | (k == 0) | (k == lz - 1)
        inflow = (i == 0) & ~side
        outflow = (i == lx - 1) & ~side
        adiabatic = (side | (i == lx - 1)) & ~inflow
        return side, inflow, outflow, adiabatic

    def program_ops(self, phase):
        """Boundary calls of one time step: those of test/nsadsens.cpp:81-103 (forward) and
        :117-133 (adjoint), with both SmoothCorner calls moved to the end of the step as in
        production/heatsink.cpp:155-168. The values are the same: the AD / AAD routines read and
        write only g (and the previous collide's velocity), the f-set smoothing reads and writes
        only f, and the outlet's adjoint pressure routine, which reads g, acts on no node the
        smoothing writes (the outlet excludes the channel walls' edges). With every smoothing
        call last, the device runs the program on its staged boundary path."""
        F = faces(self.nd, self.lx, self.ly, self.lz)
        side, inflow, outflow, adiabatic = self.masks()
        wall = side.astype(np.int32)
        m_in, m_out, m_q = inflow.astype(np.int32), outflow.astype(np.int32), adiabatic.astype(np.int32)
        u = self.inflow()
        zero = np.zeros(self.n)
        one = np.ones(self.n)
        ops = []
        if phase == "forward":
            ops += [dict(kind=A.BC_WALL, lat=0, axis=a, pos=p, dir=d, type=wall) for (a, p, d) in F]
            ops += [dict(kind=A.BC_NS_U, lat=0, axis=a, pos=p, dir=d, type=m_in, v0=u, v1=zero, v2=zero)
                    for (a, p, d) in F]
            ops += [dict(kind=A.BC_NS_RHO, lat=0, axis=a, pos=p, dir=d, type=m_out, v0=one, v1=zero, v2=zero)
                    for (a, p, d) in F]
            ops += [dict(kind=A.BC_AD_T, lat=1, axis=a, pos=p, dir=d, type=m_in, c0=0.0) for (a, p, d) in F]
            ops += [dict(kind=A.BC_AD_Q, lat=1, axis=a, pos=p, dir=d, type=m_q, c0=0.0) for (a, p, d) in F]
            ops.append(dict(kind=A.SMOOTH_CORNER, lat=0))
            ops.append(dict(kind=A.SMOOTH_CORNER, lat=1))
        else:
            ops += [dict(kind=A.BC_AAD_T, lat=1, axis=a, pos=p, dir=d, type=m_in) for (a, p, d) in F]
            ops += [dict(kind=A.BC_AAD_Q, lat=1, axis=a, pos=p, dir=d, type=m_q) for (a, p, d) in F]
            ops += [dict(kind=A.BC_IWALL, lat=0, axis=a, pos=p, dir=d, type=wall) for (a, p, d) in F]
            ops += [dict(kind=A.BC_ANS_U, lat=0, axis=a, pos=p, dir=d, type=m_in, v0=u, v1=zero, v2=zero)
                    for (a, p, d) in F]
            if self.nd == 2:
                ops += [dict(kind=A.BC_AAD_RHO, lat=0, axis=a, pos=p, dir=d, type=2 * m_out) for (a, p, d) in F]
            else:
                ops += [dict(kind=A.BC_ANS_RHO, lat=0, axis=a, pos=p, dir=d, type=m_out) for (a, p, d) in F]
            ops.append(dict(kind=A.SMOOTH_CORNER, lat=1))
            ops.append(dict(kind=A.SMOOTH_CORNER, lat=0))
        return ops

    def design(self, seed=0, sigma=8.0):
        return grf_design(self.nd, self.lx, self.ly, self.lz, seed=seed, sigma=sigma)


FWD_FIELDS = ("rho", "ux", "uy", "uz", "tem")
ADJ_FIELDS = ("ip", "iux", "iuy", "iuz", "item", "iqx", "iqy", "iqz")


class ForcedHeatSink:
    """One forced-convection heat-sink design problem on one device lattice: the design
    iteration (filter, forward and adjoint to the residual tolerance, sensitivity, filtered
    sensitivity) of production/heatsink.cpp:94-244 with this problem's physics."""

    def __init__(self, p, storage="fp64", stochastic_rounding=False):
        self.p = p
        self.q = 9 if p.nd == 2 else 15
        self.n = p.n
        self.lp = LatticePair(self.q, p.lx, p.ly, p.lz, storage)
        if stochastic_rounding:
            self.lp.set_option(A.OPT_STOCHASTIC_ROUNDING, 1)
        self.prog_f = self.lp.program(to_descs(p.program_ops("forward")))
        self.prog_a = self.lp.program(to_descs(p.program_ops("adjoint")))
        self.ph = phys(nu=p.nu)

    def close(self):
        self.lp.close()

    def filtered(self, s):
        return self.p.project(self.lp.heaviside_var(self.p.R, self.p.beta, s))

    def set_design(self, ss):
        """upload the design maps of the filtered design ss; returns (dads, dkds, dQdss)"""
        p, lp = self.p, self.lp
        alpha, kappa, dads, dkds = p.design_fields(ss)
        Q, dQ = p.heat_source(ss)
        lp.set_field(A.ALPHA, alpha)
        lp.set_field(A.KAPPA, kappa)
        lp.set_field(A.HEAT_SOURCE, Q)
        lp.set_field(A.OBJ_WEIGHT, p.objective_weight(ss))
        return dads, dkds, dQ

    def seed_forward(self, seed=None):
        """NS / AD initial condition: at rest (rho = 1, u = 0, T = 0) or from predicted fields"""
        n, lp = self.n, self.lp
        zero = np.zeros(n)
        if seed is None:
            lp.init(0, np.ones(n), ux=zero, uy=zero, uz=zero)
            lp.init(1, zero, ux=zero, uy=zero, uz=zero)
        else:
            uz = seed.get("uz", zero)
            lp.init(0, seed["rho"], ux=seed["ux"], uy=seed["uy"], uz=uz)
            lp.init(1, seed["tem"], ux=seed["ux"], uy=seed["uy"], uz=uz)

    def seed_adjoint(self, fu, seed=None):
        """ANS / AAD initial condition with the forward velocity: zero adjoint (from the frozen
        forward velocity on the device) or predicted"""
        lp, zero = self.lp, np.zeros(self.n)
        if seed is None:
            lp.init(2, None)
            lp.init(3, None)
        else:
            g = lambda k: seed.get(k, zero)  # noqa: E731
            lp.init(2, g("ip"), g("iux"), g("iuy"), g("iuz"), ux=fu[0], uy=fu[1], uz=fu[2])
            lp.init(3, g("item"), g("iqx"), g("iqy"), g("iqz"), ux=fu[0], uy=fu[1], uz=fu[2])

    def solve_pair(self, s, tol=1e-6, max_steps=100000, max_adjoint_steps=None, check_every=100):
        """forward and adjoint solves of design s from rest, leaving both solutions on the device
        (for a training sample); returns the filtered design and the (status, steps) of both"""
        lp = self.lp
        ss = self.filtered(s)
        self.set_design(ss)
        self.seed_forward(None)
        st_f, nf, _ = lp.solve(A.AD_FORCE, self.ph, self.prog_f, max_steps, check_every, tol)
        lp.freeze_forward()
        self.seed_adjoint(None)
        st_a, na, _ = lp.solve(A.AAD_FORCE, self.ph, self.prog_a, max_adjoint_steps or max_steps, check_every, tol)
        lp.synchronize()
        return ss, (st_f, nf), (st_a, na)

    def iterate(self, s, tol=1e-6, max_steps=100000, check_every=100, seed=None, filtered=None,
                fixed_steps=None, adjoint_fallback=None):
        """One design iteration. `seed` (dict of predicted fields, see FWD_FIELDS / ADJ_FIELDS)
        replaces the at-rest initial conditions (a seed without adjoint fields seeds the forward
        problem only); `fixed_steps` = (nf, na) runs exactly that many forward / adjoint steps
        instead of the residual loops (parity tests). adjoint_fallback = K: a seeded adjoint that
        has not converged after K steps is restarted from rest (its steps count in the total)."""
        p, lp, n, t = self.p, self.lp, self.n, {}
        t0 = time.perf_counter()
        ss = self.filtered(s) if filtered is None else p.project(filtered)
        dads, dkds, dQ = self.set_design(ss)
        self.seed_forward(seed)
        t["setup"] = time.perf_counter() - t0
        t1 = time.perf_counter()
        if fixed_steps is None:
            st_f, steps_f, res_f = lp.solve(A.AD_FORCE, self.ph, self.prog_f, max_steps, check_every, tol)
        else:
            steps_f = fixed_steps[0]
            lp.collide(A.AD_FORCE, self.ph)
            for m in range(1, steps_f):
                lp.step(A.AD_FORCE, self.ph, self.prog_f, save=(m == steps_f - 1))
            st_f, res_f = A.PL_MAX_STEPS, (float("nan"), float("nan"))
        lp.snapshot(0, host=False)
        lp.freeze_forward()
        lp.synchronize()
        t["forward"] = time.perf_counter() - t1
        t2 = time.perf_counter()
        fwd = {k: lp.get_field(f) for k, f in zip(FWD_FIELDS, (A.FWD_RHO, A.FWD_UX, A.FWD_UY, A.FWD_UZ, A.FWD_TEM))}
        fu = (fwd["ux"], fwd["uy"], fwd["uz"])
        adj_seed = seed if seed is not None and any(k in seed for k in ADJ_FIELDS) else None
        self.seed_adjoint(fu, adj_seed)
        fallback = False
        if fixed_steps is None:
            first = max_steps if adj_seed is None or adjoint_fallback is None else min(max_steps, adjoint_fallback)
            st_a, steps_a, res_a = lp.solve(A.AAD_FORCE, self.ph, self.prog_a, first, check_every, tol)
            if st_a != A.PL_CONVERGED and first < max_steps:
                fallback = True
                self.seed_adjoint(fu, None)
                st_a, more, res_a = lp.solve(A.AAD_FORCE, self.ph, self.prog_a, max_steps, check_every, tol)
                steps_a += more
        else:
            steps_a = fixed_steps[1]
            lp.collide(A.AAD_FORCE, self.ph, save=True)
            for m in range(1, steps_a):
                lp.step(A.AAD_FORCE, self.ph, self.prog_a, save=(m == steps_a - 1))
            st_a, res_a = A.PL_MAX_STEPS, (float("nan"), float("nan"))
        lp.snapshot(1, host=False)
        lp.synchronize()
        t["adjoint"] = time.perf_counter() - t2
        t3 = time.perf_counter()
        adj = {k: lp.get_field(f) for k, f in zip(ADJ_FIELDS, (A.IP, A.IUX, A.IUY, A.IUZ, A.ITEM, A.IQX, A.IQY,
                                                                A.IQZ))}
        J, dJ_explicit = p.objective(ss, fwd["tem"])
        # AAD::SensitivityBrinkmanDiffusivity (adjointadvection.h:1459-1493) returns the
        # reference's sign convention, -lambda^T dF/ds; the source term lambda^T dF/dQ dQ/ds is
        # formed in the same way as the heat-exchange one (adjointadvection.h:1443-1457)
        r_bd = lp.sensitivity(1, np.zeros(n), dads, dkds)
        dJdss = dJ_explicit - r_bd + adj["item"] * dQ
        dJdss[p.plate] = 0.0
        dJds = lp.heaviside_sens(p.R, p.beta, s, dJdss)
        dJds[p.plate] = 0.0
        t["sensitivity"] = time.perf_counter() - t3
        t["total"] = time.perf_counter() - t0
        return dict(objective=J, ss=ss, dJdss=dJdss, dJds=dJds, fwd=fwd, adj=adj,
                    forward=(st_f, steps_f, res_f), adjoint=(st_a, steps_a, res_a), seconds=t,
                    adjoint_restarted=fallback)
