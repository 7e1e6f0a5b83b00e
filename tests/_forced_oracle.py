"""The CPU oracle's run of the forced-convection heat-sink iteration and of the cavity, step for
step in the order the device runs them (first collide, then stream + boundary program + collide).
Test infrastructure: the library never imports this."""
import numpy as np

from panslbm2_gb300 import _capi as A
from panslbm2_gb300 import forced as FC

from tests._replay import replay

MACROS = ("rho", "ux", "uy", "uz", "tem", "qx", "qy", "qz")
ADJ = ("ip", "iux", "iuy", "iuz", "imx", "imy", "imz", "item", "iqx", "iqy", "iqz")


def cavity(o, lx, ly, steps, nu=0.1, u0=0.1):
    q, n = 9, lx * ly
    L = o.lat(q, lx, ly)
    f = np.zeros((q, n))
    zero = np.zeros(n)
    o.init(L, 0, f, o.fields(rho=np.ones(n), ux=zero, uy=zero))
    mac = {k: np.zeros(n) for k in ("rho", "ux", "uy")}
    ops = FC.cavity_ops(lx, ly, u0)
    for t in range(steps):
        if t:
            o.stream(L, f)
            replay(o, L, f, None, ops, n)
        o.collide(L, A.NS_COLLIDE, f, None, o.fields(**mac), nu=nu, save=True)
    return mac


def forced_iteration(o, p, ss, nf, na, uscale=1.0):
    """Forward nf steps from rest and adjoint na steps from zero on the filtered design ss, then
    the sensitivity terms; returns fields, objective and dJ/dss (as ForcedHeatSink.iterate)."""
    q = 9 if p.nd == 2 else 15
    n = p.n
    L = o.lat(q, p.lx, p.ly, p.lz)
    alpha, kappa, dads, dkds = p.design_fields(ss)
    Q, dQ = p.heat_source(ss)
    w = p.objective_weight(ss)
    f, g = np.zeros((q, n)), np.zeros((q, n))
    zero = np.zeros(n)
    o.init(L, 0, f, o.fields(rho=np.ones(n), ux=zero, uy=zero, uz=zero))
    o.init(L, 1, g, o.fields(tem=zero, ux=zero, uy=zero, uz=zero))
    mac = {k: np.zeros(n) for k in MACROS}
    gs = np.zeros(n * q)
    ops_f, ops_a = p.program_ops("forward"), p.program_ops("adjoint")
    for t in range(nf):
        if t:
            o.stream(L, f)
            o.stream(L, g)
            replay(o, L, f, g, ops_f, n, ux=mac["ux"], uy=mac["uy"], uz=mac["uz"], kappa=kappa, uscale=uscale)
        o.collide(L, A.AD_FORCE, f, g, o.fields(alpha=alpha, diffusivity=kappa, hsrc=Q, gsnap=gs, **mac),
                  nu=p.nu, save=True)
    fwd = {k: mac[k].copy() for k in MACROS}
    adj = {k: np.zeros(n) for k in ADJ}
    igs = np.zeros(n * q)
    o.init(L, 2, f, o.fields(ux=fwd["ux"], uy=fwd["uy"], uz=fwd["uz"], ip=zero, iux=zero, iuy=zero, iuz=zero))
    o.init(L, 3, g, o.fields(ux=fwd["ux"], uy=fwd["uy"], uz=fwd["uz"], item=zero, iqx=zero, iqy=zero, iqz=zero))
    F = o.fields(alpha=alpha, diffusivity=kappa, objw=w, gsnap=igs, **fwd, **adj)
    for t in range(na):
        if t:
            o.stream(L, f, True)
            o.stream(L, g, True)
            replay(o, L, f, g, ops_a, n, ux=fwd["ux"], uy=fwd["uy"], uz=fwd["uz"], rho=fwd["rho"], tem=fwd["tem"],
                   kappa=kappa, uscale=uscale)
        o.collide(L, A.AAD_FORCE, f, g, F, nu=p.nu, save=True)
    r_bd = np.zeros(n)
    o.sensitivity(L, 1, r_bd, o.fields(diffusivity=kappa, **fwd, **adj), dads, dkds, gs, igs)
    J, dJx = p.objective(ss, fwd["tem"])
    dJdss = dJx - r_bd + adj["item"] * dQ
    dJdss[p.plate] = 0.0
    return dict(fwd=fwd, adj=adj, objective=J, dJdss=dJdss, f=f, g=g)


def forced_transient(o, p, ss, nt, tau_in=500.0):
    """The transient sweep of panslbm2_gb300.transient for the forced-convection heat sink, every
    time level kept: forward from rest over levels 1..nt-1 with the inflow u(t) = u_max (1 -
    exp(-t / tau_in)) on the boundary calls that close step t, then the adjoint from t = nt - 2
    down to 0 in the reference transient driver's order (production/heatsink_transient.cpp:
    181-204): adjoint collide with level t (objective weight w / nt), its sensitivity terms, iStream
    and the adjoint boundary calls with u(t). Returns the time-averaged objective and dfdss in the
    reference's sign convention."""
    import math
    q = 9 if p.nd == 2 else 15
    n = p.n
    L = o.lat(q, p.lx, p.ly, p.lz)
    alpha, kappa, dads, dkds = p.design_fields(ss)
    Q, dQ = p.heat_source(ss)
    w = p.objective_weight(ss)
    sc = lambda t: 1.0 - math.exp(-t / tau_in)  # noqa: E731
    f, g = np.zeros((q, n)), np.zeros((q, n))
    zero = np.zeros(n)
    o.init(L, 0, f, o.fields(rho=np.ones(n), ux=zero, uy=zero, uz=zero))
    o.init(L, 1, g, o.fields(tem=zero, ux=zero, uy=zero, uz=zero))
    ops_f, ops_a = p.program_ops("forward"), p.program_ops("adjoint")
    lv = {0: dict(rho=np.ones(n), ux=zero.copy(), uy=zero.copy(), uz=zero.copy(), tem=zero.copy(),
                  gi=np.zeros(n * q))}
    acc = np.zeros(n)
    mac = {k: np.zeros(n) for k in MACROS}
    for t in range(1, nt):
        if t > 1:
            o.stream(L, f)
            o.stream(L, g)
            replay(o, L, f, g, ops_f, n, ux=mac["ux"], uy=mac["uy"], uz=mac["uz"], kappa=kappa, uscale=sc(t - 1))
        mac = {k: np.zeros(n) for k in MACROS}
        gs = np.zeros(n * q)
        o.collide(L, A.AD_FORCE, f, g, o.fields(alpha=alpha, diffusivity=kappa, hsrc=Q, gsnap=gs, **mac), nu=p.nu,
                  save=True)
        lv[t] = dict(rho=mac["rho"], ux=mac["ux"], uy=mac["uy"], uz=mac["uz"], tem=mac["tem"], gi=gs)
        acc += mac["tem"]
    last = lv[nt - 1]
    o.init(L, 2, f, o.fields(ux=last["ux"], uy=last["uy"], uz=last["uz"], ip=zero, iux=zero, iuy=zero, iuz=zero))
    o.init(L, 3, g, o.fields(ux=last["ux"], uy=last["uy"], uz=last["uz"], item=zero, iqx=zero, iqy=zero, iqz=zero))
    dfdss = np.zeros(n)
    wt = w / nt
    for t in range(nt - 2, -1, -1):
        s = lv[t]
        adj = {k: np.zeros(n) for k in ADJ}
        igs = np.zeros(n * q)
        fw = dict(rho=s["rho"], ux=s["ux"], uy=s["uy"], uz=s["uz"], tem=s["tem"])
        o.collide(L, A.AAD_FORCE, f, g, o.fields(alpha=alpha, diffusivity=kappa, objw=wt, gsnap=igs, **fw, **adj),
                  nu=p.nu, save=True)
        o.sensitivity(L, 1, dfdss, o.fields(diffusivity=kappa, **fw, **adj), dads, dkds, s["gi"], igs)
        if p.nd == 2:
            dfdss -= dQ * adj["item"]
        o.stream(L, f, True)
        o.stream(L, g, True)
        replay(o, L, f, g, ops_a, n, ux=s["ux"], uy=s["uy"], uz=s["uz"], rho=s["rho"], tem=s["tem"], kappa=kappa,
               uscale=sc(t))
    return dict(objective=float(np.sum(w * acc)) / nt, dfdss=dfdss, f=f, g=g)
