"""Replay op lists (panslbm2_gb300.heatsink.program_ops format) through the CPU oracle."""
import numpy as np

from panslbm2_gb300 import _capi as A

F_KINDS = (A.BC_NS_U, A.BC_NS_RHO, A.BC_ANS_U, A.BC_ANS_RHO, A.BC_AAD_RHO, A.BC_NSIN_U, A.BC_NSIN_RHO, A.BC_ANSIN_U,
           A.BC_EL_STRESS, A.BC_AEL_STRESS)


def replay(o, L, f, g, ops, n, ux=None, uy=None, uz=None, rho=None, tem=None, kappa=None, uscale=1.0):
    """Apply the op list in call order; `uscale` multiplies the prescribed velocity of NS SetU /
    ANS iSetU ops (time-varying inflow)."""
    for op in ops:
        k = op["kind"]
        lat = op.get("lat", 0)
        if k == A.SMOOTH_CORNER:
            o.smooth_corner(L, f if lat == 0 else g)
            continue
        if k == A.SMOOTH_AT:
            o.smooth_at(L, f if lat == 0 else g, op["i"], op["j"], op.get("k", 0), op["di"], op["dj"], op.get("dk", 0))
            continue
        if k == A.SMOOTH_LINE:
            o.smooth_line(L, f if lat == 0 else g, op["axis"], op["i"], op["j"], op["di"], op["dj"])
            continue
        if k in (A.BC_WALL, A.BC_IWALL):
            tgt = f if lat == 0 else g
        elif k in F_KINDS:
            tgt = f
        else:
            tgt = g
        ty = op.get("type")
        ty = np.ones(n, np.int32) if ty is None else np.ascontiguousarray(ty, np.int32)
        vals = {}
        for nm, cn in (("v0", "c0"), ("v1", "c1"), ("v2", "c2")):
            v = op.get(nm)
            vals[nm] = np.full(n, float(op.get(cn, 0.0))) if v is None else np.ascontiguousarray(v, np.float64)
        # AEL's traction is divided by the routine's rho argument, carried in v2
        brho = vals["v2"] if k == A.BC_AEL_STRESS else rho
        o.apply_bc(L, tgt, k, op["axis"], op["pos"], op["dir"], ty, g=(g if k == A.BC_AAD_RHO else None),
                   ux=ux, uy=uy, uz=uz, rho=brho, tem=tem, diffusivity=kappa, kappa=op.get("kappa", 0.0),
                   eps=op.get("eps", 0.0), uscale=uscale, **vals)
