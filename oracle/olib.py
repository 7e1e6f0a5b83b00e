"""ctypes binding of the oracle API (oracle.h) -- TEST INFRASTRUCTURE ONLY.

``Oracle("oracle")`` loads the plain-C restatement (liboracle.so); ``Oracle("ref")`` loads the
same API bound to the PANSLBM2 reference headers (oracle/_ref/libref.so, available only where
the reference sources are). Arrays are numpy float64 in the oracle's layouts:
populations f[c, idx] of shape (q, N); snapshots snap[idx, c] of shape (N, q).
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
DP = C.POINTER(C.c_double)
IP = C.POINTER(C.c_int)

# collide kinds
NS_COLLIDE, NS_BRINKMAN, AD_NATURAL, AD_FORCE, AD_HEATEX, AD_NATURAL_NOBRINK, AD_FORCE_NOBRINK = 0, 1, 2, 3, 4, 5, 6
NSIN_COLLIDE, NSIN_BRINKMAN = 7, 8
ANS_BRINKMAN, AAD_NATURAL, AAD_FORCE, AAD_HEATEX, AAD_MASSFLOW, ANSIN_BRINKMAN = 10, 11, 12, 13, 14, 15
EL_COLLIDE, EL_EXTENDED, AEL_COLLIDE = 16, 17, 18
# bc kinds
BC_WALL, BC_IWALL, BC_NS_U, BC_NS_RHO, BC_AD_T, BC_AD_Q, BC_AD_QC = 0, 1, 2, 3, 4, 5, 6
BC_ANS_U, BC_ANS_RHO, BC_AAD_T, BC_AAD_Q, BC_AAD_RHO = 7, 8, 9, 10, 11
BC_NSIN_U, BC_NSIN_RHO, BC_ANSIN_U = 12, 13, 14
BC_EL_STRESS, BC_AEL_STRESS = 15, 16


class Lat(C.Structure):
    _fields_ = [("q", C.c_int), ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int)]


FIELD_NAMES = ["rho", "ux", "uy", "uz", "tem", "qx", "qy", "qz", "ip", "iux", "iuy", "iuz",
               "imx", "imy", "imz", "item", "iqx", "iqy", "iqz", "alpha", "diffusivity", "beta",
               "dirx", "diry", "dirz", "gsnap", "sxx", "sxy", "syx", "syy", "isxx", "isxy", "isyx", "isyy",
               "gamma", "hsrc", "objw"]


class Fields(C.Structure):
    _fields_ = [(n, DP) for n in FIELD_NAMES]


class Phys(C.Structure):
    _fields_ = [("nu", C.c_double), ("diff", C.c_double), ("gx", C.c_double), ("gy", C.c_double),
                ("gz", C.c_double), ("tem0", C.c_double), ("tau", C.c_double)]


class BC(C.Structure):
    _fields_ = [("kind", C.c_int), ("axis", C.c_int), ("pos", C.c_int), ("dir", C.c_int), ("type", IP),
                ("v0", DP), ("v1", DP), ("v2", DP), ("ux", DP), ("uy", DP), ("uz", DP), ("rho", DP),
                ("tem", DP), ("diffusivity", DP), ("kappa", C.c_double), ("eps", C.c_double),
                ("uscale", C.c_double)]


def _dp(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(DP)


def _ip(a):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(IP)


def lib_path(kind):
    if kind == "oracle":
        return os.path.join(HERE, "liboracle.so")
    return os.path.join(HERE, "_ref", "libref.so")


class Oracle:
    def __init__(self, kind="oracle"):
        path = lib_path(kind)
        if not os.path.exists(path):
            import importlib.util
            spec = importlib.util.spec_from_file_location("oracle_build", os.path.join(HERE, "build.py"))
            mod = importlib.util.module_from_spec(spec)
            spec.loader.exec_module(mod)
            mod.build_oracle() if kind == "oracle" else mod.build_ref()
        self.kind = kind
        self.lib = C.CDLL(path)
        L = self.lib
        L.ol_residual.restype = C.c_double
        L.ol_nnodes.restype = C.c_int
        L.ol_filter_ntaps.restype = C.c_int

    def set_threads(self, n):
        self.lib.ol_set_threads(int(n))

    # ------------------------------------------------------------------ helpers
    @staticmethod
    def lat(q, nx, ny, nz=1):
        return Lat(q, nx, ny, nz if q == 15 else 1)

    @staticmethod
    def fields(**kw):
        F = Fields()
        keep = []
        for k, v in kw.items():
            if v is None:
                continue
            keep.append(v)
            setattr(F, k, _dp(v))
        F._keep = keep
        return F

    # ------------------------------------------------------------------ API
    def stream(self, L, f, inverse=False):
        self.lib.ol_stream(C.byref(L), _dp(f), int(inverse))

    def apply_bc(self, L, f, kind, axis, pos, dir, type, g=None, v0=None, v1=None, v2=None, ux=None, uy=None,
                 uz=None, rho=None, tem=None, diffusivity=None, kappa=0.0, eps=0.0, uscale=1.0):
        b = BC(kind, axis, pos, dir, _ip(type), _dp(v0), _dp(v1), _dp(v2), _dp(ux), _dp(uy), _dp(uz), _dp(rho),
               _dp(tem), _dp(diffusivity), float(kappa), float(eps), float(uscale))
        self.lib.ol_apply_bc(C.byref(L), _dp(f), _dp(g), C.byref(b))

    def smooth_corner(self, L, f):
        self.lib.ol_smooth_corner(C.byref(L), _dp(f))

    def smooth_at(self, L, f, i, j, k, dx, dy, dz):
        self.lib.ol_smooth_at(C.byref(L), _dp(f), i, j, k, dx, dy, dz)

    def smooth_line(self, L, f, plane, a, b, da, db):
        self.lib.ol_smooth_line(C.byref(L), _dp(f), plane, a, b, da, db)

    def collide(self, L, kind, f, g, F, nu=0.0, diff=0.0, gx=0.0, gy=0.0, gz=0.0, tem0=0.0, save=True, tau=1.0):
        P = Phys(nu, diff, gx, gy, gz, tem0, tau)
        self.lib.ol_collide(C.byref(L), int(kind), _dp(f), _dp(g), C.byref(F), C.byref(P), int(save))

    def init(self, L, which, f, F):
        self.lib.ol_init(C.byref(L), int(which), _dp(f), C.byref(F))

    def sensitivity(self, L, which, dfds, F, dads, dkds=None, g=None, ig=None, qn=None, mask=None):
        self.lib.ol_sensitivity(C.byref(L), int(which), _dp(dfds), C.byref(F), _dp(dads), _dp(dkds), _dp(g),
                                _dp(ig), _dp(qn), _ip(mask))

    def heaviside_var(self, L, R, beta, s, mask=None):
        out = np.zeros_like(s)
        self.lib.ol_heaviside_var(C.byref(L), C.c_double(R), C.c_double(beta), _dp(s), _ip(mask), _dp(out))
        return out

    def heaviside_sens(self, L, R, beta, s, dfdrho, mask=None):
        out = np.zeros_like(s)
        self.lib.ol_heaviside_sens(C.byref(L), C.c_double(R), C.c_double(beta), _dp(s), _dp(dfdrho), _ip(mask),
                                   _dp(out))
        return out

    def density_filter(self, L, R, v, mask=None):
        out = np.zeros_like(v)
        self.lib.ol_density_filter(C.byref(L), C.c_double(R), _dp(v), _ip(mask), _dp(out))
        return out

    def filter_ntaps(self, L, R):
        return int(self.lib.ol_filter_ntaps(C.byref(L), C.c_double(R)))

    def filter_table(self, L, op, R, a, w, b=None, beta=0.0):
        """the filters with a weight table w[node][tap] (op 0 / 1 / 2: Heaviside variable,
        Heaviside sensitivity with b = dfdrho, density filter)"""
        a = np.ascontiguousarray(a, np.float64)
        w = np.ascontiguousarray(w, np.float64)
        out = np.zeros_like(a)
        bb = None if b is None else np.ascontiguousarray(b, np.float64)
        self.lib.ol_filter_table(C.byref(L), op, C.c_double(R), C.c_double(beta), _dp(a), None if bb is None else _dp(bb),
                                 _dp(w), _dp(out))
        return out

    def residual(self, a, b):
        n = a[0].size
        A = (DP * len(a))(*[_dp(x) for x in a])
        B = (DP * len(b))(*[_dp(x) for x in b])
        return self.lib.ol_residual(n, len(a), A, B)

    def normalize(self, v):
        self.lib.ol_normalize(_dp(v), v.size)
