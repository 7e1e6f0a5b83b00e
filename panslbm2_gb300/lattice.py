"""Host-side mirror of the reference's lattice / equation API over the C ABI.

`LatticePair` owns one NS population set (the reference's `pf`) and one AD set (`pg`) of a
D2Q9 or D3Q15 lattice on the GPU. Methods map one-to-one onto the C entry points; arrays are
numpy float64 in the reference's node order idx = i + nx*(j + ny*k).
"""
import ctypes as C

import numpy as np

from . import _capi as A
from ._capi import check


def _dp(a):
    return None if a is None else a.ctypes.data_as(A.DP)


def _f64(a, n=None):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float64)
    if n is not None and a.size != n:
        raise ValueError("expected %d values, got %d" % (n, a.size))
    return a


def _i32(a, n=None):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.int32)
    if n is not None and a.size != n:
        raise ValueError("expected %d values, got %d" % (n, a.size))
    return a


def phys(nu=0.1, diff=0.0, gx=0.0, gy=0.0, gz=0.0, tem0=0.0, tau=0.0):
    return A.Phys(nu, diff, gx, gy, gz, tem0, tau)


class Desc:
    """One recorded boundary routine call (see pl_bc_desc)."""

    def __init__(self, kind, axis=0, pos=0, dir=-1, lat=0, type=None, v0=None, v1=None, v2=None, c0=0.0, c1=0.0,
                 c2=0.0, eps=0.0, kappa=0.0, i=0, j=0, k=0, di=0, dj=0, dk=0):
        self.kw = dict(kind=kind, axis=axis, pos=pos, dir=dir, lat=lat, c0=c0, c1=c1, c2=c2, eps=eps, kappa=kappa,
                       i=i, j=j, k=k, di=di, dj=dj, dk=dk)
        self.arrays = dict(type=type, v0=v0, v1=v1, v2=v2)


def bc(kind, axis, pos, dir, **kw):
    return Desc(kind, axis, pos, dir, **kw)


def smooth_corner(lat):
    return Desc(A.SMOOTH_CORNER, lat=lat)


def smooth_at(lat, i, j, k, di, dj, dk=0):
    return Desc(A.SMOOTH_AT, lat=lat, i=i, j=j, k=k, di=di, dj=dj, dk=dk)


def smooth_line(lat, plane, a, b, da, db):
    return Desc(A.SMOOTH_LINE, lat=lat, axis=plane, i=a, j=b, di=da, dj=db)


class LatticePair:
    def __init__(self, q, nx, ny, nz=1, storage="fp32"):
        self.lib = A.load()
        self.q, self.nx, self.ny = q, nx, ny
        self.nz = nz if q == 15 else 1
        self.nd = 2 if q == 9 else 3
        self.n = nx * ny * self.nz
        self.storage = storage
        h = C.c_void_p()
        check(self.lib.pl_create(q, nx, ny, self.nz, A.STORAGE[storage], C.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            self.lib.pl_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---------------------------------------------------------------- data exchange
    def set_stream(self, stream_ptr):
        check(self.lib.pl_set_stream(self.h, C.c_void_p(stream_ptr)))

    def set_option(self, option, value):
        check(self.lib.pl_set_option(self.h, C.c_int(option), C.c_int(int(value))))

    def set_shift(self, sf, sg):
        check(self.lib.pl_set_shift(self.h, C.c_double(sf), C.c_double(sg)))

    def set_populations(self, s, p):
        p = _f64(p, self.q * self.n)
        check(self.lib.pl_set_populations(self.h, s, _dp(p)))

    def get_populations(self, s):
        out = np.empty((self.q, self.n))
        check(self.lib.pl_get_populations(self.h, s, _dp(out)))
        return out

    def set_field(self, f, v):
        """upload field f; v = None switches the source fields (HEAT_SOURCE, OBJ_WEIGHT) off"""
        v = _f64(v, self.n)
        check(self.lib.pl_set_field(self.h, f, _dp(v)))

    def set_inflow_scale(self, s):
        check(self.lib.pl_set_inflow_scale(self.h, C.c_double(s)))

    def get_field(self, f):
        out = np.empty(self.n)
        check(self.lib.pl_get_field(self.h, f, _dp(out)))
        return out

    def set_field_ptr(self, f, host_ptr):
        """set_field from a raw host pointer (e.g. pinned memory) of n doubles"""
        check(self.lib.pl_set_field(self.h, f, C.cast(C.c_void_p(host_ptr), A.DP)))

    def get_field_ptr(self, f, host_ptr):
        check(self.lib.pl_get_field(self.h, f, C.cast(C.c_void_p(host_ptr), A.DP)))

    def freeze_forward(self):
        check(self.lib.pl_freeze_forward(self.h))

    # ---------------------------------------------------------------- programs and steps
    def program(self, descs):
        arr = (A.BcDesc * max(1, len(descs)))()
        keep = []
        for m, d in enumerate(descs):
            for k, v in d.kw.items():
                setattr(arr[m], k, v)
            t = _i32(d.arrays["type"], self.n)
            keep.append(t)
            arr[m].type = None if t is None else t.ctypes.data_as(A.IPT)
            for nm in ("v0", "v1", "v2"):
                v = _f64(d.arrays[nm], self.n)
                keep.append(v)
                setattr(arr[m], nm, _dp(v))
        prog = C.c_int()
        check(self.lib.pl_program_create(self.h, arr, len(descs), C.byref(prog)))
        return prog.value

    def init(self, which, a0, a1=None, a2=None, a3=None, ux=None, uy=None, uz=None):
        arrs = [_f64(x, self.n) for x in (a0, a1, a2, a3, ux, uy, uz)]
        check(self.lib.pl_init(self.h, which, *[_dp(x) for x in arrs]))

    def init_elastic(self, which, arrays):
        """EL (which 0: rho, ux, uy, sxx, sxy, syx, syy) or AEL (which 1: irho, imx, imy, isxx, isxy,
        isyx, isyy; gamma from the GAMMA field) initial condition."""
        arrs = [_f64(x, self.n) for x in arrays]
        if len(arrs) != 7:
            raise ValueError("seven arrays expected")
        P = (A.DP * 7)(*[_dp(x) for x in arrs])
        check(self.lib.pl_init_elastic(self.h, which, P))

    def sensitivity_compliance(self, dfds, arrays=None):
        """AEL::SensitivityCompliance: dfds + 4.5 s:is - 1.5 irho tr s over (sxx, sxy, syx, syy, irho,
        isxx, isxy, isyx, isyy), or over the last saved EL / AEL macros when arrays is None."""
        dfds = _f64(dfds, self.n).copy()
        P = None
        if arrays is not None:
            arrs = [_f64(x, self.n) for x in arrays]
            if len(arrs) != 9:
                raise ValueError("nine arrays expected")
            P = (A.DP * 9)(*[_dp(x) for x in arrs])
        check(self.lib.pl_sensitivity_compliance(self.h, _dp(dfds), P))
        return dfds

    def store(self, what, slot):
        check(self.lib.pl_store(self.h, what, slot))

    def load(self, what, slot):
        check(self.lib.pl_load(self.h, what, slot))

    def swap_snapshot(self, slot):
        check(self.lib.pl_store_swap_snapshot(self.h, slot))

    def store_release(self):
        check(self.lib.pl_store_release(self.h))

    def sensitivity_device(self, which, dads=None, dkds=None, qn=None, mask=None):
        """accumulate one sensitivity term into the device field DFDS (inputs reused when None)"""
        dads, dkds, qn = _f64(dads, self.n), _f64(dkds, self.n), _f64(qn, self.n)
        mask = _i32(mask, self.n)
        check(self.lib.pl_sensitivity_device(self.h, which, _dp(dads), _dp(dkds), _dp(qn),
                                             None if mask is None else mask.ctypes.data_as(A.IPT)))

    def accumulate(self, dst, src, a=1.0):
        check(self.lib.pl_accumulate(self.h, dst, src, C.c_double(a)))

    def collide(self, kind, ph, save=True):
        check(self.lib.pl_collide(self.h, kind, C.byref(ph), int(save)))

    def step(self, kind, ph, prog=-1, save=False):
        check(self.lib.pl_step(self.h, kind, C.byref(ph), prog, int(save)))

    def steps(self, kind, ph, prog, n):
        check(self.lib.pl_steps(self.h, kind, C.byref(ph), prog, n))

    def stream(self, mode=0, prog=-1, both=True):
        check(self.lib.pl_stream(self.h, mode, prog, int(both)))

    def solve(self, kind, ph, prog, max_steps, check_every=100, tol=1e-6):
        st, steps = C.c_int(), C.c_int()
        res = (C.c_double * 2)()
        check(self.lib.pl_solve(self.h, kind, C.byref(ph), prog, max_steps, check_every, C.c_double(tol),
                                C.byref(st), C.byref(steps), res))
        return st.value, steps.value, (res[0], res[1])

    def snapshot(self, slot, host=True):
        if not host:
            check(self.lib.pl_snapshot(self.h, slot, None))
            return None
        out = np.empty((self.n, self.q))
        check(self.lib.pl_snapshot(self.h, slot, _dp(out)))
        return out

    def set_snapshot(self, slot, snap):
        snap = _f64(snap, self.n * self.q)
        check(self.lib.pl_set_snapshot(self.h, slot, _dp(snap)))

    def residual(self, family):
        out = C.c_double()
        check(self.lib.pl_residual(self.h, family, C.byref(out)))
        return out.value

    def residual_host(self, a, b):
        a = [_f64(x) for x in a]
        b = [_f64(x) for x in b]
        A_ = (A.DP * len(a))(*[_dp(x) for x in a])
        B_ = (A.DP * len(b))(*[_dp(x) for x in b])
        out = C.c_double()
        check(self.lib.pl_residual_host(self.h, a[0].size, len(a), A_, B_, C.byref(out)))
        return out.value

    def sensitivity(self, which, dfds, dads, dkds=None, qn=None, mask=None):
        dfds = _f64(dfds, self.n).copy()
        dads, dkds, qn = _f64(dads, self.n), _f64(dkds, self.n), _f64(qn, self.n)
        mask = _i32(mask, self.n)
        check(self.lib.pl_sensitivity(self.h, which, _dp(dfds), _dp(dads), _dp(dkds), _dp(qn),
                                      None if mask is None else mask.ctypes.data_as(A.IPT)))
        return dfds

    def heaviside_var(self, R, beta, s, mask=None):
        s, mask, out = _f64(s, self.n), _i32(mask, self.n), np.empty(self.n)
        check(self.lib.pl_heaviside_var(self.h, C.c_double(R), C.c_double(beta), _dp(s),
                                        None if mask is None else mask.ctypes.data_as(A.IPT), _dp(out)))
        return out

    def heaviside_sens(self, R, beta, s, dfdrho, mask=None):
        s, d, mask, out = _f64(s, self.n), _f64(dfdrho, self.n), _i32(mask, self.n), np.empty(self.n)
        check(self.lib.pl_heaviside_sens(self.h, C.c_double(R), C.c_double(beta), _dp(s), _dp(d),
                                         None if mask is None else mask.ctypes.data_as(A.IPT), _dp(out)))
        return out

    def density_filter(self, R, v, mask=None):
        v, mask, out = _f64(v, self.n), _i32(mask, self.n), np.empty(self.n)
        check(self.lib.pl_density_filter(self.h, C.c_double(R), _dp(v),
                                         None if mask is None else mask.ctypes.data_as(A.IPT), _dp(out)))
        return out

    def filter_taps(self, R):
        """(di, dj, dk) of the filter taps of radius R in the reference's loop order"""
        nR = int(R)
        cap = (2 * nR + 1) ** 3
        n = C.c_int()
        di, dj, dk = (np.zeros(cap, np.int32) for _ in range(3))
        ip = lambda a: a.ctypes.data_as(A.IPT)  # noqa: E731
        check(self.lib.pl_filter_taps(self.h, C.c_double(R), C.byref(n), ip(di), ip(dj), ip(dk)))
        return di[:n.value].copy(), dj[:n.value].copy(), dk[:n.value].copy()

    def filter_weighted(self, op, R, a, weights, b=None, beta=0.0):
        """filters with a general weight table weights[node, tap] (op 0: Heaviside variable,
        1: Heaviside sensitivity with b = dfdrho, 2: density filter)"""
        a, out = _f64(a, self.n), np.empty(self.n)
        b = _f64(b, self.n) if b is not None else None
        w = np.ascontiguousarray(weights, np.float64)
        ntap = len(self.filter_taps(R)[0])
        if w.size != self.n * ntap:
            raise ValueError("expected %d x %d weights, got %d" % (self.n, ntap, w.size))
        check(self.lib.pl_filter_weighted(self.h, op, C.c_double(R), C.c_double(beta), _dp(a),
                                          None if b is None else _dp(b), _dp(w), _dp(out)))
        return out

    def normalize(self, v):
        v = _f64(v).copy()
        check(self.lib.pl_normalize(self.h, _dp(v), v.size))
        return v

    def synchronize(self):
        check(self.lib.pl_synchronize(self.h))

    def stats(self):
        ms, launches = C.c_double(), C.c_longlong()
        check(self.lib.pl_stats(self.h, C.byref(ms), C.byref(launches)))
        return ms.value, launches.value
