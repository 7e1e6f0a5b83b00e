"""Svanberg's method of moving asymptotes on the device (MMA<T> of the reference,
utility/mma.h:58-548), through the C ABI: pl_mma_create / pl_mma_set_param / pl_mma_update."""
import ctypes as C

import numpy as np

from . import _capi as A

PARAMS = {"move": 0, "asyinit": 1, "asydecr": 2, "asyincr": 3, "albefa": 4, "raa0": 5, "epsvalue": 6}


def _dp(v):
    return v.ctypes.data_as(C.POINTER(C.c_double))


class MMA:
    def __init__(self, n, m, a0, a, c, d, xmin, xmax, **params):
        self.lib = A.load()
        self.n, self.m = n, m
        arr = [np.ascontiguousarray(v, np.float64) for v in (a, c, d, xmin, xmax)]
        h = C.c_void_p()
        A.check(self.lib.pl_mma_create(n, m, C.c_double(a0), *[_dp(v) for v in arr], C.byref(h)))
        self.h = h
        for k, v in params.items():
            self.set(k, v)

    def set(self, name, value):
        A.check(self.lib.pl_mma_set_param(self.h, PARAMS[name], C.c_double(value)))

    def update(self, x, f, dfdx, g, dgdx):
        """One UpdateVariables: returns the new design (x is not modified)."""
        x = np.ascontiguousarray(x, np.float64).copy()
        dfdx = np.ascontiguousarray(dfdx, np.float64)
        g = np.ascontiguousarray(np.atleast_1d(g), np.float64)
        dgdx = np.ascontiguousarray(np.reshape(dgdx, (self.m, self.n)), np.float64)
        A.check(self.lib.pl_mma_update(self.h, _dp(x), C.c_double(f), _dp(dfdx), _dp(g), _dp(dgdx)))
        return x

    def close(self):
        if getattr(self, "h", None):
            self.lib.pl_mma_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
