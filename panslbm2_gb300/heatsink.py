"""Heat-sink topology-optimisation workloads: boundary programs, physics constants and seeded
synthetic designs.

The boundary programs restate the per-step boundary calls of the production heat-sink drivers
(production/heatsink.cpp:153-168 forward, 198-206 adjoint; production/heatsink3D.cpp:160-176,
205-213) as plain op lists. `to_descs` turns them into the library's boundary program; the tests
replay the same lists through the CPU oracle.
"""
import math

import numpy as np

from . import _capi as A
from .lattice import Desc


def faces(nd, lx, ly, lz=1):
    """(axis, pos, dir) of the edge/face calls of a whole-boundary routine, reference order
    xmin, xmax, ymin, ymax[, zmin, zmax] (d2q9.h:114-119, d3q15.h:182-189)."""
    out = [(0, 0, -1), (0, lx - 1, 1), (1, 0, -1), (1, ly - 1, 1)]
    if nd == 3:
        out += [(2, 0, -1), (2, lz - 1, 1)]
    return out


def grid(nd, lx, ly, lz=1):
    """Global coordinates of every node, flattened in idx = i + lx*(j + ly*k) order."""
    if nd == 2:
        j, i = np.meshgrid(np.arange(ly), np.arange(lx), indexing="ij")
        return i.reshape(-1), j.reshape(-1), np.zeros(lx * ly, dtype=np.int64)
    k, j, i = np.meshgrid(np.arange(lz), np.arange(ly), np.arange(lx), indexing="ij")
    return i.reshape(-1), j.reshape(-1), k.reshape(-1)


class Params:
    """Physics constants of the heat-sink drivers (heatsink.cpp:41-46, heatsink3D.cpp:42-48)."""

    def __init__(self, nd, lx, ly, lz=1, Pr=6.0, Ra=None, nu=0.1, tem0=0.0, qn=None, alphamax=1.0e4, qg=1.0,
                 qf=1e-2, L=None, R=2.4):
        self.nd, self.lx, self.ly, self.lz = nd, lx, ly, lz
        self.Pr, self.nu, self.tem0 = Pr, nu, tem0
        self.Ra = Ra if Ra is not None else (1e4 if nd == 2 else 1e3)
        self.qn = qn if qn is not None else (1.0e-2 if nd == 2 else 1.5e-2)
        self.alphamax, self.qg, self.qf, self.R = alphamax, qg, qf, R
        self.L = L if L is not None else (4.0 if nd == 2 else (lx - 1) / 10)
        U = nu * math.sqrt(self.Ra / Pr) / (ly - 1)
        self.diff_fluid = nu / Pr
        self.diff_solid = self.diff_fluid * 10.0
        self.gx, self.gy, self.gz = 0.0, U * U / (ly - 1), 0.0

    def design_fields(self, ss):
        """alpha, kappa and their design derivatives from the filtered design (heatsink.cpp:107-113)."""
        df, ds, qg, qf = self.diff_fluid, self.diff_solid, self.qg, self.qf
        am = self.alphamax / (self.ly - 1)
        kappa = ds + (df - ds) * ss * (1.0 + qg) / (ss + qg)
        alpha = am * qf * (1.0 - ss) / (ss + qf)
        dkds = (df - ds) * qg * (1.0 + qg) / (ss + qg) ** 2
        dads = -am * qf * (1.0 + qf) / (ss + qf) ** 2
        return alpha, kappa, dads, dkds

    def source(self):
        """heat-source flux qn and its mask on the y = 0 boundary."""
        i, j, k = grid(self.nd, self.lx, self.ly, self.lz)
        if self.nd == 2:
            m = (j == 0) & (i < self.L)
        else:
            m = (j == 0) & (i < self.L) & (k < self.L)
        return np.where(m, self.qn, 0.0), m.astype(np.int32)


def program_ops(phase, p):
    """Boundary calls of one time step, in driver order, as op dicts."""
    nd, lx, ly, lz = p.nd, p.lx, p.ly, p.lz
    i, j, k = grid(nd, lx, ly, lz)
    F = faces(nd, lx, ly, lz)
    if nd == 2:
        wall_f = np.where(i == 0, 2, 1).astype(np.int32)
        wall_g = np.where(i == 0, 2, 0).astype(np.int32)
        mask_t = ((i == lx - 1) | (j == ly - 1)).astype(np.int32)
    else:
        wall_f = np.where((i == 0) | (k == 0), 2, 1).astype(np.int32)
        wall_g = np.where((i == 0) | (k == 0), 2, 0).astype(np.int32)
        mask_t = ((i == lx - 1) | (j == ly - 1) | (k == lz - 1)).astype(np.int32)
    mask_q = (j == 0).astype(np.int32)
    qn, mask_src = p.source()
    ops = []
    if phase == "forward":
        for (a, pos, d) in F:
            ops.append(dict(kind=A.BC_WALL, lat=0, axis=a, pos=pos, dir=d, type=wall_f))
        for (a, pos, d) in F:
            ops.append(dict(kind=A.BC_AD_T, lat=1, axis=a, pos=pos, dir=d, type=mask_t, c0=p.tem0))
        for (a, pos, d) in F:
            ops.append(dict(kind=A.BC_AD_Q, lat=1, axis=a, pos=pos, dir=d, type=mask_q, v0=qn))
        for (a, pos, d) in F:
            ops.append(dict(kind=A.BC_WALL, lat=1, axis=a, pos=pos, dir=d, type=wall_g))
        ops.append(dict(kind=A.SMOOTH_CORNER, lat=0))
        ops.append(dict(kind=A.SMOOTH_CORNER, lat=1))
    else:
        for (a, pos, d) in F:
            ops.append(dict(kind=A.BC_AAD_T, lat=1, axis=a, pos=pos, dir=d, type=mask_t))
        for (a, pos, d) in F:
            ops.append(dict(kind=A.BC_AAD_Q, lat=1, axis=a, pos=pos, dir=d, type=mask_q))
        for (a, pos, d) in F:
            ops.append(dict(kind=A.BC_AAD_Q, lat=1, axis=a, pos=pos, dir=d, type=mask_src, eps=1.0))
        for (a, pos, d) in F:
            ops.append(dict(kind=A.BC_IWALL, lat=1, axis=a, pos=pos, dir=d, type=wall_g))
        for (a, pos, d) in F:
            ops.append(dict(kind=A.BC_IWALL, lat=0, axis=a, pos=pos, dir=d, type=wall_f))
        ops.append(dict(kind=A.SMOOTH_CORNER, lat=0))
        ops.append(dict(kind=A.SMOOTH_CORNER, lat=1))
    return ops


def to_descs(ops):
    out = []
    for o in ops:
        kw = dict(o)
        kind = kw.pop("kind")
        arrays = {nm: kw.pop(nm) for nm in ("type", "v0", "v1", "v2") if nm in kw}
        out.append(Desc(kind, **kw, **arrays))
    return out


def grf_design(nd, lx, ly, lz=1, seed=0, sigma=8.0):
    """Seeded Gaussian random-field design in [0, 1]: Philox white noise, separable Gaussian
    smoothing with standard deviation `sigma` cells (correlation length), standardised and
    mapped through the normal CDF."""
    rng = np.random.Generator(np.random.Philox(key=seed))
    shape = (lx, ly) if nd == 2 else (lx, ly, lz)
    z = rng.standard_normal(shape)
    try:
        from scipy.ndimage import gaussian_filter1d
        for ax in range(len(shape)):
            z = gaussian_filter1d(z, sigma, axis=ax, mode="wrap", truncate=3.0)
    except ImportError:  # pragma: no cover
        r = int(math.ceil(3 * sigma))
        x = np.arange(-r, r + 1)
        ker = np.exp(-0.5 * (x / sigma) ** 2)
        ker /= ker.sum()
        for ax in range(len(shape)):
            z = np.apply_along_axis(lambda v: np.convolve(np.pad(v, r, mode="wrap"), ker, mode="valid"), ax, z)
    z = (z - z.mean()) / z.std()
    try:
        from scipy.special import ndtr
        s = ndtr(z)
    except ImportError:  # pragma: no cover
        s = 0.5 * (1.0 + np.vectorize(math.erf)(z / math.sqrt(2.0)))
    # node order idx = i + lx*(j + ly*k)
    return np.ascontiguousarray(np.transpose(s).reshape(-1))
