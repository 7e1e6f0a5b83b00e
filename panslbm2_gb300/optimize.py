"""The topology-optimisation loop of the forced-convection heat sink (200 x 100, FP64, 20 design
iterations), on one device lattice and the device MMA.

Each design iteration takes the steps of production/heatsink.cpp:93-280, with this problem's
physics (panslbm2_gb300.forced):

  1. Heaviside-filtered design ss (HeavisideFilter::GetFilteredVariable, :97), base plate solid;
  2. design maps alpha, kappa and their derivatives (:106-111);
  3. volume constraint g = sum(1 - ss) / (weightlimit N) - 1 over the design cells, dg/dss =
     -1 / (weightlimit N) there (:113-131);
  4. forward and adjoint to the residual tolerance from rest, objective J and dJ/dss (:133-231);
  5. filtered sensitivities of J and of g (:234-235), zero outside the design cells (:236-243),
     Normalize of J's (:244);
  6. MMA update with one constraint, a0 = 1, a = 0, c = 10000, d = 0, bounds [0, 1], move limit
     0.2 (:74-81, :263), base plate cells held at 0;
  7. the largest design change dsmax (:264-283).

The reference's continuation over (qf, beta) stages is not part of this loop; beta and the
filter radius stay at the problem's values (ForcedParams).
"""
import json
import time

import numpy as np

from . import _capi as A
from .forced import ForcedHeatSink, ForcedParams
from .mma import MMA


class ForcedOptimisation:
    def __init__(self, p, storage="fp64", weightlimit=0.5, movelimit=0.2):
        self.p = p
        self.hs = ForcedHeatSink(p, storage)
        self.weightlimit = weightlimit
        self.ndesign = int(np.count_nonzero(p.design_mask))
        self.mma = MMA(p.n, 1, 1.0, [0.0], [10000.0], [0.0], np.zeros(p.n), np.ones(p.n), move=movelimit)

    def close(self):
        self.mma.close()
        self.hs.close()

    def constraint(self, ss):
        """g and dg/dss of the volume constraint (production/heatsink.cpp:113-131)"""
        dm = self.p.design_mask
        scale = 1.0 / (self.weightlimit * self.ndesign)
        g = float(np.sum((1.0 - ss)[dm])) * scale - 1.0
        dgdss = np.where(dm, -scale, 0.0)
        return g, dgdss

    def iteration(self, s, tol=1e-6, max_steps=100000):
        """one design iteration from design s; returns the updated design and its record"""
        p, hs = self.p, self.hs
        t0 = time.perf_counter()
        ss = hs.filtered(s)
        g, dgdss = self.constraint(ss)
        r = hs.iterate(s, tol=tol, max_steps=max_steps, filtered=ss)
        dfds = np.where(p.design_mask, r["dJds"], 0.0)
        dgds = np.where(p.design_mask, hs.lp.heaviside_sens(p.R, p.beta, s, dgdss), 0.0)
        dfds = hs.lp.normalize(dfds)
        s_new = self.mma.update(s, r["objective"], dfds, [g], dgds)
        s_new[~p.design_mask] = 0.0
        dsmax = float(np.max(np.abs(s_new - s)))
        mnd = float(np.sum((ss * (1.0 - ss))[p.design_mask])) * 4.0 / self.ndesign * 100.0
        rec = dict(objective=r["objective"], g=g, dsmax=dsmax, grayness_pct=mnd,
                   forward_steps=r["forward"][1], adjoint_steps=r["adjoint"][1],
                   converged=[r["forward"][0] == A.PL_CONVERGED, r["adjoint"][0] == A.PL_CONVERGED],
                   seconds=round(time.perf_counter() - t0, 4))
        return s_new, rec

    def run(self, s, iterations, tol=1e-6, max_steps=100000, log=None):
        s = np.array(s, dtype=np.float64)
        s[~self.p.design_mask] = 0.0
        recs = []
        for k in range(iterations):
            s, rec = self.iteration(s, tol, max_steps)
            rec["iteration"] = k + 1
            recs.append(rec)
            if log:
                log(rec)
        return s, recs


def main(argv=None):
    """python -m panslbm2_gb300.optimize [--shape X,Y] [--iterations K] [--storage fp64]:
    the forced heat sink's optimisation loop from the seeded GRF design 0"""
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--shape", default="200,100")
    ap.add_argument("--iterations", type=int, default=20)
    ap.add_argument("--storage", default="fp64")
    ap.add_argument("--tol", type=float, default=1e-6)
    ap.add_argument("--max-steps", type=int, default=100000)
    ap.add_argument("--seed", type=int, default=0)
    a = ap.parse_args(argv)
    lx, ly = (int(v) for v in a.shape.split(","))
    p = ForcedParams(2, lx, ly)
    opt = ForcedOptimisation(p, a.storage)
    t0 = time.perf_counter()
    _, recs = opt.run(p.design(seed=a.seed), a.iterations, a.tol, a.max_steps,
                      log=lambda r: print(json.dumps(r), flush=True))
    opt.close()
    print(json.dumps(dict(shape=[lx, ly], storage=a.storage, iterations=a.iterations, tol=a.tol,
                          seconds=round(time.perf_counter() - t0, 3),
                          objective_first=recs[0]["objective"], objective_last=recs[-1]["objective"],
                          g_last=recs[-1]["g"], all_converged=all(all(r["converged"]) for r in recs))))


if __name__ == "__main__":
    main()
