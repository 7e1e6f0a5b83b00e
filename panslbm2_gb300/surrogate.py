"""Learned warm start for the steady heat-sink design iteration.

`UNet` mirrors the library's pl_unet_* entry points: a 3D convolutional U-Net trained and
evaluated on the GPU's tensor cores (tcgen05 implicit-GEMM convolutions). `SurrogateWarmStart`
is the workflow of the forced-convection configuration on 160 x 160 x 80:

  1. training data: for seeded Gaussian-random-field designs the plain solver runs the forward and
     adjoint problems to the residual tolerance; each (filtered design, converged rho/u/T and
     adjoint fields) pair is stored on the device;
  2. training: mean squared error of the per-channel normalised fields, Adam, on the device;
  3. warm start: for a new design the network predicts the fields; the NS / AD initial
     conditions (navierstokes.h:550-572, advection.h:1048-1070) and the ANS / AAD ones
     (adjointnavierstokes.h:474-498, adjointadvection.h:1359-1381) are seeded at equilibrium
     from them, and the plain solver then runs to the same residual tolerance, so the network
     only removes iterations and the solver still judges the result.

The reference has no learned component; everything here is this library's own.
"""
import ctypes as C
import json
import os
import time

import numpy as np

from . import _capi as A
from ._capi import check

# target channels: what the four initial conditions need
TARGETS = ("rho", "ux", "uy", "uz", "tem", "ip", "iux", "iuy", "iuz", "item", "iqx", "iqy", "iqz")
FP = C.POINTER(C.c_float)


def _fp(a):
    return a.ctypes.data_as(FP)


class UNet:
    """A U-Net handle (pl_unet) over an nx x ny x nz volume."""

    def __init__(self, nx, ny, nz, levels=4, base=16, max_batch=1):
        self.lib = A.load()
        self.shape = (nx, ny, nz)
        self.nvox = nx * ny * nz
        self.levels, self.base = levels, base
        h = C.c_void_p()
        check(self.lib.pl_unet_create(nx, ny, nz, levels, base, 16, 16, max_batch, C.byref(h)))
        self.h = h
        self.lib.pl_unet_param_count.restype = C.c_longlong
        self.nparam = int(self.lib.pl_unet_param_count(self.h))
        self.ntarget = 0

    def close(self):
        if self.h:
            self.lib.pl_unet_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # parameters -----------------------------------------------------------------------------
    def init_params(self, seed):
        check(self.lib.pl_unet_init_params(self.h, C.c_ulonglong(seed)))

    def get_params(self):
        out = np.empty(self.nparam, np.float32)
        check(self.lib.pl_unet_get_params(self.h, _fp(out)))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        if p.size != self.nparam:
            raise ValueError("expected %d parameters, got %d" % (self.nparam, p.size))
        check(self.lib.pl_unet_set_params(self.h, _fp(p)))

    def gradients(self):
        out = np.empty(self.nparam, np.float32)
        check(self.lib.pl_unet_gradients(self.h, _fp(out)))
        return out

    def layer_shapes(self):
        """(cout, taps, cin) of every layer in parameter order"""
        L, c = self.levels, self.base
        ch = [c << l for l in range(L)]
        out = []
        for l in range(L):
            out.append((ch[l], 27, 16 if l == 0 else ch[l - 1]))
            out.append((ch[l], 27, ch[l]))
        for l in range(L - 2, -1, -1):
            out.append((ch[l], 27, ch[l] + ch[l + 1]))
            out.append((ch[l], 27, ch[l]))
        out.append((16, 1, ch[0]))
        return out

    # raw passes (gradient checks) -----------------------------------------------------------
    def forward(self, x):
        """x [batch][voxel][16] -> y [batch][voxel][16] (FP32)"""
        x = np.ascontiguousarray(x, np.float32)
        b = x.shape[0]
        y = np.empty((b, self.nvox, 16), np.float32)
        check(self.lib.pl_unet_forward(self.h, b, _fp(x), _fp(y)))
        return y

    def backward(self, dy):
        dy = np.ascontiguousarray(dy, np.float32)
        check(self.lib.pl_unet_backward(self.h, dy.shape[0], _fp(dy)))
        return self.gradients()

    # data, training, prediction -------------------------------------------------------------
    def reserve(self, nsamples, ntarget=len(TARGETS)):
        check(self.lib.pl_unet_dataset_reserve(self.h, nsamples, ntarget))
        self.ntarget = ntarget

    def set_static(self, feat):
        feat = np.ascontiguousarray(feat, np.float32)
        check(self.lib.pl_unet_set_static(self.h, _fp(feat), feat.shape[1]))

    def add_sample_lattice(self, slot, design, lattice):
        """targets from the lattice's frozen forward and saved adjoint fields, device to device"""
        design = np.ascontiguousarray(design, np.float64)
        check(self.lib.pl_unet_add_sample_lattice(self.h, slot, design.ctypes.data_as(A.DP), lattice.h))

    def add_sample(self, slot, design, targets):
        design = np.ascontiguousarray(design, np.float64)
        targets = np.ascontiguousarray(targets, np.float64)
        check(self.lib.pl_unet_add_sample(self.h, slot, design.ctypes.data_as(A.DP), targets.ctypes.data_as(A.DP)))

    def train(self, nsamples, epochs, batch=1, lr=1e-3, seed=0):
        loss = np.zeros(epochs)
        check(self.lib.pl_unet_train(self.h, nsamples, epochs, batch, C.c_double(lr), C.c_ulonglong(seed),
                                     loss.ctypes.data_as(A.DP)))
        return loss

    def norm(self):
        m, s = np.zeros(16, np.float32), np.zeros(16, np.float32)
        check(self.lib.pl_unet_get_norm(self.h, _fp(m), _fp(s)))
        return m[:self.ntarget].copy(), s[:self.ntarget].copy()

    def set_norm(self, mean, std):
        m, s = np.zeros(16, np.float32), np.ones(16, np.float32)
        m[:len(mean)], s[:len(std)] = mean, std
        check(self.lib.pl_unet_set_norm(self.h, _fp(m), _fp(s)))

    def predict(self, design):
        design = np.ascontiguousarray(design, np.float64)
        out = np.empty((self.ntarget, self.nvox))
        check(self.lib.pl_unet_predict(self.h, design.ctypes.data_as(A.DP), out.ctypes.data_as(A.DP)))
        return out

    def save(self, path, meta=None):
        mean, std = self.norm()
        np.savez_compressed(path, params=self.get_params(), mean=mean, std=std,
                            meta=json.dumps(dict(meta or {}, shape=self.shape, levels=self.levels, base=self.base)))

    def load(self, path):
        d = np.load(path)
        if not self.ntarget:
            self.reserve(1, len(d["mean"]))
        self.set_params(d["params"])
        self.set_norm(d["mean"], d["std"])
        return json.loads(str(d["meta"]))


def static_features(p):
    """Per-voxel inputs besides the design: base-plate mask, coordinates in [-1, 1], the inflow
    profile / u_max, channel-wall and outlet flags."""
    side, inflow, outflow, _ = p.masks()
    n = p.n
    f = np.zeros((n, 7), np.float32)
    f[:, 0] = p.plate
    f[:, 1] = 2.0 * p.i / max(1, p.lx - 1) - 1.0
    f[:, 2] = 2.0 * p.j / max(1, p.ly - 1) - 1.0
    f[:, 3] = 2.0 * p.k / max(1, p.lz - 1) - 1.0
    f[:, 4] = p.inflow() / p.umax
    f[:, 5] = side
    f[:, 6] = outflow
    return f


def targets_of(res):
    """the target fields [13][nvox] of a converged design iteration (rho stored as rho - 1)"""
    fw, ad = res["fwd"], res["adj"]
    rows = [fw["rho"] - 1.0, fw["ux"], fw["uy"], fw["uz"], fw["tem"]]
    rows += [ad[k] for k in ("ip", "iux", "iuy", "iuz", "item", "iqx", "iqy", "iqz")]
    return np.stack(rows)


def seed_of(pred):
    """ForcedHeatSink seed dict from a prediction [13][nvox]"""
    d = {k: pred[m] for m, k in enumerate(TARGETS)}
    d["rho"] = pred[0] + 1.0
    return d


class SurrogateWarmStart:
    """Training-data generation, training and warm-started design iterations for one
    forced-convection heat-sink problem (panslbm2_gb300.forced)."""

    def __init__(self, p, storage="fp32", levels=4, base=16, max_batch=1):
        from .forced import ForcedHeatSink
        self.p = p
        self.hs = ForcedHeatSink(p, storage)
        self.net = UNet(p.lx, p.ly, p.lz, levels, base, max_batch)
        self.net.set_static(static_features(p))

    def close(self):
        self.hs.close()
        self.net.close()

    def generate(self, count, first_seed=1000, tol=1e-6, max_steps=100000, max_adjoint_steps=40000, log=None,
                 max_seconds=None):
        """solve seeded designs first_seed, first_seed + 1, ... to `tol` until `count` pairs whose
        forward and adjoint both converged are stored (the others are skipped and logged), or
        until max_seconds of wall time have passed; returns the per-design records (the number
        stored is the count of records with used = True)"""
        self.net.reserve(count)
        info, slot, sd = [], 0, first_seed
        start = time.perf_counter()
        while slot < count and (max_seconds is None or time.perf_counter() - start < max_seconds):
            t0 = time.perf_counter()
            s = self.p.design(seed=sd)
            ss, (stf, nf), (sta, na) = self.hs.solve_pair(s, tol, max_steps, max_adjoint_steps)
            ok = stf == A.PL_CONVERGED and sta == A.PL_CONVERGED
            if ok:
                self.net.add_sample_lattice(slot, ss, self.hs.lp)
                slot += 1
            rec = dict(seed=int(sd), forward=nf, adjoint=na, status=[int(stf), int(sta)], used=ok,
                       seconds=round(time.perf_counter() - t0, 3))
            info.append(rec)
            if log:
                log(rec)
            sd += 1
        return info

    def train(self, nsamples, epochs, batch=1, lr=1e-3, seed=0):
        return self.net.train(nsamples, epochs, batch, lr, seed)

    def iterate(self, s, warm, tol=1e-6, max_steps=100000, mode="both", adjoint_fallback=None):
        """one design iteration; warm = True seeds the solver from the network's prediction:
        mode "both" seeds the forward and the adjoint problems, "forward" the forward one only
        (the adjoint then starts from rest); adjoint_fallback: see ForcedHeatSink.iterate"""
        seed = None
        tp = 0.0
        if warm:
            t0 = time.perf_counter()
            ss = self.hs.filtered(s)
            seed = seed_of(self.net.predict(ss))
            if mode == "forward":
                from .forced import FWD_FIELDS
                seed = {k: v for k, v in seed.items() if k in FWD_FIELDS}
            tp = time.perf_counter() - t0
            r = self.hs.iterate(s, tol=tol, max_steps=max_steps, seed=seed, filtered=ss,
                                adjoint_fallback=adjoint_fallback)
        else:
            r = self.hs.iterate(s, tol=tol, max_steps=max_steps)
        r["seconds"]["predict"] = tp
        r["seconds"]["total"] += tp
        return r


def default_weights_path():
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "unet3d_forced_160x160x80.npz")


def profile_main(argv):
    """python -m panslbm2_gb300.surrogate profile [--shape X,Y,Z] [--iters K]: K forward + backward
    + Adam passes of the U-Net on random inputs (a fixed kernel sequence for ncu captures)"""
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--shape", default="160,160,80")
    ap.add_argument("--iters", type=int, default=3)
    ap.add_argument("--levels", type=int, default=4)
    ap.add_argument("--base", type=int, default=16)
    a = ap.parse_args(argv)
    nx, ny, nz = (int(v) for v in a.shape.split(","))
    net = UNet(nx, ny, nz, a.levels, a.base, 1)
    rng = np.random.default_rng(0)
    net.reserve(1, len(TARGETS))
    net.set_static(rng.random((nx * ny * nz, 7)).astype(np.float32))
    net.add_sample(0, rng.random(nx * ny * nz), 0.01 * rng.standard_normal((len(TARGETS), nx * ny * nz)))
    t0 = time.perf_counter()
    loss = net.train(1, a.iters, 1, 1e-3, seed=0)
    print(json.dumps(dict(shape=[nx, ny, nz], iters=a.iters, seconds=round(time.perf_counter() - t0, 4),
                          loss=[float(v) for v in loss])))
    net.close()


def main(argv=None):
    """python -m panslbm2_gb300.surrogate --nsamples N --epochs E --out weights.npz [--log log.json]

    Generates N training pairs from the seeded designs 1000 .. 1000 + N - 1 on the
    forced-convection heat sink (default 160 x 160 x 80, FP32), trains the U-Net, saves the
    weights and the normalisation, and compares a cold and a warm-started design iteration on
    the held-out design of seed 0."""
    import argparse
    from .forced import ForcedParams
    ap = argparse.ArgumentParser()
    ap.add_argument("--shape", default="160,160,80")
    ap.add_argument("--nsamples", type=int, default=512)
    ap.add_argument("--first-seed", type=int, default=1000)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--batch", type=int, default=1)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--tol", type=float, default=1e-6)
    ap.add_argument("--data-tol", type=float, default=None, help="residual tolerance of the training solves")
    ap.add_argument("--levels", type=int, default=4)
    ap.add_argument("--base", type=int, default=16)
    ap.add_argument("--out", required=True)
    ap.add_argument("--log", default=None)
    ap.add_argument("--eval-seeds", default="0,1,2,3,4",
                    help="held-out designs of the cold / warm-started comparison")
    ap.add_argument("--max-generate-s", type=float, default=None,
                    help="stop generating after this many seconds and train on the pairs stored")
    ap.add_argument("--max-adjoint-steps", type=int, default=25000,
                    help="training designs whose adjoint does not converge within this are skipped")
    a = ap.parse_args(argv)
    nx, ny, nz = (int(v) for v in a.shape.split(","))
    p = ForcedParams(3, nx, ny, nz)
    sw = SurrogateWarmStart(p, "fp32", a.levels, a.base, a.batch)
    rec = dict(shape=[nx, ny, nz], nsamples=a.nsamples, epochs=a.epochs, batch=a.batch, lr=a.lr,
               first_seed=a.first_seed, params=sw.net.nparam)
    log = []

    def out(d):
        print(json.dumps(d), flush=True)

    t0 = time.perf_counter()
    rec["samples"] = sw.generate(a.nsamples, a.first_seed, tol=a.data_tol or a.tol,
                                 max_adjoint_steps=a.max_adjoint_steps,
                                 log=lambda d: (log.append(d), out(dict(sample=d))),
                                 max_seconds=a.max_generate_s)
    rec["generate_s"] = round(time.perf_counter() - t0, 2)
    used = [d["seed"] for d in rec["samples"] if d["used"]]
    nstored = len(used)
    if nstored == 0:
        raise SystemExit("no training design converged")
    rec["nsamples"] = nstored
    rec["seeds"] = [min(used), max(used)]
    rec["skipped_seeds"] = [d["seed"] for d in rec["samples"] if not d["used"]]
    t1 = time.perf_counter()
    loss = sw.train(nstored, a.epochs, a.batch, a.lr, seed=7)
    sw.hs.lp.synchronize()
    rec["train_s"] = round(time.perf_counter() - t1, 2)
    rec["loss"] = [float(v) for v in loss]
    out(dict(loss=rec["loss"], train_s=rec["train_s"], nsamples=nstored))
    sw.net.save(a.out, meta=dict(nsamples=nstored, epochs=a.epochs, seeds=rec["seeds"],
                                 skipped=rec["skipped_seeds"], data_tol=a.data_tol or a.tol))
    ev = []
    for sd in (int(v) for v in a.eval_seeds.split(",")):
        s = p.design(seed=sd)
        row = dict(seed=sd)
        for name, warm in (("plain", False), ("surrogate", True)):
            r = sw.iterate(s, warm, tol=a.tol)
            row[name] = dict(seconds=round(r["seconds"]["total"], 3),
                             phases={k: round(v, 3) for k, v in r["seconds"].items()},
                             forward_steps=r["forward"][1], adjoint_steps=r["adjoint"][1],
                             converged=[r["forward"][0] == A.PL_CONVERGED, r["adjoint"][0] == A.PL_CONVERGED],
                             objective=r["objective"])
        out(dict(eval=row))
        ev.append(row)
    rec["eval"] = ev
    if a.log:
        with open(a.log, "w") as fh:
            json.dump(rec, fh, indent=1)
    sw.close()


if __name__ == "__main__":
    import sys
    if len(sys.argv) > 1 and sys.argv[1] == "profile":
        profile_main(sys.argv[2:])
    else:
        main()
