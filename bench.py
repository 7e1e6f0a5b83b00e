"""Throughput of the fused NS+AD lattice-Boltzmann step on GB300 (one JSON line on rank 0), and
the benchmark configurations around it.

Workload (default): the 3D steady forced-convection heat sink, coupled D3Q15 NS + D3Q15
advection-diffusion, 160x160x80 lattice (2,048,000 nodes), FP32 populations and compute:
Brinkman + forced-convection collide (AD::MacroBrinkmanCollideForceConvection) with the
volumetric heat source of a 40x4x40 base plate, the boundary program of parabolic inflow,
pressure outlet with zero temperature gradient, walls and corner smoothing every step; design
from a seeded Gaussian random field (correlation length 8 cells). A bench "step" is one fused time
step over the whole lattice: pull-stream + boundary program + collide. The population buffers
(2 x 245 MB) exceed the 129 MB L2, so no flush is needed between steps.

  value          MLUPS of the device-resident fused step (sum over ranks; replicas)
  e2e            MLUPS through the C ABI with host buffers: per e2e step, upload alpha / kappa
                 from pinned host memory, run one residual-check interval of 100 time steps
                 (pl_solve), download T and u
  roofline       HBM: algorithmic bytes per node per step (read + write 2 x 15 FP32 populations,
                 read alpha, kappa and the heat source) / measured step time, vs MEASURED_PEAKS
  cpu_baseline   the C restatement of the reference's scalar OpenMP path (oracle/), FP64, on the
                 host cores: one warm-up step, then the median of 5 timed spans
  cavity_100x100 the 100x100 lid-driven cavity, 20,000 steps, FP64, GPU and the CPU port timed,
                 and their largest difference
  design_iter    one design iteration of the 200x100 FP64 forced-convection heat sink (filter,
                 forward and adjoint to residual 1e-6, sensitivity, filtered sensitivity) on the
                 GPU, and the CPU port's forward + adjoint on the same step counts (timed within a
                 budget, extrapolated beyond it and labelled so)
  design_iter_3d_surrogate  the 160x160x80 FP32 design iteration, plain (from rest) and with the
                 learned warm start (trained weights in panslbm2_gb300/weights/), to the same
                 residual tolerance
  precision_errors  objective and sensitivity errors of FP32, FP16 and BF16 storage against FP64 on
                 the 1600x800 forced-convection heat sink
  transient_iter seconds of one transient forced-convection heat-sink evaluation with the
                 time-varying inflow (4000 time steps forward and adjoint, checkpoints every 100
                 steps) on the 192x192x96 FP32 lattice

--impl reference times that CPU path alone: the reference's own implementation of the path is
header-only C++ whose sources are not present on the GPU host, so the restatement stands in.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "forced3d-160x160x80-fp32": dict(phys="forced", nd=3, lx=160, ly=160, lz=80, storage="fp32"),
    "forced3d-192x192x96-fp32": dict(phys="forced", nd=3, lx=192, ly=192, lz=96, storage="fp32"),
    "forced3d-160x160x80-fp16": dict(phys="forced", nd=3, lx=160, ly=160, lz=80, storage="fp16"),
    "forced3d-160x160x80-bf16": dict(phys="forced", nd=3, lx=160, ly=160, lz=80, storage="bf16"),
    "forced2d-1600x800-fp64": dict(phys="forced", nd=2, lx=1600, ly=800, lz=1, storage="fp64"),
    "forced2d-1600x800-fp32": dict(phys="forced", nd=2, lx=1600, ly=800, lz=1, storage="fp32"),
    "forced2d-1600x800-fp16": dict(phys="forced", nd=2, lx=1600, ly=800, lz=1, storage="fp16"),
    "forced2d-1600x800-bf16": dict(phys="forced", nd=2, lx=1600, ly=800, lz=1, storage="bf16"),
    "heatsink3d-160x160x80-fp32": dict(phys="natural", nd=3, lx=160, ly=160, lz=80, storage="fp32"),
    "heatsink3d-192x192x96-fp32": dict(phys="natural", nd=3, lx=192, ly=192, lz=96, storage="fp32"),
    "heatsink3d-160x160x80-fp16": dict(phys="natural", nd=3, lx=160, ly=160, lz=80, storage="fp16"),
    "heatsink3d-160x160x80-bf16": dict(phys="natural", nd=3, lx=160, ly=160, lz=80, storage="bf16"),
    "heatsink2d-1600x800-fp32": dict(phys="natural", nd=2, lx=1600, ly=800, lz=1, storage="fp32"),
    "heatsink2d-1600x800-fp64": dict(phys="natural", nd=2, lx=1600, ly=800, lz=1, storage="fp64"),
}
DEFAULT = "forced3d-160x160x80-fp32"
METRIC = "fused NS+AD MLUPS"


class Setup:
    """the step workload: kind, physics constants, design fields, boundary program"""

    def __init__(self, wl, seed=0):
        from panslbm2_gb300 import _capi as A
        from panslbm2_gb300 import heatsink as HS
        from panslbm2_gb300 import forced as FC
        nd, lx, ly, lz = wl["nd"], wl["lx"], wl["ly"], wl["lz"]
        self.nd, self.lx, self.ly, self.lz = nd, lx, ly, lz
        self.q = 9 if nd == 2 else 15
        self.n = lx * ly * lz
        self.storage = wl["storage"]
        ss = HS.grf_design(nd, lx, ly, lz, seed=seed, sigma=8.0)
        if wl["phys"] == "forced":
            p = FC.ForcedParams(nd, lx, ly, lz)
            ss = p.project(ss)
            alpha, kappa, _, _ = p.design_fields(ss)
            self.fields = {A.ALPHA: alpha, A.KAPPA: kappa, A.HEAT_SOURCE: p.heat_source(ss)[0]}
            self.ops = p.program_ops("forward")
            self.kind = A.AD_FORCE
            self.phys = dict(nu=p.nu, diff=0.0, gx=0.0, gy=0.0, gz=0.0, tem0=0.0)
            self.oracle_fields = dict(alpha=alpha, diffusivity=kappa, hsrc=self.fields[A.HEAT_SOURCE])
            self.nfield = 3
        else:
            p = HS.Params(nd, lx, ly, lz)
            alpha, kappa, _, _ = p.design_fields(ss)
            self.fields = {A.ALPHA: alpha, A.KAPPA: kappa}
            self.ops = HS.program_ops("forward", p)
            self.kind = A.AD_NATURAL
            self.phys = dict(nu=p.nu, diff=0.0, gx=p.gx, gy=p.gy, gz=p.gz, tem0=p.tem0)
            self.oracle_fields = dict(alpha=alpha, diffusivity=kappa)
            self.nfield = 2
        self.p = p

    def bytes_per_node(self):
        s = {"fp64": 8, "fp32": 4, "fp16": 2, "bf16": 2}[self.storage]
        c = 8 if self.storage == "fp64" else 4
        return 2 * 2 * self.q * s + self.nfield * c


class Clocks:
    """nvidia-smi sampling of SM clock and throttle reasons during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, dev):
        self.dev, self.rows, self.proc = dev, [], None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm = [float(r[0]) for r in self.rows if len(r) >= 7 and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) >= 7 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows if len(r) >= 7 for i in range(4) if r[3 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(sm)}


def replica_throughput(ms_local, nodes, steps, world, dist=None, device="cuda"):
    """Whole-job throughput of `world` independent replicas (one per rank, each `nodes` nodes and
    `steps` steps): the time is the maximum over ranks, the node updates are summed. Returns
    (max ms, MLUPS)."""
    tmax = float(ms_local)
    if dist is not None and world > 1:
        import torch
        t = torch.tensor([tmax], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        tmax = float(t.item())
    return tmax, world * nodes * steps / (tmax / 1e3) / 1e6


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_per_node(workload):
    """DRAM bytes per node of the fused step from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "step_traffic.txt")
    try:
        with open(path) as fh:
            for line in fh:
                parts = line.split()
                if len(parts) == 2 and parts[0] == workload:
                    return float(parts[1])
    except OSError:
        pass
    return None


def host_info():
    return {"nproc": os.cpu_count(), "omp_proc_bind": os.environ.get("OMP_PROC_BIND", "close"),
            "machine": os.uname().machine}


def cpu_port(S, spans=5, steps_per_span=None, budget_s=12.0):
    """The oracle restatement of the reference's scalar OpenMP path (FP64) on the host: one
    warm-up step, then the median of `spans` timed spans of the same workload."""
    os.environ.setdefault("OMP_PROC_BIND", "close")
    from oracle.olib import Oracle
    from panslbm2_gb300 import _capi as A
    from tests._replay import replay
    o = Oracle("oracle")
    cores = os.cpu_count() or 1
    o.set_threads(cores)
    q, n = S.q, S.n
    L = o.lat(q, S.lx, S.ly, S.lz)
    f, g = np.zeros((q, n)), np.zeros((q, n))
    one, zero = np.ones(n), np.zeros(n)
    o.init(L, 0, f, o.fields(rho=one, ux=zero, uy=zero, uz=zero))
    o.init(L, 1, g, o.fields(tem=zero, ux=zero, uy=zero, uz=zero))
    mac = {k: np.zeros(n) for k in ("rho", "ux", "uy", "uz", "tem", "qx", "qy", "qz")}
    F = o.fields(**S.oracle_fields, **mac)
    kappa = S.oracle_fields["diffusivity"]

    def one_step():
        o.collide(L, S.kind, f, g, F, **S.phys, save=True)
        o.stream(L, f)
        o.stream(L, g)
        replay(o, L, f, g, S.ops, n, ux=mac["ux"], uy=mac["uy"], uz=mac["uz"], kappa=kappa)

    t0 = time.perf_counter()
    one_step()   # warm-up
    t1 = time.perf_counter() - t0
    if steps_per_span is None:
        steps_per_span = max(1, min(30, int(budget_s / spans / max(t1, 1e-6))))
    rates = []
    for _ in range(spans):
        t0 = time.perf_counter()
        for _ in range(steps_per_span):
            one_step()
        rates.append(n * steps_per_span / (time.perf_counter() - t0) / 1e6)
    return {"value": float(np.median(rates)), "unit": "MLUPS", "cores": cores, "kind": "port",
            "spans_mlups": [round(r, 2) for r in rates], "method": "1 warm-up step, median of %d spans" % spans,
            "host": host_info(),
            "sample": "%d spans of %d full time steps (collide + 2 streams + boundary program) of the %dx%dx%d "
                      "lattice, FP64" % (spans, steps_per_span, S.lx, S.ly, S.lz)}


def cavity_leg():
    """the 100x100 lid-driven cavity, 20,000 steps, FP64: GPU and CPU port"""
    from oracle.olib import Oracle
    from panslbm2_gb300 import forced as FC
    from tests import _forced_oracle as FO
    FC.run_cavity(100, 100, 200)   # warm-up
    rho, ux, uy, sec = FC.run_cavity(100, 100, 20000, storage="fp64")
    o = Oracle("oracle")
    o.set_threads(os.cpu_count() or 1)
    t0 = time.perf_counter()
    mac = FO.cavity(o, 100, 100, 20000)
    cpu = time.perf_counter() - t0
    diff = max(float(np.max(np.abs(a - mac[k])) / np.max(np.abs(mac[k]))) for a, k in ((rho, "rho"), (ux, "ux"),
                                                                                        (uy, "uy")))
    return {"lattice": "cavity2d-100x100-fp64", "steps": 20000, "gpu_seconds": round(sec, 4),
            "gpu_mlups": round(1e4 * 2e4 / sec / 1e6, 1), "cpu_seconds": round(cpu, 3),
            "cpu_kind": "port, FP64, %d host threads" % (os.cpu_count() or 1),
            "max_rel_diff_gpu_vs_cpu": diff}


def design_leg(cpu=True, cpu_budget_s=120.0):
    """one forced-convection design iteration on 200x100 FP64 (filter, forward and
    adjoint to 1e-6, sensitivity, filtered sensitivity); the CPU port's forward + adjoint on the
    same step counts"""
    from panslbm2_gb300 import _capi as A
    from panslbm2_gb300 import forced as FC
    p = FC.ForcedParams(2, 200, 100)
    s = p.design(seed=0)
    hs = FC.ForcedHeatSink(p, "fp64")
    hs.iterate(s, max_steps=1000)            # warm-up: filter taps, programs
    # the 20,000-node lattice is launch-bound: time eager launches and the CUDA-graph replay of
    # the steps between residual checks, report the faster
    runs = {}
    for graphs in (0, 1):
        hs.lp.set_option(A.OPT_GRAPHS, graphs)
        hs.iterate(s, max_steps=1000)
        runs[graphs] = hs.iterate(s, tol=1e-6, max_steps=100000)
    hs.close()
    best = min(runs, key=lambda k: runs[k]["seconds"]["total"])
    r = runs[best]
    out = {"lattice": "forced2d-200x100-fp64", "tol": 1e-6, "max_steps": 100000,
           "launch": "cuda graphs" if best else "eager",
           "seconds_eager": round(runs[0]["seconds"]["total"], 4), "seconds_graphs": round(runs[1]["seconds"]["total"], 4),
           "seconds": round(r["seconds"]["total"], 4), "phases_s": {k: round(v, 4) for k, v in r["seconds"].items()},
           "forward_steps": r["forward"][1], "adjoint_steps": r["adjoint"][1],
           "converged": [r["forward"][0] == A.PL_CONVERGED, r["adjoint"][0] == A.PL_CONVERGED],
           "objective": r["objective"],
           "what": "filter, forward and adjoint to residual 1e-6 (checked every 100 steps), sensitivity, filtered "
                   "sensitivity; from rest; no MMA update"}
    if cpu:
        out.update(design_cpu(p, r["ss"], r["forward"][1], r["adjoint"][1], cpu_budget_s))
    return out


def design_cpu(p, ss, nf, na, budget_s):
    """the oracle port's forward and adjoint steps of the design iteration (FP64, all host
    threads), timed up to `budget_s`; beyond it the measured rate is extrapolated"""
    from oracle.olib import Oracle
    from panslbm2_gb300 import _capi as A
    from tests._replay import replay
    o = Oracle("oracle")
    o.set_threads(os.cpu_count() or 1)
    q, n = 9, p.n
    L = o.lat(q, p.lx, p.ly)
    alpha, kappa, _, _ = p.design_fields(ss)
    Q = p.heat_source(ss)[0]
    w = p.objective_weight(ss)
    f, g = np.zeros((q, n)), np.zeros((q, n))
    zero = np.zeros(n)
    o.init(L, 0, f, o.fields(rho=np.ones(n), ux=zero, uy=zero, uz=zero))
    o.init(L, 1, g, o.fields(tem=zero, ux=zero, uy=zero, uz=zero))
    mac = {k: np.zeros(n) for k in ("rho", "ux", "uy", "uz", "tem", "qx", "qy", "qz")}
    ops_f, ops_a = p.program_ops("forward"), p.program_ops("adjoint")
    F = o.fields(alpha=alpha, diffusivity=kappa, hsrc=Q, **mac)
    t0 = time.perf_counter()
    done_f = 0
    while done_f < nf and time.perf_counter() - t0 < budget_s / 2:
        if done_f:
            o.stream(L, f)
            o.stream(L, g)
            replay(o, L, f, g, ops_f, n, ux=mac["ux"], uy=mac["uy"], uz=mac["uz"], kappa=kappa)
        o.collide(L, A.AD_FORCE, f, g, F, nu=p.nu, save=True)
        done_f += 1
    tf = time.perf_counter() - t0
    adj = {k: np.zeros(n) for k in ("ip", "iux", "iuy", "iuz", "imx", "imy", "imz", "item", "iqx", "iqy", "iqz")}
    Fa = o.fields(alpha=alpha, diffusivity=kappa, objw=w, **mac, **adj)
    o.init(L, 2, f, o.fields(ux=mac["ux"], uy=mac["uy"], uz=mac["uz"], ip=zero, iux=zero, iuy=zero, iuz=zero))
    o.init(L, 3, g, o.fields(ux=mac["ux"], uy=mac["uy"], uz=mac["uz"], item=zero, iqx=zero, iqy=zero, iqz=zero))
    t1 = time.perf_counter()
    done_a = 0
    while done_a < na and time.perf_counter() - t1 < budget_s / 2:
        if done_a:
            o.stream(L, f, True)
            o.stream(L, g, True)
            replay(o, L, f, g, ops_a, n, ux=mac["ux"], uy=mac["uy"], uz=mac["uz"], rho=mac["rho"], tem=mac["tem"],
                   kappa=kappa)
        o.collide(L, A.AAD_FORCE, f, g, Fa, nu=p.nu, save=True)
        done_a += 1
    ta = time.perf_counter() - t1
    est = tf * nf / done_f + ta * na / done_a
    full = done_f == nf and done_a == na
    return {"cpu_seconds": round(est, 2), "cpu_timed_fully": full,
            "cpu_sample": "oracle port, FP64, %d host threads: %d of %d forward and %d of %d adjoint steps timed%s" % (
                os.cpu_count() or 1, done_f, nf, done_a, na, "" if full else ", the rest extrapolated at the measured "
                                                                             "rate")}


def surrogate_leg(tol=1e-5, seeds=(0, 1, 2, 3, 4), max_steps=40000, fallback=20000):
    """plain vs learned warm start on the 160x160x80 FP32 forced heat sink, held-out designs (seeds 0-4; the
    training designs are seeds 1000 and up). Warm starts: "both" seeds the forward and the
    adjoint problems (a seeded adjoint not converged after `fallback` steps restarts from rest),
    "forward" seeds the forward problem only."""
    from panslbm2_gb300 import _capi as A
    from panslbm2_gb300 import forced as FC
    from panslbm2_gb300.surrogate import SurrogateWarmStart, default_weights_path
    path = default_weights_path()
    if not os.path.exists(path):
        return {"error": "no trained weights at %s" % os.path.relpath(path, ROOT)}
    p = FC.ForcedParams(3, 160, 160, 80)
    sw = SurrogateWarmStart(p, "fp32")
    meta = sw.net.load(path)
    sw.iterate(p.design(seed=seeds[0]), True, tol=1e-2, max_steps=300)    # warm-up: programs, taps, kernels
    out = {"lattice": "forced3d-160x160x80-fp32", "tol": tol, "max_steps": max_steps, "fallback_steps": fallback,
           "design_seeds": list(seeds),
           "training": {k: meta.get(k) for k in ("nsamples", "epochs", "seeds", "data_tol")}, "designs": []}
    modes = (("plain", False, None), ("warm_both", True, "both"), ("warm_forward", True, "forward"))
    tot = {m[0]: [0.0, 0] for m in modes}
    for sd in seeds:
        s = p.design(seed=sd)
        row = {"seed": sd}
        for name, warm, mode in modes:
            r = sw.iterate(s, warm, tol=tol, max_steps=max_steps, mode=mode or "both",
                           adjoint_fallback=fallback if mode == "both" else None)
            row[name] = {"seconds": round(r["seconds"]["total"], 3),
                         "forward_steps": r["forward"][1], "adjoint_steps": r["adjoint"][1],
                         "converged": [r["forward"][0] == A.PL_CONVERGED, r["adjoint"][0] == A.PL_CONVERGED],
                         "adjoint_restarted": r["adjoint_restarted"], "objective": r["objective"]}
        row["counted"] = all(all(row[m[0]]["converged"]) for m in modes)
        if row["counted"]:
            for name in tot:
                tot[name][0] += row[name]["seconds"]
                tot[name][1] += row[name]["forward_steps"] + row[name]["adjoint_steps"]
            row["objective_rel_diff"] = {m: abs(row[m]["objective"] - row["plain"]["objective"]) /
                                         abs(row["plain"]["objective"]) for m in ("warm_both", "warm_forward")}
        out["designs"].append(row)
    sw.close()
    out["counted_designs"] = sum(1 for r in out["designs"] if r["counted"])
    if tot["plain"][0] > 0:
        for m in ("warm_both", "warm_forward"):
            out["speedup_" + m] = round(tot["plain"][0] / tot[m][0], 3)
            out["step_ratio_" + m] = round(tot["plain"][1] / tot[m][1], 3)
    out["what"] = ("design iteration (filter, forward, adjoint, sensitivity) from rest vs from the U-Net's predicted "
                   "fields, all to the same residual tolerance; speedups over the designs where every run converged "
                   "(some designs' adjoint residual levels off near 5e-4 from any start and never converges); FP32 "
                   "residuals on this lattice level off near 4e-6, so the comparison is at 1e-5")
    return out


def precision_leg(nf=4000, na=4000):
    """FP32 / FP16 / BF16 storage against FP64 on the 1600x800 forced heat sink"""
    from panslbm2_gb300 import forced as FC
    p = FC.ForcedParams(2, 1600, 800)
    s = p.design(seed=0)
    res = {}
    for st in ("fp64", "fp32", "fp16", "bf16", "fp16_sr", "bf16_sr"):
        hs = FC.ForcedHeatSink(p, st.split("_")[0], stochastic_rounding=st.endswith("_sr"))
        t0 = time.perf_counter()
        res[st] = hs.iterate(s, fixed_steps=(nf, na))
        res[st]["sec"] = time.perf_counter() - t0
        hs.close()
    b = res["fp64"]
    out = {"lattice": "forced2d-1600x800", "forward_steps": nf, "adjoint_steps": na, "design_seed": 0,
           "fp64_objective": b["objective"]}
    out["note"] = "fp16_sr / bf16_sr: 16-bit storage with stochastic rounding of the collide's stores"
    for st in ("fp32", "fp16", "bf16", "fp16_sr", "bf16_sr"):
        r = res[st]
        out[st] = {"objective_rel_err": abs(r["objective"] - b["objective"]) / abs(b["objective"]),
                   "sensitivity_rel_err_max": float(np.max(np.abs(r["dJdss"] - b["dJdss"])) / np.max(np.abs(b["dJdss"]))),
                   "sensitivity_rel_err_l2": float(np.linalg.norm(r["dJdss"] - b["dJdss"]) / np.linalg.norm(b["dJdss"])),
                   "seconds": round(r["sec"], 3)}
    out["fp64_seconds"] = round(b["sec"], 3)
    return out


def dropin_leg(steps=1000, short=200):
    """The drop-in: a heat-sink driver written against the reference's template API
    (tests/dropin/heatsink_driver.cpp, the calls of production/heatsink3D.cpp's forward loop in
    the same order, saving every step, residual check every 100 steps) built on dropin/src, on
    the 160x160x80 lattice with FP32 storage; its loop time against pl_step's on the same
    workload. Until the loop's first residual check the outputs are written back every step;
    the per-step rate is the difference of a long and a short run, both past that point."""
    import shutil
    import struct
    import tempfile
    from panslbm2_gb300 import heatsink as HS
    cxx = shutil.which("g++")
    if cxx is None:
        return {"error": "g++ not found"}
    tmp = tempfile.mkdtemp(prefix="dropin_")
    exe = os.path.join(tmp, "heatsink_driver")
    lib = os.path.join(ROOT, "panslbm2_gb300")
    subprocess.check_call([cxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "dropin", "heatsink_driver.cpp"), "-L", lib, "-lpanslbm_gb300",
                           "-Wl,-rpath," + lib, "-o", exe])
    p = HS.Params(3, 160, 160, 80)
    n = p.lx * p.ly * p.lz
    ss = HS.grf_design(3, 160, 160, 80, seed=0, sigma=8.0)
    alpha, kappa, dads, dkds = p.design_fields(ss)
    zero, one = np.zeros(n), np.ones(n)
    fields = [alpha, kappa, dads, dkds, one, zero, zero, zero, zero] + [zero] * 8
    fin, fout = os.path.join(tmp, "in.bin"), os.path.join(tmp, "out.bin")
    res = {}
    for nsteps in (short, steps):
        with open(fin, "wb") as fh:
            fh.write(struct.pack("6i", 3, p.lx, p.ly, p.lz, nsteps, 1))
            fh.write(struct.pack("7d", p.nu, p.gx, p.gy, p.gz, p.tem0, p.qn, p.L))
            for v in fields:
                fh.write(np.ascontiguousarray(v, np.float64).tobytes())
        env = dict(os.environ, PANSLBM2_GPU_STORAGE="fp32")
        r = subprocess.run([exe, "fwd", fin, fout], capture_output=True, text=True, env=env, check=True)
        for line in r.stderr.splitlines():
            if line.startswith("loop_seconds"):
                res[nsteps] = float(line.split()[1])
    shutil.rmtree(tmp, ignore_errors=True)
    # the per-step rate from the difference of a long and a short run (start-up excluded)
    per_step = (res[steps] - res[short]) / (steps - short)
    # pl_step on the same workload with the same every-step saves, for the ratio
    from panslbm2_gb300 import _capi as A
    from panslbm2_gb300.lattice import LatticePair, phys
    S = Setup(WORKLOADS["heatsink3d-160x160x80-fp32"])
    lp = LatticePair(S.q, S.lx, S.ly, S.lz, S.storage)
    for fid, v in S.fields.items():
        lp.set_field(fid, v)
    lp.init(0, one, ux=zero, uy=zero, uz=zero)
    lp.init(1, zero, ux=zero, uy=zero, uz=zero)
    prog = lp.program(HS.to_descs(S.ops))
    ph = phys(**S.phys)
    lp.collide(S.kind, ph)
    for _ in range(20):
        lp.step(S.kind, ph, prog, save=True)
    lp.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        lp.step(S.kind, ph, prog, save=True)
    lp.synchronize()
    api = (time.perf_counter() - t0) / steps
    lp.close()
    return {"lattice": "heatsink3d-160x160x80-fp32 (storage fp32, host arrays float64)", "steps": steps,
            "loop_seconds": round(res[steps], 4), "ms_per_step": round(per_step * 1e3, 4),
            "mlups": round(n / per_step / 1e6, 1), "pl_step_saving_ms": round(api * 1e3, 4),
            "ratio_to_pl_step": round(per_step / api, 3),
            "what": "forward loop of a driver on the template API, collide with saves every step + 2 streams + "
                    "boundary calls + smoothing + residual every 100 steps; after the first residual the outputs "
                    "stay on the device until the next phase boundary"}


def fp64_leg(steps=200):
    """FP64 step on the 1600x800 forced heat sink against both of its ceilings: HBM (312
    algorithmic bytes per node) and the FP64 FMA rate probed on this device; the FP64 operations
    per node come from the committed ncu instruction counts (profiles/fp64_step_ops.txt)"""
    import ctypes as C
    import torch
    from panslbm2_gb300 import _capi as A
    from panslbm2_gb300 import heatsink as HS
    from panslbm2_gb300.lattice import LatticePair, phys
    S = Setup(WORKLOADS["forced2d-1600x800-fp64"])
    lp = LatticePair(S.q, S.lx, S.ly, S.lz, S.storage)
    for fid, v in S.fields.items():
        lp.set_field(fid, v)
    lp.init(0, np.ones(S.n), ux=np.zeros(S.n), uy=np.zeros(S.n), uz=np.zeros(S.n))
    lp.init(1, np.zeros(S.n), ux=np.zeros(S.n), uy=np.zeros(S.n), uz=np.zeros(S.n))
    prog = lp.program(HS.to_descs(S.ops))
    ph = phys(**S.phys)
    lp.collide(S.kind, ph)
    lp.steps(S.kind, ph, prog, 20)
    lp.synchronize()
    t0 = time.perf_counter()
    lp.steps(S.kind, ph, prog, steps)
    lp.synchronize()
    ms = (time.perf_counter() - t0) / steps * 1e3
    lp.close()
    tf = C.c_double()
    A.check(A.load().pl_probe_fp64_fma(C.byref(tf)))
    peak, _ = peaks()
    bpn = S.bytes_per_node()
    out = {"lattice": "forced2d-1600x800-fp64", "ms_per_step": round(ms, 4), "bytes_per_node": bpn,
           "hbm_frac": round(S.n * bpn / (ms / 1e3) / 1e9 / peak, 4), "fp64_fma_tflops_probe": round(tf.value, 3)}
    ops, instr = None, None
    try:
        with open(os.path.join(ROOT, "profiles", "fp64_step_ops.txt")) as fh:
            for line in fh:
                k, _, v = line.partition(" ")
                if k == "flops_per_node":
                    ops = float(v)
                elif k == "dp_instr_per_node":
                    instr = float(v)
    except OSError:
        pass
    if ops:
        out["fp64_flops_per_node"] = ops
        out["fp64_frac"] = round(S.n * ops / (ms / 1e3) / 1e12 / tf.value, 4)
    if instr:
        # every DADD, DMUL and DFMA takes one FP64 pipe slot; the probe's FMA rate / 2 is the
        # pipe's instruction rate
        out["fp64_dp_instr_per_node"] = instr
        out["fp64_pipe_frac"] = round(S.n * instr / (ms / 1e3) / (tf.value * 1e12 / 2), 4)
        out["bound"] = "fp64 pipe" if out["fp64_pipe_frac"] > out["hbm_frac"] else "hbm"
    return out


TRANSIENT_LATTICE = dict(nd=3, lx=192, ly=192, lz=96, storage="fp32", levels=4000, every=100)


def transient_gpu():
    """One transient evaluation of the forced-convection heat sink (base-plate
    source, inflow u(t) = 0.02 (1 - exp(-t / 500))): forward from rest over 4000 time levels, the
    adjoint swept back with its sensitivity terms per step, checkpoints every 100 steps recomputed
    on the device, on the 192x192x96 FP32 lattice, through panslbm2_gb300.transient."""
    from panslbm2_gb300 import forced as FC
    from panslbm2_gb300.transient import TransientHeatSink
    d = TRANSIENT_LATTICE
    p = FC.ForcedParams(d["nd"], d["lx"], d["ly"], d["lz"])
    ss = p.project(p.design(seed=0))
    tr = TransientHeatSink(p, d["storage"], checkpoint_every=d["every"], tau_in=500.0)
    tr.evaluate_design(ss, 2 * d["every"] + 2, release=False)   # warm-up: programs, step slots
    t0 = time.perf_counter()
    r = tr.evaluate_design(ss, d["levels"])
    sec = time.perf_counter() - t0
    tr.close()
    n = p.lx * p.ly * p.lz
    return {"lattice": "forced3d-192x192x96-fp32", "time_levels": d["levels"], "checkpoint_every": d["every"],
            "inflow": "u(t) = 0.02 (1 - exp(-t / 500))", "segments": r["segments"], "seconds": round(sec, 3),
            "phases_s": {k: round(v, 3) for k, v in r["times"].items()},
            "forward_mlups": round(n * (d["levels"] - 1) / r["times"]["forward"] / 1e6, 1),
            "objective": r["objective"],
            "what": "forward from rest, adjoint swept back with the Brinkman and diffusivity sensitivity terms per "
                    "time step, forward states recomputed from device checkpoints; no filter or MMA"}


def transient_precision(levels=400, every=50):
    """The transient heat-sink lattice (192x192x96, forced physics, u(t)) over the first
    `levels` time levels, FP32 against FP64: objective and sensitivity errors of the transient
    sweep at full lattice size (the full 4000 levels in FP64 would take minutes)."""
    from panslbm2_gb300 import forced as FC
    from panslbm2_gb300.transient import TransientHeatSink
    d = TRANSIENT_LATTICE
    p = FC.ForcedParams(d["nd"], d["lx"], d["ly"], d["lz"])
    ss = p.project(p.design(seed=0))
    res = {}
    for st in ("fp64", "fp32"):
        tr = TransientHeatSink(p, st, checkpoint_every=every, tau_in=500.0)
        t0 = time.perf_counter()
        res[st] = tr.evaluate_design(ss, levels)
        res[st]["sec"] = time.perf_counter() - t0
        tr.close()
    a, b = res["fp32"], res["fp64"]
    return {"lattice": "forced3d-192x192x96", "time_levels": levels, "checkpoint_every": every,
            "fp64_objective": b["objective"], "fp64_seconds": round(b["sec"], 3), "fp32_seconds": round(a["sec"], 3),
            "objective_rel_err": abs(a["objective"] - b["objective"]) / abs(b["objective"]),
            "sensitivity_rel_err_l2": float(np.linalg.norm(a["dfdss"] - b["dfdss"]) / np.linalg.norm(b["dfdss"])),
            "sensitivity_rel_err_max": float(np.max(np.abs(a["dfdss"] - b["dfdss"])) / np.max(np.abs(b["dfdss"])))}


def run_reference(args, wl):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    S = Setup(wl)
    cb = cpu_port(S, spans=5, budget_s=30.0)
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": "MLUPS", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded GRF design)",
            "config": {"workload": args.workload, "nodes": S.n, "backend": "cpu"},
            "cpu_baseline": cb, "e2e": {"value": cb["value"], "unit": "MLUPS", "h2d_bytes_per_step": 0,
                                        "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def leg(line, name, fn, *a, **k):
    try:
        line[name] = fn(*a, **k)
    except Exception as e:   # reported, not fatal: the step throughput stands on its own
        line[name] = {"error": ("%s: %s" % (type(e).__name__, e))[:300]}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=50)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT, choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline legs")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--no-design", action="store_true", help="skip the configuration legs (cavity, design, "
                                                             "surrogate, precision)")
    ap.add_argument("--no-transient", action="store_true", help="skip the transient-evaluation timing")
    args = ap.parse_args()
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        return run_reference(args, wl)

    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from panslbm2_gb300 import _capi as A
    from panslbm2_gb300 import heatsink as HS
    from panslbm2_gb300.lattice import LatticePair, phys

    S = Setup(wl, seed=rank)
    q, n = S.q, S.n
    zero, one = np.zeros(n), np.ones(n)
    lp = LatticePair(q, S.lx, S.ly, S.lz, S.storage)
    stream = torch.cuda.Stream()    # a created stream: capturable into the library's CUDA graphs
    torch.cuda.set_stream(stream)
    lp.set_stream(stream.cuda_stream)
    for fid, v in S.fields.items():
        lp.set_field(fid, v)
    lp.init(0, one, ux=zero, uy=zero, uz=zero)
    lp.init(1, zero, ux=zero, uy=zero, uz=zero)
    prog = lp.program(HS.to_descs(S.ops))
    ph = phys(**S.phys)
    lp.collide(S.kind, ph)
    lp.steps(S.kind, ph, prog, max(3, args.warmup))
    torch.cuda.synchronize()
    clocks = Clocks(local)
    clocks.start()
    time.sleep(0.3)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    _, l0 = lp.stats()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    lp.steps(S.kind, ph, prog, args.steps)
    e1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ms = e0.elapsed_time(e1)
    _, l1 = lp.stats()
    ck = clocks.stop()
    lp.synchronize()
    tmax, value = replica_throughput(ms, n, args.steps, world, dist, "cuda")
    ms_step = tmax / args.steps

    # end to end through the C ABI with pinned host buffers
    ha = torch.from_numpy(S.fields[A.ALPHA]).pin_memory()
    hk = torch.from_numpy(S.fields[A.KAPPA]).pin_memory()
    outs = [torch.empty(n, dtype=torch.float64).pin_memory() for _ in range(1 + S.nd)]
    out_ids = [A.TEM, A.UX, A.UY] + ([A.UZ] if S.nd == 3 else [])
    interval = 100
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        lp.set_field_ptr(A.ALPHA, ha.data_ptr())
        lp.set_field_ptr(A.KAPPA, hk.data_ptr())
        lp.solve(S.kind, ph, prog, max_steps=interval, check_every=interval, tol=0.0)
        for fid, buf in zip(out_ids, outs):
            lp.get_field_ptr(fid, buf.data_ptr())
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / args.e2e_steps
    e2e = {"value": n * interval / e2e_s / 1e6, "unit": "MLUPS", "h2d_bytes_per_step": 2 * n * 8,
           "d2h_bytes_per_step": len(outs) * n * 8, "time_steps_per_call": interval}

    bpn = S.bytes_per_node()
    pop_mb = 2 * q * n * {"fp64": 8, "fp32": 4, "fp16": 2, "bf16": 2}[S.storage] / 1e6
    peak, src = peaks()
    achieved = n * bpn / (ms_step / 1e3) / 1e9
    tpn = traffic_per_node(args.workload)
    roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "peak_source": src, "bytes_per_node": bpn,
            "traffic": (tpn * n if tpn else None), "kernel": "fused step (interior + boundary kernels)"}
    line = {"metric": METRIC, "value": round(value, 1), "unit": "MLUPS", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_step, 5), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32" if S.storage != "fp64" else "f64",
            "data": "synthetic (seeded GRF design, correlation length 8)",
            "config": {"workload": args.workload, "nodes": n, "storage": S.storage, "parallelism": "replicas",
                       "l2": "inputs larger than L2: two population buffers of %.0f MB each" % pop_mb},
            "roofline": roof, "e2e": e2e, "clocks": ck, "gpu_launches": int(l1 - l0)}
    lp.close()
    # the configuration legs and the CPU baseline run on one GPU only (N = 1): under torchrun
    # the whole job's GPUs would otherwise wait for rank 0's minutes of single-GPU legs
    legs = rank == 0 and world == 1
    if world > 1 and rank == 0:
        line["legs"] = "configuration legs and cpu_baseline: single-GPU runs only"
    if legs and not args.no_design:
        leg(line, "cavity_100x100", cavity_leg) if not args.no_cpu else None
        leg(line, "design_iter", design_leg, cpu=not args.no_cpu)
        leg(line, "design_iter_3d_surrogate", surrogate_leg)
        leg(line, "precision_errors", precision_leg)
        leg(line, "fp64_roofline", fp64_leg)
        leg(line, "dropin", dropin_leg)
    if legs and not args.no_transient:
        leg(line, "transient_iter", transient_gpu)
        leg(line, "transient_precision", transient_precision)
    if legs and not args.no_cpu:
        line["cpu_baseline"] = cpu_port(S)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
