"""Throughput of the fused NS+AD lattice-Boltzmann step on GB300 (one JSON line on rank 0).

Workload (default): the 3D steady heat sink, coupled D3Q15 NS + D3Q15 advection-diffusion,
160x160x80 lattice (2,048,000 nodes), FP32 populations and compute, Brinkman + natural
convection collide (AD::MacroBrinkmanCollideNaturalConvection) with the production driver's
boundary program (walls, Dirichlet T, heat-flux Q, corner/edge smoothing) every step, design
from a seeded Gaussian random field (correlation length 8 cells). A bench "step" is one fused
time step over the whole lattice: pull-stream + boundary program + collide. The population
buffers (2 x 245 MB) exceed the 129 MB L2, so no flush is needed between steps.

  value        MLUPS of the device-resident fused step (sum over ranks; replicas)
  e2e          MLUPS through the C ABI with host buffers: per e2e step, upload alpha/kappa
               from pinned host memory, run one residual-check interval of 100 time steps
               (pl_solve), download T and u
  roofline     HBM: 248 algorithmic bytes per node per step (read + write 2 x 15 FP32
               populations, read alpha and kappa) / measured step time, vs MEASURED_PEAKS
  cpu_baseline the C restatement of the reference's scalar OpenMP path (oracle/), FP64, on
               the host cores, on a bounded number of steps of the same workload
  design_iter_3d the same design iteration, plain method, on the 160x160x80 FP32 lattice
  transient_iter seconds of one transient heat-sink evaluation (4000 time steps forward and
               adjoint, checkpoints every 100 steps) on the 192x192x96 FP32 lattice
  design_iter  seconds of one heat-sink design iteration (filter, forward and adjoint to residual
               1e-6, sensitivity, filtered sensitivity) on the 200x100 FP64 lattice, with the
               oracle port's time for the same step counts

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
    "heatsink3d-160x160x80-fp32": dict(nd=3, lx=160, ly=160, lz=80, storage="fp32"),
    "heatsink3d-192x192x96-fp32": dict(nd=3, lx=192, ly=192, lz=96, storage="fp32"),
    "heatsink2d-1600x800-fp32": dict(nd=2, lx=1600, ly=800, lz=1, storage="fp32"),
    "heatsink2d-1600x800-fp64": dict(nd=2, lx=1600, ly=800, lz=1, storage="fp64"),
    "heatsink2d-1600x800-fp16": dict(nd=2, lx=1600, ly=800, lz=1, storage="fp16"),
    "heatsink2d-1600x800-bf16": dict(nd=2, lx=1600, ly=800, lz=1, storage="bf16"),
    "heatsink3d-160x160x80-fp16": dict(nd=3, lx=160, ly=160, lz=80, storage="fp16"),
    "heatsink3d-160x160x80-bf16": dict(nd=3, lx=160, ly=160, lz=80, storage="bf16"),
}
DEFAULT = "heatsink3d-160x160x80-fp32"
METRIC = "fused NS+AD MLUPS"


def bytes_per_node(q, storage):
    s = {"fp64": 8, "fp32": 4, "fp16": 2, "bf16": 2}[storage]
    c = 8 if storage == "fp64" else 4
    return 2 * 2 * q * s + 2 * c


def setup(wl, seed=0):
    from panslbm2_gb300 import heatsink as HS
    p = HS.Params(wl["nd"], wl["lx"], wl["ly"], wl["lz"])
    ss = HS.grf_design(wl["nd"], wl["lx"], wl["ly"], wl["lz"], seed=seed, sigma=8.0)
    alpha, kappa, dads, dkds = p.design_fields(ss)
    ops = HS.program_ops("forward", p)
    return p, alpha, kappa, ops


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


def cpu_port(p, alpha, kappa, ops, q, budget_s=12.0, max_steps=30):
    """Time the oracle restatement of the reference's scalar OpenMP path (FP64) on the host."""
    from oracle.olib import Oracle
    from panslbm2_gb300 import _capi as A
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from _replay import replay
    o = Oracle("oracle")
    cores = os.cpu_count() or 1
    o.set_threads(cores)
    L = o.lat(q, p.lx, p.ly, p.lz)
    n = p.lx * p.ly * p.lz
    f, g = np.zeros((q, n)), np.zeros((q, n))
    one, zero = np.ones(n), np.zeros(n)
    o.init(L, 0, f, o.fields(rho=one, ux=zero, uy=zero, uz=zero))
    o.init(L, 1, g, o.fields(tem=zero, ux=zero, uy=zero, uz=zero))
    mac = {k: np.zeros(n) for k in ("rho", "ux", "uy", "uz", "tem", "qx", "qy", "qz")}
    ph = dict(nu=p.nu, diff=0.0, gx=p.gx, gy=p.gy, gz=p.gz, tem0=p.tem0)
    F = o.fields(alpha=alpha, diffusivity=kappa, **mac)

    def one_step():
        o.collide(L, A.AD_NATURAL, f, g, F, **ph, save=True)
        o.stream(L, f)
        o.stream(L, g)
        replay(o, L, f, g, ops, n, ux=mac["ux"], uy=mac["uy"], uz=mac["uz"], kappa=kappa)

    one_step()   # warm-up
    t0, steps = time.perf_counter(), 0
    while steps < max_steps and (time.perf_counter() - t0) < budget_s:
        one_step()
        steps += 1
    dt = time.perf_counter() - t0
    return {"value": n * steps / dt / 1e6, "unit": "MLUPS", "cores": cores, "kind": "port",
            "sample": "%d full time steps (collide + 2 streams + boundary program) of the %dx%dx%d lattice, FP64"
                      % (steps, p.lx, p.ly, p.lz)}


DESIGN_LATTICE = dict(nd=2, lx=200, ly=100, lz=1, storage="fp64")


def design_gpu(tol=1e-6, max_steps=100000):
    """One heat-sink design iteration (filter, forward and adjoint to `tol`, sensitivity, filtered
    and normalised sensitivity) through the library, on the 200x100 FP64 lattice."""
    from panslbm2_gb300 import heatsink as HS
    from panslbm2_gb300.design import HeatSinkDesign
    d = DESIGN_LATTICE
    p = HS.Params(d["nd"], d["lx"], d["ly"], d["lz"])
    s = HS.grf_design(d["nd"], d["lx"], d["ly"], d["lz"], seed=0, sigma=8.0)
    hs = HeatSinkDesign(p, d["storage"])
    hs.iterate(s, tol=tol, max_steps=2000)          # warm-up: builds the filter taps and programs
    r = hs.iterate(s, tol=tol, max_steps=max_steps)
    hs.close()
    return p, s, r


def design_gpu_3d(tol=1e-6, max_steps=100000):
    """The plain design iteration on the 160x160x80 FP32 lattice (the learned warm start's
    comparison point): filter, forward and adjoint from rest to `tol`, sensitivity."""
    from panslbm2_gb300 import heatsink as HS
    from panslbm2_gb300.design import HeatSinkDesign
    p = HS.Params(3, 160, 160, 80)
    s = HS.grf_design(3, 160, 160, 80, seed=0, sigma=8.0)
    hs = HeatSinkDesign(p, "fp32")
    hs.iterate(s, tol=tol, max_steps=200)          # warm-up: filter taps, programs
    r = hs.iterate(s, tol=tol, max_steps=max_steps)
    hs.close()
    from panslbm2_gb300 import _capi as A
    return {"lattice": "heatsink3d-160x160x80-fp32", "tol": tol, "max_steps": max_steps,
            "seconds": round(r["seconds"]["total"], 3),
            "phases_s": {k: round(v, 3) for k, v in r["seconds"].items()},
            "forward_steps": r["forward"][1], "adjoint_steps": r["adjoint"][1],
            "converged": [r["forward"][0] == A.PL_CONVERGED, r["adjoint"][0] == A.PL_CONVERGED],
            "objective": r["objective"],
            "what": "plain method from rest (no warm start): filter, forward and adjoint to the residual tolerance, "
                    "heat-source sensitivity, filtered and normalised sensitivity"}


TRANSIENT_LATTICE = dict(nd=3, lx=192, ly=192, lz=96, storage="fp32", levels=4000, every=100)


def transient_gpu():
    """One transient heat-sink evaluation (forward from rest over 4000 time steps, the adjoint
    swept back with a sensitivity term per step, checkpoints every 100 steps recomputed on the
    device) on the 192x192x96 FP32 lattice, through panslbm2_gb300.transient."""
    from panslbm2_gb300 import heatsink as HS
    from panslbm2_gb300.transient import TransientHeatSink
    d = TRANSIENT_LATTICE
    p = HS.Params(d["nd"], d["lx"], d["ly"], d["lz"])
    ss = HS.grf_design(d["nd"], d["lx"], d["ly"], d["lz"], seed=0, sigma=8.0)
    alpha, kappa, dads, dkds = p.design_fields(ss)
    tr = TransientHeatSink(p, d["storage"], checkpoint_every=d["every"])
    tr.evaluate(alpha, kappa, dads, dkds, 2 * d["every"] + 2, release=False)   # warm-up: programs, step slots
    t0 = time.perf_counter()
    r = tr.evaluate(alpha, kappa, dads, dkds, d["levels"])
    sec = time.perf_counter() - t0
    tr.close()
    n = p.lx * p.ly * p.lz
    return {"lattice": "heatsink3d-192x192x96-fp32", "time_levels": d["levels"], "checkpoint_every": d["every"],
            "segments": r["segments"], "seconds": round(sec, 3),
            "phases_s": {k: round(v, 3) for k, v in r["times"].items()},
            "forward_mlups": round(n * (d["levels"] - 1) / r["times"]["forward"] / 1e6, 1),
            "objective": r["objective"],
            "what": "forward from rest, adjoint swept back with one heat-source sensitivity term per time step, "
                    "forward states recomputed from device checkpoints; no filter or MMA"}


def design_cpu_per_step(p, budget_s=8.0):
    """Seconds per forward and per adjoint time step of the oracle port (FP64, all host cores) on
    the design lattice, from a bounded sample of steps with the drivers' every-step saves."""
    from oracle.olib import Oracle
    from panslbm2_gb300 import _capi as A
    from panslbm2_gb300 import heatsink as HS
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from _replay import replay
    o = Oracle("oracle")
    o.set_threads(os.cpu_count() or 1)
    q = 9 if p.nd == 2 else 15
    L = o.lat(q, p.lx, p.ly, p.lz)
    n = p.lx * p.ly * p.lz
    ss = HS.grf_design(p.nd, p.lx, p.ly, p.lz, seed=0, sigma=8.0)
    alpha, kappa, _, _ = p.design_fields(ss)
    ph = dict(nu=p.nu, diff=0.0, gx=p.gx, gy=p.gy, gz=p.gz, tem0=p.tem0)
    out = {}
    for phase, kind, inverse in (("forward", A.AD_NATURAL, False), ("adjoint", A.AAD_NATURAL, True)):
        f, g = np.zeros((q, n)), np.zeros((q, n))
        zero = np.zeros(n)
        o.init(L, 0, f, o.fields(rho=np.ones(n), ux=zero, uy=zero, uz=zero))
        o.init(L, 1, g, o.fields(tem=zero, ux=zero, uy=zero, uz=zero))
        names = ("rho", "ux", "uy", "uz", "tem", "qx", "qy", "qz", "ip", "iux", "iuy", "iuz", "imx", "imy", "imz",
                 "item", "iqx", "iqy", "iqz")
        mac = {k: np.zeros(n) for k in names}
        mac["rho"][:] = 1.0
        snap = np.zeros(n * q)
        ops = HS.program_ops(phase, p)
        F = o.fields(gsnap=snap, alpha=alpha, diffusivity=kappa, **mac)
        steps, t0 = 0, time.perf_counter()
        while time.perf_counter() - t0 < budget_s and steps < 2000:
            o.collide(L, kind, f, g, F, **ph, save=True)
            o.stream(L, f, inverse)
            o.stream(L, g, inverse)
            replay(o, L, f, g, ops, n, ux=mac["ux"], uy=mac["uy"], uz=mac["uz"], rho=mac["rho"], tem=mac["tem"],
                   kappa=kappa)
            steps += 1
        out[phase] = (time.perf_counter() - t0) / max(1, steps)
        out[phase + "_sample"] = steps
    return out


def run_reference(args, wl):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    p, alpha, kappa, ops = setup(wl)
    q = 9 if wl["nd"] == 2 else 15
    cb = cpu_port(p, alpha, kappa, ops, q, budget_s=60.0, max_steps=max(1, min(args.steps, 40)))
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": "MLUPS", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded GRF design)",
            "config": {"workload": args.workload, "nodes": p.lx * p.ly * p.lz, "backend": "cpu"},
            "cpu_baseline": cb, "e2e": {"value": cb["value"], "unit": "MLUPS", "h2d_bytes_per_step": 0,
                                        "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=50)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT, choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--no-design", action="store_true", help="skip the design-iteration timing")
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

    p, alpha, kappa, ops = setup(wl, seed=rank)
    q = 9 if wl["nd"] == 2 else 15
    n = p.lx * p.ly * p.lz
    zero, one = np.zeros(n), np.ones(n)
    lp = LatticePair(q, p.lx, p.ly, p.lz, wl["storage"])
    stream = torch.cuda.Stream()    # a created stream: capturable into the library's CUDA graphs
    torch.cuda.set_stream(stream)
    lp.set_stream(stream.cuda_stream)
    lp.set_field(A.ALPHA, alpha)
    lp.set_field(A.KAPPA, kappa)
    lp.init(0, one, ux=zero, uy=zero, uz=zero)
    lp.init(1, zero, ux=zero, uy=zero, uz=zero)
    prog = lp.program(HS.to_descs(ops))
    ph = phys(nu=p.nu, diff=0.0, gx=p.gx, gy=p.gy, gz=p.gz, tem0=p.tem0)
    lp.collide(A.AD_NATURAL, ph)
    lp.steps(A.AD_NATURAL, ph, prog, max(3, args.warmup))
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
    lp.steps(A.AD_NATURAL, ph, prog, args.steps)
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
    ha = torch.from_numpy(alpha).pin_memory()
    hk = torch.from_numpy(kappa).pin_memory()
    outs = [torch.empty(n, dtype=torch.float64).pin_memory() for _ in range(1 + wl["nd"])]
    out_ids = [A.TEM, A.UX, A.UY] + ([A.UZ] if wl["nd"] == 3 else [])
    interval = 100
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        lp.set_field_ptr(A.ALPHA, ha.data_ptr())
        lp.set_field_ptr(A.KAPPA, hk.data_ptr())
        lp.solve(A.AD_NATURAL, ph, prog, max_steps=interval, check_every=interval, tol=0.0)
        for fid, buf in zip(out_ids, outs):
            lp.get_field_ptr(fid, buf.data_ptr())
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / args.e2e_steps
    e2e = {"value": n * interval / e2e_s / 1e6, "unit": "MLUPS", "h2d_bytes_per_step": 2 * n * 8,
           "d2h_bytes_per_step": len(outs) * n * 8, "time_steps_per_call": interval}

    bpn = bytes_per_node(q, wl["storage"])
    pop_mb = 2 * q * n * {"fp64": 8, "fp32": 4, "fp16": 2, "bf16": 2}[wl["storage"]] / 1e6
    peak, src = peaks()
    achieved = n * bpn / (ms_step / 1e3) / 1e9
    tpn = traffic_per_node(args.workload)
    roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "peak_source": src, "bytes_per_node": bpn,
            "traffic": (tpn * n if tpn else None), "kernel": "fused step (interior + boundary kernels)"}
    line = {"metric": METRIC, "value": round(value, 1), "unit": "MLUPS", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_step, 5), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32" if wl["storage"] != "fp64" else "f64",
            "data": "synthetic (seeded GRF design, correlation length 8)",
            "config": {"workload": args.workload, "nodes": n, "storage": wl["storage"], "parallelism": "replicas",
                       "l2": "inputs larger than L2: two population buffers of %.0f MB each" % pop_mb},
            "roofline": roof, "e2e": e2e, "clocks": ck, "gpu_launches": int(l1 - l0)}
    if rank == 0 and not args.no_design:
        dp, _, r = design_gpu()
        di = {"lattice": "heatsink2d-200x100-fp64", "tol": 1e-6, "max_steps": 100000,
              "seconds": round(r["seconds"]["total"], 4),
              "phases_s": {k: round(v, 4) for k, v in r["seconds"].items()},
              "forward_steps": r["forward"][1], "adjoint_steps": r["adjoint"][1],
              "converged": [r["forward"][0] == A.PL_CONVERGED, r["adjoint"][0] == A.PL_CONVERGED],
              "objective": r["objective"],
              "what": "filter, forward and adjoint to residual 1e-6 (checked every 100 steps), heat-source "
                      "sensitivity, filtered and normalised sensitivity; from rest; no MMA update"}
        if not args.no_cpu:
            cs = design_cpu_per_step(dp)
            di["cpu_seconds_est"] = round(cs["forward"] * r["forward"][1] + cs["adjoint"] * r["adjoint"][1], 2)
            di["cpu_sample"] = ("oracle port, FP64, %d host threads: %d forward and %d adjoint steps timed, scaled to the "
                                "GPU's step counts" % (os.cpu_count() or 1, cs["forward_sample"], cs["adjoint_sample"]))
        line["design_iter"] = di
    if rank == 0 and not args.no_design:
        try:
            line["design_iter_3d"] = design_gpu_3d()
        except Exception as e:   # reported, not fatal
            line["design_iter_3d"] = {"error": str(e)[:300]}
    if rank == 0 and not args.no_transient:
        try:
            line["transient_iter"] = transient_gpu()
        except Exception as e:   # reported, not fatal: the step throughput above stands on its own
            line["transient_iter"] = {"error": str(e)[:300]}
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_port(p, alpha, kappa, ops, q)
        ti = line.get("transient_iter", {})
        if "seconds" in ti and line["cpu_baseline"].get("value"):
            d = TRANSIENT_LATTICE
            nodes = d["lx"] * d["ly"] * d["lz"]
            ti["cpu_seconds_est"] = round(2 * (d["levels"] - 1) * nodes / (line["cpu_baseline"]["value"] * 1e6), 1)
            ti["cpu_sample"] = ("the cpu_baseline step rate (oracle port, FP64, all host threads) applied to the "
                                "forward and adjoint steps, without recomputation")
    if rank == 0:
        print(json.dumps(line), flush=True)
    lp.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
