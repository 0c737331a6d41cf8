"""Benchmark of the GB300 SimPLIC step (cell-steps/s).

Workload (default): 256^3 uniform hex mesh on the unit cube, sphere R=0.15 at
(0.35, 0.35, 0.35), the 3-D deformation field of the reference advection
test with period T=6, fixed time step at Courant number 0.5 of the
full-speed field, controls of the reference test case (nAlphaBounds 3,
snapTol 0, clip false, mixedCellTol 1e-8, LS normals).  A step is one
reconstruct() + advect() over the whole mesh.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--n 256]
                  [--precision learned|mixed|plain]

--impl ours (default): the CUDA library, inputs resident in HBM (value) and
through the host-buffer C ABI with host<->device copies timed (e2e); plus a
bounded CPU-baseline sample of the oracle on the host cores.  The headline
form (--precision, default the learned-normal mixed form) and the other
forms (plain FP64, mixed with least-squares normals) are timed on the same
inputs ("forms", with the speed-up over plain), and every form is run over
the 128^3 comparison case to t = 3 for the L1 shape error, volume drift and
boundedness ("accuracy").
--impl reference: the reference's CPU algorithm (the FP64 restatement in
oracle/, OpenMP over all host cores) on the same workload.
Under torchrun every rank runs an independent replica on its own GPU
(the step does not shard across GPUs in this build).
"""

from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SimPLIC cell-steps/s: plain FP64 vs learned-normal mixed at equal shape error"
UNIT = "cell-steps/s"
# algorithmic bytes per cell-step of the bulk update (alpha_old, alpha_new,
# V, and per face phi, alphaPhi, owner+neighbour: 24 + 3*24)
BULK_BYTES_PER_CELL = 96.0
# DRAM bytes (read + write) of one update launch per cell, from the ncu
# capture of the 256^3 plain run (profiles/simplic_plain_256_launches.md:
# 0.582 GB + 0.490 GB for 16,777,216 cells); reported only for that workload
UPDATE_DRAM_BYTES_PER_CELL_256 = 1.0716e9 / 16777216


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def workload(n):
    from geometricvofext_gb300 import harness as H, meshgen as mg

    t0 = time.time()
    mesh = mg.hex_mesh(n)
    alpha0 = H.sphere_alpha(mesh, (0.35, 0.35, 0.35), 0.15)
    flow = H.DeformationFlow(mesh, period=6.0)
    dt = H.cfl_delta_t(mesh, flow.phi0, 0.5)
    return mesh, alpha0, flow, dt, time.time() - t0


CONTROLS = dict(mixed_cell_tol=1e-8, n_alpha_bounds=3, snap_tol=0.0, clip=0)


class ClockSampler:
    def __init__(self, index):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.f.name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(mesh, alpha0, flow, dt, max_seconds=20.0, max_steps=3):
    """The oracle (FP64 restatement of the reference CPU algorithm) with
    OpenMP over all host cores, on the first steps of the same run."""
    from oracle import oracle as O

    threads = os.cpu_count() or 1
    o = O.Oracle(mesh, n_threads=threads, mixed_cell_tol=1e-8, n_alpha_bounds=3, snap_tol=0.0, clip=False)
    a = alpha0.copy()
    t = 0.0
    done = 0
    el = 0.0
    while done < max_steps and el < max_seconds:
        t += dt
        fl = flow.at(t, dt)
        s = time.perf_counter()
        o.reconstruct(a)
        a = o.advect(a, fl.phi, fl.U, dt, U_boundary=fl.U_boundary)
        el += time.perf_counter() - s
        done += 1
    return {"value": mesh.n_cells * done / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{done} steps of the {round(mesh.n_cells ** (1 / 3))}^3 deformation run from t=0 "
                      f"({el:.1f} s of CPU work)"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    mesh, alpha0, flow, dt, tsetup = workload(args.n)
    from oracle import oracle as O

    threads = os.cpu_count() or 1
    o = O.Oracle(mesh, n_threads=threads, mixed_cell_tol=1e-8, n_alpha_bounds=3, snap_tol=0.0, clip=False)
    a = alpha0.copy()
    t = 0.0

    def step():
        nonlocal a, t
        t += dt
        fl = flow.at(t, dt)
        o.reconstruct(a)
        a = o.advect(a, fl.phi, fl.U, dt, U_boundary=fl.U_boundary)

    for _ in range(args.warmup):
        step()
    s = time.perf_counter()
    for _ in range(args.steps):
        step()
    el = time.perf_counter() - s
    v = mesh.n_cells * args.steps / el
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": config(args, mesh, "reference"),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{args.steps} full steps after {args.warmup} warm-up steps"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


FORM_NAMES = {
    "plain": "plain FP64",
    "mixed": "mixed precision (FP32 LS normals + clipping, FP64 volume)",
    "learned": "learned-normal mixed (BF16 tcgen05 network + FP32 clipping, FP64 volume)",
    "reference": "reference CPU algorithm (FP64)",
}


def config(args, mesh, form=None):
    form = FORM_NAMES[form or args.precision]
    return {"workload": f"SimPLIC {form}, {args.n}^3 hex deformation field (T=6), sphere R=0.15, CFL 0.5",
            "cells": mesh.n_cells, "faces": mesh.n_faces, "mesh": "uniform hex", "precision": args.precision,
            "controls": "nAlphaBounds 3, snapTol 0, clip false, mixedCellTol 1e-8, LS",
            "l2": ("inputs larger than L2" if 8 * (mesh.n_faces + 3 * mesh.n_cells) > 0.13e9 else
                   "inputs NOT larger than L2 (small case)")
                  + f" (phi and U are {8 * (mesh.n_faces + 3 * mesh.n_cells) / 1e9:.2f} GB per step, alpha old/new "
                  f"and V another {24 * mesh.n_cells / 1e9:.2f} GB; L2 is 0.13 GB)",
            "parallelism": f"replicas x{args.gpus}" if args.gpus > 1 else "single GPU"}


FORMS = {"plain": "PRECISION_PLAIN_FP64", "mixed": "PRECISION_MIXED", "learned": "PRECISION_LEARNED"}


def make_handle(form, mesh, stream=None):
    """A handle of one form; the learned form loads the trained network
    shipped with the package (geometricvofext_gb300/data/normal_net.npz)."""
    from geometricvofext_gb300 import capi, mlp

    kw = {"stream": stream} if stream is not None else {}
    g = capi.Simplic(mesh, precision=getattr(capi, FORMS[form]), **kw, **CONTROLS)
    if form == "learned":
        W, b = mlp.load_weights()
        g.set_network(W, b)
    return g


def time_form(form, mesh, alpha0, phis, Us, Ub, dt, args, dev, dist, local):
    """W warm-up + K timed steps of one form with inputs resident in HBM;
    CUDA events on the library's stream, kernel events inside."""
    import torch

    from geometricvofext_gb300 import capi, replicas

    stream = torch.cuda.Stream(dev)
    t0 = time.time()
    g = make_handle(form, mesh, stream.cuda_stream)
    tcreate = time.time() - t0
    g.set_alpha(alpha0)

    def step(k):
        g.reconstruct_resident()
        g.advect_resident(phis[k], Us[k], dt, U_boundary=Ub)

    for k in range(args.warmup):
        step(k)
    g.synchronize()
    g.reset_kernel_times()
    g.set_kernel_timing(True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize(dev)
    clocks = ClockSampler(local)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for k in range(args.warmup, args.warmup + args.steps):
        step(k)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1)
    if dist:
        dist.barrier()
    clk = clocks.stop()
    g.synchronize()
    kt = g.kernel_times()
    g.set_kernel_timing(False)
    nmix, passes, maxb = g.stats()
    binfo = g.bound_info()
    ms = replicas.max_over_ranks(ms, dist, dev)
    return {"g": g, "ms": ms, "clk": clk, "kt": kt, "tcreate": tcreate,
            "stats": {"mixed_cells_last_step": nmix, "bound_passes_last_step": passes, "bounded_cells_max": maxb,
                      "bound_waves_last_step": binfo[2]}}


def accuracy(dev, n=128, t_end=3.0):
    """The plain-vs-mixed comparison case: n^3 hex, deformation field T=6,
    sphere R=0.15 at (0.35, 0.35, 0.35), Courant 0.5, run to t = 3 where the
    shape returns; L1 shape error against the initial field, volume drift
    and the largest excursion outside [0, 1], per form."""
    import torch

    from geometricvofext_gb300 import capi, harness as H

    mesh, alpha0, flow, dt, _ = workload(n)
    steps = int(math.ceil(t_end / dt - 1e-9))
    dt = t_end / steps
    phi0 = torch.from_numpy(flow.phi0).to(dev)
    U0 = torch.from_numpy(flow.U0).to(dev)
    Ub = torch.zeros((mesh.n_boundary_faces, 3), dtype=torch.float64, device=dev)
    phi = torch.empty_like(phi0)
    U = torch.empty_like(U0)
    vol0 = float(np.sum(alpha0 * mesh.V))
    out = {"case": f"{n}^3 hex deformation (T=6), sphere R=0.15, Courant 0.5, t=0..{t_end:g}, {steps} steps"}
    # one stream for the per-step scaling of phi / U and the library, so each
    # step reads the fields written for it
    stream = torch.cuda.Stream(dev)
    torch.cuda.synchronize(dev)
    for form in FORMS:
        g = make_handle(form, mesh, stream.cuda_stream)
        g.set_alpha(alpha0)
        s = time.perf_counter()
        with torch.cuda.stream(stream):
            for k in range(steps):
                t = (k + 1) * dt
                f = H.time_factor(t, dt, flow.period)
                torch.mul(phi0, f, out=phi)
                torch.mul(U0, f, out=U)
                g.reconstruct_resident()
                g.advect_resident(phi, U, dt, U_boundary=Ub)
        g.synchronize()
        a = g.get_alpha()
        el = time.perf_counter() - s
        e = H.errors(a, alpha0, mesh.V, vol0)
        out[form] = {"shape_error_L1": e.shape_error, "volume_drift": e.volume_error,
                     "max_bound_violation": e.boundedness, "wall_s": round(el, 2)}
        del g
    return out


def run_ours(args):
    import torch

    from geometricvofext_gb300 import replicas

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)

    mesh, alpha0, flow, dt, tsetup = workload(args.n)
    nsteps = args.warmup + args.steps
    phi0 = torch.from_numpy(flow.phi0).to(dev)
    U0 = torch.from_numpy(flow.U0).to(dev)
    Ub = torch.zeros((mesh.n_boundary_faces, 3), dtype=torch.float64, device=dev)
    from geometricvofext_gb300 import harness as H

    facs = [H.time_factor((k + 1) * dt, dt, flow.period) for k in range(nsteps)]
    phis = [phi0 * f for f in facs]
    Us = [U0 * f for f in facs]
    torch.cuda.synchronize(dev)

    # the headline form, then the other form on the same inputs for the
    # comparison the metric names
    head = args.precision
    forms = [head] + ([] if args.single_form else [f for f in FORMS if f != head])
    res = {f: time_form(f, mesh, alpha0, phis, Us, Ub, dt, args, dev, dist, local) for f in forms}
    r = res[head]
    ms, kt, clk = r["ms"], r["kt"], r["clk"]
    value = replicas.replica_throughput(world, mesh.n_cells, args.steps, ms)
    launches = sum(v[1] for v in kt.values())  # counters were reset after the warm-up

    # --- per-kernel roofline (live CUDA-event durations inside the timed region)
    hbm, src = peaks()
    kavg = {k: (v[0] / max(1, v[1])) for k, v in kt.items()}
    ktot = {k: v[0] for k, v in kt.items() if k != "faceFlatness"}
    dominant = max(ktot, key=ktot.get)
    nc = mesh.n_cells
    upd_ms = kavg["update"]
    upd_bytes = BULK_BYTES_PER_CELL * nc
    traffic = UPDATE_DRAM_BYTES_PER_CELL_256 * nc if args.n == 256 else None
    roof = {"bound": "hbm", "kernel": "update", "achieved": upd_bytes / (upd_ms * 1e-3) / 1e9,
            "peak": hbm, "unit": "GB/s", "frac": None, "traffic": traffic,
            "bytes_per_launch": upd_bytes, "peak_source": f"{src} hbm_gbs (burst copy)",
            "dominant_kernel": dominant,
            # whole step against HBM: the 96 B/cell bulk bytes over the step time
            "step_achieved_gbs": upd_bytes / (ms / args.steps * 1e-3) / 1e9,
            "kernel_ms_per_step": {k: round(v / args.steps, 4) for k, v in ktot.items()},
            "kernel_share": {k: round(v / max(1e-12, sum(ktot.values())), 4) for k, v in ktot.items()}}
    roof["frac"] = roof["achieved"] / hbm

    forms_out = {}
    for f, rf in res.items():
        forms_out[f] = {"value": replicas.replica_throughput(world, nc, args.steps, rf["ms"]),
                        "ms_per_step": rf["ms"] / args.steps,
                        "kernel_ms_per_step": {k: round(v[0] / args.steps, 4) for k, v in rf["kt"].items()
                                               if k != "faceFlatness"},
                        "stats": rf["stats"]}
    if "plain" in res and head != "plain":
        forms_out["speedup_vs_plain"] = res["plain"]["ms"] / ms

    # --- end to end through the host-buffer C ABI (pinned buffers, copies timed)
    e2e = run_e2e(r["g"], mesh, alpha0, flow, dt, args, dev) if not args.no_e2e else None

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {"plain": "f64", "mixed": "f64+f32", "learned": "f64+f32+bf16"}[head], "data": "synthetic", "config": config(args, mesh),
        "roofline": roof, "gpu_launches": launches, "clocks": clk, "forms": forms_out,
        "stats": dict(r["stats"], setup_s={"mesh_and_fields": round(tsetup, 1), "create": round(r["tcreate"], 1)}),
    }
    if e2e:
        line["e2e"] = e2e
    for f in list(res):
        del res[f]["g"]
    if rank == 0 and world == 1 and not args.no_accuracy:
        line["accuracy"] = accuracy(dev)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(mesh, alpha0, flow, dt)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def run_e2e(g, mesh, alpha0, flow, dt, args, dev):
    import torch

    from geometricvofext_gb300 import capi

    K = max(1, min(args.steps, args.e2e_steps))
    nc, nf, nfb = mesh.n_cells, mesh.n_faces, mesh.n_boundary_faces

    def pinned(shape):
        return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()

    alpha = pinned(nc)
    alpha[:] = alpha0
    phis, Us = [], []
    from geometricvofext_gb300 import harness as H

    for k in range(K + 1):
        f = H.time_factor((k + 1) * dt, dt, flow.period)
        p = pinned(nf)
        p[:] = flow.phi0 * f
        u = pinned((nc, 3))
        u[:] = flow.U0 * f
        phis.append(p)
        Us.append(u)
    Ub = pinned((nfb, 3))
    Ub[:] = 0.0
    # one untimed step
    g.reconstruct_ptr(alpha)
    g.advect_inplace(alpha, phis[0], Us[0], dt, U_boundary=Ub)
    torch.cuda.synchronize(dev)
    s = time.perf_counter()
    for k in range(1, K + 1):
        g.reconstruct_ptr(alpha)                                          # H2D alpha
        g.advect_inplace(alpha, phis[k], Us[k], dt, U_boundary=Ub)        # H2D phi, U, Ub; D2H alpha
    el = time.perf_counter() - s
    h2d = 8 * nc + 8 * nf + 24 * nc + 24 * nfb
    d2h = 8 * nc
    return {"value": nc * K / el, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "steps": K, "path": "simplic_reconstruct + simplic_advect (host pinned buffers)"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--precision", default="learned", choices=list(FORMS))
    ap.add_argument("--single-form", action="store_true", help="time the headline form only")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the 128^3 t=3 plain-vs-mixed accuracy run")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.steps < 1:
        raise SystemExit("steps >= 1 required")
    args.warmup = max(3, args.warmup)  # at least three warm-up steps
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
