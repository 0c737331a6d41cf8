"""Benchmark of the GB300 SimPLIC step (cell-steps/s).

Workload (default): 256^3 uniform hex mesh on the unit cube, sphere R=0.15 at
(0.35, 0.35, 0.35), the 3-D deformation field of the reference advection
test with period T=6, fixed time step at Courant number 0.5 of the
full-speed field (rounded so that a whole number of steps reaches t = 3),
controls of the reference test case (nAlphaBounds 3, snapTol 0, clip false,
mixedCellTol 1e-8, LS normals).  A step is one reconstruct() + advect() over
the whole mesh.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--n 256]
                  [--precision learned|mixed|plain] [--case deformation|scale|unstructured]

--impl ours (default): the CUDA library.  For every form (the headline
--precision, default the learned-normal mixed form, then plain FP64 and the
mixed form with least-squares normals), on the same inputs:
  * the contract window: W warm-up steps, then K steps timed with CUDA events
    on the library's stream, inputs resident in HBM, no per-kernel events
    (this is `value` for the headline form);
  * a kernel pass: K further steps with an event pair around every kernel
    launch (per-kernel times, the roofline of the update kernel);
  * the full period t = 0 .. 3 (about 3,800 steps at 256^3) with the
    velocity scaled per step on the same stream; the device time of the
    library's calls only (the handle's reconstruction and advection timers,
    the reference's reconstructionTime / advectionTime), and at t = 3 the
    L1 shape error against the initial field, the volume drift and the
    largest excursion outside [0, 1].
Then the end-to-end figure through the host-buffer C ABI (copies timed), and
a bounded CPU-baseline sample of the oracle (1 thread and all host cores).
The unstructured-mesh configuration (96^3 jittered hex, 64^3 x 6 tets, to
t = 3, every form) is appended as `configs.unstructured` unless
--no-unstructured.
--case scale: the 320^3 scale case (spheres and slab, T = 6, 500 steps).
--case unstructured: the unstructured-mesh configuration alone.
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
# ncu summary of the update kernel: "dram_bytes_per_cell <value>" and the
# workload line, read for the roofline's traffic figure
UPDATE_PROFILE = os.path.join(ROOT, "profiles", "simplic_update_256_dram.md")


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def update_traffic(n):
    """DRAM bytes (read + write) per launch of the update kernel from its
    committed ncu summary, scaled to n^3 cells by the cells processed."""
    try:
        with open(UPDATE_PROFILE) as fh:
            for line in fh:
                if line.startswith("dram_bytes_per_cell"):
                    return float(line.split()[1]) * n ** 3, os.path.relpath(UPDATE_PROFILE, ROOT)
    except OSError:
        pass
    return None, None


def deformation_workload(n):
    from geometricvofext_gb300 import harness as H, meshgen as mg

    t0 = time.time()
    mesh = mg.hex_mesh(n)
    alpha0 = H.sphere_alpha(mesh, (0.35, 0.35, 0.35), 0.15)
    flow = H.DeformationFlow(mesh, period=6.0)
    dt = H.cfl_delta_t(mesh, flow.phi0, 0.5)
    steps = int(math.ceil(3.0 / dt - 1e-9))
    return mesh, alpha0, flow, 3.0 / steps, steps, time.time() - t0


CONTROLS = dict(mixed_cell_tol=1e-8, n_alpha_bounds=3, snap_tol=0.0, clip=0)
CONTROLS_TEXT = "nAlphaBounds 3, snapTol 0, clip false, mixedCellTol 1e-8, LS"


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


def oracle_steps(mesh, alpha0, flow, dt, threads, max_seconds, max_steps):
    """Reconstruct + advect steps of the oracle from t = 0; returns the
    steps done and their wall time (velocity generation excluded)."""
    from oracle import oracle as O

    o = O.Oracle(mesh, n_threads=threads, **dict(CONTROLS, clip=False))
    a = alpha0.copy()
    done, el = 0, 0.0
    while done < max_steps and el < max_seconds:
        fl = flow.at((done + 1) * dt, dt)
        s = time.perf_counter()
        o.reconstruct(a)
        a = o.advect(a, fl.phi, fl.U, dt, U_boundary=fl.U_boundary)
        el += time.perf_counter() - s
        done += 1
    return done, el


def cpu_baseline(mesh, alpha0, flow, dt):
    """The oracle (FP64 restatement of the reference CPU algorithm) on the
    first steps of the same run: one thread (one reference MPI rank) and
    OpenMP over all host cores."""
    threads = os.cpu_count() or 1
    n = round(mesh.n_cells ** (1 / 3))
    d1, e1 = oracle_steps(mesh, alpha0, flow, dt, 1, 8.0, 1)
    dn, en = oracle_steps(mesh, alpha0, flow, dt, threads, 12.0, 3)
    return {"value": mesh.n_cells * dn / en, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{dn} steps of the {n}^3 deformation run from t=0 ({en:.1f} s of CPU work, OpenMP)",
            "single_thread": {"value": mesh.n_cells * d1 / e1, "unit": UNIT, "cores": 1,
                              "sample": f"{d1} step of the same run ({e1:.1f} s)"}}


FORM_NAMES = {
    "plain": "plain FP64",
    "mixed": "mixed precision (FP32 LS normals + clipping, FP64 volume)",
    "learned": "learned-normal mixed (BF16 tcgen05 network + FP32 clipping, FP64 volume)",
    "reference": "reference CPU algorithm (FP64 restatement, OpenMP)",
}


def config(args, mesh):
    """The workload; the same for both arms (the form is a separate key)."""
    nb = 8 * (mesh.n_faces + 3 * mesh.n_cells)
    return {"workload": f"SimPLIC step, {args.n}^3 hex, 3-D deformation field (T=6), sphere R=0.15 at "
                        f"(0.35,0.35,0.35), Courant 0.5",
            "cells": mesh.n_cells, "faces": mesh.n_faces, "mesh": "uniform hex", "controls": CONTROLS_TEXT,
            "l2": ("inputs larger than L2" if nb > 0.13e9 else "inputs NOT larger than L2 (small case)")
                  + f" (phi and U are {nb / 1e9:.2f} GB per step, alpha old/new and V another "
                  f"{24 * mesh.n_cells / 1e9:.2f} GB; L2 is 0.13 GB)",
            "parallelism": f"replicas x{args.gpus}" if args.gpus > 1 else "single GPU",
            **({"window_start_t": args.t0} if args.t0 > 0 else {})}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    mesh, alpha0, flow, dt, _, _ = deformation_workload(args.n)
    from oracle import oracle as O

    threads = os.cpu_count() or 1
    o = O.Oracle(mesh, n_threads=threads, **dict(CONTROLS, clip=False))
    a = alpha0.copy()
    k = 0

    def step():
        nonlocal a, k
        k += 1
        fl = flow.at(k * dt, dt)
        o.reconstruct(a)
        a = o.advect(a, fl.phi, fl.U, dt, U_boundary=fl.U_boundary)

    for _ in range(args.warmup):
        step()
    el = 0.0
    for _ in range(args.steps):
        s = time.perf_counter()
        step()
        el += time.perf_counter() - s
    v = mesh.n_cells * args.steps / el
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "form": FORM_NAMES["reference"], "config": config(args, mesh),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{args.steps} full steps after {args.warmup} warm-up steps"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


FORMS = {"plain": "PRECISION_PLAIN_FP64", "mixed": "PRECISION_MIXED", "learned": "PRECISION_LEARNED"}


def make_handle(form, mesh, stream=None, **extra):
    """A handle of one form; the learned form loads the trained network
    shipped with the package (geometricvofext_gb300/data/normal_net.npz)."""
    from geometricvofext_gb300 import capi, mlp

    kw = {"stream": stream} if stream is not None else {}
    ctrl = dict(CONTROLS, **extra)
    g = capi.Simplic(mesh, precision=getattr(capi, FORMS[form]), **kw, **ctrl)
    if form == "learned":
        W, b = mlp.load_weights()
        g.set_network(W, b)
    return g


class ScaledFlow:
    """phi0 and U0 resident in HBM; each step's fields are the product with
    the step's time factor, written on the library's stream."""

    def __init__(self, phi0, U0, n_bfaces, dev, period):
        import torch

        self.phi0 = torch.from_numpy(phi0).to(dev)
        self.U0 = torch.from_numpy(U0).to(dev)
        self.Ub = torch.zeros((n_bfaces, 3), dtype=torch.float64, device=dev)
        self.phi = torch.empty_like(self.phi0)
        self.U = torch.empty_like(self.U0)
        self.period = period

    def set(self, t, dt, stream):
        import torch

        from geometricvofext_gb300 import harness as H

        f = H.time_factor(t, dt, self.period)
        with torch.cuda.stream(stream):
            torch.mul(self.phi0, f, out=self.phi)
            torch.mul(self.U0, f, out=self.U)


def full_period(g, flow, alpha0, mesh, dt, steps, stream, vol0):
    """All steps t = 0 .. steps*dt; device time of the library's calls from
    the handle's timers; the errors at the end against the initial field."""
    from geometricvofext_gb300 import harness as H

    g.set_alpha(alpha0)
    r0, a0, _ = g.timers()
    s = time.perf_counter()
    maxmix = 0
    for k in range(steps):
        flow.set((k + 1) * dt, dt, stream)
        g.reconstruct_resident()
        g.advect_resident(flow.phi, flow.U, dt, U_boundary=flow.Ub)
    g.synchronize()
    wall = time.perf_counter() - s
    r1, a1, _ = g.timers()
    dev_s = (r1 - r0) + (a1 - a0)
    a = g.get_alpha()
    e = H.errors(a, alpha0, mesh.V, vol0)
    return a, {"value": mesh.n_cells * steps / dev_s, "unit": UNIT, "steps": steps, "t_end": steps * dt,
               "device_s": round(dev_s, 4), "ms_per_step": 1e3 * dev_s / steps,
               "reconstruct_s": round(r1 - r0, 4), "advect_s": round(a1 - a0, 4), "loop_wall_s": round(wall, 3),
               "shape_error_L1": e.shape_error, "volume_drift": e.volume_error,
               "max_bound_violation": e.boundedness}


def run_form(form, mesh, alpha0, flow, dt, steps_full, args, dev, dist, local):
    """Contract window, kernel pass and full period of one form."""
    import torch

    from geometricvofext_gb300 import replicas

    stream = torch.cuda.Stream(dev)
    t0 = time.time()
    g = make_handle(form, mesh, stream.cuda_stream)
    tcreate = time.time() - t0
    g.set_alpha(alpha0)
    k = 0

    def step():
        nonlocal k
        k += 1
        flow.set(k * dt, dt, stream)
        g.reconstruct_resident()
        g.advect_resident(flow.phi, flow.U, dt, U_boundary=flow.Ub)

    # a window later in the period (profiling): the steps up to t0 untimed
    for _ in range(int(round(args.t0 / dt))):
        step()
    for _ in range(args.warmup):
        step()
    g.synchronize()
    g.set_kernel_timing(False)
    # the per-step velocity scaling would count in a CUDA-event window, so
    # the window's fields are written up front (K x 0.8 GB at 256^3 would
    # not fit for large K: at most 16 precomputed, the rest reuse them)
    from geometricvofext_gb300 import harness as H

    nbuf = min(args.steps, 16)
    phis = [flow.phi0 * H.time_factor((k + 1 + j) * dt, dt, flow.period) for j in range(nbuf)]
    Us = [flow.U0 * H.time_factor((k + 1 + j) * dt, dt, flow.period) for j in range(nbuf)]
    torch.cuda.synchronize(dev)
    if dist:
        dist.barrier()
    torch.cuda.synchronize(dev)
    clocks = ClockSampler(local)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for j in range(args.steps):
        g.reconstruct_resident()
        g.advect_resident(phis[j % nbuf], Us[j % nbuf], dt, U_boundary=flow.Ub)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1)
    if dist:
        dist.barrier()
    win_clk = clocks.stop()
    ms = replicas.max_over_ranks(ms, dist, dev)
    nmix, passes, maxb = g.stats()
    binfo = g.bound_info()
    bprof = g.bound_profile()
    # kernel pass: K more steps with an event pair around each launch, on
    # the same precomputed inputs as the window
    g.reset_kernel_times()
    g.set_kernel_timing(True)
    for j in range(args.steps):
        g.reconstruct_resident()
        g.advect_resident(phis[j % nbuf], Us[j % nbuf], dt, U_boundary=flow.Ub)
    g.synchronize()
    k += 2 * args.steps
    kt = g.kernel_times()
    g.set_kernel_timing(False)
    del phis, Us
    out = {"g": g, "ms": ms, "clk": win_clk, "kt": kt, "tcreate": tcreate, "stream": stream,
           "stats": {"mixed_cells_window_end": nmix, "bound_passes": passes, "bounded_cells_max": maxb,
                     "bound_chain_starts": binfo[2], "bound_longest_warp_chain": bprof[0],
                     "bound_us_last_step": bprof[3], "bound_dependency_us_last_step": bprof[2]}}
    if form == "learned":
        out["stats"]["network_rows_overflow"] = g.network_overflow()
    if not args.no_full_period:
        vol0 = float(np.sum(alpha0 * mesh.V))
        clocks = ClockSampler(local)
        a, fp = full_period(g, flow, alpha0, mesh, dt, steps_full, stream, vol0)
        fp["clocks"] = clocks.stop()
        out["full"] = fp
        out["alpha_end"] = a
    return out


def clocks_of(r):
    """Clock samples of the headline form: the K-step window is shorter than
    the 200 ms sampling period at 256^3, so the full-period run that
    follows it (seconds of the same step) supplies the samples; the
    window's own samples are kept beside them."""
    win = r["clk"]
    if "full" not in r:
        return win
    c = dict(r["full"]["clocks"])
    c["sampled_over"] = "full-period run of the headline form (directly after the window)"
    c["window"] = win
    return c


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

    mesh, alpha0, hflow, dt, steps_full, tsetup = deformation_workload(args.n)
    flow = ScaledFlow(hflow.phi0, hflow.U0, mesh.n_boundary_faces, dev, hflow.period)
    torch.cuda.synchronize(dev)

    head = args.precision
    forms = [head] + ([] if args.single_form else [f for f in FORMS if f != head])
    res = {}
    for f in forms:
        res[f] = run_form(f, mesh, alpha0, flow, dt, steps_full, args, dev, dist, local)
        res[f].pop("alpha_end", None)
        if f != head:
            res[f].pop("g")
    r = res[head]
    ms, kt, clk = r["ms"], r["kt"], r["clk"]
    value = replicas.replica_throughput(world, mesh.n_cells, args.steps, ms)
    # launches of the library's kernels in the timed window: the kernel pass
    # runs the same K steps (its counters start after the window)
    launches = sum(v[1] for v in kt.values())

    # --- roofline of the update kernel (event-timed launches of the kernel pass)
    hbm, src = peaks()
    kavg = {k: (v[0] / max(1, v[1])) for k, v in kt.items()}
    ktot = {k: v[0] for k, v in kt.items() if k not in ("faceFlatness", "faceFull")}
    dominant = max(ktot, key=ktot.get)
    nc = mesh.n_cells
    upd_ms = kavg["update"]
    upd_bytes = BULK_BYTES_PER_CELL * nc
    traffic, tsrc = update_traffic(args.n)
    step_ms = ms / args.steps
    roof = {"bound": "hbm", "kernel": "update", "achieved": upd_bytes / (upd_ms * 1e-3) / 1e9,
            "peak": hbm, "unit": "GB/s", "frac": None, "traffic": traffic, "traffic_source": tsrc,
            "bytes_per_launch": upd_bytes, "peak_source": f"{src} hbm_gbs (burst copy)",
            "timing": "CUDA events around each update launch in the kernel pass (K steps after the window)",
            "dominant_kernel": dominant,
            # whole step against HBM: the 96 B/cell bulk bytes over the step time
            "step_achieved_gbs": upd_bytes / (step_ms * 1e-3) / 1e9,
            "step_frac": upd_bytes / (step_ms * 1e-3) / 1e9 / hbm,
            "kernel_ms_per_step": {k: round(v / args.steps, 4) for k, v in ktot.items()},
            "kernel_share": {k: round(v / max(1e-12, sum(ktot.values())), 4) for k, v in ktot.items()}}
    roof["frac"] = roof["achieved"] / hbm

    forms_out = {}
    for f, rf in res.items():
        fms = rf["ms"] / args.steps
        forms_out[f] = {"window": {"value": replicas.replica_throughput(world, nc, args.steps, rf["ms"]),
                                   "ms_per_step": fms, "steps": args.steps,
                                   "step_frac_hbm": BULK_BYTES_PER_CELL * nc / (fms * 1e-3) / 1e9 / hbm},
                        "kernel_ms_per_step": {k: round(v[0] / args.steps, 4) for k, v in rf["kt"].items()
                                               if k not in ("faceFlatness", "faceFull")},
                        "stats": rf["stats"]}
        if "full" in rf:
            fp = rf["full"]
            fp["step_frac_hbm"] = BULK_BYTES_PER_CELL * nc / (fp["ms_per_step"] * 1e-3) / 1e9 / hbm
            forms_out[f]["full_period"] = fp
    if "plain" in res:
        for f in res:
            if f == "plain":
                continue
            forms_out[f]["speedup_vs_plain_window"] = res["plain"]["ms"] / res[f]["ms"]
            if "full" in res[f] and "full" in res["plain"]:
                forms_out[f]["speedup_vs_plain_full_period"] = (res["plain"]["full"]["device_s"]
                                                                / res[f]["full"]["device_s"])

    # --- end to end through the host-buffer C ABI (pinned buffers, copies timed)
    e2e = run_e2e(r["g"], mesh, alpha0, hflow, dt, args, dev) if not args.no_e2e else None
    r.pop("g")

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {"plain": "f64", "mixed": "f64+f32", "learned": "f64+f32+bf16"}[head], "data": "synthetic",
        "form": FORM_NAMES[head], "config": config(args, mesh),
        "roofline": roof, "gpu_launches": launches, "clocks": clocks_of(r), "forms": forms_out,
        "stats": dict(r["stats"], setup_s={"mesh_and_fields": round(tsetup, 1), "create": round(r["tcreate"], 1)}),
    }
    if "full" in r:
        line["accuracy"] = {
            "case": f"{args.n}^3 hex deformation (T=6), sphere R=0.15, Courant 0.5, t=0..3, {steps_full} steps "
                    f"(the full-period runs above)",
            **{f: {k: res[f]["full"][k] for k in ("shape_error_L1", "volume_drift", "max_bound_violation")}
               for f in res if "full" in res[f]}}
    if e2e:
        line["e2e"] = e2e
    if rank == 0 and world == 1 and not args.no_unstructured:
        line["configs"] = {"unstructured": unstructured_case(dev, forms)}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(mesh, alpha0, hflow, dt)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def run_e2e(g, mesh, alpha0, flow, dt, args, dev):
    """K steps through simplic_reconstruct + simplic_advect with pinned host
    buffers, the way a solver calls it: its alpha, phi and U arrays are the
    same buffers every step, updated in place between the calls (the
    velocity update is the caller's work and is not timed).  Timed: the two
    calls of every step, which copy alpha, phi, U, U_boundary to the device
    and alpha back.  The split: the device time of the library's calls (its
    timers) and the rest (copies and host work), with the link bandwidth
    measured beside it by one pinned copy of each direction."""
    import torch

    from geometricvofext_gb300 import harness as H

    K = max(1, min(args.steps, args.e2e_steps))
    nc, nf, nfb = mesh.n_cells, mesh.n_faces, mesh.n_boundary_faces
    keep = []

    def pinned(shape):
        t = torch.empty(shape, dtype=torch.float64, pin_memory=True)
        keep.append(t)
        return t.numpy()

    alpha, phi, U, Ub = pinned(nc), pinned(nf), pinned((nc, 3)), pinned((nfb, 3))
    alpha[:] = alpha0
    Ub[:] = 0.0

    def fill(k):
        f = H.time_factor((k + 1) * dt, dt, flow.period)
        np.multiply(flow.phi0, f, out=phi)
        np.multiply(flow.U0, f, out=U)

    fill(0)
    g.reconstruct_ptr(alpha)  # one untimed step
    g.advect_inplace(alpha, phi, U, dt, U_boundary=Ub)
    torch.cuda.synchronize(dev)
    r0, a0, _ = g.timers()
    el = 0.0
    for k in range(1, K + 1):
        fill(k)
        s = time.perf_counter()
        g.reconstruct_ptr(alpha)                                  # H2D alpha
        g.advect_inplace(alpha, phi, U, dt, U_boundary=Ub)        # H2D phi, U, Ub; D2H alpha
        el += time.perf_counter() - s
    r1, a1, _ = g.timers()
    dev_s = (r1 - r0) + (a1 - a0)
    h2d = 8 * nc + 8 * nf + 24 * nc + 24 * nfb
    d2h = 8 * nc
    # the link: one pinned copy of each direction of the same sizes
    hsrc = torch.empty(h2d // 8, dtype=torch.float64, pin_memory=True)
    ddst = torch.empty(h2d // 8, dtype=torch.float64, device=dev)
    hout = torch.empty(d2h // 8, dtype=torch.float64, pin_memory=True)
    st = torch.cuda.Stream(dev)
    bw = {}
    for name, (dst, srcb, nbytes) in {"h2d": (ddst, hsrc, h2d), "d2h": (hout, ddst[: d2h // 8], d2h)}.items():
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        best = None
        for _ in range(3):
            with torch.cuda.stream(st):
                e0.record(st)
                dst.copy_(srcb, non_blocking=True)
                e1.record(st)
            st.synchronize()
            t = e0.elapsed_time(e1) * 1e-3
            best = t if best is None else min(best, t)
        bw[name] = nbytes / best / 1e9
    del hsrc, ddst, hout, keep
    return {"value": nc * K / el, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "steps": K, "path": "simplic_reconstruct + simplic_advect (host pinned buffers reused per step)",
            "ms_per_step": 1e3 * el / K, "device_ms_per_step": 1e3 * dev_s / K,
            "copy_and_host_ms_per_step": 1e3 * (el - dev_s) / K,
            "effective_copy_gbs": (h2d + d2h) / max(1e-12, el - dev_s) / 1e9,
            "link_gbs": {k: round(v, 1) for k, v in bw.items()},
            "link_bound_ms_per_step": 1e3 * (h2d / (bw["h2d"] * 1e9) + d2h / (bw["d2h"] * 1e9))}


def unstructured_case(dev, forms, steps_cap=None):
    """The unstructured-mesh configuration: 96^3 hex with interior points
    jittered by +-0.2 h (seed 12345) and 64^3 hexes split into 6 tets,
    sphere R=0.15 at (0.35, 0.35, 0.35) in the deformation field T=6,
    Courant 0.5 (fixed step), t = 0 .. 3; per form the device-timed
    throughput and the errors at t = 3."""
    import torch

    from geometricvofext_gb300 import harness as H, meshgen as mg

    out = {}
    for kind, n in (("jitter", 96), ("tet", 64)):
        mesh = mg.make_mesh(kind, n, seed=12345)
        alpha0 = H.sphere_alpha(mesh, (0.35, 0.35, 0.35), 0.15)
        hf = H.DeformationFlow(mesh, period=6.0)
        dt = H.cfl_delta_t(mesh, hf.phi0, 0.5)
        steps = int(math.ceil(3.0 / dt - 1e-9))
        dt = 3.0 / steps
        if steps_cap:
            steps = min(steps, steps_cap)
        flow = ScaledFlow(hf.phi0, hf.U0, mesh.n_boundary_faces, dev, hf.period)
        vol0 = float(np.sum(alpha0 * mesh.V))
        res = {"mesh": f"{n}^3 hex" + (" jittered +-0.2h (seed 12345)" if kind == "jitter" else " x 6 tets"),
               "cells": mesh.n_cells, "steps": steps}
        plain_alpha = None
        for f in ["plain"] + [x for x in forms if x != "plain"]:
            stream = torch.cuda.Stream(dev)
            g = make_handle(f, mesh, stream.cuda_stream)
            a, fp = full_period(g, flow, alpha0, mesh, dt, steps, stream, vol0)
            if f == "plain":
                plain_alpha = a
            else:
                fp["L1_vs_plain"] = float(np.sum(np.abs(a - plain_alpha) * mesh.V) / vol0)
            res[f] = fp
            del g
        out[kind] = res
    return out


def run_scale(args):
    """The 320^3 scale case: seeded union of 200 spheres (R 0.01 .. 0.04)
    plus a slab alpha = 1 for z < 0.2, deformation field with T = 6, 500
    steps at Courant 0.5; per form the device-timed throughput, the HBM
    fraction of the bulk bytes, the volume drift and the L1 difference of
    the final field from the plain FP64 form's."""
    import torch

    from geometricvofext_gb300 import harness as H, meshgen as mg

    dev = torch.device("cuda", 0)
    n = args.n if args.n != 256 else 320
    t0 = time.time()
    mesh = mg.hex_mesh(n)
    alpha0 = H.spheres_and_slab_alpha(mesh)
    hf = H.DeformationFlow(mesh, period=6.0)
    dt = H.cfl_delta_t(mesh, hf.phi0, 0.5)
    tsetup = time.time() - t0
    steps = args.scale_steps
    flow = ScaledFlow(hf.phi0, hf.U0, mesh.n_boundary_faces, dev, hf.period)
    vol0 = float(np.sum(alpha0 * mesh.V))
    hbm, src = peaks()
    out = {}
    plain_alpha = None
    for f in ["plain"] + [x for x in FORMS if x != "plain"]:
        stream = torch.cuda.Stream(dev)
        g = make_handle(f, mesh, stream.cuda_stream)
        for _ in range(3):  # warm-up on the initial field
            flow.set(dt, dt, stream)
            g.set_alpha(alpha0)
            g.reconstruct_resident()
            g.advect_resident(flow.phi, flow.U, dt, U_boundary=flow.Ub)
        g.synchronize()
        clocks = ClockSampler(0)
        a, fp = full_period(g, flow, alpha0, mesh, dt, steps, stream, vol0)
        fp["clocks"] = clocks.stop()
        fp["step_frac_hbm"] = BULK_BYTES_PER_CELL * mesh.n_cells / (fp["ms_per_step"] * 1e-3) / 1e9 / hbm
        fp["mixed_cells_last_step"] = g.stats()[0]
        if f == "plain":
            plain_alpha = a
        else:
            fp["L1_vs_plain"] = float(np.sum(np.abs(a - plain_alpha) * mesh.V) / vol0)
            fp["speedup_vs_plain"] = out["plain"]["device_s"] / fp["device_s"]
        if f == "learned":
            fp["network_rows_overflow"] = g.network_overflow()
        del fp["shape_error_L1"]  # no reference shape at t = 500 dt; L1_vs_plain instead
        out[f] = fp
        del g
    line = {"metric": METRIC, "value": out["learned"]["value"], "unit": UNIT, "n_gpus": 1, "steps": steps,
            "higher_is_better": True, "dtype": "f64+f32+bf16", "data": "synthetic",
            "case": "scale", "config": {"workload": f"SimPLIC step, {n}^3 hex, 200 seeded spheres (R 0.01-0.04, "
                                                   f"seed 2024) + slab z<0.2, deformation field T=6, Courant 0.5, "
                                                   f"{steps} steps", "cells": mesh.n_cells, "controls": CONTROLS_TEXT},
            "peak_hbm_gbs": hbm, "peak_source": src, "forms": out, "setup_s": round(tsetup, 1)}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--case", default="deformation", choices=["deformation", "scale", "unstructured"])
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--precision", default="learned", choices=list(FORMS))
    ap.add_argument("--single-form", action="store_true", help="time the headline form only")
    ap.add_argument("--no-full-period", action="store_true", help="skip the t=0..3 runs")
    ap.add_argument("--no-unstructured", action="store_true", help="skip the unstructured-mesh configuration")
    ap.add_argument("--scale-steps", type=int, default=500)
    ap.add_argument("--t0", type=float, default=0.0,
                    help="start the timed window at this time of the period (steps before it untimed)")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.steps < 1:
        raise SystemExit("steps >= 1 required")
    args.warmup = max(3, args.warmup)  # at least three warm-up steps
    if args.impl == "reference":
        run_reference(args)
    elif args.case == "scale":
        run_scale(args)
    elif args.case == "unstructured":
        import torch

        print(json.dumps({"metric": METRIC, "unit": UNIT, "case": "unstructured",
                          "configs": unstructured_case(torch.device("cuda", 0), list(FORMS))}), flush=True)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
