"""Benchmark: split-step KDK steps/s of the Schroedinger-Poisson solver on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl native|reference]

Default workload (N=1): 384^3, L = 40, complex FP32 psi, dt = dx^2/6, Strang KDK
with the time-dependent Hernquist tidal tensor (host-integrated FP64 orbit) and
1e5 static Plummer baryons CIC-deposited every step; seeded synthetic input.

One JSON line is printed by rank 0:
* value      steps/s with psi resident in HBM (one wdm_step_async call of K steps,
             CUDA events on the library's stream; psi is 453 MB > L2 so no flush)
* e2e        steps/s through the C ABI with host buffers: per step the pinned
             host psi is copied in (wdm_set_psi), one step runs (wdm_step) and
             psi is copied back (wdm_get_psi)
* roofline   the dominant pass: its algorithmic bytes per launch / its mean
             event-timed duration, against the measured HBM copy bandwidth
* cpu_baseline  the FP64 oracle (numpy + scipy.fft, all host cores) on a
             bounded sample of the same workload
--impl reference times that CPU restatement alone (the reference is Julia and
cannot run here; its FFTW CPU path is restated by the oracle).
Under torchrun (N>1) every rank runs an independent replica (one halo per GPU;
the path has no data exchange), value = total steps/s over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

B_ALG_PER_CELL = 192.0  # 4 C2C 3D FFTs x 3 axis passes x (8 B read + 8 B write) of complex64

# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per launch of each
# pass, read from the ncu capture summarised in this file, together with the
# hash of the kernel sources it was captured on.
TRAFFIC_FILE = os.path.join(ROOT, "profiles", "step384_traffic.json")
CSRC = os.path.join(ROOT, "wavedm.jl_gb300", "csrc")


def kernel_source_hash(csrc=None):
    """sha256 (first 16 hex digits) of the kernel sources (every csrc file but the
    host-only pipeline wdm_api.cu) with comments and blank space removed, the key a
    traffic capture is valid for (an edit of a comment does not change it)."""
    import hashlib
    import re

    csrc = csrc or CSRC
    h = hashlib.sha256()
    for f in sorted(os.listdir(csrc)):
        if f.endswith((".cu", ".cuh", ".h")) and f != "wdm_api.cu":
            h.update(f.encode())
            with open(os.path.join(csrc, f), encoding="utf-8") as fh:
                text = fh.read()
            text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
            text = re.sub(r"//[^\n]*", " ", text)
            h.update(" ".join(text.split()).encode())
    return h.hexdigest()[:16]


def ncu_traffic(pass_name, n, workload, sched):
    """(DRAM bytes per launch of the pass, provenance) from the committed capture,
    or (None, reason) when the capture does not cover this run."""
    if n != 384 or workload != 3 or not sched:
        return None, "no capture of this workload"
    if not os.path.exists(TRAFFIC_FILE):
        return None, "no capture file"
    with open(TRAFFIC_FILE) as f:
        cap = json.load(f)
    impl = {"kick_xfft_fwd": "x_kick", "kick_final": "x_kick", "psi_y_fwd": "psi_y", "psi_z_drift": "psi_z",
            "psi_y_inv": "psi_y", "psi_x_inv_rho": "x_rho_b", "rho_y_fwd": "h_y", "rho_z_poisson": "h_z",
            "phi_y_inv": "h_y"}.get(pass_name)
    if impl is None or impl not in sched:
        return None, "pass not captured"
    v = cap["passes"].get(f"{pass_name}/{sched[impl]['impl']}")
    if v is None:
        return None, "pass and implementation not captured"
    same = cap.get("kernel_source_hash") == kernel_source_hash()
    return v, {"capture": os.path.relpath(TRAFFIC_FILE, ROOT), "command": cap.get("command"),
               "kernels_unchanged_since_capture": same}


def free_port():
    import socket

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def launch_ranks(argv, n):
    """Run this script again as n ranks on this node, one process per GPU, the
    way the torchrun launch does; returns the launcher's exit status."""
    # the launcher's own parser would take an abbreviation such as --n for one of its options
    argv = ["--grid" + a[3:] if a == "--n" or a.startswith("--n=") else a for a in argv]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), os.path.abspath(__file__), *argv]
    return subprocess.call(cmd)


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.f = None

    def start(self):
        """Start sampling every 10 ms (a 20-step timed region at 384^3 lasts
        about 30 ms); returns once the first sample is in, so the samples cover
        a timed region that starts afterwards."""
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "10"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < 5.0 and self.proc.poll() is None:
            if os.path.getsize(self.f.name) > 0:
                break
            time.sleep(0.01)

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
                for nm, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def max_over_ranks(x, world):
    """The largest x over the ranks: a job of independent replicas ends with its slowest rank."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(steps, world, seconds):
    """Whole-job steps/s of `world` replicas that each ran `steps` steps in `seconds` (the max over ranks)."""
    return steps * world / seconds


def workload_config(wl, args, world):
    """The config object of a bench line (the same for both arms)."""
    N = wl["n"]
    return {"workload": wl["name"], "grid": [N, N, N], "box": wl["L"], "dt": wl["dt"], "mode": args.mode,
            "phase_mode": args.phase, "tidal": wl["tidal"] is not None,
            "baryon_particles": 0 if wl["particles"] is None else len(wl["particles"][1]),
            "baryons": None if wl["particles"] is None else
            "static: one CIC deposit before the timed steps, added to the density of every step's Poisson solve "
            "(the reference computes the static baryons' potential once, src/simulation_main.jl:248-261)",
            "l2": "inputs larger than L2 (psi 8 B/cell)", "parallelism": f"replicas x{world}"}


def setup_context(wdm, wl, phase_mode, steps_total):
    N, L = wl["n"], wl["L"]
    ctx = wdm.SPEContext((N, N, N), (L, L, L), poisson_coeff=wl["poisson_coeff"], phase_mode=phase_mode)
    psi0 = wl["psi0"].astype(np.complex64)
    ctx.set_psi(psi0)
    if wl["tidal"] is not None:
        ctx.set_tidal(wl["tidal"](np.arange(steps_total + 1) * wl["dt"]))
    if wl["particles"] is not None:
        ctx.set_particles(*wl["particles"])
    return ctx, psi0


def run_native(args, rank, world):
    import torch

    import wavedm_gb300 as wdm

    wdm.build_library()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    wl = wdm.ics.workload(args.workload, n=args.n)
    N, dt = wl["n"], wl["dt"]
    K, W = args.steps, args.warmup
    ctx, psi0 = setup_context(wdm, wl, args.phase, max(K, W, 1))
    stream = torch.cuda.ExternalStream(ctx.stream)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # warm-up (also builds the potential of psi0)
    ctx.step(W, dt, mode=args.mode)
    tide = wl["tidal"](np.arange(K + 1) * dt) if wl["tidal"] is not None else None
    # per-pass breakdown: a run of the same workload with every pass bracketed by events
    n_brk = min(K, 50)
    ctx.set_psi(psi0)
    ctx.get_phi()
    ctx.set_tidal(tide)
    ctx.set_profiling(True)
    ctx.step(n_brk, dt, mode=args.mode)
    prof = ctx.profile()
    ctx.set_profiling(False)
    top_name = max(prof.items(), key=lambda kv: kv[1]["ms"])[0]
    # timed region: events around the whole run and around the dominant pass only
    ctx.set_psi(psi0)
    ctx.get_phi()  # potential of psi0 outside the timed region
    ctx.set_tidal(tide)
    ctx.set_profile_mask([top_name])
    ctx.set_profiling(True)
    torch.cuda.synchronize()
    barrier()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", 0)))
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = ctx.launch_count
    torch.cuda.synchronize()
    ev0.record(stream)
    ctx.step(K, dt, mode=args.mode, sync=False)
    ev1.record(stream)
    torch.cuda.synchronize()
    launches = ctx.launch_count - l0
    clk = clocks.stop()
    barrier()
    ms = ev0.elapsed_time(ev1)
    prof_top = ctx.profile()[top_name]
    ctx.set_profiling(False)
    ctx.set_profile_mask(None)
    ms = max_over_ranks(ms, world)
    value = replica_throughput(K, world, ms / 1e3)

    # e2e: host psi in, one step, psi out, per step (pinned host buffers)
    e2e = None
    if not args.no_e2e:
        host_in = torch.from_numpy(psi0.view(np.float32).reshape(-1)).pin_memory()
        host_out = torch.empty_like(host_in).pin_memory()
        ne = max(1, min(K, args.e2e_steps))
        ctx.set_tidal(wl["tidal"](np.arange(2) * dt) if wl["tidal"] is not None else None)
        import ctypes as C

        lib = ctx.lib
        for _ in range(2):
            wdm._abi.check(lib.wdm_set_psi(ctx.handle, C.c_void_p(host_in.data_ptr()), 0), ctx.handle)
            wdm._abi.check(lib.wdm_step(ctx.handle, 1, dt, 0.0, 0), ctx.handle)
            wdm._abi.check(lib.wdm_get_psi(ctx.handle, C.c_void_p(host_out.data_ptr()), 0), ctx.handle)
        barrier()
        t0 = time.perf_counter()
        for _ in range(ne):
            wdm._abi.check(lib.wdm_set_psi(ctx.handle, C.c_void_p(host_in.data_ptr()), 0), ctx.handle)
            wdm._abi.check(lib.wdm_step(ctx.handle, 1, dt, 0.0, 0), ctx.handle)
            wdm._abi.check(lib.wdm_get_psi(ctx.handle, C.c_void_p(host_out.data_ptr()), 0), ctx.handle)
        el = time.perf_counter() - t0
        el = max_over_ranks(el, world)
        nb = psi0.nbytes
        e2e = {"value": ne * world / el, "unit": "steps/s", "h2d_bytes_per_step": nb, "d2h_bytes_per_step": nb,
               "steps": ne, "calls_per_step": ["wdm_set_psi(host)", "wdm_step(1)", "wdm_get_psi(host)"]}
    # The reference loop with its per-step diagnostics: K(dt/2) D(dt) per
    # iteration (src/simulation_main.jl:538-547), then findmax, the radii
    # quantiles, R and the mass (:551-558, :641-653), here on the device.
    loop = None
    if not args.no_e2e:
        nl = max(1, min(K, args.e2e_steps))
        ctx.set_psi(psi0)
        for _ in range(2):
            ctx.step(1, dt, mode="reference_loop")
            ctx.diagnostics()
        barrier()
        t0 = time.perf_counter()
        for _ in range(nl):
            ctx.step(1, dt, mode="reference_loop")
            ctx.diagnostics()
        el = max_over_ranks(time.perf_counter() - t0, world)
        loop = {"value": nl * world / el, "unit": "steps/s", "steps": nl,
                "calls_per_step": ["wdm_step(1, reference_loop)", "wdm_diagnostics"]}
    sched = ctx.line_schedule()
    ctx.close()

    # roofline of the dominant pass
    peak, peak_kind = measured_peaks()
    name, p = top_name, prof_top  # the dominant pass, timed inside the timed region
    mean_ms = p["ms"] / max(p["launches"], 1)
    achieved = p["bytes_per_launch"] / (mean_ms / 1e3) / 1e9
    passes = {k: {"launches": v["launches"], "ms": round(v["ms"], 4),
                  "share": round(v["ms"] / max(sum(q["ms"] for q in prof.values()), 1e-12), 4),
                  "GBps": round(v["bytes_per_launch"] / (v["ms"] / max(v["launches"], 1) / 1e3) / 1e9, 1)}
              for k, v in prof.items() if v["launches"]}
    ncell = N ** 3
    traffic, traffic_src = ncu_traffic(name, N, args.workload, sched)
    rec = {
        "metric": f"KDK steps/s at {N}^3 (Strang, complex FP32 psi, {args.phase} phases)",
        "value": round(value, 3),
        "unit": "steps/s",
        "n_gpus": world,
        "steps": K,
        "warmup": W,
        "ms_per_step": round(ms / K, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "c64",
        "data": "synthetic (seeded soliton + 4096-plane-wave NFW halo; Hernquist tide; 1e5 Plummer baryons)",
        "config": workload_config(wl, args, world),
        "roofline": {"bound": "hbm", "kernel": name, "achieved": round(achieved, 1), "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "traffic": traffic, "traffic_source": traffic_src,
                     "bytes_per_launch": p["bytes_per_launch"], "mean_launch_ms": round(mean_ms, 5)},
        "step_effective": {"B_alg_per_cell": B_ALG_PER_CELL,
                           "GBps": round(B_ALG_PER_CELL * ncell * value / world / 1e9, 1),
                           "frac_of_peak": round(B_ALG_PER_CELL * ncell * value / world / 1e9 / peak, 4)},
        "passes": passes,
        "line_schedule": sched,
        "gpu_launches": int(launches),
        "e2e": e2e,
        "loop_with_diagnostics": loop,
        "clocks": clk,
    }
    return rec


ENSEMBLE_FULL = {64: 96, 96: 24, 128: 8}
ENSEMBLE_SMALL = {64: 8, 96: 2, 128: 1}  # few halos per size: grids that do not fill the GPU


def ensemble_contexts(wdm, phase, counts=None):
    """Workload 4: one context per grid size, batch = halos of that size, per-halo tides
    (counts: halos per size, the first of workload 4's seeded halos of each size)."""
    counts = counts or ENSEMBLE_FULL
    members = wdm.ics.ensemble_members()
    sizes = sorted({m[0] for m in members})
    ctxs, inputs, dts = [], [], []
    for N in sizes:
        mem = [m for m in members if m[0] == N][: counts[N]]
        L = mem[0][1]
        ctx = wdm.SPEContext((N, N, N), (L, L, L), poisson_coeff=1.0, phase_mode=phase, batch=len(mem))
        psi = np.stack([m[2] for m in mem]).astype(np.complex64)
        ctx.set_psi(psi)
        ctx.set_tidal(np.stack([m[3] for m in mem]), per_item=True)
        ctxs.append(ctx)
        inputs.append(psi)
        dts.append(wdm.ics.dt_for(N, L))
    return ctxs, inputs, dts, sizes


def run_ensemble(args, rank, world, counts=None):
    """96 x 64^3 + 24 x 96^3 + 8 x 128^3 halos (or `counts` per size) advanced by one
    captured CUDA graph replay per call."""
    import ctypes as C

    import torch

    import wavedm_gb300 as wdm

    wdm.build_library()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    K, W = args.steps, args.warmup
    counts = counts or ENSEMBLE_FULL
    ctxs, inputs, dts, sizes = ensemble_contexts(wdm, args.phase, counts)
    psi_mb = sum(p.nbytes for p in inputs) / 1e6
    ncell = sum(c.batch * int(np.prod(c.n)) for c in ctxs)
    ens = wdm.Ensemble(ctxs)
    # warm-up: capture and run the K-step graph (and W more steps if W > K)
    ens.step(K, dts)
    if W > K:
        ens.step(W - K, dts)
    for c, p in zip(ctxs, inputs):
        c.set_psi(p)
    for c in ctxs:
        c.get_phi()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", 0)))
    clocks.start()
    gs = torch.cuda.ExternalStream(ens.stream)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = ens.launch_count
    torch.cuda.synchronize()
    ev0.record(gs)
    ens.step(K, dts, sync=False)  # one graph replay on the group's stream
    ev1.record(gs)
    torch.cuda.synchronize()
    el = ev0.elapsed_time(ev1) / 1e3
    launches = ens.launch_count - l0
    clk = clocks.stop()
    sched, sched_ms = ens.schedule
    if not all(c.is_finite() for c in ctxs):
        raise RuntimeError("ensemble state became non-finite")
    el = max_over_ranks(el, world)
    value = replica_throughput(K, world, el)
    # per-pass profile from one eager step of each member
    prof = {}
    for c in ctxs:
        c.set_profiling(True)
        c.step(1, dts[ctxs.index(c)])
        for k, v in c.profile().items():
            if v["launches"]:
                q = prof.setdefault(k, {"launches": 0, "ms": 0.0, "bytes": 0.0})
                q["launches"] += v["launches"]
                q["ms"] += v["ms"]
                q["bytes"] += v["bytes_per_launch"] * v["launches"]
        c.set_profiling(False)
    e2e = None
    if not args.no_e2e:
        host_in = [torch.from_numpy(p.view(np.float32).reshape(-1)).pin_memory() for p in inputs]
        host_out = [torch.empty_like(h).pin_memory() for h in host_in]
        lib = ens.lib
        ne = max(1, min(K, args.e2e_steps))

        def one():
            for c, h in zip(ctxs, host_in):
                wdm._abi.check(lib.wdm_set_psi(c.handle, C.c_void_p(h.data_ptr()), 0), c.handle)
            ens.step(1, dts)
            for c, h in zip(ctxs, host_out):
                wdm._abi.check(lib.wdm_get_psi(c.handle, C.c_void_p(h.data_ptr()), 0), c.handle)

        one()
        t0 = time.perf_counter()
        for _ in range(ne):
            one()
        e_el = time.perf_counter() - t0
        nb = sum(p.nbytes for p in inputs)
        e2e = {"value": ne * world / e_el, "unit": "ensemble steps/s", "h2d_bytes_per_step": nb,
               "d2h_bytes_per_step": nb, "steps": ne,
               "calls_per_step": ["wdm_set_psi(host) x3", "wdm_group_step(1)", "wdm_get_psi(host) x3"]}
    ens.close()
    for c in ctxs:
        c.close()
    peak, peak_kind = measured_peaks()
    name, p = max(prof.items(), key=lambda kv: kv[1]["ms"])
    mean_ms = p["ms"] / p["launches"]
    achieved = (p["bytes"] / p["launches"]) / (mean_ms / 1e3) / 1e9
    halos = sum(c.batch for c in ctxs)
    return {
        "metric": "ensemble KDK steps/s (" + " + ".join(f"{counts[n]}x{n}^3" for n in sizes)
                  + " halos, one CUDA graph replay per call)",
        "value": round(value, 3), "unit": "ensemble steps/s", "n_gpus": world, "steps": K, "warmup": max(W, K),
        "ms_per_step": round(el / K * 1e3, 4), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64", "data": "synthetic (seeded solitons rc~U[0.8,2] + 1024-wave halos; tidal amp~U[0,0.05])",
        "config": {"workload": "ensemble_" + "_".join(f"{n}x{counts[n]}" for n in sizes), "sizes": sizes,
                   "halos": halos, "cells": ncell,
                   "dts": dts, "phase_mode": args.phase, "l2": (f"inputs larger than L2 ({psi_mb:.0f} MB of psi)" if psi_mb > 129 else
                          f"psi ({psi_mb:.0f} MB) fits in the 129 MB L2: the steps of a call run L2-resident, "
                          "as such a small ensemble does in use; no flush"),
                   "parallelism": f"replicas x{world}"},
        "halo_steps_per_s": round(value * halos, 1),
        "roofline": {"bound": "hbm", "kernel": name, "achieved": round(achieved, 1), "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": None},
        "step_effective": {"B_alg_per_cell": B_ALG_PER_CELL,
                           "GBps": round(B_ALG_PER_CELL * ncell * value / world / 1e9, 1)},
        "passes": {k: {"launches": v["launches"], "ms": round(v["ms"], 4)} for k, v in prof.items()},
        "schedule": {"chosen": sched, "ms_two_steps": sched_ms,
                     "what": "graph: the members' pass launches in one captured graph; persistent: one cooperative "
                             "kernel for every pass, member and step of a call; streams: the pass launches of each "
                             "member on its own stream inside the graph"},
        "gpu_launches": int(launches), "launches_per_step": round(launches / K, 3), "e2e": e2e, "clocks": clk,
    }


def oracle_setup(wl, nsteps):
    from oracle import spe

    N, L, dt = wl["n"], wl["L"], wl["dt"]
    g = spe.Grid((N, N, N), (L, L, L))
    rho_b = spe.cic_deposit(g, *wl["particles"]) if wl["particles"] is not None else None
    sched = wl["tidal"](np.arange(nsteps + 2) * dt) if wl["tidal"] is not None else None
    tidal = (lambda t: tuple(sched[int(round(t / dt))])) if sched is not None else None
    phys = spe.Physics(poisson_coeff=wl["poisson_coeff"], rho_b=rho_b, tidal=tidal)
    return spe, g, phys


def time_oracle(wl, budget_s, max_steps, warm=1):
    """FP64 oracle Strang steps on all host cores; returns (steps/s, steps timed, cores)."""
    spe, g, phys = oracle_setup(wl, max_steps + warm)
    dt = wl["dt"]
    psi = wl["psi0"].astype(np.complex64).astype(np.complex128)
    for s in range(warm):
        psi = spe.kdk_step(psi, g, phys, s * dt, dt)
    t0 = time.perf_counter()
    n = 0
    while n < max_steps:
        psi = spe.kdk_step(psi, g, phys, (warm + n) * dt, dt)
        n += 1
        if time.perf_counter() - t0 > budget_s:
            break
    el = time.perf_counter() - t0
    return n / el, n, spe.WORKERS


def time_oracle_loop(wl, budget_s):
    """The reference loop on the host cores: one literal K(dt/2) D(dt) iteration of
    the FP64 oracle plus the loop's per-step diagnostics (the potential, findmax,
    the weighted radii quantiles, R, mass), until the budget is spent."""
    spe, g, phys = oracle_setup(wl, 4)
    dt = wl["dt"]
    psi = wl["psi0"].astype(np.complex64).astype(np.complex128)
    t0 = time.perf_counter()
    n = 0
    while True:
        psi = spe.kdk_step(psi, g, phys, n * dt, dt, mode="reference_loop")
        spe.loop_diagnostics(psi, spe.potential(psi, g, phys, (n + 1) * dt), g)
        spe.mass(psi, g)
        n += 1
        if time.perf_counter() - t0 > budget_s or n >= 3:
            break
    return n / (time.perf_counter() - t0), n, spe.WORKERS


def adjoint_part(wdm, phase, N=128, nsteps=200, ck=20, reps=1):
    """Workload 5: adjoint of nsteps Strang steps at N^3 (checkpoints every ck) against the forward run."""
    import torch

    ics = wdm.ics
    L = 20.0
    dt = ics.dt_for(N, L)
    D = np.array([2.0, -1.0, -1.0, 0.0, 0.0, 0.0])
    amp, rc = 0.02, 1.2
    psi0 = ics.soliton_halo_ic((N, N, N), (L, L, L), rc=rc, rng=ics.rng_for(5)).astype(np.complex64)
    target = (np.abs(ics.soliton_halo_ic((N, N, N), (L, L, L), rc=1.1 * rc, rng=ics.rng_for(5))) ** 2
              ).astype(np.float32)
    ctx = wdm.SPEContext((N, N, N), (L, L, L), poisson_coeff=1.0, phase_mode=phase)
    ctx.set_psi(psi0)
    ctx.set_tidal([amp * D])
    rho_d = torch.from_numpy(target).cuda()
    grad_d = torch.empty(psi0.shape, dtype=torch.complex64, device="cuda")
    # warm-up of both
    ctx.step(nsteps, dt)
    ctx.set_psi(psi0)
    ctx.adjoint(nsteps, dt, rho_d, ckpt_every=ck, tidal_dir=D, grad_out=grad_d)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        ctx.set_psi(psi0)
        ctx.step(nsteps, dt)
    t_fwd = (time.perf_counter() - t0) / reps
    l0 = ctx.launch_count
    t0 = time.perf_counter()
    for _ in range(reps):
        ctx.set_psi(psi0)
        loss, _, da = ctx.adjoint(nsteps, dt, rho_d, ckpt_every=ck, tidal_dir=D, grad_out=grad_d)
    t_adj = (time.perf_counter() - t0) / reps
    launches = (ctx.launch_count - l0) // reps
    # where the adjoint's time goes: one more run with per-pass events (not timed above)
    ctx.set_psi(psi0)
    ctx.set_profiling(True)
    ctx.adjoint(nsteps, dt, rho_d, ckpt_every=ck, tidal_dir=D, grad_out=grad_d)
    prof = {k: {"launches": v["launches"], "ms": round(v["ms"], 3)} for k, v in ctx.profile().items() if v["launches"]}
    ctx.set_profiling(False)
    ctx.close()
    return {"ratio": round(t_adj / t_fwd, 3), "grid": [N, N, N], "steps": nsteps, "ckpt_every": ck, "dt": dt,
            "repeats": reps, "forward_steps_per_s": round(nsteps / t_fwd, 2),
            "adjoint_steps_per_s": round(nsteps / t_adj, 2), "loss": float(loss), "dL_damp": float(da),
            "gpu_launches": int(launches), "passes_adjoint_run": prof,
            "timing": "host wall clock around synchronous calls, whole runs (forward: set_psi + wdm_step of all "
                      "steps; adjoint: set_psi + wdm_adjoint)"}


def run_adjoint(args, rank, world):
    """Workload 5 as its own bench line: the adjoint/forward time ratio."""
    import torch

    import wavedm_gb300 as wdm

    wdm.build_library()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    a = adjoint_part(wdm, args.phase, N=args.n or 128, reps=max(1, args.steps // 10))
    N, nsteps, ck = a["grid"][0], a["steps"], a["ckpt_every"]
    return {
        "passes_adjoint_run": a["passes_adjoint_run"],
        "metric": f"adjoint/forward time ratio, {nsteps} Strang steps at {N}^3, checkpoints every {ck}",
        "value": a["ratio"], "unit": "ratio", "n_gpus": world, "steps": nsteps, "warmup": nsteps,
        "ms_per_step": round(1e3 / a["adjoint_steps_per_s"], 4), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "c64", "data": "synthetic (seeded soliton + halo; target from rc x 1.1)",
        "config": {"workload": "adjoint128", "grid": a["grid"], "dt": a["dt"], "ckpt_every": ck,
                   "repeats": a["repeats"], "phase_mode": args.phase},
        "forward_steps_per_s": a["forward_steps_per_s"], "adjoint_steps_per_s": a["adjoint_steps_per_s"],
        "loss": a["loss"], "dL_damp": a["dL_damp"], "gpu_launches": a["gpu_launches"],
    }


def plain_part(wdm, wl, K, W, mode):
    """steps/s of the plain FP32 phase form on the same workload, timed like `value`."""
    import torch

    dt = wl["dt"]
    ctx, psi0 = setup_context(wdm, wl, "plain", max(K, W, 1))
    stream = torch.cuda.ExternalStream(ctx.stream)
    ctx.step(W, dt, mode=mode)
    ctx.set_psi(psi0)
    ctx.get_phi()
    if wl["tidal"] is not None:
        ctx.set_tidal(wl["tidal"](np.arange(K + 1) * dt))
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    ctx.step(K, dt, mode=mode, sync=False)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    ok = ctx.is_finite()
    ctx.close()
    return {"value": round(K / (ms / 1e3), 3), "unit": "steps/s", "steps": K, "ms_per_step": round(ms / K, 4),
            "phase_mode": "plain", "finite": bool(ok)}


def accuracy_part(wdm, wl, oracle_steps, mass_steps):
    """psi and rho rel-L2 against the FP64 oracle after oracle_steps Strang steps of
    the workload (precise and plain phase forms), and the relative mass drift of
    both forms over mass_steps steps (GPU only: the FP64 path conserves mass to
    ~1e-13, so the drift needs no reference run)."""
    from oracle import spe

    N, L, dt = wl["n"], wl["L"], wl["dt"]
    psi0 = wl["psi0"].astype(np.complex64)
    spe_, g, phys = oracle_setup(wl, oracle_steps)
    t0 = time.perf_counter()
    ref = spe.run(psi0.astype(np.complex128), g, phys, dt, oracle_steps)
    t_oracle = time.perf_counter() - t0
    rho_ref = np.abs(ref) ** 2
    out = {"oracle_steps": oracle_steps, "oracle_seconds": round(t_oracle, 1), "oracle_threads": spe.WORKERS,
           "tolerance_psi_rel_l2": 1e-5, "mass_steps": mass_steps, "tolerance_mass_drift": 1e-6}
    rows = wl["tidal"](np.arange(mass_steps + 1) * dt) if wl["tidal"] is not None else None
    for mode in ("precise", "plain"):
        ctx = wdm.SPEContext((N, N, N), (L, L, L), poisson_coeff=wl["poisson_coeff"], phase_mode=mode)
        ctx.set_psi(psi0)
        if rows is not None:
            ctx.set_tidal(rows, t_first=0.0, t_step=dt)
        if wl["particles"] is not None:
            ctx.set_particles(*wl["particles"])
        m0 = ctx.reduce()["mass"]
        ctx.step(oracle_steps, dt, t0=0.0)
        psi = ctx.get_psi()
        r = {"psi_rel_l2": spe.rel_l2(psi, ref), "rho_rel_l2": spe.rel_l2(np.abs(psi) ** 2, rho_ref)}
        ctx.step(mass_steps - oracle_steps, dt, t0=oracle_steps * dt)
        r["mass_drift"] = float(ctx.reduce()["mass"] / m0 - 1.0)
        ctx.close()
        out[mode] = r
    out["pass"] = bool(out["precise"]["psi_rel_l2"] <= 1e-5 and abs(out["precise"]["mass_drift"]) <= 1e-6)
    return out


def ensemble_cpu_baseline(budget_s):
    """Oracle time of one step of one halo per size, weighted by the halo counts."""
    import wavedm_gb300 as wdm
    from oracle import spe

    members = wdm.ics.ensemble_members(nwaves=64)
    total, detail = 0.0, []
    for N in sorted({m[0] for m in members}):
        mem = [m for m in members if m[0] == N]
        n0, L, psi, T6 = mem[0]
        g = spe.Grid((N, N, N), (L, L, L))
        phys = spe.Physics(poisson_coeff=1.0, tidal=lambda t, T6=T6: tuple(T6))
        dt = wdm.ics.dt_for(N, L)
        p = spe.kdk_step(psi, g, phys, 0.0, dt)
        t0 = time.perf_counter()
        reps = 0
        while reps < 1 or time.perf_counter() - t0 < budget_s / 6:
            p = spe.kdk_step(p, g, phys, 0.0, dt)
            reps += 1
        per = (time.perf_counter() - t0) / reps
        total += per * len(mem)
        detail.append(f"{N}^3: {reps} steps, {per * 1e3:.1f} ms/halo-step x {len(mem)} halos")
    return {"value": round(1.0 / total, 6), "unit": "ensemble steps/s", "cores": spe.WORKERS, "kind": "port",
            "sample": "; ".join(detail)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["native", "reference"], default="native")
    ap.add_argument("--workload", type=int, default=3)
    ap.add_argument("--grid", "--n", dest="n", type=int, default=None, help="override the grid size of the workload")
    ap.add_argument("--phase", choices=["precise", "plain"], default="precise")
    ap.add_argument("--mode", choices=["strang", "reference_loop", "lie"], default="strang")
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=20.0, help="seconds of oracle time for cpu_baseline")
    ap.add_argument("--no-extras", action="store_true",
                    help="leave out the metric's other parts (accuracy vs the FP64 oracle, mass drift over the "
                         "workload's steps, the plain phase form, the adjoint ratio, the ensemble)")
    ap.add_argument("--acc-steps", type=int, default=10, help="Strang steps of the accuracy check against the oracle")
    ap.add_argument("--mass-steps", type=int, default=None, help="steps of the mass-drift check (default: the "
                                                                   "workload's own step count)")
    args = ap.parse_args()

    if "WORLD_SIZE" not in os.environ and args.gpus > 1:
        # one process per GPU, launched here the way torchrun launches them
        sys.exit(launch_ranks(sys.argv[1:], args.gpus))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world != args.gpus:
        raise SystemExit(f"bench.py: --gpus {args.gpus} but WORLD_SIZE={world}")

    if args.impl == "reference":
        if rank != 0:
            return
        import wavedm_gb300 as wdm

        wl = wdm.ics.workload(args.workload, n=args.n)
        v, n, cores = time_oracle(wl, budget_s=150.0, max_steps=args.steps, warm=min(args.warmup, 1))
        N = wl["n"]
        sample = f"{n} timed FP64 Strang steps of the full {N}^3 workload after {min(args.warmup, 1)} warm-up"
        print(json.dumps({
            "impl": "reference",
            "metric": f"KDK steps/s at {N}^3 (Strang, complex FP32 psi, {args.phase} phases)",
            "value": round(v, 5), "unit": "steps/s", "n_gpus": args.gpus, "steps": n, "warmup": min(args.warmup, 1),
            "ms_per_step": round(1e3 / v, 2), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c128", "data": "synthetic (same seeded workload)",
            "config": workload_config(wl, args, args.gpus),
            "cpu_baseline": {"value": round(v, 5), "unit": "steps/s", "cores": cores, "kind": "port",
                             "sample": sample,
                             "what": "oracle/spe.py: numpy/scipy.fft FP64 restatement of the reference's FFTW "
                                     "CPU path (Julia absent)"},
            "e2e": {"value": round(v, 5), "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }), flush=True)
        return

    if world > 1:
        import torch

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        torch.distributed.init_process_group("nccl")
    if args.workload == 5:
        rec = run_adjoint(args, rank, world)
        if world > 1:
            import torch

            torch.distributed.destroy_process_group()
        if rank == 0:
            print(json.dumps(rec), flush=True)
        return
    if args.workload == 4:
        rec = run_ensemble(args, rank, world)
        if rank == 0 and not args.no_cpu_baseline:
            rec["cpu_baseline"] = ensemble_cpu_baseline(args.cpu_budget)
        if world > 1:
            import torch

            torch.distributed.destroy_process_group()
        if rank == 0:
            print(json.dumps(rec), flush=True)
        return
    rec = run_native(args, rank, world)
    if rank == 0 and not args.no_extras and args.workload == 3:
        # the rest of the metric: accuracy at the stated tolerance, the plain
        # FP32 form beside the precise one, the adjoint/forward ratio, the ensemble
        import copy

        import wavedm_gb300 as wdm

        wl = wdm.ics.workload(args.workload, n=args.n)
        rec["plain"] = plain_part(wdm, wl, args.steps, args.warmup, args.mode)
        rec["accuracy"] = accuracy_part(wdm, wl, args.acc_steps, args.mass_steps or wl["steps"])
        rec["adjoint"] = adjoint_part(wdm, args.phase)
        ea = copy.copy(args)
        ea.no_e2e, ea.n = True, None
        e = run_ensemble(ea, 0, 1)
        keys = ("metric", "value", "unit", "steps", "ms_per_step", "halo_steps_per_s", "gpu_launches",
                "launches_per_step", "schedule", "config", "roofline")
        rec["ensemble"] = {k: e[k] for k in keys}
        e = run_ensemble(ea, 0, 1, counts=ENSEMBLE_SMALL)
        rec["ensemble_small"] = {k: e[k] for k in keys}
    if rank == 0 and not args.no_cpu_baseline:
        import wavedm_gb300 as wdm

        wl = wdm.ics.workload(args.workload, n=args.n)
        v, n, cores = time_oracle(wl, budget_s=args.cpu_budget, max_steps=1000, warm=1)
        rec["cpu_baseline"] = {"value": round(v, 5), "unit": "steps/s", "cores": cores, "kind": "port",
                               "sample": f"{n} FP64 Strang steps of the full {wl['n']}^3 workload (1 warm-up)"}
        if not args.no_e2e:
            v, n, cores = time_oracle_loop(wl, budget_s=args.cpu_budget)
            rec["cpu_baseline_loop"] = {
                "value": round(v, 5), "unit": "steps/s", "cores": cores, "kind": "port",
                "sample": f"{n} FP64 reference-loop iterations of the full {wl['n']}^3 workload, each with the "
                          "loop's host diagnostics (potential, findmax, radii quantiles, R, mass)",
                "compare_with": "loop_with_diagnostics"}
    if world > 1:
        import torch

        torch.distributed.destroy_process_group()
    if rank == 0:
        print(json.dumps(rec), flush=True)


if __name__ == "__main__":
    main()
