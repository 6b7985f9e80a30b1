"""Accuracy of the CUDA path against the FP64 oracle on the benchmark workloads (needs a GPU).

    python tests/accuracy.py --workload 2 [--steps 1000] [--n 256] [--out report.json]

For the precise and the plain phase forms it runs the workload's seeded input
for `steps` Strang steps through the library (complex64 psi) and through the
oracle (complex128, all host cores), and reports the relative L2 error of psi
and of rho = |psi|^2 (test/simulation_SPE3D_validation.jl:85-88) and the
relative mass drift sum|psi|^2 dV (src/simulation_main.jl:652) of both.
Workload 4 (the ensemble) is checked on its first halo of each grid size;
workload 5 (the adjoint) is checked by tests/test_gpu_adjoint.py instead.

This is test infrastructure: it runs the oracle as the checker.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from oracle import spe  # noqa: E402


def oracle_physics(wl, nsteps):
    N, L, dt = wl["n"], wl["L"], wl["dt"]
    g = spe.Grid((N, N, N), (L, L, L))
    rho_b = spe.cic_deposit(g, *wl["particles"]) if wl.get("particles") is not None else None
    sched = wl["tidal"](np.arange(nsteps + 2) * dt) if wl.get("tidal") is not None else None
    tidal = (lambda t: tuple(sched[int(round(t / dt))])) if sched is not None else None
    return g, spe.Physics(poisson_coeff=wl["poisson_coeff"], rho_b=rho_b, tidal=tidal), sched


def compare(wdm, wl, steps):
    """Errors of both phase forms against one oracle run of the workload."""
    N, L, dt = wl["n"], wl["L"], wl["dt"]
    psi0 = wl["psi0"].astype(np.complex64)
    g, phys, sched = oracle_physics(wl, steps)
    t0 = time.perf_counter()
    ref = spe.run(psi0.astype(np.complex128), g, phys, dt, steps)
    t_oracle = time.perf_counter() - t0
    m0_ref = spe.mass(psi0.astype(np.complex128), g)
    rho_ref = np.abs(ref) ** 2
    out = {"n": N, "L": L, "dt": dt, "steps": steps, "oracle_seconds": round(t_oracle, 1),
           "oracle_threads": spe.WORKERS, "oracle_mass_drift": spe.mass(ref, g) / m0_ref - 1.0}
    for mode in ("precise", "plain"):
        with wdm.SPEContext((N, N, N), (L, L, L), poisson_coeff=wl["poisson_coeff"], phase_mode=mode) as ctx:
            ctx.set_psi(psi0)
            if sched is not None:
                ctx.set_tidal(sched[: steps + 1])
            if wl.get("particles") is not None:
                ctx.set_particles(*wl["particles"])
            m0 = ctx.reduce()["mass"]
            ctx.step(steps, dt)
            psi = ctx.get_psi()
            m1 = ctx.reduce()["mass"]
        out[mode] = {"psi_rel_l2": spe.rel_l2(psi, ref), "rho_rel_l2": spe.rel_l2(np.abs(psi) ** 2, rho_ref),
                     "mass_drift": float(m1 / m0 - 1.0)}
    return out


def mass_drift_only(wdm, wl, steps, every=100):
    """Relative mass drift of both phase forms every `every` steps up to `steps`."""
    N, L, dt = wl["n"], wl["L"], wl["dt"]
    psi0 = wl["psi0"].astype(np.complex64)
    sched = wl["tidal"](np.arange(steps + 2) * dt) if wl.get("tidal") is not None else None
    out = {"n": N, "L": L, "dt": dt, "steps": steps, "every": every}
    for mode in ("precise", "plain"):
        with wdm.SPEContext((N, N, N), (L, L, L), poisson_coeff=wl["poisson_coeff"], phase_mode=mode) as ctx:
            ctx.set_psi(psi0)
            if wl.get("particles") is not None:
                ctx.set_particles(*wl["particles"])
            m0 = ctx.reduce()["mass"]
            drift = []
            for s0 in range(0, steps, every):
                k = min(every, steps - s0)
                if sched is not None:
                    ctx.set_tidal(sched[s0: s0 + k + 1])
                ctx.step(k, dt, t0=s0 * dt)
                drift.append(float(ctx.reduce()["mass"] / m0 - 1.0))
        out[mode] = {"mass_drift": drift[-1], "mass_drift_every": drift}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", type=int, required=True, choices=[1, 2, 3, 4])
    ap.add_argument("--steps", type=int, default=None, help="default: the workload's own step count")
    ap.add_argument("--n", type=int, default=None, help="override the grid size")
    ap.add_argument("--out", default=None)
    ap.add_argument("--gpu-only", action="store_true",
                    help="no oracle: the mass drift of both phase forms over the step count (the FP64 path conserves "
                         "mass to ~1e-13, so the drift needs no reference run)")
    a = ap.parse_args()

    import wavedm_gb300 as wdm

    wdm.build_library()
    report = {"workload": a.workload}
    if a.gpu_only and a.workload != 4:
        wl = wdm.ics.workload(a.workload, n=a.n)
        report.update(mass_drift_only(wdm, wl, a.steps or wl["steps"]))
    elif a.workload == 4:
        seen = set()
        report["halos"] = []
        for N, L, psi0, T6 in wdm.ics.ensemble_members():
            if N in seen:
                continue
            seen.add(N)
            wl = dict(n=N, L=L, dt=wdm.ics.dt_for(N, L), psi0=psi0, poisson_coeff=1.0, particles=None,
                      tidal=lambda t, T6=T6: np.tile(T6, (len(t), 1)))
            report["halos"].append(compare(wdm, wl, a.steps or 500))
    else:
        wl = wdm.ics.workload(a.workload, n=a.n)
        report.update(compare(wdm, wl, a.steps or wl["steps"]))
    line = json.dumps(report)
    print(line)
    if a.out:
        with open(a.out, "w") as f:
            f.write(line + "\n")


if __name__ == "__main__":
    main()
