"""Generate the golden fixtures of tests/golden/ with the FP64 oracle.

    python tests/golden/make_golden.py

Each case is a small seeded grid advanced by the oracle (oracle/spe.py); the
fixture stores the inputs (psi0, physics, schedule) and the FP64 outputs, so
the GPU tests can compare the CUDA path with them and the CPU tests can check
that the oracle still reproduces them.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import spe  # noqa: E402

CASES = {
    # name: n, L, convention, mode, steps, dt, poisson_coeff, kerr, alpha, tidal, vstatic, particles
    "strang_16_gravity": dict(n=(16, 16, 16), L=(8.0, 8.0, 8.0), convention="periodic", mode="strang", steps=8,
                              dt=0.02, c=1.0, kerr=0.0, alpha=0.0, tidal=False, vstatic=False, particles=0),
    "strang_24x16x12_all": dict(n=(24, 16, 12), L=(9.0, 6.0, 4.5), convention="periodic", mode="strang", steps=6,
                                dt=0.01, c=4 * np.pi, kerr=-0.2, alpha=0.0, tidal=True, vstatic=True, particles=40),
    "refloop_16_mask": dict(n=(16, 16, 16), L=(8.0, 8.0, 8.0), convention="reference", mode="reference_loop",
                            steps=5, dt=0.02, c=4 * np.pi, kerr=0.0, alpha=5.0, tidal=False, vstatic=False,
                            particles=0),
    "lie_12x16x8_tidal": dict(n=(12, 16, 8), L=(6.0, 8.0, 4.0), convention="periodic", mode="lie", steps=5,
                              dt=0.015, c=1.0, kerr=0.1, alpha=0.0, tidal=True, vstatic=False, particles=0),
}


def tidal_fn(t):
    return (0.02 + 0.01 * t, -0.01, -0.01 + 0.002 * t, 0.003, -0.002, 0.001)


def make_case(spec, seed):
    rng = np.random.default_rng(seed)
    nx, ny, nz = spec["n"]
    g = spe.Grid(spec["n"], spec["L"], spec["convention"])
    X, Y, Z = g.coords()
    r2 = X ** 2 / (spec["L"][0] / 4) ** 2 + Y ** 2 / (spec["L"][1] / 4) ** 2 + Z ** 2 / (spec["L"][2] / 4) ** 2
    psi0 = np.exp(-r2) * np.exp(1j * 0.4 * rng.standard_normal((nz, ny, nx))) + 0.05 * (
        rng.standard_normal((nz, ny, nx)) + 1j * rng.standard_normal((nz, ny, nx)))
    psi0 = psi0.astype(np.complex64).astype(np.complex128)  # exactly representable on the GPU
    V = None
    if spec["vstatic"]:
        V = (0.05 * (X ** 2 + Y ** 2) + 0.02 * np.sin(2 * np.pi * Z / spec["L"][2])) * np.ones((nz, ny, nx))
        V = V.astype(np.float32).astype(np.float64)
    pos = mass = None
    rho_b = None
    if spec["particles"]:
        pos = rng.uniform(-0.4, 0.4, size=(spec["particles"], 3)) * np.array(spec["L"])
        mass = rng.uniform(0.05, 0.2, size=spec["particles"])
        rho_b = spe.cic_deposit(g, pos, mass)
    steps, dt = spec["steps"], spec["dt"]
    sched = np.array([tidal_fn(s * dt) for s in range(steps + 1)]) if spec["tidal"] else None
    phys = spe.Physics(poisson_coeff=spec["c"], kerr=spec["kerr"], absorb_alpha=spec["alpha"], V_static=V,
                       rho_b=rho_b, tidal=(lambda t: tidal_fn(t)) if spec["tidal"] else None)
    psi = spe.run(psi0, g, phys, dt, steps, mode=spec["mode"])
    phi = spe.potential(psi, g, spe.Physics(poisson_coeff=spec["c"], rho_b=rho_b), 0.0)
    out = dict(psi0=psi0, psi=psi, phi=phi, n=np.array(spec["n"]), L=np.array(spec["L"]),
               convention=spec["convention"], mode=spec["mode"], steps=steps, dt=dt, c=spec["c"],
               kerr=spec["kerr"], alpha=spec["alpha"])
    if V is not None:
        out["V"] = V
    if sched is not None:
        out["tidal"] = sched
    if pos is not None:
        out["pos"] = pos
        out["mass"] = mass
    return out


def main():
    for i, (name, spec) in enumerate(sorted(CASES.items())):
        data = make_case(spec, seed=1000 + i)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **data)
        print(name, data["psi"].shape)


if __name__ == "__main__":
    main()
