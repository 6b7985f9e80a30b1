"""FP64 CPU adjoint of the Strang KDK run (the oracle of the adjoint path).

TEST INFRASTRUCTURE ONLY: used by tests/ and by bench.py's CPU baseline.  The
reference has no adjoint (Zygote is imported but never called); the quantity
differentiated is the one of the adjoint workload:

    L = sum_cells (|psi_N|^2 - rho_target)^2 dV

after N Strang steps from psi_0 (the run of spe.run with mode "strang").  The
gradient convention is dL = Re sum conj(g) dpsi_0, i.e. g = dL/d(Re psi_0) + i
dL/d(Im psi_0).

A Strang run is a chain of kicks and drifts; between two drifts the half kicks
of consecutive steps see the same density and merge into one kick of dt, so
the run has N+1 kicks at the boundaries b = 0..N (dt/2, dt, ..., dt, dt/2) and N
drifts.  For a kick psi+ = exp(-i th) psi with th = dt_k (G |psi|^2 + V + kappa
|psi|^2), G the (self-adjoint) Poisson operator, the adjoint map is

    lam = exp(i th) lam+ + 2 (G mu + kappa mu) psi,  mu = dt_k Im(conj(lam+) psi+)

and a tidal amplitude a with V = a v(x) contributes dL/da += sum mu v.  The
drift adjoint is the drift with -dt, the absorbing mask is its own adjoint.
"""
from __future__ import annotations

import numpy as np

from . import spe


def _kick_theta(psi_pre, grid, phys, t, dtk):
    pot = spe.potential(psi_pre, grid, phys, t)
    if phys.kerr:
        pot = pot + phys.kerr * np.abs(psi_pre) ** 2
    return dtk * pot


def forward_states(psi0, grid, phys, dt, nsteps, t0=0.0):
    """Pre-kick states s_b (b = 0..N) of the merged-kick Strang run, and psi_N."""
    mask = spe.absorption_mask(grid, phys.absorb_alpha, dt) if phys.absorb_alpha else None
    s = [np.asarray(psi0, np.complex128)]
    psi = s[0]
    for b in range(nsteps):
        dtk = dt / 2 if b == 0 else dt
        psi = np.exp(-1j * _kick_theta(psi, grid, phys, t0 + b * dt, dtk)) * psi
        psi = spe.drift(psi, grid, dt)
        if mask is not None:
            psi = psi * mask
        s.append(psi)
    psiN = np.exp(-1j * _kick_theta(psi, grid, phys, t0 + nsteps * dt, dt / 2)) * psi
    return s, psiN


def loss(psiN, rho_target, grid):
    return float(np.sum((np.abs(psiN) ** 2 - rho_target) ** 2) * grid.dV)


def adjoint(psi0, grid, phys, dt, nsteps, rho_target, tidal_dir=None, t0=0.0):
    """Returns (loss, grad_psi0, dL/d amp) for V_tidal = amp * 1/2 x^T D x (D = tidal_dir)."""
    mask = spe.absorption_mask(grid, phys.absorb_alpha, dt) if phys.absorb_alpha else None
    s, psiN = forward_states(psi0, grid, phys, dt, nsteps, t0)
    L = loss(psiN, rho_target, grid)
    lam = 4.0 * (np.abs(psiN) ** 2 - rho_target) * psiN * grid.dV
    vdir = spe.tidal_potential(grid, tidal_dir) if tidal_dir is not None else None
    damp = 0.0
    for b in range(nsteps, -1, -1):
        dtk = dt / 2 if b in (0, nsteps) else dt
        pre = s[b]
        th = _kick_theta(pre, grid, phys, t0 + b * dt, dtk)
        post = np.exp(-1j * th) * pre
        mu = dtk * np.imag(np.conj(lam) * post)
        if vdir is not None:
            damp += float(np.sum(mu * vdir))
        gmu = spe.poisson(mu, grid, phys.poisson_coeff) if phys.poisson_coeff != 0 else 0.0
        if phys.kerr:
            gmu = gmu + phys.kerr * mu
        lam = np.exp(1j * th) * lam + 2.0 * gmu * pre
        if b > 0:
            if mask is not None:
                lam = lam * mask
            lam = spe.drift(lam, grid, -dt)
    return L, lam, damp


def fd_directional(psi0, grid, phys, dt, nsteps, rho_target, direction, h=1e-4):
    """Central difference of L along a complex direction of psi_0."""
    def L_of(p):
        _, psiN = forward_states(p, grid, phys, dt, nsteps)
        return loss(psiN, rho_target, grid)
    return (L_of(psi0 + h * direction) - L_of(psi0 - h * direction)) / (2 * h)
