"""Closed-form answers on the CUDA path itself.

These are the analytic cases that the reference's own tests and docs use:
- the harmonic-oscillator ground state (test/simulation_SPE1D.jl), with Strang's
  second order in dt;
- the travelling Kerr soliton;
- free Gaussian dispersion.
Each runs through the C ABI on a line grid (x resolved; y and z of 8 points
carry a uniform state, so only their k = 0 mode is populated) and is compared
with its closed form directly, not with the oracle (tests/test_oracle.py holds
the same cases for the oracle)."""
import numpy as np
import pytest

from oracle import spe

pytestmark = pytest.mark.gpu


def _line(nx, L):
    g = spe.Grid((nx, 8, 8), (L, 1.0, 1.0))
    X, _, _ = g.coords()
    return g, np.broadcast_to(X, (8, 8, nx))


def _harmonic(wdm, dt, tmax, nx=64, L=20.0):
    g, X = _line(nx, L)
    psi0 = np.exp(-X ** 2 / 2).astype(np.complex64)
    nst = int(round(tmax / dt))
    with wdm.SPEContext(g.n, g.L, poisson_coeff=0.0) as ctx:
        ctx.set_psi(psi0)
        ctx.set_tidal([[1.0, 0.0, 0.0, 0.0, 0.0, 0.0]])  # V = x^2 / 2
        ctx.step(nst, dt)
        psi = ctx.get_psi()
    exact = psi0.astype(np.complex128) * np.exp(-0.5j * nst * dt)  # E0 = 1/2
    return spe.rel_l2(psi, exact)


def test_harmonic_oscillator_ground_state(wdm):
    assert _harmonic(wdm, 0.01, 1.0) < 1e-4


def test_strang_is_second_order(wdm):
    e1 = _harmonic(wdm, 0.1, 2.0)
    e2 = _harmonic(wdm, 0.05, 2.0)
    assert 3.5 < e1 / e2 < 4.5


def test_kerr_soliton_travels(wdm):
    A, v = np.sqrt(2.0), 0.5
    B = A / 2
    kappa = -(B ** 2) / A ** 2
    g, X = _line(256, 60.0)

    def sol(t):
        return A / np.cosh(B * (X - v * t)) * np.exp(1j * (v * X - 0.5 * (v * v - B * B) * t))

    dt, nst = 0.005, 400
    with wdm.SPEContext(g.n, g.L, poisson_coeff=0.0, kerr=kappa) as ctx:
        ctx.set_psi(sol(0.0).astype(np.complex64))
        ctx.step(nst, dt)
        psi = ctx.get_psi()
    assert spe.rel_l2(psi, sol(nst * dt)) < 1e-4


def test_free_gaussian_dispersion(wdm):
    s2, t = 1.0, 3.0
    g, X = _line(256, 80.0)
    psi0 = np.exp(-X ** 2 / (2 * s2))
    exact = np.sqrt(s2 / (s2 + 1j * t)) * np.exp(-X ** 2 / (2 * (s2 + 1j * t)))
    with wdm.SPEContext(g.n, g.L, poisson_coeff=0.0) as ctx:
        ctx.set_psi(psi0.astype(np.complex64))
        ctx.drift(t)
        psi = ctx.get_psi()
    assert spe.rel_l2(psi, exact) < 1e-5
