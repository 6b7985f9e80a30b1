"""The FP64 oracle adjoint against central finite differences (h = 1e-4), CPU only."""
import numpy as np
import pytest

from oracle import adjoint as adj
from oracle import spe


def _setup(n=16, L=8.0, kerr=0.0, alpha=0.0, seed=0):
    g = spe.Grid((n, n, n), (L, L, L))
    X, Y, Z = g.coords()
    rng = np.random.default_rng(seed)
    r2 = X ** 2 + Y ** 2 + Z ** 2
    psi0 = np.exp(-r2 / 3) * np.exp(0.3j * rng.standard_normal((n, n, n))) + 0.02
    D = np.array([2.0, -1.0, -1.0, 0.0, 0.0, 0.0])
    amp = 0.03
    phys = spe.Physics(poisson_coeff=1.5, kerr=kerr, absorb_alpha=alpha, tidal=lambda t: tuple(amp * D))
    target = np.exp(-r2 / 2.5) * 0.8
    return g, psi0, phys, D, amp, target


@pytest.mark.parametrize("kerr,alpha", [(0.0, 0.0), (0.3, 0.0), (0.0, 2.0)])
def test_psi0_gradient_matches_finite_differences(kerr, alpha):
    g, psi0, phys, D, amp, target = _setup(kerr=kerr, alpha=alpha)
    dt, n = 0.05, 6
    L, grad, damp = adj.adjoint(psi0, g, phys, dt, n, target, tidal_dir=D)
    rng = np.random.default_rng(1)
    for _ in range(3):
        e = rng.standard_normal(psi0.shape) + 1j * rng.standard_normal(psi0.shape)
        fd = adj.fd_directional(psi0, g, phys, dt, n, target, e)
        an = float(np.real(np.sum(np.conj(grad) * e)))
        assert an == pytest.approx(fd, rel=1e-6, abs=1e-10)


def test_tidal_amplitude_gradient_matches_finite_differences():
    g, psi0, phys, D, amp, target = _setup()
    dt, n, h = 0.05, 6, 1e-4
    L, grad, damp = adj.adjoint(psi0, g, phys, dt, n, target, tidal_dir=D)

    def L_amp(a):
        ph = spe.Physics(poisson_coeff=phys.poisson_coeff, tidal=lambda t: tuple(a * D))
        _, psiN = adj.forward_states(psi0, g, ph, dt, n)
        return adj.loss(psiN, target, g)

    fd = (L_amp(amp + h) - L_amp(amp - h)) / (2 * h)
    assert damp == pytest.approx(fd, rel=1e-6)


def test_core_radius_gradient_by_chain_rule():
    g, _, phys, D, amp, target = _setup()
    X, Y, Z = g.coords()
    r = np.sqrt(X ** 2 + Y ** 2 + Z ** 2)
    phase = np.exp(0.2j * np.sin(X))

    def psi_of(rc):
        return np.sqrt(1.0 / (1.0 + 0.091 * (r / rc) ** 2) ** 8) * phase

    rc, h, dt, n = 1.3, 1e-4, 0.05, 6
    L, grad, _ = adj.adjoint(psi_of(rc), g, phys, dt, n, target)
    dpsi = (psi_of(rc + 1e-6) - psi_of(rc - 1e-6)) / 2e-6
    chain = float(np.real(np.sum(np.conj(grad) * dpsi)))

    def L_rc(x):
        _, psiN = adj.forward_states(psi_of(x), g, phys, dt, n)
        return adj.loss(psiN, target, g)

    fd = (L_rc(rc + h) - L_rc(rc - h)) / (2 * h)
    assert chain == pytest.approx(fd, rel=1e-5)


def test_forward_states_reproduce_spe_run():
    g, psi0, phys, D, amp, target = _setup()
    s, psiN = adj.forward_states(psi0, g, phys, 0.05, 5)
    ref = spe.run(psi0, g, phys, 0.05, 5)
    assert spe.rel_l2(psiN, ref) < 1e-12
