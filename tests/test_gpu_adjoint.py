"""GPU adjoint against the FP64 CPU adjoint (oracle/adjoint.py) and finite differences.

Tolerances: the gradient is compared in relative L2 (5e-4: FP32 forward and
backward sweeps over the run), the loss to 1e-5 and dL/da to 1e-3 relative.
"""
import numpy as np
import pytest

from oracle import adjoint as adj
from oracle import spe

pytestmark = pytest.mark.gpu


def _case(n=32, L=8.0, kerr=0.0, alpha=0.0, seed=4):
    g = spe.Grid((n, n, n), (L, L, L))
    X, Y, Z = g.coords()
    rng = np.random.default_rng(seed)
    r2 = X ** 2 + Y ** 2 + Z ** 2
    psi0 = (np.exp(-r2 / 3) * np.exp(0.3j * rng.standard_normal((n, n, n))) + 0.02).astype(np.complex64)
    D = np.array([2.0, -1.0, -1.0, 0.0, 0.0, 0.0])
    amp = 0.03
    target = (np.exp(-r2 / 2.5) * 0.8).astype(np.float32)
    return g, psi0, D, amp, target


@pytest.mark.parametrize("kerr,alpha,ckpt", [(0.0, 0.0, 4), (0.2, 0.0, 7), (0.0, 0.0, 20), (0.0, 2.0, 4),
                                             (0.0, 2.0, 20)])
def test_adjoint_matches_fp64_adjoint(wdm, kerr, alpha, ckpt):
    g, psi0, D, amp, target = _case(kerr=kerr, alpha=alpha)
    dt, nsteps = 0.03, 12
    phys = spe.Physics(poisson_coeff=1.5, kerr=kerr, absorb_alpha=alpha, tidal=lambda t: tuple(amp * D))
    L_ref, g_ref, da_ref = adj.adjoint(psi0.astype(np.complex128), g, phys, dt, nsteps,
                                       target.astype(np.float64), tidal_dir=D)
    with wdm.SPEContext(g.n, g.L, poisson_coeff=1.5, kerr=kerr, absorb_alpha=alpha) as ctx:
        ctx.set_psi(psi0)
        ctx.set_tidal([amp * D])
        loss, grad, da = ctx.adjoint(nsteps, dt, target, ckpt_every=ckpt, tidal_dir=D)
        psi_after = ctx.get_psi()
    assert loss == pytest.approx(L_ref, rel=1e-5)
    assert spe.rel_l2(grad, g_ref) < 5e-4
    assert da == pytest.approx(da_ref, rel=1e-3)
    assert np.array_equal(psi_after, psi0)


def test_autograd_function_matches_fp64_adjoint(wdm):
    torch = pytest.importorskip("torch")
    from wavedm_gb300.autograd import evolve_loss

    g, psi0, D, amp, target = _case(n=32)
    dt, nsteps = 0.03, 8
    phys = spe.Physics(poisson_coeff=1.5, tidal=lambda t: tuple(amp * D))
    L_ref, g_ref, da_ref = adj.adjoint(psi0.astype(np.complex128), g, phys, dt, nsteps,
                                       target.astype(np.float64), tidal_dir=D)
    p = torch.from_numpy(psi0).cuda().requires_grad_(True)
    a = torch.tensor(amp, dtype=torch.float64, requires_grad=True)
    rho = torch.from_numpy(target).cuda()
    with wdm.SPEContext(g.n, g.L, poisson_coeff=1.5) as ctx:
        loss = evolve_loss(p, a, ctx, nsteps, dt, rho, D, ckpt_every=3)
        (2.0 * loss).backward()
    assert float(loss.detach()) == pytest.approx(L_ref, rel=1e-5)
    assert spe.rel_l2(p.grad.cpu().numpy() / 2.0, g_ref) < 5e-4
    assert float(a.grad) / 2.0 == pytest.approx(da_ref, rel=1e-3)
    # without a gradient to compute, the loss comes from the forward run alone
    with torch.no_grad(), wdm.SPEContext(g.n, g.L, poisson_coeff=1.5) as ctx:
        l0 = ctx.launch_count
        loss_only = evolve_loss(p.detach(), a.detach(), ctx, nsteps, dt, rho, D, ckpt_every=3)
        assert ctx.launch_count - l0 < 12 * nsteps  # a forward run: ~9 launches per step
    assert float(loss_only) == pytest.approx(L_ref, rel=1e-5)


def test_adjoint_workload5_shape_at_64(wdm):
    """The adjoint workload's loss and parameters on a 64^3 grid, against the FP64
    CPU adjoint, including dL/drc through the chain rule of the initial state
    (the finite-difference pins of the adjoint are FP64 tests of oracle/adjoint.py)."""
    w = wdm.ics
    N, L, dt, nsteps, ck = 64, 20.0, w.dt_for(64, 20.0), 20, 5
    D = np.array([2.0, -1.0, -1.0, 0.0, 0.0, 0.0])
    amp, rc = 0.02, 1.2
    rng = w.rng_for(5)
    psi_of = lambda r_c: w.soliton_halo_ic((N, N, N), (L, L, L), rc=r_c, rng=np.random.default_rng(55), nwaves=256)
    psi0 = psi_of(rc).astype(np.complex64)
    del rng
    target = (np.abs(psi_of(1.3 * rc)) ** 2).astype(np.float32)
    g = spe.Grid((N, N, N), (L, L, L))
    phys = spe.Physics(poisson_coeff=1.0, tidal=lambda t: tuple(amp * D))
    L_ref, g_ref, da_ref = adj.adjoint(psi0.astype(np.complex128), g, phys, dt, nsteps, target.astype(np.float64),
                                       tidal_dir=D)
    with wdm.SPEContext((N, N, N), (L, L, L), poisson_coeff=1.0) as ctx:
        ctx.set_psi(psi0)
        ctx.set_tidal([amp * D])
        loss, grad, da = ctx.adjoint(nsteps, dt, target, ckpt_every=ck, tidal_dir=D)
    assert loss == pytest.approx(L_ref, rel=1e-5)
    assert spe.rel_l2(grad, g_ref) < 5e-4
    assert da == pytest.approx(da_ref, rel=1e-3)
    dpsi = (psi_of(rc + 1e-5) - psi_of(rc - 1e-5)) / 2e-5
    drc = float(np.real(np.sum(np.conj(grad.astype(np.complex128)) * dpsi)))
    drc_ref = float(np.real(np.sum(np.conj(g_ref) * dpsi)))
    assert drc == pytest.approx(drc_ref, rel=1e-3)


ADJ_IMPL_CASES = [(32, 24, 16), (64, 16, 8), (128, 16, 16), (96, 8, 8)]


@pytest.mark.parametrize("n", ADJ_IMPL_CASES, ids=["x".join(map(str, n)) for n in ADJ_IMPL_CASES])
def test_adjoint_kick_implementations_agree(wdm, n, monkeypatch):
    """The staged adjoint kick (rows copied to shared memory one unit ahead) and
    the direct one share their arithmetic: forced onto either, an adjoint run
    with tide, Kerr term and absorbing mask gives bit-identical gradients."""
    L = (4.0, 3.0, 5.0)
    g = spe.Grid(n, L)
    X, Y, Z = g.coords()
    rng = np.random.default_rng(8)
    shape = (n[2], n[1], n[0])
    psi0 = (np.exp(-(X ** 2 + Y ** 2 + Z ** 2)) * np.exp(1j * rng.uniform(0, 1, shape)) + 0.01).astype(np.complex64)
    target = (0.5 * np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / 1.5)).astype(np.float32)
    D = np.array([2.0, -1.0, -1.0, 0.1, 0.0, 0.0])
    out = {}
    for x_impl in ("staged", "direct"):
        monkeypatch.setenv("WDM_X_IMPL", x_impl)
        with wdm.SPEContext(n, L, poisson_coeff=2.0, kerr=0.3, absorb_alpha=0.5) as ctx:
            ctx.set_psi(psi0)
            ctx.set_tidal([0.02 * D])
            out[x_impl] = ctx.adjoint(6, 0.01, target, ckpt_every=4, tidal_dir=D)
    # the loss and dL/da are FP64 sums of per-block partials added atomically,
    # so only their last bits depend on the order the blocks finish in
    assert out["staged"][0] == pytest.approx(out["direct"][0], rel=1e-12)
    assert np.array_equal(out["staged"][1], out["direct"][1])
    assert out["staged"][2] == pytest.approx(out["direct"][2], rel=1e-12)
