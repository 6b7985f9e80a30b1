"""Pins of the FP64 oracle against the reference's own known answers and analytic cases.

The reference stores no golden vectors; its tests pin the path by formulas and
bounds, which are restated here:

* grid spacing and cell volume            test/unit_test.jl:1-24
* Poisson on a 32^3 Gaussian, loose bounds test/test_parallel.jl:70-97
* harmonic oscillator exp(-x^2/2)exp(-it/2) test/simulation_SPE1D.jl:8-10,197-212
* sech soliton A sech(A x/2) with a Kerr term test/simulation_SPE1D.jl:12-18,214-229
  (the reference's phase omega = A^2/2 is not a solution of its own equation;
  the self-consistent kappa = -(A/2)^2/A^2 and phase are used)
* relative L2 metric                       test/simulation_SPE3D_validation.jl:85-88
* drift factor of setup_fft_operators      src/solver/fft_operators.jl:8-15
"""
import numpy as np
import pytest

from oracle import spe


def test_setup_grid_matches_reference_unit_test():
    x, y, z, d, vol = spe.setup_grid(2.0, 2.0, 2.0, 64, 64, 64)
    assert np.isclose(x.min(), -2.0) and np.isclose(x.max(), 2.0)
    assert len(x) == len(y) == len(z) == 64
    assert np.allclose(d, 4.0 / 63)
    assert np.isclose(vol, np.prod(d))
    x8, _, _, d8, _ = spe.setup_grid(1.0, 1.0, 1.0, 8, 8, 8)
    assert len(x8) == 8 and np.isclose(d8[0], 2.0 / 7)
    g = spe.Grid((64, 64, 64), (4.0, 4.0, 4.0), "reference")
    assert np.allclose(g.spacing, 4.0 / 63)


def test_rel_l2_definition():
    a = np.array([1.0 + 1j, 2.0, 3.0])
    b = np.array([1.0, 2.0, 3.0 + 0.5j])
    ref = np.sqrt(np.mean(np.abs(a - b) ** 2)) / np.sqrt(np.mean(np.abs(b) ** 2))
    assert spe.rel_l2(a, b) == pytest.approx(ref)


def test_poisson_single_mode_exact():
    n, L = (16, 12, 8), (2.0, 3.0, 1.5)
    g = spe.Grid(n, L)
    X, Y, Z = g.coords()
    k = 2 * np.pi * np.array([2 / L[0], 1 / L[1], 3 / L[2]])
    rho = np.cos(k[0] * X + k[1] * Y + k[2] * Z) * np.ones((n[2], n[1], n[0]))
    phi = spe.poisson(rho, g, coeff=4 * np.pi)
    expect = -4 * np.pi * rho / np.dot(k, k)
    assert np.abs(phi - expect).max() < 1e-12


def test_poisson_gaussian_bounds_of_reference_test():
    # test/test_parallel.jl:70-97: 32^3 Gaussian on LinRange(-pi, pi, 32), Delta = 1
    x = np.linspace(-np.pi, np.pi, 32)
    rho = np.exp(-(x[None, None, :] ** 2 + x[None, :, None] ** 2 + x[:, None, None] ** 2))
    g = spe.Grid((32, 32, 32), (32.0, 32.0, 32.0))  # spacing 1
    phi = spe.poisson(rho, g, coeff=1.0)
    assert np.all(np.isfinite(phi))
    assert 1e-6 < np.abs(phi).max() < 100.0


def test_drift_factor_matches_setup_fft_operators():
    X, N, dt = 5.0, 16, 0.013
    dense = spe.setup_fft_operators(X, X, X, N, N, N, dt)
    g = spe.Grid((N, N, N), (2 * X, 2 * X, 2 * X), "reference")
    assert np.abs(dense - np.exp(-0.5j * dt * g.k2())).max() < 1e-12


def _line_grid(nx, L):
    return spe.Grid((nx, 4, 4), (L, 1.0, 1.0))


def _harmonic(dt, tmax, nx=64, L=20.0):
    g = _line_grid(nx, L)
    X, _, _ = g.coords()
    psi0 = np.exp(-X ** 2 / 2) * np.ones((4, 4, nx))
    phys = spe.Physics(poisson_coeff=0.0, tidal=lambda t: (1.0, 0, 0, 0, 0, 0))
    nst = int(round(tmax / dt))
    psi = spe.run(psi0, g, phys, dt, nst)
    exact = psi0 * np.exp(-0.5j * nst * dt)
    return spe.rel_l2(psi, exact)


def test_harmonic_oscillator_ground_state():
    assert _harmonic(0.01, 1.0) < 1e-4


def test_strang_is_second_order():
    e1 = _harmonic(0.1, 2.0)
    e2 = _harmonic(0.05, 2.0)
    assert 3.5 < e1 / e2 < 4.5


def test_kerr_soliton_travels():
    A, v = np.sqrt(2.0), 0.5
    B = A / 2
    kappa = -(B ** 2) / A ** 2
    nx, L = 256, 60.0
    g = _line_grid(nx, L)
    X, _, _ = g.coords()

    def sol(t):
        return (A / np.cosh(B * (X - v * t)) * np.exp(1j * (v * X - 0.5 * (v * v - B * B) * t))) * np.ones((4, 4, nx))

    phys = spe.Physics(poisson_coeff=0.0, kerr=kappa)
    dt, nst = 0.005, 400
    psi = spe.run(sol(0.0), g, phys, dt, nst)
    assert spe.rel_l2(psi, sol(nst * dt)) < 1e-4


def test_free_gaussian_dispersion():
    s2, nx, L, t = 1.0, 256, 80.0, 3.0
    g = _line_grid(nx, L)
    X, _, _ = g.coords()
    psi0 = np.exp(-X ** 2 / (2 * s2)) * np.ones((4, 4, nx))
    exact = np.sqrt(s2 / (s2 + 1j * t)) * np.exp(-X ** 2 / (2 * (s2 + 1j * t))) * np.ones((4, 4, nx))
    assert spe.rel_l2(spe.drift(psi0, g, t), exact) < 1e-10


def _random_state(n, L, seed=1):
    rng = np.random.default_rng(seed)
    g = spe.Grid(n, L)
    X, Y, Z = g.coords()
    r2 = X ** 2 + Y ** 2 + Z ** 2
    psi = np.exp(-r2 / 4) * np.exp(1j * 0.3 * rng.standard_normal((n[2], n[1], n[0])))
    return g, psi


def test_strang_conserves_mass_and_is_time_reversible():
    g, psi0 = _random_state((16, 16, 16), (8.0, 8.0, 8.0))
    phys = spe.Physics(poisson_coeff=1.0, kerr=0.1,
                       tidal=lambda t: (0.01 + 0.001 * t, -0.005, -0.005, 0.002, 0.0, 0.0))
    dt = 0.02
    psi = spe.run(psi0, g, phys, dt, 6)
    assert abs(spe.mass(psi, g) / spe.mass(psi0, g) - 1) < 1e-12
    back = spe.run(psi, g, phys, -dt, 6, t0=6 * dt)
    assert spe.rel_l2(back, psi0) < 1e-12


def test_reference_loop_is_half_kick_then_drift():
    g, psi0 = _random_state((8, 8, 8), (6.0, 6.0, 6.0))
    phys = spe.Physics(poisson_coeff=2.0)
    dt = 0.05
    one = spe.kdk_step(psi0, g, phys, 0.0, dt, mode="reference_loop")
    manual = spe.drift(spe.kick(psi0, spe.potential(psi0, g, phys, 0.0), dt / 2), g, dt)
    assert spe.rel_l2(one, manual) < 1e-14
    lie = spe.kdk_step(psi0, g, phys, 0.0, dt, mode="lie")
    manual = spe.drift(spe.kick(psi0, spe.potential(psi0, g, phys, 0.0), dt), g, dt)
    assert spe.rel_l2(lie, manual) < 1e-14


def test_absorbing_mask_values():
    g = spe.Grid((16, 16, 16), (10.0, 10.0, 10.0), "reference")
    m = spe.absorption_mask(g, alpha=10.0, dt=0.01)
    assert np.all(m > 0) and np.all(m <= 1.0 + 1e-15)
    # centre ~ 1; a face centre (x = X, y = z = 0) ~ exp(-alpha dt)
    c = 8
    assert m[c, c, c] == pytest.approx(1.0, abs=0.05)
    assert m[c, c, -1] == pytest.approx(np.exp(-0.1), rel=1e-6)


def test_cic_deposit_and_interpolation():
    g = spe.Grid((16, 16, 16), (4.0, 4.0, 4.0))
    rng = np.random.default_rng(3)
    pos = rng.uniform(-2.0, 2.0, size=(500, 3))
    m = rng.uniform(0.5, 1.5, size=500)
    rho = spe.cic_deposit(g, pos, m)
    assert np.sum(rho) * g.dV == pytest.approx(m.sum(), rel=1e-12)
    X, Y, Z = g.coords()
    f = (0.3 * X + 0.2 * Y - 0.1 * Z) * np.ones((16, 16, 16))
    inside = np.all((pos > -2.0) & (pos < 2.0 - 0.25), axis=1)
    val = spe.cic_interpolate(g, f, pos[inside])
    exact = pos[inside] @ np.array([0.3, 0.2, -0.1])
    assert np.abs(val - exact).max() < 1e-12


def test_virial_terms_plane_wave():
    n, L = (16, 16, 16), (8.0, 8.0, 8.0)
    g = spe.Grid(n, L)
    X, Y, Z = g.coords()
    kx = 2 * np.pi * 2 / L[0]
    psi = np.exp(1j * kx * X) * np.ones((16, 16, 16))
    phi = np.zeros((16, 16, 16))
    v = spe.virial_terms(psi, phi, g)
    dx = g.spacing[0]
    j = np.sin(kx * dx) / dx
    nint = 14 ** 3
    assert v["TotalKineticE"] == pytest.approx(0.5 * j * j * nint * g.dV, rel=1e-12)
    assert abs(v["TotalQuantumE"]) < 1e-20
    assert v["MomentumX"] == pytest.approx(j * nint * g.dV, rel=1e-12)


def test_weighted_quantile_equal_weights_is_type7_quantile():
    """StatsBase documents that with equal weights the weighted quantile is the
    unweighted one (Hyndman-Fan type 7, numpy's default 'linear')."""
    rng = np.random.default_rng(11)
    v = rng.normal(size=257)
    p = np.linspace(0.0, 1.0, 21)
    got = spe.weighted_quantile(v, np.full(v.size, 0.37), p)
    assert np.allclose(got, np.quantile(v, p), rtol=0, atol=1e-12)


def test_weighted_quantile_hand_example():
    """v = (1, 2, 3, 4), w = (2, 1, 1, 4): S = (2, 3, 4, 8), w_1 = 2,
    h = p (8 - 2) + 2.  p = 0.5: h = 5 -> first S_k > 5 is S_4 = 8, so
    3 + (5 - 4)/(8 - 4) (4 - 3) = 3.25.  p = 0.1: h = 2.6 -> S_2 = 3,
    1 + 0.6 (2 - 1) = 1.6.  p = 0: h = 2 -> S_2 = 3 > 2, 1 + 0 = 1.
    p = 1: h = 8 -> no S_k > 8, the largest value 4.  A zero weight drops out."""
    v = np.array([4.0, 2.0, 9.0, 1.0, 3.0])
    w = np.array([4.0, 1.0, 0.0, 2.0, 1.0])
    got = spe.weighted_quantile(v, w, [0.5, 0.1, 0.0, 1.0])
    assert np.allclose(got, [3.25, 1.6, 1.0, 4.0], rtol=0, atol=1e-15)


def test_loop_diagnostics_of_a_gaussian():
    """Radii about the maximum of a centred Gaussian blob grow with p, R of
    the middle slice is positive, a plane-wave factor gives the momentum of
    virial_terms and the timestep limits follow compute_timestep."""
    n, L = (24, 24, 24), (6.0, 6.0, 6.0)
    g = spe.Grid(n, L)
    X, Y, Z = g.coords()
    k = 2 * np.pi / L[0]
    psi = np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / 2) * np.exp(1j * k * X)
    phi = -np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / 4)
    d = spe.loop_diagnostics(psi, phi, g, kappa=0.5)
    assert np.all(np.diff(d["radii"]) > 0) and d["radii"][0] > 0
    assert d["argmax"] == np.argmax(np.abs(psi) ** 2)
    assert d["R"] > 0
    assert d["MomentumX"] == pytest.approx(spe.virial_terms(psi, phi, g)["MomentumX"], rel=1e-14)
    assert d["dt_phase"] == pytest.approx(2 * g.spacing[0] ** 2 / np.pi)
    assert d["dt_grav"] == pytest.approx(2 * np.pi / np.abs(phi).max())
    assert d["dt_self"] == pytest.approx(2 * np.pi / 0.5 / np.abs(psi).max())


def _quadratic_tide_case(convention):
    g = spe.Grid((20, 16, 12), (10.0, 8.0, 6.0), convention)
    X, Y, Z = g.coords()
    rng = np.random.default_rng(3)
    # a positive density with a unique interior maximum off the box centre
    rho = 0.1 + np.exp(-((X - 1.3) ** 2 + (Y + 0.7) ** 2 + (Z - 0.9) ** 2)) + 0.01 * rng.random((12, 16, 20))
    T6 = (0.3, -0.1, -0.2, 0.05, -0.04, 0.02)
    return g, rho, T6, (X, Y, Z)


@pytest.mark.parametrize("convention", ["periodic", "reference"])
def test_tide_about_density_max_closed_form(convention):
    """The reference's value and gradient removal at the density maximum
    (src/physics/tidal_fields.jl:114-146, restated step by step with its 1-based
    ramps about div(N, 2)) equals, for the quadratic tide, the closed form
    1/2 (x-x_c)^T T (x-x_c) + (T x_c).(<x> - x_c) the kernels evaluate."""
    g, rho, T6, (X, Y, Z) = _quadratic_tide_case(convention)
    c = np.unravel_index(int(np.argmax(rho)), rho.shape)
    xc = np.array([X[0, 0, c[2]], Y[0, c[1], 0], Z[c[0], 0, 0]])
    m = np.array([np.sum(rho * X), np.sum(rho * Y), np.sum(rho * Z)]) / np.sum(rho)
    txx, tyy, tzz, txy, txz, tyz = T6
    T = np.array([[txx, txy, txz], [txy, tyy, tyz], [txz, tyz, tzz]])
    d = [X - xc[0], Y - xc[1], Z - xc[2]]
    closed = 0.5 * sum(T[a, b] * d[a] * d[b] for a in range(3) for b in range(3)) + (T @ xc) @ (m - xc)
    got = spe.centred_tidal_potential(g, T6, rho, "density_max")
    assert np.allclose(got, closed, rtol=0, atol=1e-12 * np.abs(closed).max())
    # what the reference's code leaves: only the value at x_c removed
    ref = spe.centred_tidal_potential(g, T6, rho, "reference")
    assert np.allclose(ref, spe.tidal_potential(g, T6) - 0.5 * xc @ T @ xc, rtol=0, atol=1e-13)


def test_tide_gradient_cancellation_needs_an_interior_maximum():
    g, rho, T6, _ = _quadratic_tide_case("periodic")
    rho[0, 0, 0] = 10.0
    with pytest.raises(IndexError):
        spe.centred_tidal_potential(g, T6, rho, "density_max")
