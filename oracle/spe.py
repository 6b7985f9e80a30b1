"""FP64 CPU restatement of WaveDM.jl's split-step Fourier KDK path (the oracle).

TEST INFRASTRUCTURE ONLY.  This module is the oracle that the CUDA library is
compared against; it is imported by ``tests/``, by ``__graft_entry__.smoke()``
and by the ``cpu_baseline`` / ``--impl reference`` legs of ``bench.py``.  The
product path (``wavedm.jl_gb300``) never imports it.

Everything is complex128 / float64 numpy with ``scipy.fft`` (pocketfft, threads
= ``workers``) standing in for FFTW.jl.  Array layout is ``psi[z, y, x]`` (x
fastest in memory), i.e. the C-order view of Julia's column-major
``psi[x, y, z]``.

Reference sources restated here (paths inside the WaveDM.jl project):

* ``src/physics/poisson.jl:8-15``      setup_grid (endpoint-inclusive LinRange grid)
* ``src/solver/fft_operators.jl:8-15`` drift factor exp(i*Lap*dt/2), k = m/(2X) cycles
* ``src/solver/fft_operators.jl:22-27`` tanh absorbing mask
* ``src/solver/gravity.jl:13-27``      rho = |psi|^2 - <|psi|^2>, Phi = 4pi*Poisson(rho) (+Phi_b)
* ``src/parallel_poisson.jl:3-4``      Phi_hat = -4pi rho_hat / |k|^2, k=0 removed
* ``src/solver/KDK.jl:52-73,88-101``   kick exp(-i dt Phi) psi, fft, phase, ifft, mask
* ``src/simulation_main.jl:536-547``   literal loop order K(dt/2) D(dt) per iteration
* ``docs/src/algorithms.md:120-142``   symmetric Strang K(dt/2) D(dt) K(dt/2)
* ``src/physics/tidal_fields.jl:114-146`` tidal potential with its value (and,
  as an option, its gradient) removed at the density maximum
* ``src/visualization/runtime.jl:210-238`` virial / kinetic / quantum / momentum sums
* ``test/simulation_SPE3D_validation.jl:85-88`` relative L2 error definition

Parity note: the Poisson solve lives in the unvendored PhysicalFFT.jl
(``fft_poisson``, compat "0.1", no Manifest pin), so its k-grid and k=0
handling are not visible in the reference; this oracle fixes them explicitly
(periodic k of the grid convention, Phi_hat(0) = 0).  Poisson parity is
therefore *unpinned* against PhysicalFFT and pinned only by analytic cases.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np
import scipy.fft as sfft

WORKERS = os.cpu_count() or 1


# ---------------------------------------------------------------------------
# grid conventions
# ---------------------------------------------------------------------------

@dataclass
class Grid:
    """Uniform 3D grid.

    ``convention="periodic"``: box [-L/2, L/2) with spacing L/N and angular
    wavenumbers 2*pi*fftfreq(N, L/N).
    ``convention="reference"``: the reference's endpoint-inclusive grid
    x = LinRange(-X, X, N) with X = L/2, spacing 2X/(N-1)
    (``src/physics/poisson.jl:8-15``) and drift wavenumbers 2*pi*m/(2X)
    (``src/solver/fft_operators.jl:9-13``: LinRange(-N/4X, N/4X-1/2X, N)
    fftshift-ed is m/(2X) cycles per unit length).
    """

    n: tuple  # (nx, ny, nz)
    L: tuple  # (Lx, Ly, Lz) full box lengths
    convention: str = "periodic"

    def axis(self, a):
        n, L = self.n[a], self.L[a]
        if self.convention == "periodic":
            d = L / n
            x = -L / 2 + d * np.arange(n)
        elif self.convention == "reference":
            X = L / 2
            x = np.linspace(-X, X, n)
            d = x[1] - x[0]
        else:
            raise ValueError(self.convention)
        k = 2 * np.pi * sfft.fftfreq(n) * n / L  # m * 2pi / L in both conventions
        return x, d, k

    @property
    def spacing(self):
        return tuple(self.axis(a)[1] for a in range(3))

    @property
    def dV(self):
        dx, dy, dz = self.spacing
        return dx * dy * dz

    def coords(self):
        """Broadcastable (z, y, x)-ordered coordinate arrays X, Y, Z."""
        x = self.axis(0)[0]
        y = self.axis(1)[0]
        z = self.axis(2)[0]
        return x[None, None, :], y[None, :, None], z[:, None, None]

    def k2(self):
        kx = self.axis(0)[2]
        ky = self.axis(1)[2]
        kz = self.axis(2)[2]
        return kx[None, None, :] ** 2 + ky[None, :, None] ** 2 + kz[:, None, None] ** 2


def setup_grid(Xmax, Ymax, Zmax, Nx, Ny, Nz):
    """Restates ``src/physics/poisson.jl:8-15``: endpoint-inclusive axes and spacing."""
    x = np.linspace(-Xmax, Xmax, Nx)
    y = np.linspace(-Ymax, Ymax, Ny)
    z = np.linspace(-Zmax, Zmax, Nz)
    d = np.array([x[1] - x[0], y[1] - y[0], z[1] - z[0]])
    return x, y, z, d, float(np.prod(d))


def setup_fft_operators(Xmax, Ymax, Zmax, Nx, Ny, Nz, dt):
    """Restates ``src/solver/fft_operators.jl:8-15`` (dense fftshift-ed drift factor).

    Returned in (z, y, x) order, i.e. the transpose of the Julia array.
    """
    def kax(N, X):
        return np.linspace(-N / 4 / X, N / 4 / X - 1 / 2 / X, N)

    kx, ky, kz = kax(Nx, Xmax), kax(Ny, Ymax), kax(Nz, Zmax)
    lap = (2j * np.pi * kx[None, None, :]) ** 2 + (2j * np.pi * ky[None, :, None]) ** 2 \
        + (2j * np.pi * kz[:, None, None]) ** 2
    return np.fft.fftshift(np.exp(1j * lap * dt / 2))


def absorption_mask(grid: Grid, alpha, dt):
    """Restates ``src/solver/fft_operators.jl:22-27`` with X = L/2 and w = X/50."""
    X, Y, Z = grid.coords()
    Xm, Ym, Zm = grid.L[0] / 2, grid.L[1] / 2, grid.L[2] / 2
    wx, wy, wz = Xm / 50, Ym / 50, Zm / 50
    s = (6 - np.tanh((X + Xm) / wx) + np.tanh((X - Xm) / wx)
         - np.tanh((Y + Ym) / wy) + np.tanh((Y - Ym) / wy)
         - np.tanh((Z + Zm) / wz) + np.tanh((Z - Zm) / wz))
    return np.exp(-alpha * s * dt)


# ---------------------------------------------------------------------------
# operators
# ---------------------------------------------------------------------------

def fftn(a):
    return sfft.fftn(a, workers=WORKERS)


def ifftn(a):
    return sfft.ifftn(a, workers=WORKERS)


def poisson(rho, grid: Grid, coeff):
    """Phi with lap(Phi) = coeff * (rho - <rho>): Phi_hat = -coeff rho_hat / k^2, Phi_hat(0)=0.

    ``src/solver/gravity.jl:13-23`` (mean removal, 4pi prefactor) and
    ``src/parallel_poisson.jl:3-4`` (spectral form).
    """
    k2 = grid.k2()
    rk = sfft.rfftn(rho, workers=WORKERS)
    nxh = rk.shape[2]
    k2h = k2[:, :, :nxh]
    with np.errstate(divide="ignore", invalid="ignore"):
        g = np.where(k2h > 0, -coeff / np.where(k2h > 0, k2h, 1.0), 0.0)
    return sfft.irfftn(rk * g, s=rho.shape, workers=WORKERS)


def tidal_potential(grid: Grid, T6):
    """1/2 x^T T x with T = (Txx, Tyy, Tzz, Txy, Txz, Tyz) about the box centre.

    Stands in for ``src/physics/tidal_fields.jl:64-146``: the reference subtracts
    the host potential's value and gradient at the centre, leaving the
    quadratic (tidal) part that this form models.
    """
    X, Y, Z = grid.coords()
    txx, tyy, tzz, txy, txz, tyz = T6
    return 0.5 * (txx * X * X + tyy * Y * Y + tzz * Z * Z) + txy * X * Y + txz * X * Z + tyz * Y * Z


def cancel_field_gradient_at_center(field, center, rho):
    """Restatement of ``cancel_field_gradient_at_center!`` (``src/physics/tidal_fields.jl:126-146``),
    returning the field it computes.

    ``center`` is the (z, y, x) index of the density maximum.  The gradient is
    the central difference at the centre in index units (``:127-129``); a
    linear ramp (i - div(N, 2)) * gradient per axis, with the 1-based index i
    (``:131-141``), is subtracted, and the density-weighted mean of the ramps
    added back (``:143``).  Like Julia's indexing, a centre on the edge of the
    grid has no central difference and raises.

    The reference's function assigns ``field -= dp_field``, which rebinds its
    local ``field`` to a new array, and its caller (``:115``) discards the
    return value: the caller's potential keeps its gradient.  Callers of this
    restatement choose whether to use the returned field.
    """
    nz, ny, nx = field.shape
    cz, cy, cx = center
    if not (0 < cx < nx - 1 and 0 < cy < ny - 1 and 0 < cz < nz - 1):
        raise IndexError("density maximum on the edge of the grid: no central difference (BoundsError in Julia)")
    dp_dx = (field[cz, cy, cx + 1] - field[cz, cy, cx - 1]) / 2
    dp_dy = (field[cz, cy + 1, cx] - field[cz, cy - 1, cx]) / 2
    dp_dz = (field[cz + 1, cy, cx] - field[cz - 1, cy, cx]) / 2
    out = np.array(field, dtype=np.float64, copy=True)
    ramp_x = (np.arange(1, nx + 1) - nx // 2)[None, None, :] * dp_dx * np.ones_like(out)
    out = out - ramp_x
    sum_pe = np.sum(ramp_x * rho)
    ramp_y = (np.arange(1, ny + 1) - ny // 2)[None, :, None] * dp_dy * np.ones_like(out)
    out = out - ramp_y
    sum_pe += np.sum(ramp_y * rho)
    ramp_z = (np.arange(1, nz + 1) - nz // 2)[:, None, None] * dp_dz * np.ones_like(out)
    out = out - ramp_z
    sum_pe += np.sum(ramp_z * rho)
    return out + sum_pe / np.sum(rho)


def centred_tidal_potential(grid: Grid, T6, rho, centering):
    """The tidal potential after add_tidal_potential!'s treatment at the density
    maximum (``src/physics/tidal_fields.jl:114-115``), for the quadratic tide.

    ``rho`` is |psi|^2 of the state being kicked (the loop's ``rho``,
    ``src/simulation_main.jl:550``); its maximum is the first in memory order,
    as Julia's findmax takes it.
    * ``"reference"``: the value at the maximum subtracted (``:114``), and the
      gradient cancellation computed but not applied, as in the reference
      (see cancel_field_gradient_at_center);
    * ``"density_max"``: the field the gradient cancellation computes.
    """
    pot = tidal_potential(grid, T6) * np.ones(rho.shape)
    c = np.unravel_index(int(np.argmax(rho)), rho.shape)
    pot = pot - pot[c]
    cancelled = cancel_field_gradient_at_center(pot, c, rho)
    if centering == "reference":
        return pot
    if centering == "density_max":
        return cancelled
    raise ValueError(centering)


def cic_deposit(grid: Grid, pos, mass):
    """Cloud-in-cell density (mass / dV per cell), periodic wrap.

    Particle position p maps to the continuous index u = (p - x0)/dx where x0
    is the first grid coordinate of the axis.
    """
    nx, ny, nz = grid.n
    rho = np.zeros((nz, ny, nx))
    idx = []
    for a in range(3):
        x, d, _ = grid.axis(a)
        u = (pos[:, a] - x[0]) / d
        i0 = np.floor(u).astype(np.int64)
        f = u - i0
        idx.append((i0, f))
    (ix, fx), (iy, fy), (iz, fz) = idx
    for dz in (0, 1):
        wz = fz if dz else 1 - fz
        for dy in (0, 1):
            wy = fy if dy else 1 - fy
            for dx in (0, 1):
                wx = fx if dx else 1 - fx
                np.add.at(rho, ((iz + dz) % nz, (iy + dy) % ny, (ix + dx) % nx), mass * wx * wy * wz)
    return rho / grid.dV


def cic_interpolate(grid: Grid, field3, pos):
    """Cloud-in-cell interpolation of a real mesh field at particle positions."""
    nx, ny, nz = grid.n
    idx = []
    for a in range(3):
        x, d, _ = grid.axis(a)
        u = (pos[:, a] - x[0]) / d
        i0 = np.floor(u).astype(np.int64)
        idx.append((i0, u - i0))
    (ix, fx), (iy, fy), (iz, fz) = idx
    out = np.zeros(len(pos))
    for dz in (0, 1):
        wz = fz if dz else 1 - fz
        for dy in (0, 1):
            wy = fy if dy else 1 - fy
            for dx in (0, 1):
                wx = fx if dx else 1 - fx
                out += wx * wy * wz * field3[(iz + dz) % nz, (iy + dy) % ny, (ix + dx) % nx]
    return out


# ---------------------------------------------------------------------------
# the KDK step
# ---------------------------------------------------------------------------

@dataclass
class Physics:
    """Per-run physics switches (keywords of ``SPE3D_waveDM`` that the path uses)."""

    poisson_coeff: float = 1.0          # 4*pi*G; the reference uses 4pi with G=1 (gravity.jl:23)
    kerr: float = 0.0                   # local potential kappa*|psi|^2 (simulation_main.jl:56 kappa)
    absorb_alpha: float = 0.0           # fft_operators.jl:22-27 (0 => mask == 1)
    V_static: np.ndarray | None = None  # static external potential (z,y,x)
    rho_b: np.ndarray | None = None     # static baryon density added before the Poisson solve
    tidal: object = None                # callable t -> T6, or None
    tidal_centering: str = "box_centre"  # "box_centre", "reference" or "density_max" (centred_tidal_potential)

    def tidal_at(self, t):
        if self.tidal is None:
            return None
        return self.tidal(t)


def potential(psi, grid: Grid, phys: Physics, t):
    """Phi_total = Poisson(|psi|^2 (+rho_b)) + V_static + V_tidal(t)  (gravity.jl:13-27; KDK.jl:59-65)."""
    rho = np.abs(psi) ** 2
    if phys.rho_b is not None:
        rho = rho + phys.rho_b
    phi = poisson(rho, grid, phys.poisson_coeff) if phys.poisson_coeff != 0 else np.zeros(psi.shape)
    if phys.V_static is not None:
        phi = phi + phys.V_static
    T6 = phys.tidal_at(t)
    if T6 is not None:
        if phys.tidal_centering == "box_centre":
            phi = phi + tidal_potential(grid, T6)
        else:
            phi = phi + centred_tidal_potential(grid, T6, np.abs(psi) ** 2, phys.tidal_centering)
    return phi


def kick(psi, phi, dt, kerr=0.0):
    """psi <- exp(-i dt (Phi + kerr |psi|^2)) psi   (``src/solver/KDK.jl:65-69``)."""
    pot = phi if kerr == 0 else phi + kerr * np.abs(psi) ** 2
    return np.exp(-1j * dt * pot) * psi


def drift(psi, grid: Grid, dt):
    """psi <- ifft(exp(-i k^2 dt/2) fft(psi))   (``src/solver/KDK.jl:88-91``)."""
    return ifftn(fftn(psi) * np.exp(-0.5j * dt * grid.k2()))


def kdk_step(psi, grid: Grid, phys: Physics, t, dt, mode="strang", mask=None):
    """One step.

    ``mode="strang"``: K(dt/2) D(dt) [mask] K(dt/2) with the second kick's
    potential recomputed from the drifted density (``docs/src/algorithms.md:120-142``).
    ``mode="reference_loop"``: the literal reference iteration K(dt/2) D(dt) [mask]
    (``src/simulation_main.jl:538-547``, KDK_flag=true).
    ``mode="lie"``: K(dt) D(dt) [mask] (KDK_flag=false).
    The absorbing mask is applied right after the inverse FFT as in
    ``src/solver/KDK.jl:95-96``.
    """
    if mode == "strang":
        psi = kick(psi, potential(psi, grid, phys, t), dt / 2, phys.kerr)
        psi = drift(psi, grid, dt)
        if mask is not None:
            psi = psi * mask
        psi = kick(psi, potential(psi, grid, phys, t + dt), dt / 2, phys.kerr)
        return psi
    if mode in ("reference_loop", "lie"):
        dk = dt / 2 if mode == "reference_loop" else dt
        psi = kick(psi, potential(psi, grid, phys, t), dk, phys.kerr)
        psi = drift(psi, grid, dt)
        if mask is not None:
            psi = psi * mask
        return psi
    raise ValueError(mode)


def run(psi0, grid: Grid, phys: Physics, dt, nsteps, t0=0.0, mode="strang"):
    """Advance ``nsteps`` steps from time t0."""
    mask = absorption_mask(grid, phys.absorb_alpha, dt) if phys.absorb_alpha else None
    psi = np.asarray(psi0, dtype=np.complex128)
    t = t0
    for _ in range(nsteps):
        psi = kdk_step(psi, grid, phys, t, dt, mode, mask)
        t += dt
    return psi


# ---------------------------------------------------------------------------
# diagnostics and metrics
# ---------------------------------------------------------------------------

def rel_l2(a, b):
    """sqrt(mean|a-b|^2)/sqrt(mean|b|^2)  (``test/simulation_SPE3D_validation.jl:85-88``)."""
    a = np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    return float(np.sqrt(np.mean(np.abs(a - b) ** 2)) / np.sqrt(np.mean(np.abs(b) ** 2)))


def mass(psi, grid: Grid):
    """sum(|psi|^2) dV   (``src/simulation_main.jl:652``)."""
    return float(np.sum(np.abs(psi) ** 2) * grid.dV)


def _grad_central(f, d):
    """Second-order central differences (z,y,x order of d) on the interior."""
    dz, dy, dx = d
    gx = (f[1:-1, 1:-1, 2:] - f[1:-1, 1:-1, :-2]) / (2 * dx)
    gy = (f[1:-1, 2:, 1:-1] - f[1:-1, :-2, 1:-1]) / (2 * dy)
    gz = (f[2:, 1:-1, 1:-1] - f[:-2, 1:-1, 1:-1]) / (2 * dz)
    return gx, gy, gz


def virial_terms(psi, phi, grid: Grid):
    """Restates ``src/visualization/runtime.jl:210-238`` on the interior cells.

    Returns dict with VirialPotential = -1/2 sum rho*Phi dV, TotalKineticE =
    1/2 sum (rho v)^2/rho dV, TotalQuantumE = 1/2 sum |grad sqrt rho|^2 dV,
    Virial = 2K + 2Q - VirialPotential and Momentum{X,Y,Z} = sum rho v dV.
    grad_central (PhysicalFDM, unvendored) is taken as the second-order
    central difference; only interior cells [2:end-1] enter every sum.
    """
    dx, dy, dz = grid.spacing
    d = (dz, dy, dx)
    rho = np.abs(psi) ** 2
    sq = np.sqrt(rho)
    px, py, pz = _grad_central(psi, d)
    c = np.conj(psi[1:-1, 1:-1, 1:-1])
    p = psi[1:-1, 1:-1, 1:-1]
    # rho v = (psi* grad psi - psi grad psi*)/(2i) = Im(psi* grad psi)
    jx = np.imag(c * px)
    jy = np.imag(c * py)
    jz = np.imag(c * pz)
    ri = rho[1:-1, 1:-1, 1:-1]
    dV = grid.dV
    W = -0.5 * np.sum(ri * phi[1:-1, 1:-1, 1:-1]) * dV
    with np.errstate(divide="ignore", invalid="ignore"):
        K = 0.5 * np.sum(np.where(ri > 0, (jx ** 2 + jy ** 2 + jz ** 2) / np.where(ri > 0, ri, 1), 0.0)) * dV
    sx, sy, sz = _grad_central(sq, d)
    Q = 0.5 * np.sum(sx ** 2 + sy ** 2 + sz ** 2) * dV
    del p
    return {
        "VirialPotential": float(W),
        "TotalKineticE": float(K),
        "TotalQuantumE": float(Q),
        "Virial": float(2 * K + 2 * Q - W),
        "MomentumX": float(np.sum(jx) * dV),
        "MomentumY": float(np.sum(jy) * dV),
        "MomentumZ": float(np.sum(jz) * dV),
    }


def weighted_quantile(v, w, p):
    """Weighted quantiles of ``v`` at probabilities ``p`` with weights ``w``.

    Restates StatsBase's ``quantile(v, w::AbstractWeights, p)`` for weights other
    than FrequencyWeights (StatsBase compat "0.34", ``Project.toml:103``; called
    as ``quantile(r_mass_center[:], weights(rho[:]), 0.1:0.1:0.9)`` at
    ``src/simulation_main.jl:641``), element by element:
    zero weights are dropped; the pairs (v, w) are sorted; with S_k the
    cumulative weight and h = p (sum w - w_1) + w_1, the first k with S_k > h
    gives v_{k-1} + (h - S_{k-1}) / (S_k - S_{k-1}) (v_k - v_{k-1}), where v_0 = 0
    and S_0 = 0; when no S_k exceeds h the result is the largest v.
    Cumulative sums are FP64 here; the reference accumulates in the weights'
    element type.
    """
    v = np.asarray(v, np.float64).ravel()
    w = np.asarray(w, np.float64).ravel()
    keep = w != 0
    v, w = v[keep], w[keep]
    order = np.lexsort((w, v))
    v, w = v[order], w[order]
    S = np.cumsum(w)
    total, w1 = S[-1], w[0]
    out = []
    for pp in np.atleast_1d(p):
        h = pp * (total - w1) + w1
        k = int(np.searchsorted(S, h, side="right"))
        if k >= len(v):
            out.append(v[-1])
            continue
        vprev = v[k - 1] if k else 0.0
        sprev = S[k - 1] if k else 0.0
        out.append(vprev + (h - sprev) / (S[k] - sprev) * (v[k] - vprev))
    return np.array(out)


def loop_diagnostics(psi, phi, grid: Grid, kappa=0.0):
    """The per-step host diagnostics of the reference loop, restated in FP64.

    * ``rho_max, rho_max_id = findmax(rho)`` and the distances from that cell,
      ``r_mass_center`` (``src/simulation_main.jl:553-555``; first maximum in
      x-fastest order);
    * ``R = std(r[:, :, div(end, 2)], aweights(|psi|^2 on that slice))``
      (``:558``), with r the distance from the coordinate origin and the
      uncorrected weighted variance (StatsBase's default for ``std`` with
      weights);
    * the radii ``quantile(r_mass_center[:], weights(rho[:]), 0.1:0.1:0.9)``
      (``:641``) by ``weighted_quantile``;
    * momentum sums of ``src/visualization/runtime.jl:229-231`` (interior cells,
      as ``virial_terms``);
    * the timestep limits of ``compute_timestep`` (``src/physics/poisson.jl:35-50``):
      2 dx^2/pi, 2 pi / max|Phi|, 2 pi / (|kappa| max|psi|).
    """
    rho = np.abs(psi) ** 2
    nz, ny, nx = rho.shape
    arg = int(np.argmax(rho))
    cz, rem = divmod(arg, nx * ny)
    cy, cx = divmod(rem, nx)
    X, Y, Z = grid.coords()
    dx, dy, dz = grid.spacing
    if np.isclose(dx, dy, rtol=1e-12, atol=0) and np.isclose(dx, dz, rtol=1e-12, atol=0):
        # cubic cells: distances from integer cell offsets, so equal distances
        # tie exactly (FP64 coordinate differences would break such ties by
        # rounding noise and make the tie order, which the interpolation at a
        # group's first element depends on, arbitrary)
        i = np.arange(nx)[None, None, :] - cx
        j = np.arange(ny)[None, :, None] - cy
        k = np.arange(nz)[:, None, None] - cz
        r_mc = dx * np.sqrt((i * i + j * j + k * k).astype(np.float64))
    else:
        r_mc = np.sqrt((X - X[0, 0, cx]) ** 2 + (Y - Y[0, cy, 0]) ** 2 + (Z - Z[cz, 0, 0]) ** 2)
    zs = max(nz // 2 - 1, 0)
    r0 = np.sqrt(X[0] ** 2 + Y[0] ** 2 + Z[zs] ** 2)
    w0 = rho[zs]
    mean = np.sum(w0 * r0) / np.sum(w0)
    R = np.sqrt(np.sum(w0 * (r0 - mean) ** 2) / np.sum(w0))
    vt = virial_terms(psi, phi, grid)
    phimax = float(np.max(np.abs(phi)))
    psimax = float(np.sqrt(rho.max()))
    return {
        "rho_max": float(rho.max()),
        "argmax": arg,
        "R": float(R),
        "radii": weighted_quantile(r_mc, rho, np.arange(1, 10) / 10.0),
        "MomentumX": vt["MomentumX"],
        "MomentumY": vt["MomentumY"],
        "MomentumZ": vt["MomentumZ"],
        "phi_abs_max": phimax,
        "psi_abs_max": psimax,
        "dt_phase": 2 * dx * dx / np.pi,
        "dt_grav": 2 * np.pi / phimax if phimax > 0 else np.inf,
        "dt_self": 2 * np.pi / abs(kappa) / psimax if kappa != 0 and psimax > 0 else np.inf,
    }


def spectral_energy(psi, grid: Grid, phys: Physics, t=0.0):
    """Total energy E = 1/2 sum |grad psi|^2 dV + 1/2 sum rho Phi_grav dV + sum rho V_ext dV."""
    dV = grid.dV
    N = psi.size
    ek = 0.5 * np.sum(grid.k2() * np.abs(fftn(psi)) ** 2) * dV / N
    rho = np.abs(psi) ** 2
    e = ek
    if phys.poisson_coeff != 0:
        pg = poisson(rho + (phys.rho_b if phys.rho_b is not None else 0), grid, phys.poisson_coeff)
        e += 0.5 * np.sum(rho * pg) * dV
    if phys.V_static is not None:
        e += np.sum(rho * phys.V_static) * dV
    T6 = phys.tidal_at(t)
    if T6 is not None:
        e += np.sum(rho * tidal_potential(grid, T6)) * dV
    if phys.kerr:
        e += 0.5 * phys.kerr * np.sum(rho * rho) * dV
    return float(e)
