"""Seeded synthetic initial conditions and host-side schedules for the workloads.

No dataset is involved: every workload is generated in FP64 on the host with
``numpy.random.default_rng(20261203 + workload_index)`` and uploaded.

* soliton density rho_sol(r) = rho_c / (1 + 0.091 (r/r_c)^2)^8 (rho_c = 1);
* random-phase halo: ``nwaves`` plane waves with Maxwellian |k| (a 3D normal
  vector of per-axis width sigma_k), isotropic directions and uniform phases,
  snapped to the box's Fourier lattice so the field is periodic, normalised
  to <|W|^2> = 1 and shaped by sqrt(rho_NFW(r; r_s)) with the NFW profile
  scaled to a mean density of ``halo_mean`` over the box and softened at
  r = dx;
* a Gaussian random phase field (white noise smoothed by exp(-k^2 l^2/2),
  l = 2 dx, rescaled to standard deviation sigma);
* Plummer baryon particles (mass M, scale b), radius truncated at 0.45 L;
* the tidal tensor T(t) of a Hernquist host (M, a) along an eccentric orbit
  (pericentre, apocentre), integrated by leapfrog in FP64 with substeps.

Arrays are complex128 in C order [nz][ny][nx] (cast to complex64 for the GPU).
"""
from __future__ import annotations

import numpy as np

SEED0 = 20261203


def rng_for(workload):
    return np.random.default_rng(SEED0 + int(workload))


def axis_coords(n, L, convention="periodic"):
    if convention == "reference":
        return np.linspace(-L / 2, L / 2, n)
    return -L / 2 + (L / n) * np.arange(n)


def coords(n, L, convention="periodic"):
    nx, ny, nz = n
    Lx, Ly, Lz = L
    x = axis_coords(nx, Lx, convention)
    y = axis_coords(ny, Ly, convention)
    z = axis_coords(nz, Lz, convention)
    return x[None, None, :], y[None, :, None], z[:, None, None]


def radius(n, L, convention="periodic", centre=(0.0, 0.0, 0.0)):
    X, Y, Z = coords(n, L, convention)
    return np.sqrt((X - centre[0]) ** 2 + (Y - centre[1]) ** 2 + (Z - centre[2]) ** 2)


def rho_soliton(r, rc, rho_c=1.0):
    return rho_c / (1.0 + 0.091 * (r / rc) ** 2) ** 8


def gaussian_phase(n, L, rng, sigma=0.1, ell_cells=2.0):
    nx, ny, nz = n
    w = rng.standard_normal((nz, ny, nx))
    k2 = 0.0
    for a, (m, Lm) in enumerate(zip(n, L)):
        k = 2 * np.pi * np.fft.fftfreq(m, Lm / m)
        shape = [1, 1, 1]
        shape[2 - a] = m
        k2 = k2 + (k ** 2).reshape(shape)
    ell = ell_cells * (L[0] / n[0])
    th = np.real(np.fft.ifftn(np.fft.fftn(w) * np.exp(-0.5 * k2 * ell ** 2)))
    th -= th.mean()
    return th * (sigma / th.std())


def plane_wave_halo(n, L, rng, nwaves=4096, sigma_k=2.0):
    """Unit-variance periodic sum of plane waves with Maxwellian |k| and random phases."""
    nx, ny, nz = n
    k = rng.normal(0.0, sigma_k, size=(nwaves, 3))
    ph = rng.uniform(0.0, 2 * np.pi, size=nwaves)
    m = np.rint(k * np.array(L) / (2 * np.pi)).astype(np.int64)
    A = np.zeros((nz, ny, nx), np.complex128)
    np.add.at(A, (m[:, 2] % nz, m[:, 1] % ny, m[:, 0] % nx), np.exp(1j * ph))
    W = np.fft.ifftn(A) * (nx * ny * nz)
    return W / np.sqrt(np.mean(np.abs(W) ** 2))


def rho_nfw(r, rs, mean_density, soft):
    prof = 1.0 / (np.maximum(r, soft) / rs * (1 + np.maximum(r, soft) / rs) ** 2)
    return prof * (mean_density / prof.mean())


def soliton_noise_ic(n, L, rc, rng, sigma=0.1, convention="periodic"):
    """sqrt(rho_sol(r)) exp(i theta), theta a smoothed Gaussian random field."""
    r = radius(n, L, convention)
    th = gaussian_phase(n, L, rng, sigma=sigma)
    return np.sqrt(rho_soliton(r, rc)) * np.exp(1j * th)


def soliton_halo_ic(n, L, rc, rng, nwaves=4096, sigma_k=2.0, rs=4.0, halo_mean=0.01, convention="periodic"):
    """sqrt(rho_sol) plus a random-phase NFW-shaped halo."""
    r = radius(n, L, convention)
    W = plane_wave_halo(n, L, rng, nwaves=nwaves, sigma_k=sigma_k)
    env = np.sqrt(rho_nfw(r, rs, halo_mean, soft=L[0] / n[0]))
    return np.sqrt(rho_soliton(r, rc)) + env * W


def plummer_particles(rng, npart=100_000, M=10.0, b=0.5, rmax=None):
    """Isotropic Plummer sphere centred at the origin: positions [n,3], masses [n]."""
    pos = np.empty((0, 3))
    while len(pos) < npart:
        u = rng.uniform(0.0, 1.0, size=2 * npart)
        r = b / np.sqrt(u ** (-2.0 / 3.0) - 1.0)
        if rmax is not None:
            r = r[r < rmax]
        cz = rng.uniform(-1, 1, size=len(r))
        phi = rng.uniform(0, 2 * np.pi, size=len(r))
        sz = np.sqrt(1 - cz ** 2)
        p = np.stack([r * sz * np.cos(phi), r * sz * np.sin(phi), r * cz], axis=1)
        pos = np.concatenate([pos, p])
    pos = pos[:npart]
    return pos, np.full(npart, M / npart)


# ---------------------------------------------------------------------------
# Hernquist host tidal tensor along an orbit
# ---------------------------------------------------------------------------
FOUR_PI_G = 1.0


def hernquist_phi(r, M, a, G):
    return -G * M / (r + a)


def hernquist_hessian(R, M, a, G):
    """d_i d_j Phi at position R: Phi'' Rh Rh^T + Phi'/r (I - Rh Rh^T)."""
    r = np.linalg.norm(R)
    rh = R / r
    d1 = G * M / (r + a) ** 2
    d2 = -2 * G * M / (r + a) ** 3
    P = np.outer(rh, rh)
    return d2 * P + (d1 / r) * (np.eye(3) - P)


def hernquist_orbit_tidal(times, M=1e4, a=20.0, peri=30.0, apo=90.0, substeps=10, dt_hint=None):
    """T6 rows (xx, yy, zz, xy, xz, yz) of the host Hessian at each time.

    The orbit starts at apocentre on the +x axis moving along +y with the
    tangential speed that gives the requested pericentre (energy and angular
    momentum conservation), and is integrated with kick-drift-kick leapfrog in
    FP64, ``substeps`` substeps per interval of ``dt_hint`` (default: the
    spacing of ``times``).
    """
    G = FOUR_PI_G / (4 * np.pi)
    times = np.asarray(times, dtype=np.float64)
    dphi = hernquist_phi(peri, M, a, G) - hernquist_phi(apo, M, a, G)
    va = np.sqrt(2 * dphi / (1 - apo ** 2 / peri ** 2))
    x = np.array([apo, 0.0, 0.0])
    v = np.array([0.0, va, 0.0])

    def acc(p):
        r = np.linalg.norm(p)
        return -G * M / (r + a) ** 2 * p / r

    if dt_hint is None:
        dt_hint = float(np.min(np.diff(times))) if len(times) > 1 else 1.0
    h = dt_hint / substeps
    out = np.zeros((len(times), 6))
    t = 0.0
    for i, tt in enumerate(times):
        while t < tt - 1e-15:
            step = min(h, tt - t)
            v += 0.5 * step * acc(x)
            x += step * v
            v += 0.5 * step * acc(x)
            t += step
        Hm = hernquist_hessian(x, M, a, G)
        out[i] = [Hm[0, 0], Hm[1, 1], Hm[2, 2], Hm[0, 1], Hm[0, 2], Hm[1, 2]]
    return out


# ---------------------------------------------------------------------------
# the workloads
# ---------------------------------------------------------------------------
WORKLOADS = {
    1: dict(name="spe64_soliton_noise", n=64, L=20.0, steps=100),
    2: dict(name="spe256_soliton_halo", n=256, L=30.0, steps=1000),
    3: dict(name="spe384_tidal_cic", n=384, L=40.0, steps=2000),
    4: dict(name="ensemble_64x96_96x24_128x8", steps=500),
    5: dict(name="adjoint128", n=128, L=20.0, steps=200),
}


def dt_for(n, L):
    dx = L / n
    return dx * dx / 6.0


def workload(idx, n=None):
    """Return dict(psi0, n, L, dt, steps, poisson_coeff, tidal_schedule_fn, particles) for a workload.

    ``n`` overrides the grid size (same box and physics) for scaled-down cases.
    """
    w = dict(WORKLOADS[idx])
    rng = rng_for(idx)
    if idx == 1:
        N = n or w["n"]
        L = w["L"]
        psi = soliton_noise_ic((N, N, N), (L, L, L), rc=1.5, rng=rng, sigma=0.1)
        return dict(w, n=N, psi0=psi, L=L, dt=dt_for(N, L), poisson_coeff=1.0, tidal=None, particles=None)
    if idx == 2:
        N = n or w["n"]
        L = w["L"]
        psi = soliton_halo_ic((N, N, N), (L, L, L), rc=1.0, rng=rng)
        return dict(w, n=N, psi0=psi, L=L, dt=dt_for(N, L), poisson_coeff=1.0, tidal=None, particles=None)
    if idx == 3:
        N = n or w["n"]
        L = w["L"]
        psi = soliton_halo_ic((N, N, N), (L, L, L), rc=1.0, rng=rng)
        pos, m = plummer_particles(rng, 100_000, M=10.0, b=0.5, rmax=0.45 * L)
        dt = dt_for(N, L)
        return dict(w, n=N, psi0=psi, L=L, dt=dt, poisson_coeff=1.0,
                    tidal=lambda times: hernquist_orbit_tidal(times, dt_hint=dt), particles=(pos, m))
    raise KeyError(idx)


def ensemble_members(seed_idx=4, nwaves=1024):
    """Halos of workload 4: list of (n, L, psi0, T6) with rc ~ U[0.8, 2], amp ~ U[0, 0.05]."""
    rng = rng_for(seed_idx)
    out = []
    for N, count in ((64, 96), (96, 24), (128, 8)):
        L = 20.0
        for _ in range(count):
            rc = rng.uniform(0.8, 2.0)
            amp = rng.uniform(0.0, 0.05)
            psi = soliton_halo_ic((N, N, N), (L, L, L), rc=rc, rng=rng, nwaves=nwaves)
            out.append((N, L, psi, np.array([2 * amp, -amp, -amp, 0.0, 0.0, 0.0])))
    return out
