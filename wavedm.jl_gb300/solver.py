"""Reference-shaped operator API of the gpu=true path, on top of libwavedm.

Names, argument meanings and error behaviour follow WaveDM.jl (paths inside
that project); the state lives on the GPU in an SPEContext instead of being
passed around as host/device arrays:

* setup_grid                 src/physics/poisson.jl:8-15
* compute_timestep           src/physics/poisson.jl:35-50
* setup_fft_operators        src/solver/fft_operators.jl:8-15   (descriptor; the phase is built on the GPU)
* setup_absorption_boundary  src/solver/fft_operators.jl:22-27  (descriptor; separable tables on the GPU)
* apply_kick_step            src/solver/KDK.jl:37-77   (apply_kick_step!)
* apply_drift_step           src/solver/KDK.jl:88-101  (apply_drift_step!)
* compute_gravitational_potential  src/solver/gravity.jl:7-35
* parallel_poisson           src/parallel_poisson.jl:36-68
* SPE3D_waveDM               src/simulation_main.jl:41-865 (the loop of :536-559 and its
                             per-step diagnostics :551-653; graphics and IO are not part of the path)

A generic potential closure V(x, y, z, psi) cannot run inside the kernels
(src/solver/KDK.jl:64 evaluates it on the host every step); V is accepted as
None, a static array, or the built-in local term kappa |psi|^2, and a callable
raises ArgumentError-style ValueError as the Julia glue does.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .core import SPEContext


def setup_grid(Xmax, Ymax, Zmax, Nx, Ny, Nz):
    """x = LinRange(-X, X, N) per axis; returns (x, y, z, Delta, unit_cell_volumn)."""
    x = np.linspace(-Xmax, Xmax, Nx)
    y = np.linspace(-Ymax, Ymax, Ny)
    z = np.linspace(-Zmax, Zmax, Nz)
    d = np.array([x[1] - x[0], y[1] - y[0], z[1] - z[0]])
    return x, y, z, d, float(np.prod(d))


def compute_timestep(dx, Phi_all, kappa, psi, Tmax, Nt, autoset_timestep=False, autoset_timestep_ratio=0.5):
    """CFL bounds [2 dx^2/pi, 2 pi/max|Phi|, 2 pi/(|kappa| max|psi|)]; dt = Float32(Tmax/Nt)."""
    dt_phase = 2 * dx ** 2 / np.pi
    pmax = float(np.max(np.abs(Phi_all))) if Phi_all is not None else 0.0
    dt_grav = 2 * np.pi / pmax if pmax > 0 else np.inf
    amax = float(np.max(np.abs(psi))) if psi is not None else 0.0
    dt_si = 2 * np.pi / abs(kappa) / amax if kappa and amax > 0 else np.inf
    if autoset_timestep:
        lim = min(dt_phase, dt_grav, dt_si)
        Nt = int(np.ceil(Tmax / (autoset_timestep_ratio * lim)))
    t = np.linspace(0, Tmax, Nt)
    dt = float(np.float32(Tmax / Nt))
    return t, dt, Nt


@dataclass(frozen=True)
class LinearPhase:
    """Stands for the dense fftshift-ed exp(i Lap dt/2) of setup_fft_operators: the
    factor exp(-i k^2 dt/2) is built per mode on the GPU (FP64-built per-axis phases)."""

    dt: float


@dataclass(frozen=True)
class Border:
    """Stands for the dense tanh mask of setup_absorption_boundary (alpha, dt)."""

    absorb_coeff: float
    dt: float


def setup_fft_operators(Xmax, Ymax, Zmax, Nx, Ny, Nz, dt):
    return LinearPhase(float(dt))


def setup_absorption_boundary(Xmax, Ymax, Zmax, x, y, z, absorb_coeff, dt):
    return Border(float(absorb_coeff), float(dt))


def _check_V(V):
    if callable(V):
        raise ValueError("a potential closure V(x, y, z, psi) cannot run on the GPU path: pass None, a static "
                         "array [nz][ny][nx], or use kappa for the local term kappa |psi|^2")


def apply_kick_step(ctx: SPEContext, dt, t=0.0, return_potential=False):
    """psi <- exp(-i dt Phi_total) psi with Phi_total from the current |psi|^2.

    Mirrors apply_kick_step! (KDK.jl:37-77) except that psi stays on the device;
    with return_potential the host potential Phi (gravity part) is returned as
    the reference's Phi_all/Phi_WaveDM pair.
    """
    phi = ctx.get_phi() if return_potential else None
    ctx.kick(dt, t)
    return (phi, phi) if return_potential else None


def apply_drift_step(ctx: SPEContext, dt, border: Border | None = None):
    """psi <- border * ifft(exp(-i k^2 dt/2) fft(psi)) (KDK.jl:88-101); the border
    coefficient is the context's absorb_alpha (must match ``border``)."""
    ctx.drift(dt)


def compute_gravitational_potential(ctx: SPEContext):
    """Phi from |psi|^2 (gravity.jl:7-35): returns the host potential."""
    return ctx.get_phi()


_poisson_ctx = {}


def parallel_poisson(delta, N, rho, boundary="Periodic", backend="gpu"):
    """Phi with lap Phi = rho - <rho> on the periodic box of spacing delta (parallel_poisson.jl:36-68).

    ``N`` is accepted for signature compatibility (the reference passes
    [Nx-1, Ny-1, Nz-1]); the grid shape is rho's.  Callers multiply by 4 pi as
    gravity.jl:23 does.  Only periodic boundaries and the gpu backend exist
    here; other values raise like the reference's distributed backend.
    """
    if str(boundary).lower().startswith("vacuum"):
        raise NotImplementedError("vacuum boundaries (James algorithm / tree) are not on the GPU path")
    if backend not in ("gpu", "cuda"):
        raise NotImplementedError(f"backend {backend!r}: only the gpu backend exists in this library")
    rho = np.asarray(rho)
    if np.iscomplexobj(rho):
        rho = rho.real
    nz, ny, nx = rho.shape
    d = np.broadcast_to(np.asarray(delta, np.float64), (3,))
    key = (nx, ny, nz, float(d[0]), float(d[1]), float(d[2]))
    ctx = _poisson_ctx.get(key)
    if ctx is None:
        ctx = SPEContext((nx, ny, nz), (d[0] * nx, d[1] * ny, d[2] * nz), poisson_coeff=1.0)
        _poisson_ctx[key] = ctx
    return ctx.poisson(np.ascontiguousarray(rho, dtype=np.float32)).astype(np.float64)


def SPE3D_waveDM(*, Nx=64, Ny=None, Nz=None, Xmax=10.0, Ymax=None, Zmax=None, Nt=100, Tmax=1.0, IC=None, V=None,
                 KDK_flag=True, absorb_coeff=0.0, kappa=0.0, poisson_coeff=4 * np.pi, grid_convention="reference",
                 StepsBetweenSnapshots=None, tidal=None, particles=None, phase_mode="precise", mode=None,
                 gpu=True, keep_snapshots=False):
    """The gpu=true solver entry of SPE3D_waveDM with its keyword arguments for the path.

    IC: callable IC(x, y, z) -> complex (broadcast over the grid) or an array
    [Nz][Ny][Nx].  mode: "strang" (the documented KDK), "reference_loop" (the
    literal K(dt/2) D(dt) iteration, the default when KDK_flag is true as in
    simulation_main.jl:538) or "lie" (KDK_flag false).  tidal: callable t ->
    (Txx, Tyy, Tzz, Txy, Txz, Tyz) for the 1/2 x^T T x tide.  particles:
    (pos [n,3], mass [n]) CIC-deposited each step.  Returns a dict with psi, t,
    dt and per-snapshot diagnostics (mass, rho_max, centre of mass, virial sums).
    """
    if not gpu:
        raise ValueError("this library is the gpu=true path; there is no CPU fallback")
    _check_V(V)
    Ny = Ny or Nx
    Nz = Nz or Nx
    Ymax = Ymax or Xmax
    Zmax = Zmax or Xmax
    if mode is None:
        mode = "reference_loop" if KDK_flag else "lie"
    x, y, z, d, vol = setup_grid(Xmax, Ymax, Zmax, Nx, Ny, Nz)
    if grid_convention == "periodic":
        x = -Xmax + (2 * Xmax / Nx) * np.arange(Nx)
        y = -Ymax + (2 * Ymax / Ny) * np.arange(Ny)
        z = -Zmax + (2 * Zmax / Nz) * np.arange(Nz)
    if callable(IC):
        psi0 = np.asarray(IC(x[None, None, :], y[None, :, None], z[:, None, None]), np.complex128)
        psi0 = np.broadcast_to(psi0, (Nz, Ny, Nx))
    else:
        psi0 = np.asarray(IC)
    t = np.linspace(0, Tmax, Nt)
    dt = float(np.float32(Tmax / Nt))  # poisson.jl:47
    stride = StepsBetweenSnapshots or (Nt - 1)
    ctx = SPEContext((Nx, Ny, Nz), (2 * Xmax, 2 * Ymax, 2 * Zmax), convention=grid_convention,
                     poisson_coeff=poisson_coeff, kerr=kappa, absorb_alpha=absorb_coeff, phase_mode=phase_mode)
    try:
        ctx.set_psi(np.ascontiguousarray(psi0, np.complex64))
        if V is not None:
            ctx.set_static_potential(np.asarray(V, np.float32))
        if particles is not None:
            ctx.set_particles(*particles)
        records, snaps = [], []
        done = 0
        total = Nt - 1
        while done < total:
            n = min(stride, total - done)
            if tidal is not None:
                ctx.set_tidal([tidal(t0) for t0 in (done + np.arange(n + 1)) * dt])
            ctx.step(n, dt, t0=done * dt, mode=mode)
            done += n
            rec = ctx.reduce()
            rec["t"] = done * dt
            records.append(rec)
            if keep_snapshots:
                snaps.append(ctx.get_psi())
        out = {"psi": ctx.get_psi(), "t": t, "dt": dt, "Nt": Nt, "Prop": records}
        if keep_snapshots:
            out["snapshots"] = snaps
        return out
    finally:
        ctx.close()
