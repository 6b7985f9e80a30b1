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
                 gpu=True, keep_snapshots=False, outputdir=None, title="WaveDM", suffix="GB300", plot_virial=True,
                 uL=1.0):
    """The gpu=true solver entry of SPE3D_waveDM with its keyword arguments for the path.

    IC: callable IC(x, y, z) -> complex (broadcast over the grid) or an array
    [Nz][Ny][Nx].  mode: "strang" (the documented KDK), "reference_loop" (the
    literal K(dt/2) D(dt) iteration, the default when KDK_flag is true as in
    simulation_main.jl:538) or "lie" (KDK_flag false).  tidal: callable t ->
    (Txx, Tyy, Tzz, Txy, Txz, Tyz) for the 1/2 x^T T x tide.  particles:
    (pos [n,3], mass [n]) CIC-deposited once (static).  Returns a dict with psi, t,
    dt and the per-snapshot diagnostics of the reference loop (wdm_diagnostics:
    mass, density maximum and its index, the radii R1..R9 about it, R, virial
    and momentum sums, timestep limits).  With outputdir, writes the
    reference's "<title>, <suffix> - Prop.csv" (save_property_dataframe,
    src/io/save.jl:41-72) and the final state "<title>, <suffix> - Prop.npz"
    with the keys of save_evolution_results (src/io/save.jl:25-34); the .npz
    stands in for JLD2, which needs an HDF5 library (the Julia module writes
    the .jld2 itself).
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
        psi_last_t = None
        if tidal is not None:
            # one clocked schedule for the run: row s is the tide at time s dt
            ctx.set_tidal([tidal(t0) for t0 in np.arange(total + 1) * dt], t_first=0.0, t_step=dt)
        while done < total:
            n = min(stride, total - done)
            if outputdir is not None and done + n == total and n > 1:
                # the state one step before the end (psi_last_t of the reference loop)
                ctx.step(n - 1, dt, t0=done * dt, mode=mode)
                psi_last_t = ctx.get_psi()
                ctx.step(1, dt, t0=(done + n - 1) * dt, mode=mode)
            else:
                if outputdir is not None and done + n == total:
                    psi_last_t = ctx.get_psi()
                ctx.step(n, dt, t0=done * dt, mode=mode)
            done += n
            rec = ctx.diagnostics()
            rec["t"] = done * dt
            records.append(rec)
            if keep_snapshots:
                snaps.append(ctx.get_psi())
        out = {"psi": ctx.get_psi(), "t": t, "dt": dt, "Nt": Nt, "Prop": records}
        if keep_snapshots:
            out["snapshots"] = snaps
        if outputdir is not None:
            out["Prop.csv"] = save_property_dataframe(records, outputdir, title, suffix, plot_virial=plot_virial, uL=uL)
            out["Prop.npz"] = save_evolution_results(out["psi"], ctx.get_phi(), psi_last_t, None, outputdir, title,
                                                     suffix)
        return out
    finally:
        ctx.close()


PROP_COLUMNS = ("t", "R", "R1", "R2", "R3", "R4", "R5", "R6", "R7", "R8", "R9", "TotalMass")
PROP_VIRIAL_COLUMNS = ("PE_abs", "KE", "QE", "Virial", "MomentumX", "MomentumY", "MomentumZ")


def save_property_dataframe(records, outputdir, title, suffix, plot_virial=True, uL=1.0):
    """Write "<title>, <suffix> - Prop.csv" as src/io/save.jl:41-72 does: one row
    per record of SPEContext.diagnostics() (plus its "t"), columns t, R,
    R1..R9 (lengths times uL, as the loop stores them), TotalMass and, with
    plot_virial, PE_abs KE QE Virial MomentumX..Z.  Returns the path."""
    import csv
    import os

    cols = PROP_COLUMNS + (PROP_VIRIAL_COLUMNS if plot_virial else ())
    path = os.path.join(outputdir, f"{title}, {suffix} - Prop.csv")
    with open(path, "w", newline="") as f:
        w = csv.writer(f)
        w.writerow(cols)
        for r in records:
            row = [r["t"], r["R"] * uL] + [r[f"radius_{k}0"] * uL for k in range(1, 10)] + [r["mass"]]
            if plot_virial:
                row += [r["VirialPotential"], r["TotalKineticE"], r["TotalQuantumE"], r["Virial"],
                        r["MomentumX"], r["MomentumY"], r["MomentumZ"]]
            w.writerow([repr(float(v)) for v in row])
    return path


def save_evolution_results(psi, phi_all, psi_last_t, averaged_psi2, outputdir, title, suffix):
    """The final state with the keys of src/io/save.jl:25-34 ("ψ", "Φ_all",
    "ψ_last_t", "ψ2_averaged"), as "<title>, <suffix> - Prop.npz" (arrays in the
    library's [nz][ny][nx] order; an absent array is stored as an empty one).
    Returns the path."""
    import os

    path = os.path.join(outputdir, f"{title}, {suffix} - Prop.npz")
    empty = np.zeros(0)
    np.savez(path, **{"ψ": psi, "Φ_all": phi_all,
                      "ψ_last_t": psi_last_t if psi_last_t is not None else empty,
                      "ψ2_averaged": averaged_psi2 if averaged_psi2 is not None else empty})
    return path
