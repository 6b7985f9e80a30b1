"""Host-side handle on one libwavedm context (one grid size, `batch` halos).

Arrays may be numpy arrays (host memory; copied through the C ABI's host
path) or CUDA tensors exposing ``data_ptr()`` and ``is_cuda`` (device memory;
used in place).  Layout is C order [batch][nz][ny][nx].
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from ._abi import DEVICE, HOST, check


def _is_device(a):
    return getattr(a, "is_cuda", False)


def _ptr(a):
    if _is_device(a):
        return C.c_void_p(a.data_ptr()), DEVICE
    if not isinstance(a, np.ndarray):
        raise TypeError(f"expected a numpy array or a CUDA tensor, got {type(a)!r}")
    if not a.flags.c_contiguous:
        raise ValueError("arrays must be C-contiguous ([nz][ny][nx], x fastest)")
    return C.c_void_p(a.ctypes.data), HOST


class SPEContext:
    """A device-resident Schroedinger-Poisson state and its fused KDK pipeline.

    Parameters mirror ``wdm_desc``: grid points ``n=(nx, ny, nz)``, box
    lengths ``L=(Lx, Ly, Lz)``, grid ``convention`` ("periodic" or
    "reference"), ``poisson_coeff`` (4 pi G), ``kerr`` (kappa of kappa|psi|^2),
    ``absorb_alpha`` (tanh mask), ``phase_mode`` ("plain" or "precise") and
    ``batch`` (independent halos of this size).
    """

    def __init__(self, n, L, convention="periodic", poisson_coeff=1.0, kerr=0.0, absorb_alpha=0.0,
                 phase_mode="precise", batch=1):
        self.lib = _abi.load()
        nx, ny, nz = (int(v) for v in n)
        lx, ly, lz = (float(v) for v in L)
        self.n = (nx, ny, nz)
        self.L = (lx, ly, lz)
        self.convention = convention
        self.batch = int(batch)
        self.shape = (nz, ny, nx) if self.batch == 1 else (self.batch, nz, ny, nx)
        d = _abi.WdmDesc(nx, ny, nz, lx, ly, lz, _abi.CONVENTIONS[convention], float(poisson_coeff),
                         float(kerr), float(absorb_alpha), _abi.PHASE_MODES[phase_mode], self.batch)
        h = C.c_void_p()
        check(self.lib.wdm_create(C.byref(d), C.byref(h)))
        self._h = h

    @property
    def cell_volume(self):
        """dx dy dz of the grid convention (periodic: L/n, reference: L/(n - 1))."""
        k = 0 if self.convention == "periodic" else 1
        return float(np.prod([L / (n - k) for L, n in zip(self.L, self.n)]))

    # lifecycle -------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self.lib.wdm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        if not self._h:
            raise RuntimeError("context is closed")
        return self._h

    def _check(self, st):
        return check(st, self.handle)

    # state -----------------------------------------------------------------
    def set_psi(self, psi):
        if not _is_device(psi):
            psi = np.ascontiguousarray(psi, dtype=np.complex64)
            if psi.size != int(np.prod(self.shape)):
                raise ValueError(f"psi has {psi.size} elements, the grid needs {int(np.prod(self.shape))}")
        p, w = _ptr(psi)
        self._check(self.lib.wdm_set_psi(self.handle, p, w))

    def get_psi(self, out=None):
        if out is None:
            out = np.empty(self.shape, np.complex64)
        p, w = _ptr(out)
        self._check(self.lib.wdm_get_psi(self.handle, p, w))
        return out

    def get_rho(self, out=None):
        if out is None:
            out = np.empty(self.shape, np.float32)
        p, w = _ptr(out)
        self._check(self.lib.wdm_get_rho(self.handle, p, w))
        return out

    def get_phi(self, out=None):
        if out is None:
            out = np.empty(self.shape, np.float32)
        p, w = _ptr(out)
        self._check(self.lib.wdm_get_phi(self.handle, p, w))
        return out

    def set_static_potential(self, V):
        if V is None:
            self._check(self.lib.wdm_set_static_potential(self.handle, None, HOST))
            return
        if not _is_device(V):
            V = np.ascontiguousarray(V, dtype=np.float32)
        p, w = _ptr(V)
        self._check(self.lib.wdm_set_static_potential(self.handle, p, w))

    def set_tidal(self, schedule, per_item=False, t_first=None, t_step=None):
        """Rows of (Txx, Tyy, Tzz, Txy, Txz, Tyz).

        Without ``t_step`` row s is used by the s-th kick of every following
        step call.  With ``t_step`` (and ``t_first``, default 0) row s is the
        tensor at time t_first + s t_step and each kick takes the row nearest
        to its own time (step's t0 + s dt, kick's t)."""
        if schedule is None:
            self._check(self.lib.wdm_set_tidal(self.handle, None, 0, 0))
            return
        s = np.ascontiguousarray(np.asarray(schedule, dtype=np.float64).reshape(-1, 6))
        self._tidal_keep = s
        self._check(self.lib.wdm_set_tidal(self.handle, C.c_void_p(s.ctypes.data), len(s), int(per_item)))
        if t_step is not None:
            self._check(self.lib.wdm_set_tidal_clock(self.handle, float(t_first or 0.0), float(t_step)))

    def set_tidal_centering(self, mode):
        """Anchor of the tide: "box_centre" (default), "reference" (its value at the
        density maximum removed, as src/physics/tidal_fields.jl:114 leaves it) or
        "density_max" (value and gradient removed there)."""
        self._check(self.lib.wdm_set_tidal_centering(self.handle, _abi.TIDE_CENTERING[mode]))

    def set_particles(self, pos, mass):
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        mass = np.ascontiguousarray(np.broadcast_to(np.asarray(mass, np.float64), (len(pos),)))
        self._check(self.lib.wdm_set_particles(self.handle, C.c_void_p(pos.ctypes.data),
                                               C.c_void_p(mass.ctypes.data), len(pos)))

    # the path ----------------------------------------------------------------
    def step(self, nsteps, dt, t0=0.0, mode="strang", sync=True):
        fn = self.lib.wdm_step if sync else self.lib.wdm_step_async
        self._check(fn(self.handle, int(nsteps), float(dt), float(t0), _abi.STEP_MODES[mode]))

    def step_graph(self, nsteps, dt, mode="strang"):
        """Same as step(), replayed from a captured CUDA graph."""
        self._check(self.lib.wdm_step_graph(self.handle, int(nsteps), float(dt), _abi.STEP_MODES[mode]))

    def adjoint(self, nsteps, dt, rho_target, ckpt_every=20, tidal_dir=None, grad_out=None):
        """Loss, gradient and tidal-amplitude derivative of L = sum(|psi_N|^2 - rho_target)^2 dV.

        Returns (loss, grad, dL/da): grad = dL/dRe psi_0 + i dL/dIm psi_0 (complex64, the
        context's layout); dL/da is None without ``tidal_dir``.  psi is left at psi_0.
        """
        if not _is_device(rho_target):
            rho_target = np.ascontiguousarray(rho_target, dtype=np.float32)
        if grad_out is None:
            grad_out = np.empty(self.shape, np.complex64)
        pt, wt = _ptr(rho_target)
        pg, wg = _ptr(grad_out)
        loss = np.zeros(self.batch, np.float64)
        damp = np.zeros(self.batch, np.float64)
        d6 = None if tidal_dir is None else np.ascontiguousarray(np.asarray(tidal_dir, np.float64).reshape(6))
        self._check(self.lib.wdm_adjoint(self.handle, int(nsteps), float(dt), int(ckpt_every), pt, wt,
                                         None if d6 is None else C.c_void_p(d6.ctypes.data), pg, wg,
                                         C.c_void_p(loss.ctypes.data), C.c_void_p(damp.ctypes.data)))
        one = self.batch == 1
        return (loss[0] if one else loss), grad_out, (None if d6 is None else (damp[0] if one else damp))

    def kick(self, dt, t=0.0):
        self._check(self.lib.wdm_kick(self.handle, float(dt), float(t)))

    def drift(self, dt):
        self._check(self.lib.wdm_drift(self.handle, float(dt)))

    def poisson(self, rho, out=None):
        if not _is_device(rho):
            rho = np.ascontiguousarray(rho, dtype=np.float32)
            if out is None:
                out = np.empty(self.shape, np.float32)
        pr, wr = _ptr(rho)
        po, wo = _ptr(out)
        if wr != wo:
            raise ValueError("rho and phi must both be host or both be device arrays")
        self._check(self.lib.wdm_poisson(self.handle, pr, po, wr))
        return out

    def fft3d(self, data_dev, inverse=False):
        if not _is_device(data_dev):
            raise TypeError("fft3d works in place on a CUDA tensor")
        self._check(self.lib.wdm_fft3d(self.handle, C.c_void_p(data_dev.data_ptr()), 1 if inverse else -1))
        return data_dev

    # diagnostics ---------------------------------------------------------------
    FIELDS = ("mass", "rho_max", "argmax", "com_x", "com_y", "com_z",
              "VirialPotential", "TotalKineticE", "TotalQuantumE", "Virial")

    def reduce(self):
        out = np.zeros((self.batch, 10), np.float64)
        self._check(self.lib.wdm_reduce(self.handle, C.c_void_p(out.ctypes.data)))
        recs = [dict(zip(self.FIELDS, row.tolist())) for row in out]
        return recs[0] if self.batch == 1 else recs

    DIAG_FIELDS = FIELDS + ("MomentumX", "MomentumY", "MomentumZ", "phi_abs_max", "psi_abs_max",
                            "dt_phase", "dt_grav", "dt_self", "R") + tuple(f"radius_{k}0" for k in range(1, 10))

    def diagnostics(self):
        """The loop diagnostics of the reference's SPE3D_waveDM (mass, density maximum
        and its index, Lagrangian radii about it, R, virial and momentum sums) and
        the compute_timestep limits, on the device (wdm_diagnostics)."""
        n = len(self.DIAG_FIELDS)
        out = np.zeros((self.batch, n), np.float64)
        self._check(self.lib.wdm_diagnostics(self.handle, C.c_void_p(out.ctypes.data)))
        recs = [dict(zip(self.DIAG_FIELDS, row.tolist())) for row in out]
        return recs[0] if self.batch == 1 else recs

    def interpolate_phi(self, pos):
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        out = np.zeros(len(pos), np.float64)
        self._check(self.lib.wdm_interpolate_phi(self.handle, C.c_void_p(pos.ctypes.data), len(pos),
                                                 C.c_void_p(out.ctypes.data)))
        return out

    def is_finite(self):
        f = C.c_int32(0)
        self._check(self.lib.wdm_check_finite(self.handle, C.byref(f)))
        return bool(f.value)

    @property
    def stream(self):
        return self.lib.wdm_stream(self.handle)

    # profiling -------------------------------------------------------------------
    def set_profiling(self, on=True):
        self._check(self.lib.wdm_set_profiling(self.handle, int(bool(on))))

    def set_profile_mask(self, passes=None):
        """Bracket only the named passes with events while profiling (None: all)."""
        if passes is None:
            mask = (1 << 64) - 1
        else:
            names = [self.lib.wdm_pass_name(p).decode() for p in range(self.lib.wdm_num_passes())]
            mask = 0
            for name in passes:
                if name not in names:
                    raise ValueError(f"unknown pass {name!r}; passes: {names}")
                mask |= 1 << names.index(name)
        self._check(self.lib.wdm_set_profile_mask(self.handle, C.c_uint64(mask)))

    def profile(self):
        """{pass name: dict(launches, ms, bytes_per_launch)} since profiling was turned on."""
        n = self.lib.wdm_num_passes()
        la = np.zeros(n, np.int64)
        ms = np.zeros(n, np.float64)
        by = np.zeros(n, np.float64)
        self._check(self.lib.wdm_get_profile(self.handle, C.c_void_p(la.ctypes.data), C.c_void_p(ms.ctypes.data),
                                             C.c_void_p(by.ctypes.data)))
        return {self.lib.wdm_pass_name(p).decode(): dict(launches=int(la[p]), ms=float(ms[p]),
                                                          bytes_per_launch=float(by[p])) for p in range(n)}

    # tuned passes and the names of their two implementations
    SCHEDULE = (("psi_y", ("tma", "tile")), ("psi_z", ("tma", "tile")), ("h_y", ("tma", "tile")),
                ("h_z", ("tma", "tile")), ("x_kick", ("staged", "direct")), ("x_rho", ("staged", "direct")),
                ("x_rho_b", ("staged", "direct")))

    def line_schedule(self):
        """{pass: dict(impl, ms={impl name: best ms})} as chosen by the autotuner at creation."""
        n = len(self.SCHEDULE)
        impl = np.zeros(n, np.int32)
        ms = np.zeros(2 * n, np.float64)
        self._check(self.lib.wdm_get_line_schedule(self.handle, C.c_void_p(impl.ctypes.data),
                                                   C.c_void_p(ms.ctypes.data)))
        return {name: dict(impl=names[int(impl[k])], ms={names[0]: float(ms[2 * k]), names[1]: float(ms[2 * k + 1])})
                for k, (name, names) in enumerate(self.SCHEDULE)}

    @property
    def launch_count(self):
        return int(self.lib.wdm_launch_count(self.handle))


class Ensemble:
    """Independent halos of several grid sizes advanced together.

    ``members`` are SPEContexts (one per grid size, each with ``batch`` halos);
    every call to step() runs all their steps from one captured CUDA graph
    (wdm_group_step).  The contexts stay owned by the caller.
    """

    def __init__(self, members):
        self.lib = _abi.load()
        self.members = list(members)
        arr = (C.c_void_p * len(self.members))(*[m.handle.value for m in self.members])
        h = C.c_void_p()
        check(self.lib.wdm_group_create(arr, len(self.members), C.byref(h)))
        self._h = h

    def step(self, nsteps, dts, mode="strang", sync=True):
        """Advance every member; sync=False returns once the graph is enqueued on self.stream."""
        d = np.ascontiguousarray(np.broadcast_to(np.asarray(dts, np.float64), (len(self.members),)))
        fn = self.lib.wdm_group_step if sync else self.lib.wdm_group_step_async
        check(fn(self._h, int(nsteps), C.c_void_p(d.ctypes.data), _abi.STEP_MODES[mode]))

    @property
    def stream(self):
        """The group's cudaStream_t (as an integer handle)."""
        return int(self.lib.wdm_group_stream(self._h) or 0)

    @property
    def launch_count(self):
        return int(self.lib.wdm_group_launch_count(self._h))

    @property
    def schedule(self):
        """("graph" | "persistent" | "streams" | None, {schedule: timed ms of two steps})."""
        sched = C.c_int32(-1)
        ms = (C.c_double * 3)()
        check(self.lib.wdm_group_schedule(self._h, C.byref(sched), C.cast(ms, C.c_void_p)))
        names = {0: "graph", 1: "persistent", 2: "streams"}
        return names.get(sched.value), {"graph": ms[0], "persistent": ms[1], "streams": ms[2]}

    def close(self):
        if getattr(self, "_h", None):
            self.lib.wdm_group_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def weighted_quantiles_grouped(value, wsum, wmin, p):
    """The library's grouped weighted quantile (host code, no GPU): groups of equal
    value ascending, with total and smallest element weight per group."""
    lib = _abi.load()
    value = np.ascontiguousarray(value, np.float64)
    wsum = np.ascontiguousarray(wsum, np.float64)
    wmin = np.ascontiguousarray(wmin, np.float64)
    p = np.ascontiguousarray(p, np.float64)
    out = np.zeros(len(p), np.float64)
    check(lib.wdm_weighted_quantiles_grouped(value.ctypes.data, wsum.ctypes.data, wmin.ctypes.data, len(value),
                                             p.ctypes.data, len(p), out.ctypes.data))
    return out


def size_supported(n):
    return bool(_abi.load().wdm_size_supported(int(n)))
