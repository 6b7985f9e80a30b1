"""CUDA-graph replay and multi-size ensembles (needs a GPU).

A captured graph replays exactly the launches of wdm_step, so its results must
match wdm_step bit for bit; an ensemble of contexts of different grid sizes in
one graph must match each context stepped on its own, and the FP64 oracle.
"""
import glob
import os

import numpy as np
import pytest

from oracle import spe

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))


def _halo(n, L, rc, seed):
    rng = np.random.default_rng(seed)
    g = spe.Grid((n, n, n), (L, L, L))
    X, Y, Z = g.coords()
    r2 = X ** 2 + Y ** 2 + Z ** 2
    psi = np.sqrt(1.0 / (1.0 + 0.091 * r2 / rc ** 2) ** 8) * np.exp(0.2j * rng.standard_normal((n, n, n)))
    return psi.astype(np.complex64)


def test_step_graph_matches_step(wdm):
    d = dict(np.load([f for f in GOLDEN if "strang_24x16x12_all" in f][0]))
    n = tuple(int(v) for v in d["n"])
    L = tuple(float(v) for v in d["L"])
    out = []
    for use_graph in (False, True):
        with wdm.SPEContext(n, L, poisson_coeff=float(d["c"]), kerr=float(d["kerr"])) as ctx:
            ctx.set_psi(d["psi0"])
            ctx.set_static_potential(d["V"])
            ctx.set_tidal(d["tidal"])
            ctx.set_particles(d["pos"], d["mass"])
            if use_graph:
                ctx.step_graph(int(d["steps"]), float(d["dt"]))
            else:
                ctx.step(int(d["steps"]), float(d["dt"]))
            out.append(ctx.get_psi())
    assert np.array_equal(out[0], out[1])
    assert spe.rel_l2(out[1], d["psi"]) < 2e-5


def test_graph_replay_continues_the_run(wdm):
    n, L, dt = (32, 32, 32), (10.0, 10.0, 10.0), 0.01
    psi0 = _halo(32, 10.0, 1.2, 3)
    with wdm.SPEContext(n, L) as a, wdm.SPEContext(n, L) as b:
        a.set_psi(psi0)
        b.set_psi(psi0)
        for _ in range(3):
            a.step_graph(4, dt)  # captured once, replayed twice
            b.step(4, dt)
        assert np.array_equal(a.get_psi(), b.get_psi())


def test_graph_replay_follows_a_particle_change(wdm):
    """New particles between two graph calls: the graph is captured again and
    the kept deposit is remade, as in the eager run (particles on a lattice
    three cells apart, so that the FP32 atomic deposit has one order)."""
    n, L, dt = (32, 32, 32), (10.0, 10.0, 10.0), 0.01
    psi0 = _halo(32, 10.0, 1.2, 5)
    d = 10.0 / 32
    lat = np.stack(np.meshgrid(*[np.arange(4)] * 3, indexing="ij"), -1).reshape(-1, 3)
    pos_a = -5.0 + (lat * 3.0 + 2.3) * d
    pos_b = -5.0 + (lat * 3.0 + 14.6) * d
    out = []
    for use_graph in (True, False):
        with wdm.SPEContext(n, L) as ctx:
            ctx.set_psi(psi0)
            for pos in (pos_a, pos_b):
                ctx.set_particles(pos, 0.02)
                if use_graph:
                    ctx.step_graph(3, dt)
                else:
                    ctx.step(3, dt)
            out.append(ctx.get_psi())
    assert np.array_equal(out[0], out[1])


def test_ensemble_of_three_sizes(wdm):
    specs = [(16, 3, 8.0), (24, 2, 8.0), (32, 1, 8.0)]
    members, inputs, tides, dts = [], [], [], []
    for k, (n, batch, L) in enumerate(specs):
        ctx = wdm.SPEContext((n, n, n), (L, L, L), poisson_coeff=1.0, batch=batch)
        psis = np.stack([_halo(n, L, 1.0 + 0.3 * b, 10 * k + b) for b in range(batch)])
        T = np.array([[0.02 * (b + 1), -0.01 * (b + 1), -0.01 * (b + 1), 0, 0, 0] for b in range(batch)])
        ctx.set_psi(psis)
        ctx.set_tidal(T, per_item=True)
        members.append(ctx)
        inputs.append(psis)
        tides.append(T)
        dts.append((L / n) ** 2 / 6)
    steps = 5
    with wdm.Ensemble(members) as ens:
        ens.step(steps, dts)
        assert ens.launch_count > 0
    for k, (n, batch, L) in enumerate(specs):
        got = members[k].get_psi().reshape(batch, n, n, n)
        with wdm.SPEContext((n, n, n), (L, L, L), poisson_coeff=1.0, batch=batch) as solo:
            solo.set_psi(inputs[k])
            solo.set_tidal(tides[k], per_item=True)
            solo.step(steps, dts[k])
            assert np.array_equal(got, solo.get_psi().reshape(batch, n, n, n))
        g = spe.Grid((n, n, n), (L, L, L))
        for b in range(batch):
            phys = spe.Physics(poisson_coeff=1.0, tidal=lambda t, T=tides[k][b]: tuple(T))
            ref = spe.run(inputs[k][b].astype(np.complex128), g, phys, dts[k], steps)
            assert spe.rel_l2(got[b], ref) < 2e-5
        members[k].close()


# Baryon particles of one member, 1.5 length units (9 cells) apart along x, so
# that no two CIC stencils share a cell and the FP32 atomic deposit is the
# same in every run.
PARTS_POS = np.array([[-3.0 + 1.5 * p, 0.1 * p, 0.05] for p in range(4)])
PARTS_MASS = np.array([0.5, 0.3, 0.4, 0.2])


def _members(wdm, specs, centering=None, particles_for=None):
    out = []
    for k, (n, batch, L) in enumerate(specs):
        nx, ny, nz = n if isinstance(n, tuple) else (n, n, n)
        ctx = wdm.SPEContext((nx, ny, nz), (L, L * ny / nx, L * nz / nx), poisson_coeff=1.0, batch=batch)
        rng = np.random.default_rng(100 + k)
        g = spe.Grid((nx, ny, nz), ctx.L)
        X, Y, Z = g.coords()
        psis = []
        for b in range(batch):
            amp = np.exp(-((X - 0.3 * b - 0.2) ** 2 + (Y + 0.1 * b) ** 2 + (Z - 0.15) ** 2) / (1.0 + 0.2 * b))
            psis.append((amp * np.exp(0.2j * rng.standard_normal((nz, ny, nx)))).astype(np.complex64))
        psis = np.stack(psis)
        T = np.array([[0.05 * (b + 1), -0.02, -0.03 * (b + 1), 0.01, 0.0, 0.005] for b in range(batch)])
        ctx.set_psi(psis)
        ctx.set_tidal(T, per_item=True)
        if centering and k == 0:
            ctx.set_tidal_centering(centering)
        if particles_for == k:
            ctx.set_particles(PARTS_POS, PARTS_MASS)
        out.append((ctx, psis, T, (L / nx) ** 2 / 6))
    return out


ENS_SPECS = [(16, 3, 8.0), (24, 2, 8.0), ((48, 32, 16), 1, 8.0), (64, 2, 10.0)]


@pytest.mark.parametrize("mode", ["strang", "reference_loop", "lie"])
def test_persistent_ensemble_equals_its_pass_launches(wdm, monkeypatch, mode):
    """One cooperative launch per call (all passes, members and steps) gives the
    bits of the same passes launched one by one with the register-tile line
    passes and the direct x passes, including a tide anchored at the density
    maximum (its words zeroed and refilled inside the launch) and a member with
    baryon particles (their deposit made once, before the launch)."""
    monkeypatch.setenv("WDM_GROUP_SCHEDULE", "persistent")
    monkeypatch.setenv("WDM_SCHEDULE", "tile,tile,tile,tile,direct,direct,direct")
    steps = 4
    mem = _members(wdm, ENS_SPECS, centering="density_max", particles_for=2)
    with wdm.Ensemble([m[0] for m in mem]) as ens:
        l0 = ens.launch_count
        ens.step(steps, [m[3] for m in mem], mode=mode)
        ens.step(steps, [m[3] for m in mem], mode=mode)  # a replay continues the run
        assert ens.schedule[0] == "persistent"
        # per call: the persistent kernel, and the small frame kernel of the one
        # member whose tide is anchored at its density maximum
        assert ens.launch_count - l0 == 2 * 2
    for k, (ctx, psis, T, dt) in enumerate(mem):
        got = ctx.get_psi()
        with wdm.SPEContext(ctx.n, ctx.L, poisson_coeff=1.0, batch=ctx.batch) as solo:
            solo.set_psi(psis)
            solo.set_tidal(T, per_item=True)
            if k == 0:
                solo.set_tidal_centering("density_max")
            if k == 2:
                solo.set_particles(PARTS_POS, PARTS_MASS)
            solo.step(steps, dt, mode=mode)
            solo.step(steps, dt, mode=mode)
            assert np.array_equal(got, solo.get_psi()), k
        ctx.close()


def test_ensemble_schedule_choice_keeps_the_state(wdm, monkeypatch):
    """The first call times both schedules on the members' own state and puts
    it back: the run then equals a run under the chosen schedule forced."""
    steps = 3
    mem = _members(wdm, ENS_SPECS[:3])
    with wdm.Ensemble([m[0] for m in mem]) as ens:
        ens.step(steps, [m[3] for m in mem])
        sched, ms = ens.schedule
    assert sched in ("graph", "persistent", "streams")
    assert ms["graph"] > 0 and ms["persistent"] > 0 and ms["streams"] > 0
    auto = [m[0].get_psi() for m in mem]
    for m in mem:
        m[0].close()
    monkeypatch.setenv("WDM_GROUP_SCHEDULE", sched)
    mem = _members(wdm, ENS_SPECS[:3])
    with wdm.Ensemble([m[0] for m in mem]) as ens:
        ens.step(steps, [m[3] for m in mem])
    for a, m in zip(auto, mem):
        assert np.array_equal(a, m[0].get_psi())
        m[0].close()


def test_ensemble_on_forked_streams_equals_one_stream(wdm, monkeypatch):
    """Each member on a stream of its own inside the group's graph (the sizes
    run concurrently) gives the bits of the members stepped one after another."""
    steps = 3
    out = {}
    for sched in ("graph", "streams"):
        monkeypatch.setenv("WDM_GROUP_SCHEDULE", sched)
        mem = _members(wdm, ENS_SPECS)
        with wdm.Ensemble([m[0] for m in mem]) as ens:
            ens.step(steps, [m[3] for m in mem])
            ens.step(steps, [m[3] for m in mem])
            assert ens.schedule[0] == sched
        out[sched] = [m[0].get_psi() for m in mem]
        for m in mem:
            m[0].close()
    for a, b in zip(out["graph"], out["streams"]):
        assert np.array_equal(a, b)
