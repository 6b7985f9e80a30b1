"""The reference-shaped host API (wavedm.jl_gb300/solver.py)."""
import numpy as np
import pytest

from oracle import spe


def test_setup_grid_matches_reference_unit_test(wdm):
    from wavedm_gb300 import solver

    x, y, z, d, vol = solver.setup_grid(2.0, 2.0, 2.0, 64, 64, 64)
    assert np.isclose(x.min(), -2.0) and np.isclose(x.max(), 2.0)
    assert np.allclose(d, 4.0 / 63) and np.isclose(vol, np.prod(d))
    ref = spe.setup_grid(2.0, 2.0, 2.0, 64, 64, 64)
    assert np.allclose(x, ref[0]) and np.allclose(d, ref[3])


def test_compute_timestep_follows_reference(wdm):
    from wavedm_gb300 import solver

    phi = np.array([-3.0, 1.0])
    psi = np.array([2.0, 0.5])
    t, dt, Nt = solver.compute_timestep(0.1, phi, 0.5, psi, 1.0, 10)
    assert Nt == 10 and len(t) == 10 and dt == float(np.float32(0.1))
    _, _, Nt2 = solver.compute_timestep(0.1, phi, 0.5, psi, 1.0, 10, autoset_timestep=True,
                                        autoset_timestep_ratio=0.5)
    lim = min(2 * 0.01 / np.pi, 2 * np.pi / 3.0, 2 * np.pi / 0.5 / 2.0)
    assert Nt2 == int(np.ceil(1.0 / (0.5 * lim)))


def test_gpu_path_refuses_closures_and_cpu(wdm):
    from wavedm_gb300 import solver

    with pytest.raises(ValueError):
        solver.SPE3D_waveDM(Nx=16, IC=lambda x, y, z: 1.0 + 0 * x, V=lambda x, y, z, p: 0.0)
    with pytest.raises(ValueError):
        solver.SPE3D_waveDM(Nx=16, IC=lambda x, y, z: 1.0 + 0 * x, gpu=False)
    with pytest.raises(NotImplementedError):
        solver.parallel_poisson(1.0, [15, 15, 15], np.zeros((16, 16, 16)), "Vacuum")


def test_descriptors_stand_for_dense_operators(wdm):
    from wavedm_gb300 import solver

    assert solver.setup_fft_operators(1, 1, 1, 8, 8, 8, 0.01).dt == 0.01
    b = solver.setup_absorption_boundary(1, 1, 1, None, None, None, 10.0, 0.02)
    assert (b.absorb_coeff, b.dt) == (10.0, 0.02)


@pytest.mark.gpu
def test_spe3d_wavedm_gpu_matches_oracle(wdm):
    """The keyword entry on the reference grid convention, literal reference loop, mask and 4 pi."""
    from wavedm_gb300 import solver

    N, X, Nt, Tmax, alpha = 32, 6.0, 11, 0.2, 5.0
    IC = lambda x, y, z: np.exp(-(x ** 2 + y ** 2 + z ** 2) / 4) * np.exp(0.2j * x)
    out = solver.SPE3D_waveDM(Nx=N, Xmax=X, Nt=Nt, Tmax=Tmax, IC=IC, absorb_coeff=alpha, StepsBetweenSnapshots=5)
    g = spe.Grid((N, N, N), (2 * X, 2 * X, 2 * X), "reference")
    Xc, Yc, Zc = g.coords()
    psi0 = np.broadcast_to(IC(Xc, Yc, Zc), (N, N, N)).astype(np.complex64).astype(np.complex128)
    dt = float(np.float32(Tmax / Nt))
    ref = spe.run(psi0, g, spe.Physics(poisson_coeff=4 * np.pi, absorb_alpha=alpha), dt, Nt - 1,
                  mode="reference_loop")
    assert spe.rel_l2(out["psi"], ref) < 2e-5
    assert len(out["Prop"]) == 2
    assert out["Prop"][-1]["mass"] == pytest.approx(spe.mass(ref, g), rel=1e-5)


@pytest.mark.gpu
def test_parallel_poisson_mirror(wdm):
    from wavedm_gb300 import solver

    rng = np.random.default_rng(0)
    rho = rng.uniform(0, 1, (16, 24, 32))
    phi = 4 * np.pi * solver.parallel_poisson([0.5, 0.25, 0.125], [31, 23, 15], rho)
    g = spe.Grid((32, 24, 16), (16.0, 6.0, 2.0))
    assert spe.rel_l2(phi, spe.poisson(rho, g, 4 * np.pi)) < 4e-6


def test_prop_csv_has_the_reference_columns(wdm, tmp_path):
    """save_property_dataframe writes the columns of src/io/save.jl:46-68 in order,
    lengths scaled by uL, one row per record."""
    from wavedm_gb300 import solver

    rec = {f: float(i + 1) for i, f in enumerate(wdm.SPEContext.DIAG_FIELDS)}
    rec["t"] = 0.5
    path = solver.save_property_dataframe([rec, dict(rec, t=1.0)], str(tmp_path), "T", "S", plot_virial=True, uL=2.0)
    assert path.endswith("T, S - Prop.csv")
    lines = open(path).read().splitlines()
    assert lines[0].split(",") == ["t", "R", "R1", "R2", "R3", "R4", "R5", "R6", "R7", "R8", "R9", "TotalMass",
                                   "PE_abs", "KE", "QE", "Virial", "MomentumX", "MomentumY", "MomentumZ"]
    row = [float(v) for v in lines[1].split(",")]
    assert row[0] == 0.5
    assert row[1] == 2.0 * rec["R"]
    assert row[2:11] == [2.0 * rec[f"radius_{k}0"] for k in range(1, 10)]
    assert row[11] == rec["mass"]
    assert row[12:] == [rec[k] for k in ("VirialPotential", "TotalKineticE", "TotalQuantumE", "Virial",
                                         "MomentumX", "MomentumY", "MomentumZ")]
    assert len(lines) == 3
    path = solver.save_property_dataframe([rec], str(tmp_path), "T", "S2", plot_virial=False)
    assert open(path).read().splitlines()[0].split(",")[-1] == "TotalMass"


@pytest.mark.gpu
def test_spe3d_wavedm_writes_prop_files(wdm, tmp_path):
    """With outputdir the entry writes Prop.csv from the device diagnostics and the
    final state with psi_last_t one step before the end."""
    from wavedm_gb300 import solver

    N, X, Nt, Tmax = 32, 6.0, 9, 0.16
    IC = lambda x, y, z: np.exp(-(x ** 2 + y ** 2 + z ** 2) / 4) * np.exp(0.2j * x)
    out = solver.SPE3D_waveDM(Nx=N, Xmax=X, Nt=Nt, Tmax=Tmax, IC=IC, StepsBetweenSnapshots=4,
                              outputdir=str(tmp_path), title="run", suffix="x")
    lines = open(out["Prop.csv"]).read().splitlines()
    assert len(lines) == 1 + 2
    last = dict(zip(lines[0].split(","), map(float, lines[-1].split(","))))
    assert last["TotalMass"] == pytest.approx(out["Prop"][-1]["mass"], rel=1e-15)
    assert 0 < last["R1"] < last["R5"] < last["R9"]
    z = np.load(out["Prop.npz"])
    assert np.array_equal(z["ψ"], out["psi"])
    # psi_last_t is the state after Nt - 2 steps of the same dt
    short = solver.SPE3D_waveDM(Nx=N, Xmax=X, Nt=Nt - 1, Tmax=Tmax * (Nt - 1) / Nt, IC=IC)
    assert short["dt"] == out["dt"]
    assert np.allclose(z["ψ_last_t"], short["psi"], rtol=0, atol=1e-6 * np.abs(short["psi"]).max())
    assert not np.allclose(z["ψ_last_t"], out["psi"], rtol=0, atol=1e-6 * np.abs(out["psi"]).max())
    assert z["Φ_all"].shape == out["psi"].shape and z["ψ2_averaged"].size == 0
