"""Device loop diagnostics (wdm_diagnostics) against the FP64 oracle's restatement
of the reference loop's host diagnostics (oracle.spe.loop_diagnostics).

Both sides see the same complex64 psi and float32 Phi read back from the
library, so these tests check the reductions, the histogram and the quantile,
not the step: the momentum sums to 2e-6 relative (FP32 per-cell terms summed
in FP64), the R and radii sums to 1e-9 relative (FP64 throughout), maxima and
indices exactly.
"""
import numpy as np
import pytest

from oracle import spe

pytestmark = pytest.mark.gpu


def _state(wdm, n, L, batch=1, kerr=0.0, seed=2):
    g = spe.Grid(n, L)
    X, Y, Z = g.coords()
    rng = np.random.default_rng(seed)
    items = []
    for b in range(batch):
        c = rng.uniform(-0.5, 0.5, 3)
        r2 = (X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2
        psi = (np.exp(-r2 / (1.5 + b)) * np.exp(1j * (2 * np.pi / L[0] * X + 0.2 * rng.standard_normal(r2.shape)))
               + 0.01)
        items.append(psi.astype(np.complex64))
    psi0 = np.stack(items) if batch > 1 else items[0]
    ctx = wdm.SPEContext(n, L, poisson_coeff=1.0, kerr=kerr, batch=batch)
    ctx.set_psi(psi0)
    ctx.step(3, 0.01)
    return g, ctx


@pytest.mark.parametrize("n,batch", [((48, 32, 24), 1), ((32, 32, 32), 2)], ids=["48x32x24", "32cube-b2"])
def test_diagnostics_match_oracle(wdm, n, batch):
    dx = 0.15
    L = tuple(dx * m for m in n)
    g, ctx = _state(wdm, n, L, batch=batch, kerr=0.3)
    with ctx:
        got = ctx.diagnostics()
        psi = ctx.get_psi()
        phi = ctx.get_phi()
    got = got if batch > 1 else [got]
    psi = psi.reshape((batch,) + psi.shape[-3:])
    phi = phi.reshape((batch,) + phi.shape[-3:])
    for b in range(batch):
        ref = spe.loop_diagnostics(psi[b].astype(np.complex128), phi[b].astype(np.float64), g, kappa=0.3)
        d = got[b]
        assert int(d["argmax"]) == ref["argmax"]
        assert d["rho_max"] == pytest.approx(ref["rho_max"], rel=1e-12)
        assert d["psi_abs_max"] == pytest.approx(ref["psi_abs_max"], rel=1e-12)
        assert d["phi_abs_max"] == pytest.approx(ref["phi_abs_max"], rel=1e-12)
        for k in ("MomentumX", "MomentumY", "MomentumZ"):
            assert d[k] == pytest.approx(ref[k], rel=2e-6, abs=2e-6 * abs(ref["MomentumX"]))
        assert abs(d["MomentumX"]) > 10 * max(abs(d["MomentumY"]), abs(d["MomentumZ"]))
        for k in ("dt_phase", "dt_grav", "dt_self"):
            assert d[k] == pytest.approx(ref[k], rel=1e-12)
        assert d["R"] == pytest.approx(ref["R"], rel=1e-9)
        radii = np.array([d[f"radius_{k}0"] for k in range(1, 10)])
        assert np.allclose(radii, ref["radii"], rtol=1e-9, atol=0)
        assert np.all(np.diff(radii) >= 0)


def test_diagnostics_radii_need_cubic_cells(wdm):
    n, L = (32, 32, 32), (4.0, 4.8, 4.0)
    g, ctx = _state(wdm, n, L)
    with ctx:
        d = ctx.diagnostics()
        red = ctx.reduce()
    assert all(np.isnan(d[f"radius_{k}0"]) for k in range(1, 10))
    assert np.isfinite(d["R"])
    for k, v in red.items():
        assert d[k] == pytest.approx(v, rel=1e-12)


def test_diagnostics_without_kerr_or_gravity_report_infinite_limits(wdm):
    n = (32, 32, 32)
    g = spe.Grid(n, (4.0, 4.0, 4.0))
    X, Y, Z = g.coords()
    psi = (np.exp(-(X ** 2 + Y ** 2 + Z ** 2)) + 0j).astype(np.complex64)
    with wdm.SPEContext(n, (4.0, 4.0, 4.0), poisson_coeff=0.0) as ctx:
        ctx.set_psi(psi)
        d = ctx.diagnostics()
    assert d["dt_grav"] == np.inf and d["dt_self"] == np.inf
    assert d["dt_phase"] == pytest.approx(2 * g.spacing[0] ** 2 / np.pi)
