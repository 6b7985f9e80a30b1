"""Per-pass profiling (wdm_set_profiling / wdm_set_profile_mask / wdm_get_profile; needs a GPU).

Profiling brackets passes with CUDA events on the context's stream; it must not
change the results, and the mask must restrict the events to the named passes
without changing which kernels run.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STEP_PASSES = ("kick_xfft_fwd", "psi_y_fwd", "psi_z_drift", "psi_y_inv", "psi_x_inv_rho", "rho_y_fwd",
               "rho_z_poisson", "phi_y_inv")


def _psi(n, seed=5):
    rng = np.random.default_rng(seed)
    return (1.0 + 0.1 * rng.standard_normal((n, n, n)) + 0.1j * rng.standard_normal((n, n, n))).astype(np.complex64)


def _run(wdm, psi0, steps, dt, profiling=False, mask=None):
    n = psi0.shape[0]
    with wdm.SPEContext((n, n, n), (10.0, 10.0, 10.0)) as ctx:
        ctx.set_psi(psi0)
        ctx.get_phi()
        if mask is not None:
            ctx.set_profile_mask(mask)
        ctx.set_profiling(profiling)
        l0 = ctx.launch_count
        ctx.step(steps, dt)
        launches = ctx.launch_count - l0
        prof = ctx.profile() if profiling else None
        return ctx.get_psi(), launches, prof


def test_profiling_counts_every_pass_and_leaves_results_unchanged(wdm):
    psi0 = _psi(48)
    ref, la_ref, _ = _run(wdm, psi0, 5, 0.01)
    out, la, prof = _run(wdm, psi0, 5, 0.01, profiling=True)
    assert np.array_equal(out, ref)
    assert la == la_ref
    for name in STEP_PASSES:
        assert prof[name]["launches"] == 5, name
        assert prof[name]["ms"] > 0.0 and prof[name]["bytes_per_launch"] > 0.0, name


def test_profile_mask_restricts_the_events(wdm):
    psi0 = _psi(48)
    ref, la_ref, _ = _run(wdm, psi0, 4, 0.01)
    out, la, prof = _run(wdm, psi0, 4, 0.01, profiling=True, mask=["psi_z_drift"])
    assert np.array_equal(out, ref)
    assert la == la_ref  # the mask changes the events, not the kernels
    assert prof["psi_z_drift"]["launches"] == 4 and prof["psi_z_drift"]["ms"] > 0.0
    for name, p in prof.items():
        if name != "psi_z_drift":
            assert p["launches"] == 0 and p["ms"] == 0.0, name


def test_profile_mask_rejects_unknown_pass(wdm):
    with wdm.SPEContext((16, 16, 16), (10.0, 10.0, 10.0)) as ctx:
        with pytest.raises(ValueError):
            ctx.set_profile_mask(["no_such_pass"])
