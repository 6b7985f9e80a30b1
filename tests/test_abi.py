"""The C-ABI library loads and exports every declared entry point (no GPU needed)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "wavedm.h")


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(wdm_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_path(wdm):
    syms = declared_symbols()
    for s in ("wdm_create", "wdm_step", "wdm_kick", "wdm_drift", "wdm_poisson", "wdm_reduce"):
        assert s in syms


def test_library_exports_every_declared_symbol(wdm):
    lib = C.CDLL(wdm.lib_path())
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_binding_covers_every_symbol(wdm):
    bound = {name for name, _, _ in wdm._abi.SIGNATURES}
    assert bound == set(declared_symbols())


def test_size_table(wdm):
    lib = wdm._abi.load()
    for n in (8, 12, 16, 24, 32, 48, 64, 96, 128, 192, 256, 384, 512):
        assert lib.wdm_size_supported(n) == 1
    for n in (0, 7, 10, 100, 1024, -8):
        assert lib.wdm_size_supported(n) == 0


def _desc(wdm, **kw):
    base = dict(nx=16, ny=16, nz=16, lx=1.0, ly=1.0, lz=1.0, convention=0, poisson_coeff=1.0, kerr=0.0,
                absorb_alpha=0.0, phase_mode=1, batch=1)
    base.update(kw)
    return wdm._abi.WdmDesc(**base)


@pytest.mark.parametrize("kw,status", [
    (dict(nx=100), 2), (dict(nz=7), 2), (dict(lx=0.0), 1), (dict(batch=0), 1), (dict(convention=5), 1),
    (dict(phase_mode=9), 1),
])
def test_create_rejects_bad_descriptors_before_touching_the_gpu(wdm, kw, status):
    lib = wdm._abi.load()
    h = C.c_void_p()
    d = _desc(wdm, **kw)
    st = lib.wdm_create(C.byref(d), C.byref(h))
    assert st == status
    assert not h.value
    assert lib.wdm_last_error(None)


def test_null_arguments_are_errors(wdm):
    lib = wdm._abi.load()
    assert lib.wdm_create(None, None) == 1
    assert lib.wdm_destroy(None) == 0
    assert lib.wdm_step(None, 1, 0.1, 0.0, 0) == 1
    assert lib.wdm_set_psi(None, None, 0) == 1
    assert lib.wdm_stream(None) is None


def test_python_api_fails_loudly_without_library(wdm, tmp_path):
    with pytest.raises(ImportError):
        wdm._abi.load(str(tmp_path / "missing.so"))


def test_grouped_weighted_quantile_matches_the_oracle(wdm):
    """The library's host-side quantile over groups of equal values (the form the
    device histogram of the radii gives) equals the oracle's element-wise
    StatsBase restatement on data with many ties and zero weights."""
    from oracle import spe

    rng = np.random.default_rng(5)
    for trial in range(20):
        vals = np.sort(rng.choice(np.arange(1, 200) * 0.37, size=rng.integers(1, 40), replace=False))
        v = rng.choice(vals, size=rng.integers(1, 400))
        w = rng.exponential(size=v.size) * (rng.random(v.size) > 0.1)
        if not np.any(w > 0):
            continue
        groups = np.unique(v)
        wsum = np.array([w[v == u].sum() for u in groups])
        wmin = np.array([w[(v == u) & (w > 0)].min() if np.any((v == u) & (w > 0)) else 0.0 for u in groups])
        p = np.concatenate([[0.0, 1.0], rng.random(30)])
        got = wdm.weighted_quantiles_grouped(groups, wsum, wmin, p)
        ref = spe.weighted_quantile(v, w, p)
        assert np.allclose(got, ref, rtol=1e-12, atol=1e-12), trial


def test_grouped_weighted_quantile_rejects_unsorted_groups(wdm):
    with pytest.raises(wdm._abi.WdmError):
        wdm.weighted_quantiles_grouped([1.0, 1.0], [1.0, 1.0], [1.0, 1.0], [0.5])
