"""Failure paths driven from the host (needs a GPU; no GPU fault is caused).

The library reads WDM_FAULT at every allocation and finite check, so setting
it in this process injects the failure:
* WDM_FAULT=alloc:N  the N-th device allocation fails: wdm_create must return
  WDM_ERR_ALLOC and give back everything it had allocated before that point;
* WDM_FAULT=nonfinite  the finite check of a step reports a NaN density:
  wdm_step returns WDM_ERR_NONFINITE and the context stays usable.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _free_bytes(torch):
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


@pytest.mark.parametrize("nth", [1, 2, 5, 9])
def test_failed_allocation_in_create_frees_what_it_had(wdm, torch_cuda, monkeypatch, nth):
    n, L = (256, 256, 128), (10.0, 10.0, 5.0)  # psi 64 MiB, H 33 MiB: a leak would show
    with wdm.SPEContext(n, L) as ctx:  # tunes the schedule once, so the retry below allocates the same
        pass
    before = _free_bytes(torch_cuda)
    monkeypatch.setenv("WDM_FAULT", f"alloc:{nth}")
    with pytest.raises(wdm._abi.WdmError, match="WDM_ERR_ALLOC"):
        wdm.SPEContext(n, L)
    monkeypatch.delenv("WDM_FAULT")
    after = _free_bytes(torch_cuda)
    assert abs(before - after) <= 4 << 20, f"{(before - after) / 2**20:.1f} MiB not given back"
    with wdm.SPEContext(n, L) as ctx:  # the library still works
        ctx.set_psi(np.ones((n[2], n[1], n[0]), np.complex64))
        ctx.step(1, 1e-3)


def test_injected_nonfinite_density_is_reported(wdm, torch_cuda, monkeypatch):
    n, L = (32, 32, 32), (8.0, 8.0, 8.0)
    with wdm.SPEContext(n, L) as ctx:
        psi0 = np.ones((32, 32, 32), np.complex64)
        ctx.set_psi(psi0)
        monkeypatch.setenv("WDM_FAULT", "nonfinite")
        with pytest.raises(wdm._abi.WdmError, match="WDM_ERR_NONFINITE"):
            ctx.step(1, 1e-3)
        monkeypatch.delenv("WDM_FAULT")
        ctx.set_psi(psi0)
        ctx.step(2, 1e-3)
        assert ctx.is_finite()
        assert np.allclose(np.abs(ctx.get_psi()), 1.0, atol=1e-5)
