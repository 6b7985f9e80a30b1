"""wdm_poisson_noalloc against wdm_poisson, through the C ABI (needs a GPU).

wdm_poisson_noalloc serves callers that cannot allocate device memory (a host
runtime that owns the GPU memory pool, or a loop that must not pay for the
device synchronisation of cudaMalloc/cudaFree): its scratch is a static device
array, so it must agree with the context-based wdm_poisson, which allocates its
own scratch.  Calls in a row check that nothing left in the shared array by
one call leaks into the next: the same input solved again after a call on
another grid shape must give the same bits.  This file is collected last so
that a run stopping at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import spe

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _noalloc(lib, rho, phi, n, L, coeff):
    nx, ny, nz = n
    return lib.wdm_poisson_noalloc(C.c_void_p(rho.data_ptr()), C.c_void_p(phi.data_ptr()), nx, ny, nz,
                                   L[0], L[1], L[2], coeff, None)


def test_noalloc_poisson_matches_wdm_poisson_twice(wdm, torch_cuda):
    torch = torch_cuda
    lib = wdm._abi.load()
    cases = [((32, 48, 24), (3.0, 2.0, 4.0), 4 * np.pi, 11), ((64, 64, 64), (20.0, 20.0, 20.0), 1.0, 12)]
    results = []
    for n, L, coeff, seed in cases:
        nx, ny, nz = n
        rng = np.random.default_rng(seed)
        rho_h = rng.uniform(0.0, 2.0, size=(nz, ny, nx)).astype(np.float32)
        rho = torch.from_numpy(rho_h).cuda()
        phi_na = torch.full_like(rho, float("nan"))
        assert _noalloc(lib, rho, phi_na, n, L, coeff) == 0, lib.wdm_last_error(None)
        with wdm.SPEContext(n, L, poisson_coeff=coeff) as ctx:
            phi_ref = torch.empty_like(rho)
            ctx.poisson(rho, phi_ref)
        got, ref = phi_na.cpu().numpy(), phi_ref.cpu().numpy()
        assert np.all(np.isfinite(got))
        # same kernels on the same data: the test_gpu_parity Poisson tolerance
        assert spe.rel_l2(got, ref) < 2e-6
        # and the FP64 oracle's solve of the same density (white noise: the
        # tolerance of test_poisson_matches_oracle)
        oracle = spe.poisson(rho_h.astype(np.float64), spe.Grid(n, L), coeff)
        assert spe.rel_l2(got, oracle) < 4e-6
        results.append((n, L, coeff, rho, got))
    # Solve the first case again, now that the second (larger) case has filled
    # the shared array: bit for bit the first answer.
    n, L, coeff, rho, first = results[0]
    again = torch.full_like(rho, float("nan"))
    assert _noalloc(lib, rho, again, n, L, coeff) == 0, lib.wdm_last_error(None)
    assert np.array_equal(again.cpu().numpy(), first)


def test_noalloc_rejects_grids_beyond_the_static_scratch(wdm, torch_cuda):
    torch = torch_cuda
    lib = wdm._abi.load()
    rho = torch.zeros(8, device="cuda")
    st = lib.wdm_poisson_noalloc(C.c_void_p(rho.data_ptr()), C.c_void_p(rho.data_ptr()), 256, 256, 256,
                                 1.0, 1.0, 1.0, 1.0, None)
    assert st == 1
    assert b"static scratch" in lib.wdm_last_error(None)
    st = lib.wdm_poisson_noalloc(C.c_void_p(rho.data_ptr()), C.c_void_p(rho.data_ptr()), 100, 8, 8,
                                 1.0, 1.0, 1.0, 1.0, None)
    assert st == 2
