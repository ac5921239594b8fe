"""The allocation-free spectral solve (erp_spectral_solve_noalloc).

It exists for callers that cannot call cudaMalloc: hosts whose device memory is
owned by another allocator's pool, and loops that must not stall on cudaFree.
Its intermediates live in one file-scope device array, so it is checked here
against the allocating entry point (erp_spectral_create + erp_spectral_solve) on
the same inputs, twice in a row, through the C ABI.  The buffers it is given are
allocated by the test; the entry point itself allocates nothing.

This file is collected last on purpose, so that a run stopping at the first
failure has already run every other test; it also passes on its own in a fresh
process (the first call does the per-device set-up).
"""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-5   # the relative-L2 bar of the FP32 parity tests


@pytest.fixture(scope="module")
def R(built):
    import reda_erplacer_gb300 as R
    return R


# group and warp transform forms (512, 64-256), and the generic radix-2 forms
# (sides 16, 32 and 4096) with the largest twiddle-table offsets
@pytest.mark.parametrize("m,n,bw,bh", [(512, 512, 1.3, 1.1), (64, 256, 0.7, 2.1), (4096, 64, 0.9, 1.4),
                                       (32, 4096, 1.1, 0.8), (16, 16, 1.0, 1.0)])
def test_noalloc_matches_allocating_solve(R, m, n, bw, bh):
    import torch
    lib = R.lib.load()
    rng = np.random.default_rng(17)
    rho = torch.tensor((0.7 + 0.3 * rng.random((m, n))).astype(np.float32), device="cuda")
    want = [torch.empty_like(rho) for _ in range(3)]
    sol = R.SpectralSolver(m, n, bw, bh)
    sol.solve(rho.data_ptr(), *[t.data_ptr() for t in want])
    torch.cuda.synchronize()
    sol.close()
    first = None
    for call in range(2):
        got = [torch.full_like(rho, float("nan")) for _ in range(3)]
        st = lib.erp_spectral_solve_noalloc(m, n, bw, bh, C.c_void_p(rho.data_ptr()),
                                            *[C.c_void_p(t.data_ptr()) for t in got], None)
        R.lib.check(st)
        torch.cuda.synchronize()
        for g, w in zip(got, want):
            assert rel_l2(g.cpu().numpy(), w.cpu().numpy()) <= TOL, call
        if first is None:
            first = [g.clone() for g in got]
        else:   # the shared scratch keeps no state between calls
            for g, f in zip(got, first):
                assert torch.equal(g, f)


def test_noalloc_rejects_grids_above_its_limit(R):
    import torch
    lib = R.lib.load()
    t = torch.zeros(1024 * 1024, device="cuda")
    p = C.c_void_p(t.data_ptr())
    st = lib.erp_spectral_solve_noalloc(1024, 1024, 1.0, 1.0, p, p, p, None, None)
    assert st == R.lib.EINVAL
    assert b"512 x 512" in lib.erp_last_error(None)
