"""The allocation-free residual entry point against the allocating one.

dg_residual_csr_noalloc serves callers that cannot allocate device memory
when they need the residual (a caller-owned memory pool, a stream under
graph capture, a loop that must not synchronise on cudaMalloc).  It must give
the same r = b - A x and ||r||^2 as dg_residual_csr, on consecutive calls
that reuse its fixed scratch array.  The file is named so that pytest
collects it last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(L, name, n, ptrs, stream=0):
    return getattr(L, name)(n, *ptrs, stream)


def test_noalloc_residual_matches_allocating_entry_twice():
    torch = pytest.importorskip("torch")
    import scipy.sparse as sp
    import doug_gb300 as D
    from doug_gb300 import problems as P

    L = D.load_library()
    results = []
    for seed in (11, 12):  # two calls in a row, different sizes and data
        N = 20 + 4 * (seed - 11)
        n, r, c, v, b = P.diffusion3d_fv(N, seed=seed)
        A = sp.csr_matrix((v, (r - 1, c - 1)), shape=(n, n))
        rp = torch.tensor(A.indptr, dtype=torch.int64, device="cuda")
        ci = torch.tensor(A.indices, dtype=torch.int32, device="cuda")
        vv = torch.tensor(A.data, dtype=torch.float64, device="cuda")
        x = torch.tensor(np.random.default_rng(seed).uniform(-1, 1, n), device="cuda")
        bt = torch.tensor(b, device="cuda")
        r_a = torch.empty_like(x)
        n_a = torch.zeros(1, dtype=torch.float64, device="cuda")
        r_b = torch.empty_like(x)
        n_b = torch.zeros(1, dtype=torch.float64, device="cuda")
        common = [rp.data_ptr(), ci.data_ptr(), vv.data_ptr(), x.data_ptr(), bt.data_ptr()]
        assert _call(L, "dg_residual_csr", n, common + [r_a.data_ptr(), n_a.data_ptr()]) == D.DG_OK
        assert _call(L, "dg_residual_csr_noalloc", n, common + [r_b.data_ptr(), n_b.data_ptr()]) == D.DG_OK
        torch.cuda.synchronize()
        ra, rb = r_a.cpu().numpy(), r_b.cpu().numpy()
        scale = np.abs(ra).max()
        assert np.allclose(rb, ra, rtol=0, atol=1e-12 * scale)
        assert abs(n_b.item() - n_a.item()) <= 1e-12 * n_a.item()
        ref = b - A @ x.cpu().numpy()
        assert abs(n_b.item() - ref @ ref) <= 1e-12 * (ref @ ref)
        results.append(n_b.item())
    assert results[0] != results[1]


def test_noalloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    import doug_gb300 as D

    L = D.load_library()
    t = torch.zeros(8, dtype=torch.float64, device="cuda")
    ti = torch.zeros(8, dtype=torch.int64, device="cuda")
    # the size check comes before any device access
    rc = _call(L, "dg_residual_csr_noalloc", 67_108_865,
               [ti.data_ptr(), ti.data_ptr(), t.data_ptr(), t.data_ptr(), t.data_ptr(),
                t.data_ptr(), t.data_ptr()])
    assert rc == D.DG_BAD_INPUT
