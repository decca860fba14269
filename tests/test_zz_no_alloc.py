"""fkg_eigh_logz_noalloc: the eigen-solve + logZ for callers that cannot
allocate device memory (their device memory is owned by someone else's pool,
or a synchronising cudaMalloc is not allowed where they call from). Its
scratch is a fixed-size device array inside the library, so the test checks
that two calls in a row, on different inputs, both agree with the allocating
entry point fkg_eigh_logz and with the CPU oracle within the FP64 tolerance of
the other parity tests (|dlambda| <= 1e-10 ||H||_2, logZ relative 1e-10),
that sizes beyond the stated maximum are rejected with an error, and that a
CSR column outside [0, n) is skipped and reported instead of being written."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_matches_allocating_entry_point(cuda_ok, fkg_lib, oracle):
    import torch
    import fk_mc_gb300
    from fk_mc_gb300._lib import SIGNATURES
    from fk_mc_gb300.lattice import hopping_csr
    assert "fkg_eigh_logz_noalloc" in SIGNATURES
    L, B = 10, 5  # n = 100 <= FKG_NOALLOC_MAX_N, batch 5 <= FKG_NOALLOC_MAX_BATCH
    n, rp, col, val = hopping_csr("cubic2d", L)
    ref = fk_mc_gb300.Solver(max_n=n, max_batch=B)
    ref.set_hopping(0, rp, col, val)
    dev = torch.device("cuda", 0)
    d_rp = torch.tensor(rp, dtype=torch.int32, device=dev)
    d_col = torch.tensor(col, dtype=torch.int32, device=dev)
    d_val = torch.tensor(val, dtype=torch.float64, device=dev)
    err = ctypes.create_string_buffer(256)
    rng = np.random.default_rng(11)
    for call in range(2):
        U = 1.0 + call
        f = rng.integers(0, 2, (B, n))
        diag = (-U / 2 + U * f).ravel()
        beta = rng.uniform(1, 10, B)
        d_diag = torch.tensor(diag, dtype=torch.float64, device=dev)
        d_beta = torch.tensor(beta, dtype=torch.float64, device=dev)
        d_w = torch.full((B * n,), float("nan"), dtype=torch.float64, device=dev)
        d_z = torch.full((B,), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        rc = fkg_lib.fkg_eigh_logz_noalloc(B, n, _dev(d_rp), _dev(d_col), _dev(d_val), _dev(d_diag), _dev(d_beta),
                                           _dev(d_w), _dev(d_z), None, err, 256)
        assert rc == 0, err.value
        w, z = d_w.cpu().numpy(), d_z.cpu().numpy()
        out = ref.eigh_logz(np.zeros(B, np.int32), diag, beta)
        hn = np.abs(out["evals"]).max()
        assert np.abs(w - out["evals"]).max() <= 1e-10 * hn
        assert np.all(np.abs(z - out["logz"]) <= 1e-10 * np.abs(out["logz"]))
        for c in range(B):  # and the oracle's calc_ed of the same configuration
            o = oracle.calc_ed("cubic2d", L, f[c], beta[c], U, U / 2)
            assert np.abs(w[c * n:(c + 1) * n] - o["spectrum"]).max() <= 1e-10 * hn
            assert abs(z[c] - o["logZ"]) <= 1e-10 * abs(o["logZ"])
    ref.close()


def test_noalloc_rejects_out_of_range_column(cuda_ok, fkg_lib):
    """The matrix build checks every CSR column against [0, n): one entry set to -1 is skipped (nothing is
    written outside the chain's part of the scratch array) and the call fails with FKG_ERR_ARG; the next call
    with a valid CSR succeeds."""
    import torch
    from fk_mc_gb300.lattice import hopping_csr
    n, rp, col, val = hopping_csr("cubic2d", 6)
    dev = torch.device("cuda", 0)
    bad = col.copy()
    bad[3] = -1
    d_rp = torch.tensor(rp, dtype=torch.int32, device=dev)
    d_val = torch.tensor(val, dtype=torch.float64, device=dev)
    d_diag = torch.zeros(n, dtype=torch.float64, device=dev)
    d_beta = torch.ones(1, dtype=torch.float64, device=dev)
    d_w = torch.zeros(n, dtype=torch.float64, device=dev)
    d_z = torch.zeros(1, dtype=torch.float64, device=dev)
    err = ctypes.create_string_buffer(256)
    for cols, want in ((bad, -1), (col, 0)):
        d_col = torch.tensor(cols, dtype=torch.int32, device=dev)
        torch.cuda.synchronize()
        rc = fkg_lib.fkg_eigh_logz_noalloc(1, n, _dev(d_rp), _dev(d_col), _dev(d_val), _dev(d_diag), _dev(d_beta),
                                           _dev(d_w), _dev(d_z), None, err, 256)
        assert rc == want, err.value
        if want:
            assert b"outside [0, n)" in err.value


def test_noalloc_rejects_oversize(cuda_ok, fkg_lib):
    err = ctypes.create_string_buffer(256)
    # the size check comes first, before any pointer is looked at
    rc = fkg_lib.fkg_eigh_logz_noalloc(1, 129, None, None, None, None, None, None, None, None, err, 256)
    assert rc == -1 and b"FKG_NOALLOC_MAX_N" in err.value
    rc = fkg_lib.fkg_eigh_logz_noalloc(9, 16, None, None, None, None, None, None, None, None, err, 256)
    assert rc == -1 and b"FKG_NOALLOC_MAX_BATCH" in err.value
