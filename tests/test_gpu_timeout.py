"""The timeout path of the bounded mbarrier waits in the tcgen05 kernels.

The mixed path's tcgen05 back-transformation (backtransform_tc5.cu) and the
two-stage reduction's first stage (sy2sb.cu) bound every main-loop wait.
fkg_set_wait_limit(ctx, 0) makes each such wait give up without checking, so
the first wait of every CTA runs out: the kernel must set the timeout status,
wait for the copies and MMAs it has issued, free its tensor memory and return;
the call must fail with FKG_ERR_TIMEOUT (not a numeric error), and the same
context must then solve correctly again with the default limit (eigenvalues
within 1e-9 ||H|| and logZ within 1e-9 relative of the oracle, the mixed path's
tolerance). No GPU fault is involved: the wait is cut short on purpose, the
copies and MMAs themselves are valid.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kernel", ["backtransform_tc5", "sy2sb"])
def test_tcgen05_wait_timeout_is_reported_and_recovers(cuda_ok, fkg_lib, oracle, kernel):
    import fk_mc_gb300
    from fk_mc_gb300 import _lib
    L, B, U, beta = 16, 3, 2.0, 5.0
    n = L * L
    s = fk_mc_gb300.Solver(max_n=n, max_batch=B, precision="mixed")
    try:
        s.set_lattice(0, "cubic2d", L)
        for n_max in range(64, 1025, 64):  # the kernel under test for every size
            if kernel == "backtransform_tc5":
                s.set_tuning_back(n_max, 1)
            else:
                s.set_tuning("mixed", n_max, 3)  # the two-stage reduction
        rng = np.random.default_rng(7)
        f = rng.integers(0, 2, (B, n))
        diag = (-U / 2 + U * f).ravel().astype(float)
        ids = np.zeros(B, np.int32)
        s.set_wait_limit(0)
        w = np.zeros(B * n)
        lz = np.zeros(B)
        rc = s.lib.fkg_eigh_logz(s.ctx, B, _lib.i32(ids), _lib.f64(diag), _lib.f64(np.full(B, beta)), _lib.f64(w),
                                 None, None, None, _lib.f64(lz))
        assert rc == -5, f"expected FKG_ERR_TIMEOUT, got {rc}: {s.lib.fkg_last_error(s.ctx)}"
        assert b"bounded device wait" in s.lib.fkg_last_error(s.ctx)
        s.set_wait_limit(-1)
        for _ in range(2):  # the context is usable again, with correct results
            out = s.eigh_logz(ids, diag, beta)
            for c in range(B):
                ref = oracle.calc_ed("cubic2d", L, f[c], beta, U, U / 2)
                hn = np.abs(ref["spectrum"]).max()
                assert np.abs(out["evals"][c * n:(c + 1) * n] - ref["spectrum"]).max() <= 1e-9 * hn
                assert abs(out["logz"][c] - ref["logZ"]) <= 1e-9 * abs(ref["logZ"])
    finally:
        s.close()
