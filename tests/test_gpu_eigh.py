"""GPU parity of the batched calc_ed (fkg_eigh_logz) against the CPU oracle.

Tolerances (FP64 path): eigenvalues |dlambda| <= 1e-10 * ||H||_2 (norm-wise
relative, the accuracy any backward-stable FP64 solver, Eigen included,
guarantees), logZ relative 1e-10, exp/fermi relative 1e-10.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")
NDIM = {"cubic1d": 1, "cubic2d": 2, "cubic3d": 3, "triangular": 2}


@pytest.fixture(scope="module")
def solver(cuda_ok, fkg_lib):
    import fk_mc_gb300
    s = fk_mc_gb300.Solver(max_n=1024, max_batch=64)
    yield s
    s.close()


def _check(out, refs, tol=1e-10):
    off = 0
    for c, ref in enumerate(refs):
        n = ref["spectrum"].size
        w = out["evals"][off:off + n]
        hn = np.abs(ref["spectrum"]).max()
        assert np.all(np.diff(w) >= 0), "spectrum not ascending"
        assert np.abs(w - ref["spectrum"]).max() <= tol * hn, f"chain {c}: eigenvalues differ"
        assert abs(out["logz"][c] - ref["logZ"]) <= tol * abs(ref["logZ"]), f"chain {c}: logZ differs"
        if "exp" in out:
            assert np.allclose(out["exp"][off:off + n], ref["exp"], rtol=tol, atol=0)
            assert np.allclose(out["fermi"][off:off + n], ref["fermi"], rtol=tol, atol=1e-300)
        off += n


@pytest.mark.parametrize("kind,L,U,beta", [("cubic2d", 8, 1.0, 1.0), ("cubic2d", 16, 2.0, 5.0),
                                           ("cubic3d", 8, 2.0, 5.0), ("triangular", 12, 1.5, 3.0),
                                           ("cubic1d", 37, 4.0, 10.0), ("cubic2d", 24, 2.0, 4.0)])
def test_eigh_logz_matches_oracle(solver, oracle, kind, L, U, beta):
    solver.set_lattice(0, kind, L)
    n = L ** NDIM[kind]
    rng = np.random.default_rng(L)
    B = 3
    f = rng.integers(0, 2, (B, n))
    diag = (-U / 2 + U * f).ravel()
    out = solver.eigh_logz(np.zeros(B, np.int32), diag, beta, exp_fermi=True)
    refs = [oracle.calc_ed(kind, L, f[c], beta, U, U / 2) for c in range(B)]
    _check(out, refs)


def test_uneven_batch(solver, oracle):
    lat = [("cubic2d", 12), ("cubic2d", 16), ("triangular", 12), ("cubic2d", 5), ("cubic1d", 3), ("cubic3d", 3)]
    for i, (k, L) in enumerate(lat):
        solver.set_lattice(i, k, L)
    rng = np.random.default_rng(5)
    ids, diags, refs, betas = [], [], [], []
    for c in range(12):
        i = c % len(lat)
        k, L = lat[i]
        n = L ** NDIM[k]
        U, beta = rng.uniform(0.5, 4), rng.uniform(1, 10)
        f = rng.integers(0, 2, n)
        ids.append(i)
        betas.append(beta)
        diags.append(-U / 2 + U * f)
        refs.append(oracle.calc_ed(k, L, f, beta, U, U / 2))
    out = solver.eigh_logz(np.array(ids), np.concatenate(diags), np.array(betas), exp_fermi=True)
    _check(out, refs)


def test_golden_fixture_cases(solver):
    g = json.load(open(os.path.join(GOLD, "oracle_cases.json")))
    for case in g["calc_ed"]:
        solver.set_lattice(0, case["kind"], case["L"], case["t"])
        f = np.array(case["f"])
        out = solver.eigh_logz([0], -case["mu_c"] + case["U"] * f, case["beta"])
        spec = np.array(case["spectrum"])
        assert np.abs(out["evals"] - spec).max() <= 1e-10 * np.abs(spec).max()
        assert abs(out["logz"][0] - case["logZ"]) <= 1e-10 * abs(case["logZ"])


def test_large_n_properties(solver):
    # N = 1024 (cubic2d L=32): trace and Frobenius norm are preserved, spectrum sorted
    from fk_mc_gb300.lattice import dense
    solver.set_lattice(0, "cubic2d", 32)
    rng = np.random.default_rng(1)
    f = rng.integers(0, 2, 1024)
    U = 3.0
    d = -U / 2 + U * f
    out = solver.eigh_logz([0], d, 2.0)
    w = out["evals"]
    H = dense("cubic2d", 32) + np.diag(d)
    assert np.all(np.diff(w) >= 0)
    assert abs(w.sum() - np.trace(H)) < 1e-9 * np.abs(w).sum()
    assert abs((w ** 2).sum() - (H ** 2).sum()) < 1e-10 * (H ** 2).sum()
    assert abs(out["logz"][0] - np.logaddexp(0, -2.0 * w).sum()) < 1e-12 * abs(out["logz"][0])


def test_analytic_band_n576(solver):
    # U = 0 on cubic2d L=24: eps(k) = -2t (cos kx + cos ky) - mu
    L = 24
    solver.set_lattice(0, "cubic2d", L)
    k = 2 * np.pi * np.arange(L) / L
    eps0 = np.sort((-2 * (np.cos(k)[:, None] + np.cos(k)[None, :])).ravel())
    out = solver.eigh_logz([0], np.full(L * L, -0.3), 4.0)
    assert np.abs(out["evals"] - (eps0 - 0.3)).max() < 1e-12 * 4


def test_bad_arguments_raise(solver):
    from fk_mc_gb300 import _lib
    from fk_mc_gb300._lib import FkgError
    ids = np.array([62], np.int32)  # never registered
    d, b, w, z = np.zeros(16), np.ones(1), np.zeros(16), np.zeros(1)
    rc = solver.lib.fkg_eigh_logz(solver.ctx, 1, _lib.i32(ids), _lib.f64(d), _lib.f64(b), _lib.f64(w), None, None,
                                  None, _lib.f64(z))
    assert rc == -1 and b"not registered" in solver.lib.fkg_last_error(solver.ctx)
    with pytest.raises(FkgError):
        solver.set_hopping(1, np.array([0, 1], np.int32), np.array([5], np.int32), np.array([1.0]))
    solver.set_lattice(0, "cubic2d", 4)
    with pytest.raises(FkgError):
        solver.eigh_logz([0], np.zeros(16), -1.0)  # beta must be > 0


def test_stream_and_profile(solver, oracle):
    import torch
    st = torch.cuda.Stream()
    solver.set_stream(st.cuda_stream)
    solver.set_lattice(0, "cubic2d", 8)
    solver.profile(True)
    f = np.zeros(64)
    out = solver.eigh_logz([0, 0], np.concatenate([f - 0.5, f + 0.5]), 1.0)
    ms, n = solver.stage_time("reduce")
    assert n == 1 and ms > 0
    solver.profile(False)
    solver.set_stream(0)
    ref = oracle.calc_ed("cubic2d", 8, np.zeros(64, np.int32), 1.0, 1.0, 0.5)
    assert np.abs(out["evals"][:64] - ref["spectrum"]).max() < 1e-12 * 4
