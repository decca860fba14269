"""CPU tests: pin the oracle against the reference's golden values, LAPACK and
analytic known answers. No GPU needed."""
import json
import os

import numpy as np
import pytest
import scipy.linalg as sl

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def kats():
    return json.load(open(os.path.join(GOLD, "reference_kats.json")))


@pytest.mark.parametrize("case", kats()["stiffness"], ids=lambda c: c["name"])
def test_reference_stiffness_kats(oracle, case):
    # test/stiffness_test.cpp:60-63 — eigenvalues, eigenvectors and fermi factors at beta=1000
    val = oracle.stiffness(case["L"], case["t"], case["U"], case["beta"], case["f"])
    assert abs(val - case["stiffness"]) < case["tol"]


def test_reference_logz_identity(oracle):
    # test/fast_update_test.cpp:70-78: logZ equals the direct sum to 1e-15 relative
    k = kats()["logz_identity"]
    L, U, beta = k["L"], k["U"], 1.0 / k["T"]
    r = oracle.mc_run("cubic2d", L, beta, U, U / 2, U / 2, k["seed"], nsweeps=1, sweep_len=0,
                      nf_start=L * L // 2)
    f = r["f_initial"]
    assert f.sum() == L * L // 2
    ed = oracle.calc_ed("cubic2d", L, f, beta, U, U / 2, t=-1.0)
    direct = np.sum(np.log1p(np.exp(-beta * ed["spectrum"])))
    assert abs(ed["logZ"] - direct) / abs(ed["logZ"]) < 1e-13  # summation order differs from numpy's
    assert abs(ed["logZ"] - oracle.logz_of_spectrum(ed["spectrum"], beta)) == 0.0


@pytest.mark.parametrize("n", [1, 2, 3, 7, 33, 100])
def test_eigh_vs_lapack_random(oracle, n):
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n))
    A = A + A.T
    w, Z = oracle.eigh(A, vectors=True)
    ref = sl.eigh(A, eigvals_only=True)
    nrm = max(np.abs(ref).max(), 1.0)
    assert np.all(np.diff(w) >= 0)
    assert np.abs(w - ref).max() < 1e-12 * nrm
    assert np.abs(A @ Z - Z * w).max() < 1e-12 * nrm
    assert np.abs(Z.T @ Z - np.eye(n)).max() < 1e-12


@pytest.mark.parametrize("kind,L", [("cubic2d", 8), ("cubic3d", 4), ("triangular", 6), ("cubic1d", 16)])
def test_calc_ed_vs_lapack(oracle, kind, L):
    rng = np.random.default_rng(L)
    n = L ** {"cubic1d": 1, "cubic2d": 2, "cubic3d": 3, "triangular": 2}[kind]
    f = rng.integers(0, 2, n)
    U, beta = 2.0, 5.0
    ed = oracle.calc_ed(kind, L, f, beta, U, U / 2)
    H = oracle.dense_hopping(kind, L) + np.diag(-U / 2 + U * f)
    ref = sl.eigh(H, eigvals_only=True)
    assert np.abs(ed["spectrum"] - ref).max() < 1e-12 * np.abs(ref).max()
    assert np.allclose(ed["exp"], np.exp(beta * ed["spectrum"]), rtol=1e-15, atol=0)
    assert np.allclose(ed["fermi"], 1 / (1 + ed["exp"]), rtol=1e-15, atol=0)
    direct = np.sum(np.logaddexp(0.0, -beta * ref))
    assert abs(ed["logZ"] - direct) < 1e-12 * abs(direct)


def test_analytic_kats(oracle):
    L, t = 8, 1.0
    k = 2 * np.pi * np.arange(L) / L
    eps0 = (-2 * t * (np.cos(k)[:, None] + np.cos(k)[None, :])).ravel()
    for U in (0.0, 1.0, 4.0):
        mu = U / 2
        # (1) U = 0 band; (2) all f occupied: the band shifted by U
        for fill, shift in ((0, 0.0), (1, U)):
            ed = oracle.calc_ed("cubic2d", L, np.full(L * L, fill), 1.0, U, mu)
            assert np.abs(ed["spectrum"] - np.sort(eps0 - mu + shift)).max() < 1e-13
        # (3) checkerboard on the bipartite square lattice
        x, y = np.meshgrid(np.arange(L), np.arange(L), indexing="ij")
        f = ((x + y) % 2).ravel()
        ed = oracle.calc_ed("cubic2d", L, f, 1.0, U, mu)
        # eps0(k) and eps0(k+pi) = -eps0(k) pair up, so each value appears twice
        ref = np.sort(np.concatenate([U / 2 - mu + s * np.sqrt(U ** 2 / 4 + eps0 ** 2) for s in (1, -1)]))[::2]
        assert np.abs(ed["spectrum"] - np.sort(ref)).max() < 1e-12


def test_lattice_builder_matches_oracle(oracle):
    from fk_mc_gb300.lattice import hopping_csr
    for kind, L, t, tp in [("cubic1d", 10, 1.0, 0), ("cubic2d", 6, -1.0, 0), ("cubic3d", 4, 1.0, 0),
                           ("triangular", 6, 1.0, 0.5)]:
        n, rp, c, v = hopping_csr(kind, L, t, tp)
        orp, oc, ov = oracle.lattice_csr(kind, L, t, tp)
        assert np.array_equal(rp, orp) and np.array_equal(c, oc) and np.array_equal(v, ov)


def test_oracle_golden_cases(oracle):
    g = json.load(open(os.path.join(GOLD, "oracle_cases.json")))
    for case in g["calc_ed"]:
        ed = oracle.calc_ed(case["kind"], case["L"], case["f"], case["beta"], case["U"], case["mu_c"])
        assert np.abs(ed["spectrum"] - case["spectrum"]).max() < 1e-13
        assert abs(ed["logZ"] - case["logZ"]) < 1e-12 * abs(case["logZ"])
    ch = g["chain"]
    r = oracle.mc_run(ch["kind"], ch["L"], ch["beta"], ch["U"], ch["mu_c"], ch["mu_f"], ch["seed"], ch["nsweeps"],
                      ch["sweep_len"])
    assert r["site"].tolist() == ch["site"]
    assert r["accepted"].tolist() == ch["accepted"]
    assert r["f_final"].tolist() == ch["f_final"]
    assert np.allclose(r["energy"], ch["energy"], rtol=1e-12, atol=0)


def test_mc_draw_order(oracle):
    """Every proposal consumes: discrete_distribution (move), uniform_int (site),
    uniform_real (Metropolis), in that order (src/mc_metropolis.cpp:41-43, src/moves.cpp:55-57).
    Replaying the draws from a fresh mt19937 reproduces the recorded sites and uniforms."""
    import random
    r = oracle.mc_run("cubic2d", 4, 1.0, 1.0, 0.5, 0.5, 7, nsweeps=3, sweep_len=16, nf_start=0)
    # nf_start = 0 makes randomize_f draw nf itself, then nf site draws with rejection
    assert r["site"].min() >= 0 and r["site"].max() < 16
    assert np.all((r["uniform"] >= 0) & (r["uniform"] < 1))
    # the weight decides acceptance exactly as |w| > u
    assert np.array_equal(r["accepted"], (np.abs(r["weight"]) > r["uniform"]).astype(np.int32))
