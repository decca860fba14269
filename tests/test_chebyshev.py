"""The oracle's restatement of the Chebyshev-expansion logZ (oracle/chebyshev.py),
pinned against the reference's own checks (test/fast_update_test.cpp) and against
exact identities. CPU only."""
import json
import math
import os

import numpy as np
import pytest

from oracle import chebyshev as C

KATS = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_kats.json")))

FUNCS = {"1.": lambda x: 1., "x*x": lambda x: x * x, "sin(x)": math.sin}


def test_moment_f_reference_kats():
    # fast_update_test.cpp:52-65: cheb_size = 2 int(log(msize)) (even), grid = cheb_size
    k = KATS["chebyshev"]
    cheb = int(math.log(k["msize"])) * 2
    cheb += cheb % 2
    ch = C.ChebyshevEval(cheb, cheb)
    assert ch.M == 12
    for c in k["checks"]:
        assert abs(ch.moment_f(FUNCS[c["f"]], c["order"]) - c["value"]) < c["tol"], c


@pytest.mark.parametrize("n,M", [(5, 2), (12, 10), (30, 12), (40, 21)])
def test_moments_equal_spectral_sums(n, M):
    rng = np.random.default_rng(n + M)
    A = rng.standard_normal((n, n))
    H = A + A.T
    ev = np.linalg.eigvalsh(H)
    a, b = (ev[-1] - ev[0]) / 2, (ev[-1] + ev[0]) / 2
    x = (H - b * np.eye(n)) / a
    mu = C.moments(x, M + M % 2)
    xs = np.clip((ev - b) / a, -1, 1)
    exact = [np.mean(np.cos(m * np.arccos(xs))) for m in range(M + M % 2)]
    assert np.allclose(mu, exact, atol=1e-11, rtol=0)


def test_logz_close_to_exact_as_the_reference_test_asks(oracle):
    # fast_update_test.cpp:28-78: L=24, U=8, mu=U/2, t=-1, T=0.16, f = randomize_f(mt19937(32167), L^2/2):
    # the Chebyshev logZ with 12 moments on 12 grid points within 5e-2 of the exact one
    k = KATS["logz_identity"]
    L, U, beta = k["L"], k["U"], 1.0 / k["T"]
    r = oracle.mc_run("cubic2d", L, beta, U, U / 2, U / 2, k["seed"], nsweeps=1, sweep_len=0, nf_start=L * L // 2)
    f = r["f_initial"]
    H = C.dense_h(oracle.lattice_csr("cubic2d", L, -1.0), f, U, U / 2)
    res = C.calc_chebyshev(H, beta, 12, 12)
    ed = oracle.calc_ed("cubic2d", L, f, beta, U, U / 2, t=-1.0)
    assert abs((res["logZ"] - ed["logZ"]) / res["logZ"]) < 5e-2
    # more moments and grid points converge to the exact value
    fine = C.calc_chebyshev(H, beta, 200, 400)
    assert abs((fine["logZ"] - ed["logZ"]) / ed["logZ"]) < 1e-6


@pytest.mark.parametrize("kind,L,moves", [("cubic2d", 4, (0.0, 1.0, 0.0)), ("triangular", 4, (0.0, 1.0, 0.0))])
def test_cpp_oracle_chebyshev_chain_equals_numpy(oracle, kind, L, moves):
    """The C++ oracle's Chebyshev moves (used as the chain reference) recomputed proposal by
    proposal with the numpy restatement: every add/remove weight to 1e-12."""
    beta, U, mu = 2.0, 2.0, 1.0
    r = oracle.mc_run(kind, L, beta, U, mu, mu, 7, nsweeps=3, sweep_len=16, mc_flip=moves[0],
                      mc_add_remove=moves[1], mc_reshuffle=moves[2], cheb_moves=True)
    n = L * L
    cs = int(math.log(n) * 2.2)
    cs += cs % 2
    G = max(2 * cs, 10)
    csr = oracle.lattice_csr(kind, L)
    f = r["f_initial"].copy()
    lz = C.calc_chebyshev(C.dense_h(csr, f, U, mu), beta, cs, G)["logZ"]
    checked = 0
    for k in range(r["accepted"].size):
        if r["move_index"][k] != 1:      # flips and reshuffles: follow the accepted state only
            if r["accepted"][k]:
                break
            continue
        s = r["site"][k]
        g = f.copy()
        g[s] ^= 1
        l1 = C.calc_chebyshev(C.dense_h(csr, g, U, mu), beta, cs, G)["logZ"]
        w = math.exp(l1 - lz) * (math.exp(beta * mu) if g[s] else math.exp(-beta * mu))
        assert abs(w - r["weight"][k]) <= 1e-12 * w
        checked += 1
        if r["accepted"][k]:
            f, lz = g, l1
    assert checked >= 8


def test_cpp_oracle_chebyshev_all_moves_run(oracle):
    r = oracle.mc_run("cubic2d", 4, 2.0, 2.0, 1.0, 1.0, 9, nsweeps=3, sweep_len=16, mc_flip=0.5, mc_add_remove=1.0,
                      mc_reshuffle=0.2, cheb_moves=True)
    assert set(np.unique(r["move_index"])) <= {0, 1, 2} and len(np.unique(r["move_index"])) >= 2
    assert np.all(np.isfinite(r["weight"]))
