"""Chebyshev-expansion logZ on the GPU (fkg_chebyshev_logz, chebyshev.cu)
against the oracle's numpy restatement of calc_chebyshev (oracle/chebyshev.py).

Tolerances: spectral bounds within 1e-12 of the spectral width of the exact
extreme eigenvalues (the reference takes ARPACK's converged values); moments
to 1e-11 absolute (|mu_m| <= 1); logZ to 1e-10 relative. Device-resident chains
under FKG_METHOD_CHEBYSHEV: every accept/reject decision equal to the oracle's
except near-ties |w - u| < 1e-8 max(1, w)."""
import json
import math
import os

import numpy as np
import pytest

from oracle import chebyshev as C

pytestmark = pytest.mark.gpu
NDIM = {"cubic1d": 1, "cubic2d": 2, "cubic3d": 3, "triangular": 2}
KATS = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_kats.json")))


@pytest.fixture(scope="module")
def solver(cuda_ok, fkg_lib):
    import fk_mc_gb300
    s = fk_mc_gb300.Solver(max_n=1024, max_batch=64, precision="f64")
    yield s
    s.close()


def _check(solver, oracle, kind, L, U, beta, M, G, nconf=3, seed=1, t=1.0):
    n = L ** NDIM[kind]
    solver.set_lattice(0, kind, L, t)
    solver.set_chebyshev(M, G)
    rng = np.random.default_rng(seed)
    fs = rng.integers(0, 2, (nconf, n))
    mu_c = U / 2
    diag = (-mu_c + U * fs).ravel().astype(float)
    r = solver.chebyshev_logz(np.zeros(nconf, np.int32), diag, beta, moments=True)
    csr = oracle.lattice_csr(kind, L, t)
    for c in range(nconf):
        ref = C.calc_chebyshev(C.dense_h(csr, fs[c], U, mu_c), beta, M, G)
        width = ref["e_max"] - ref["e_min"]
        assert abs(r["e_min"][c] - ref["e_min"]) <= 1e-12 * width
        assert abs(r["e_max"][c] - ref["e_max"]) <= 1e-12 * width
        assert np.allclose(r["moments"][c], ref["moments"], atol=1e-11, rtol=0)
        assert abs(r["logz"][c] - ref["logZ"]) <= 1e-10 * abs(ref["logZ"])
        assert 0 < r["lanczos_steps"][c] < min(2 * n + 64, 2048)   # converged before the cap
    return r


@pytest.mark.parametrize("kind,L,U,beta,M,G", [
    ("cubic2d", 8, 1.0, 1.0, 12, 24),      # M/2 even
    ("cubic2d", 16, 2.0, 5.0, 14, 28),     # M/2 odd: mu_{M/2} from the product
    ("triangular", 6, 3.0, 2.0, 10, 10),
    ("cubic3d", 4, 1.0, 10.0, 20, 40),     # balls cover the whole lattice
    ("cubic1d", 40, 4.0, 3.0, 8, 16),
    ("cubic2d", 6, 2.0, 1.0, 2, 10),       # two moments: bounds and Tr x only
])
def test_chebyshev_logz_matches_oracle(solver, oracle, kind, L, U, beta, M, G):
    _check(solver, oracle, kind, L, U, beta, M, G)


def test_reference_chebyshev_case(solver, oracle):
    """fast_update_test.cpp:28-78 on the GPU: L=24 (N=576), U=8, t=-1, T=0.16, 12 moments on 12 points;
    equal to the oracle's expansion and within the reference's 5e-2 of the exact logZ."""
    k = KATS["logz_identity"]
    L, U, beta = k["L"], k["U"], 1.0 / k["T"]
    r0 = oracle.mc_run("cubic2d", L, beta, U, U / 2, U / 2, k["seed"], nsweeps=1, sweep_len=0, nf_start=L * L // 2)
    f = r0["f_initial"]
    solver.set_lattice(0, "cubic2d", L, -1.0)
    solver.set_chebyshev(12, 12)
    r = solver.chebyshev_logz(np.zeros(1, np.int32), (-U / 2 + U * f).astype(float), beta, moments=True)
    ref = C.calc_chebyshev(C.dense_h(oracle.lattice_csr("cubic2d", L, -1.0), f, U, U / 2), beta, 12, 12)
    assert abs(r["logz"][0] - ref["logZ"]) <= 1e-10 * abs(ref["logZ"])
    ed = oracle.calc_ed("cubic2d", L, f, beta, U, U / 2, t=-1.0)
    assert abs((r["logz"][0] - ed["logZ"]) / r["logz"][0]) < 5e-2


def test_uneven_batch(solver, oracle):
    """Chains on lattices of different size and ball size in one call."""
    import fk_mc_gb300
    s = fk_mc_gb300.Solver(max_n=1024, max_batch=16, precision="f64")
    try:
        cases = [("cubic2d", 8), ("triangular", 10), ("cubic3d", 5), ("cubic1d", 64)]
        for i, (kind, L) in enumerate(cases):
            s.set_lattice(i, kind, L)
        s.set_chebyshev(16, 32)
        rng = np.random.default_rng(5)
        ids = np.array([0, 1, 2, 3, 2, 0], np.int32)
        U, beta = 2.5, 4.0
        fs = [rng.integers(0, 2, L ** NDIM[kind]) for kind, L in (cases[i] for i in ids)]
        diag = np.concatenate([-U / 2 + U * f for f in fs]).astype(float)
        r = s.chebyshev_logz(ids, diag, beta)
        for c, i in enumerate(ids):
            kind, L = cases[i]
            ref = C.calc_chebyshev(C.dense_h(oracle.lattice_csr(kind, L), fs[c], U, U / 2), beta, 16, 32)
            assert abs(r["logz"][c] - ref["logZ"]) <= 1e-10 * abs(ref["logZ"]), (kind, L)
    finally:
        s.close()


def test_set_chebyshev_arguments(solver):
    from fk_mc_gb300._lib import FkgError
    import fk_mc_gb300
    with pytest.raises(FkgError):
        solver.set_chebyshev(1, 10)
    with pytest.raises(FkgError):
        solver.set_chebyshev(12, 1)
    s = fk_mc_gb300.Solver(max_n=64, max_batch=2)
    try:
        s.set_lattice(0, "cubic2d", 4)
        with pytest.raises(FkgError, match="fkg_set_chebyshev"):
            s.chebyshev_logz(np.zeros(1, np.int32), np.zeros(16), 1.0)
    finally:
        s.close()


def test_device_chains_with_chebyshev_moves(solver, oracle):
    """fkg_chains_init / fkg_propose_accept under FKG_METHOD_CHEBYSHEV: the single-site-flip Metropolis
    decisions of chebyshev::move_addremove (src/moves_chebyshev.cpp:54-72) against the oracle's expansion."""
    import fk_mc_gb300
    kind, L, U, mu_f, beta, M, G = "cubic2d", 6, 2.0, 1.0, 3.0, 12, 24
    n = L * L
    B, steps = 8, 12
    s = fk_mc_gb300.Solver(max_n=64, max_batch=B, precision="f64")
    try:
        s.set_lattice(0, kind, L)
        s.set_chebyshev(M, G)
        s.set_method("chebyshev")
        rng = np.random.default_rng(11)
        f = rng.integers(0, 2, (B, n)).astype(np.int32)
        s.chains_init(np.zeros(B, np.int32), f.ravel(), U, U / 2, mu_f, beta)
        site = rng.integers(0, n, (steps, B)).astype(np.int32)
        u = rng.random((steps, B))
        acc, dl = s.propose_accept(site, u)
        csr = oracle.lattice_csr(kind, L)
        cur = f.copy()
        logz = [C.calc_chebyshev(C.dense_h(csr, cur[c], U, U / 2), beta, M, G)["logZ"] for c in range(B)]
        ties = 0
        for k in range(steps):
            for c in range(B):
                g = cur[c].copy()
                g[site[k, c]] ^= 1
                lz = C.calc_chebyshev(C.dense_h(csr, g, U, U / 2), beta, M, G)["logZ"]
                ratio = math.exp(lz - logz[c])
                w = ratio * math.exp(beta * mu_f) if g[site[k, c]] else ratio / math.exp(beta * mu_f)
                assert abs(dl[k, c] - (lz - logz[c])) < 2e-10 * (abs(lz) + abs(logz[c]))
                if abs(abs(w) - u[k, c]) < 1e-8 * max(1.0, abs(w)):
                    ties += 1
                    if acc[k, c]:
                        cur[c], logz[c] = g, lz
                    continue
                assert bool(acc[k, c]) == (abs(w) > u[k, c]), (k, c)
                if acc[k, c]:
                    cur[c], logz[c] = g, lz
        fg, lzg, _ = s.chains_get()
        assert np.array_equal(fg.reshape(B, n), cur)
        assert np.allclose(lzg, logz, rtol=1e-10, atol=0)
    finally:
        s.close()


@pytest.mark.parametrize("kind,L,moves", [("cubic2d", 6, (0.0, 1.0, 0.0)), ("triangular", 5, (0.5, 1.0, 0.2))])
def test_host_adapter_chebyshev_chain(oracle, kind, L, moves):
    """fkh_run_chain with the Chebyshev moves (chebyshev::move_flip / move_addremove / move_randomize on
    calc_chebyshev on the GPU) against the oracle's Chebyshev chain, same seed: identical draws, decisions
    equal except near-ties."""
    from fk_mc_gb300 import host_lib
    kw = dict(kind=kind, L=L, beta=2.0, U=2.0, mu_c=1.0, mu_f=1.0, seed=34792, nsweeps=6, sweep_len=L * L,
              mc_flip=moves[0], mc_add_remove=moves[1], mc_reshuffle=moves[2])
    g = host_lib.run_chain(cheb_moves=True, **kw)
    r = oracle.mc_run(cheb_moves=True, **kw)
    assert np.array_equal(g["f_initial"], r["f_initial"])
    assert np.array_equal(g["move_index"], r["move_index"])
    near = np.abs(np.abs(r["weight"]) - r["uniform"]) < 1e-8
    first = np.nonzero((g["accepted"] != r["accepted"]) & ~near)[0]
    assert first.size == 0, f"decisions differ at {first[:5]}"
    if not near.any():
        assert np.array_equal(g["uniform"], r["uniform"])
        assert np.allclose(g["weight"], r["weight"], rtol=1e-9, atol=1e-300)
        assert np.array_equal(g["f_final"], r["f_final"])


def test_batched_chebyshev_chains_equal_single_chains(oracle):
    """fkh_run_batched with the Chebyshev moves: chain c equals the oracle's chain of seed SEED + c."""
    from fk_mc_gb300 import host_lib
    kw = dict(kind="cubic2d", L=6, beta=2.0, U=2.0, mu_c=1.0, mu_f=1.0, nsweeps=4, sweep_len=36)
    B, seed = 4, 34793
    g = host_lib.run_batched(seed=seed, batch=B, cheb_moves=True, **kw)
    for c in range(B):
        r = oracle.mc_run(seed=seed + c, cheb_moves=True, **kw)
        assert np.array_equal(g["f_initial"][c], r["f_initial"])
        near = np.abs(np.abs(r["weight"]) - r["uniform"]) < 1e-8
        assert not np.any((g["accepted"][c] != r["accepted"]) & ~near)
