"""Single-site-flip proposals by the rank-one update (fkg_rank1_logz, rank1.cu):
the eigenvalues and logZ of the flipped configuration from the current
eigen-decomposition, against the oracle's full re-solve of the flipped
configuration (calc_ed). Tolerances: eigenvalues |dl| <= 1e-12 ||H||; logZ
1e-12 relative (the rank-one update is as accurate as the FP64 eigenvectors
it starts from)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
NDIM = {"cubic1d": 1, "cubic2d": 2, "cubic3d": 3, "triangular": 2}


@pytest.fixture(scope="module")
def solver(cuda_ok, fkg_lib):
    import fk_mc_gb300
    s = fk_mc_gb300.Solver(max_n=1024, max_batch=64, precision="f64")
    yield s
    s.close()


def _proposals(oracle, kind, L, U, beta, fs, sites, mu=None):
    mu = U / 2 if mu is None else mu
    ev, Z, rho, ref_ev, ref_lz = [], [], [], [], []
    for f, s in zip(fs, sites):
        cur = oracle.calc_ed(kind, L, f, beta, U, mu, vectors=True)
        g = f.copy()
        g[s] ^= 1
        new = oracle.calc_ed(kind, L, g, beta, U, mu)
        ev.append(cur["spectrum"])
        Z.append(cur["evecs"][s])          # row s of the eigenvector matrix
        rho.append(U if g[s] else -U)
        ref_ev.append(new["spectrum"])
        ref_lz.append(new["logZ"])
    return np.array(ev), np.array(Z), np.array(rho), np.array(ref_ev), np.array(ref_lz)


@pytest.mark.parametrize("kind,L,U,beta", [("cubic2d", 8, 1.0, 1.0), ("cubic2d", 16, 2.0, 5.0),
                                           ("triangular", 10, 3.0, 2.0), ("cubic3d", 6, 4.0, 10.0),
                                           ("cubic1d", 100, 0.5, 3.0)])
def test_rank1_matches_full_resolve(solver, oracle, kind, L, U, beta):
    n = L ** NDIM[kind]
    rng = np.random.default_rng(n)
    B = 6
    fs = rng.integers(0, 2, (B, n))
    sites = rng.integers(0, n, B)
    ev, Z, rho, ref_ev, ref_lz = _proposals(oracle, kind, L, U, beta, fs, sites)
    lz, evn = solver.rank1_logz(ev, Z, rho, beta, evals_new=True)
    scale = np.max(np.abs(ref_ev), axis=1, keepdims=True)
    assert np.all(np.abs(evn - ref_ev) <= 1e-12 * scale)
    assert np.all(np.abs(lz - ref_lz) <= 1e-12 * np.abs(ref_lz))


def test_rank1_deflation_cases(solver, oracle):
    """Degenerate spectra (clean lattices: every f equal, so many equal eigenvalues and zero
    components of z), U = 0 (no change), a single site."""
    L, beta = 8, 2.0
    n = L * L
    cases = [np.zeros(n, int), np.ones(n, int)]
    checker = np.indices((L, L)).sum(axis=0).ravel() % 2
    cases.append(checker)
    for f in cases:
        for U in (2.0, 0.0):
            ev, Z, rho, ref_ev, ref_lz = _proposals(oracle, "cubic2d", L, U, beta, [f, f], [0, 27], mu=1.0)
            lz, evn = solver.rank1_logz(ev, Z, rho, beta, evals_new=True)
            assert np.all(np.abs(evn - ref_ev) <= 1e-12 * np.max(np.abs(ref_ev)))
            assert np.all(np.abs(lz - ref_lz) <= 1e-12 * np.abs(ref_lz))
    lz, evn = solver.rank1_logz(np.array([[0.3]]), np.array([[1.0]]), [2.0], 1.0, evals_new=True)
    assert abs(evn[0, 0] - 2.3) < 1e-13 and abs(lz[0] - np.log1p(np.exp(-2.3))) < 1e-13


def test_rank1_on_gpu_eigenvectors(solver, oracle):
    """The eigen-decomposition from the library's own FP64 path (fkg_eigh_logz with evecs)."""
    L, U, beta = 12, 2.0, 4.0
    n = L * L
    solver.set_precision("f64")
    solver.set_lattice(0, "cubic2d", L)
    rng = np.random.default_rng(9)
    B = 8
    fs = rng.integers(0, 2, (B, n))
    out = solver.eigh_logz(np.zeros(B, np.int32), (-U / 2 + U * fs).ravel().astype(float), beta, vectors=True)
    sites = rng.integers(0, n, B)
    ev = out["evals"].reshape(B, n)
    Z = np.array([out["evecs"][c][sites[c]] for c in range(B)])
    rho = np.where(fs[np.arange(B), sites] == 0, U, -U)
    lz = solver.rank1_logz(ev, Z, rho, beta)
    for c in range(B):
        g = fs[c].copy()
        g[sites[c]] ^= 1
        ref = oracle.calc_ed("cubic2d", L, g, beta, U, U / 2)
        assert abs(lz[c] - ref["logZ"]) <= 1e-12 * abs(ref["logZ"])


def test_rank1_arguments(solver):
    from fk_mc_gb300._lib import FkgError
    with pytest.raises(FkgError, match="ascending"):
        solver.rank1_logz(np.array([[1.0, 0.0]]), np.array([[0.6, 0.8]]), [1.0], 1.0)
    with pytest.raises(FkgError, match="beta"):
        solver.rank1_logz(np.array([[0.0, 1.0]]), np.array([[0.6, 0.8]]), [1.0], -1.0)


@pytest.mark.parametrize("kind,L,U,beta", [("cubic2d", 8, 1.0, 1.0), ("triangular", 6, 4.0, 8.0)])
def test_host_adapter_rank1_chain(oracle, kind, L, U, beta):
    """move_addremove_rank1 in the host adapter (proposal spectra by the rank-one update, a re-solve
    with eigenvectors only after an accept) against the oracle's plain chain, same seed: the same
    draws, decisions equal except near-ties |w - u| < 1e-10, energies to 1e-10."""
    from fk_mc_gb300 import host_lib
    n = L * L
    kw = dict(kind=kind, L=L, beta=beta, U=U, mu_c=U / 2, mu_f=U / 2, seed=34794, nsweeps=10, sweep_len=n)
    g = host_lib.run_chain(rank1_moves=True, **kw)
    r = oracle.mc_run(**kw)
    assert np.array_equal(g["f_initial"], r["f_initial"])
    near = np.abs(np.abs(r["weight"]) - r["uniform"]) < 1e-10
    assert not np.any((g["accepted"] != r["accepted"]) & ~near)
    if not near.any():
        assert np.array_equal(g["uniform"], r["uniform"])
        assert np.allclose(g["weight"], r["weight"], rtol=1e-9, atol=0)
        assert np.array_equal(g["f_final"], r["f_final"])
        assert np.allclose(g["energy"], r["energy"], rtol=1e-10, atol=0)
