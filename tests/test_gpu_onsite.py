"""Graph lattices whose hopping matrix has on-site (diagonal) entries, through the C ABI.

In the reference, calc_hamiltonian adds -mu_c + U f_i onto hopping_m()'s
diagonal (src/configuration.cpp:83-88), and a graph lattice read by
read_lattice_hdf5 (src/lattice/graph.cpp:52-80) may carry on-site terms in that
diagonal. fkg_set_hopping registers the whole hopping matrix, on-site entries
included, and fkg_eigh_logz's `diag` is only the -mu_c + U f_i part: each
on-site energy must enter H exactly once. The lattice here is written to .npy
datasets and read back by the host adapter's graph loader; H is checked
against the oracle's eigen-solve of the dense matrix.

Tolerances: FP64 eigenvalues within 1e-10 ||H||, logZ relative 1e-10; mixed
path eigenvalues within 1e-9 ||H||, logZ relative 1e-9.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _graph_with_onsite(tmp_path, L=12, seed=5):
    """A periodic L x L square lattice with random bond amplitudes and random on-site energies."""
    from fk_mc_gb300 import stats
    rng = np.random.default_rng(seed)
    n = L * L
    rows = []
    for x in range(L):
        for y in range(L):
            i = x * L + y
            rows.append([i, i, rng.uniform(-1.5, 1.5)])  # on-site energy
            for j in (((x + 1) % L) * L + y, x * L + (y + 1) % L):
                t = -rng.uniform(0.5, 1.5)
                rows.append([i, j, t])
                rows.append([j, i, t])
    coords = [[x, y] for x in range(L) for y in range(L)]
    d = str(tmp_path / "onsite_lattice")
    stats.write_graph_lattice(d, [L, L], 1, coords, np.array(rows, dtype=np.float64))
    rowptr, col, val = stats.graph_lattice_csr(d)
    H = np.zeros((n, n))
    for i in range(n):
        for p in range(rowptr[i], rowptr[i + 1]):
            H[i, col[p]] += val[p]
    assert np.abs(np.diag(H)).max() > 0.5, "the lattice must carry on-site entries"
    return n, rowptr, col, val, H


@pytest.mark.parametrize("precision,tol", [("f64", 1e-10), ("mixed", 1e-9)])
def test_onsite_hopping_counted_once(cuda_ok, fkg_lib, oracle, tmp_path, precision, tol):
    import fk_mc_gb300
    n, rowptr, col, val, H0 = _graph_with_onsite(tmp_path)
    s = fk_mc_gb300.Solver(max_n=n, max_batch=4, precision=precision)
    try:
        s.set_hopping(0, rowptr, col, val)
        rng = np.random.default_rng(11)
        B, U, mu, beta = 3, 2.0, 1.0, 4.0
        f = rng.integers(0, 2, (B, n))
        diag = (-mu + U * f).ravel().astype(float)  # the -mu_c + U f_i part only
        out = s.eigh_logz(np.zeros(B, np.int32), diag, beta)
        for c in range(B):
            H = H0 + np.diag(-mu + U * f[c])
            ref = oracle.eigh(H)
            lz = oracle.logz_of_spectrum(ref, beta)
            w = out["evals"][c * n:(c + 1) * n]
            hn = np.abs(ref).max()
            assert np.abs(w - ref).max() <= tol * hn, f"chain {c}: eigenvalues differ from the oracle"
            assert abs(out["logz"][c] - lz) <= tol * abs(lz), f"chain {c}: logZ differs from the oracle"
            # the double-count the boundary must not make: H0's diagonal added a second time
            wrong = oracle.eigh(H + np.diag(np.diag(H0)))
            assert np.abs(w - wrong).max() > 1e-3
    finally:
        s.close()
