"""GPU eigenvector measures against the oracle: measure_ipr
(include/fk_mc/measures/ipr.hpp:39-56) and the Drude stiffness of
measure_stiffness (include/fk_mc/measures/stiffness.hpp:129-187), on both
precisions, on single chains, uneven batches and the reference's stiffness
KATs (test/stiffness_test.cpp:60-63).

Tolerances: stiffness within 1e-9 (FP64 path) or 1e-5 (mixed path) relative
to the oracle, KATs within their stated 1e-3; ipr within 1e-10 / 1e-5 for
eigenvalues at least 1e-6 ||H|| from their neighbours (inside a degenerate
subspace the vectors, and so their ipr, are not unique)."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
NDIM = {"cubic2d": 2, "cubic3d": 3, "triangular": 2}


@pytest.fixture(scope="module")
def solvers(cuda_ok, fkg_lib):
    import fk_mc_gb300
    s64 = fk_mc_gb300.Solver(max_n=576, max_batch=8, precision="f64")
    s32 = fk_mc_gb300.Solver(max_n=576, max_batch=8, precision="mixed")
    yield s64, s32
    s64.close()
    s32.close()


@pytest.mark.parametrize("kind,L,U", [("cubic2d", 8, 2.0), ("triangular", 6, 3.0), ("cubic3d", 4, 1.0)])
def test_ipr_matches_oracle(solvers, oracle, kind, L, U):
    n = L ** NDIM[kind]
    f = np.random.default_rng(L + 11).integers(0, 2, n)
    ref = oracle.calc_ed(kind, L, f, 2.0, U, U / 2, vectors=True)
    want = oracle.ipr(ref["evecs"])
    w = ref["spectrum"]
    gap = np.minimum(np.r_[np.inf, np.diff(w)], np.r_[np.diff(w), np.inf])
    iso = gap > 1e-6 * np.abs(w).max()
    assert iso.sum() > n // 2
    for s, tol in ((solvers[0], 1e-10), (solvers[1], 1e-5)):
        s.set_lattice(0, kind, L)
        got = s.measure_ipr([0], -U / 2 + U * f, 2.0)[0]
        assert np.abs(got - want)[iso].max() < tol


@pytest.mark.parametrize("L,U,beta", [(6, 1.0, 2.0), (8, 4.0, 10.0), (8, 2.0, 1.0)])
def test_stiffness_matches_oracle(solvers, oracle, L, U, beta):
    f = np.random.default_rng(7 * L + int(U)).integers(0, 2, L * L)
    want = oracle.stiffness(L, 1.0, U, beta, f)
    for s, tol in ((solvers[0], 1e-9), (solvers[1], 1e-5)):
        s.set_lattice(0, "cubic2d", L)
        s.set_stiffness_ops(0, "cubic2d", L)
        got = s.measure_stiffness([0], -U / 2 + U * f, beta)[0]
        assert abs(got - want) < tol * max(1.0, abs(want)), (s.precision, got, want)


@pytest.mark.parametrize("case", json.load(open(os.path.join(GOLD, "reference_kats.json")))["stiffness"],
                         ids=lambda c: c["name"])
def test_stiffness_reference_kats(solvers, oracle, case):
    L, U = case["L"], case["U"]
    f = np.array(case["f"])
    for s in solvers:
        s.set_lattice(0, "cubic2d", L, case["t"])
        s.set_stiffness_ops(0, "cubic2d", L)
        got = s.measure_stiffness([0], -U / 2 + U * f, case["beta"])[0]
        assert abs(got - case["stiffness"]) < case["tol"]
    assert abs(got - oracle.stiffness(L, case["t"], U, case["beta"], f)) < 1e-5


def test_measures_uneven_batch(solvers, oracle):
    # two lattices of different N in one batch give each chain its own result
    rng = np.random.default_rng(5)
    f6, f8 = rng.integers(0, 2, 36), rng.integers(0, 2, 64)
    U, beta = 2.0, 3.0
    for s in solvers:
        s.set_lattice(0, "cubic2d", 6)
        s.set_stiffness_ops(0, "cubic2d", 6)
        s.set_lattice(1, "cubic2d", 8)
        s.set_stiffness_ops(1, "cubic2d", 8)
        diag = np.concatenate([-U / 2 + U * f8, -U / 2 + U * f6, -U / 2 + U * f8])
        st = s.measure_stiffness([1, 0, 1], diag, beta)
        tol = 1e-9 if s.precision == "f64" else 1e-5
        for got, L, f in zip(st, (8, 6, 8), (f8, f6, f8)):
            assert abs(got - oracle.stiffness(L, 1.0, U, beta, f)) < tol
        ip = s.measure_ipr([1, 0], np.concatenate([-U / 2 + U * f8, -U / 2 + U * f6]), beta)
        assert [a.size for a in ip] == [64, 36]


def test_stiffness_needs_operators(solvers):
    import fk_mc_gb300
    s = solvers[0]
    s.set_lattice(2, "cubic2d", 4)  # registering a lattice drops its operators
    with pytest.raises(fk_mc_gb300._lib.FkgError):
        s.measure_stiffness([2], np.zeros(16), 1.0)


def _cond_reference(L, X, ev, fermi, wgrid, eta):
    # the resonant terms of measure_stiffness::accumulate (stiffness.hpp:160-185)
    # summed on the grid: for i > j with |e_i - e_j| > 1e-12 and |sigma| > 1e-13,
    # sigma (L(w + e_j - e_i) - L(w + e_i - e_j)), L(x) = eta / pi / (x^2 + eta^2)
    from fk_mc_gb300.lattice import stiffness_ops
    n = L * L
    rp, c, tv, jv = stiffness_ops("cubic2d", L)
    Jm = np.zeros((n, n))
    for i in range(n):
        for p in range(rp[i], rp[i + 1]):
            Jm[i, c[p]] += jv[p]
    mJ = X.T @ Jm @ X
    lor = lambda x: eta / np.pi / (x * x + eta * eta)
    out = np.zeros(len(wgrid))
    for i in range(n):
        for j in range(i):
            if abs(ev[i] - ev[j]) > 1e-12:
                sv = np.pi * (fermi[j] - fermi[i]) * mJ[j, i] * mJ[i, j]
                if abs(sv) > 1e-13:
                    out += sv * (lor(wgrid + ev[j] - ev[i]) - lor(wgrid + ev[i] - ev[j]))
    return out


@pytest.mark.parametrize("L,U,beta", [(6, 2.0, 3.0), (8, 1.0, 5.0)])
def test_conductivity_history(solvers, oracle, L, U, beta):
    f = np.random.default_rng(L + 3).integers(0, 2, L * L)
    ref = oracle.calc_ed("cubic2d", L, f, beta, U, U / 2, vectors=True)
    wgrid = np.linspace(-4.0, 4.0, 41)
    eta = 0.1
    want = _cond_reference(L, ref["evecs"], ref["spectrum"], ref["fermi"], wgrid, eta)
    for s, tol in ((solvers[0], 1e-9), (solvers[1], 1e-5)):
        s.set_lattice(0, "cubic2d", L)
        s.set_stiffness_ops(0, "cubic2d", L)
        st, cond = s.measure_stiffness([0], -U / 2 + U * f, beta, wgrid, eta)
        assert cond.shape == (1, wgrid.size)
        assert np.abs(cond[0] - want).max() < tol * max(1.0, np.abs(want).max())
        assert abs(st[0] - oracle.stiffness(L, 1.0, U, beta, f)) < tol * max(1.0, abs(st[0]))


def test_host_adapter_measures(oracle):
    # the adapter's measure_stiffness / measure_ipr classes (C++) over the C ABI
    from fk_mc_gb300 import host_lib
    L, U, beta = 6, 2.0, 4.0
    f = np.random.default_rng(21).integers(0, 2, L * L)
    wgrid = np.linspace(-3.0, 3.0, 13)
    st, cond, ipr = host_lib.measure_eigen("cubic2d", L, f, beta, U, U / 2, wgrid, 0.2)
    assert abs(st - oracle.stiffness(L, 1.0, U, beta, f)) < 1e-9
    ref = oracle.calc_ed("cubic2d", L, f, beta, U, U / 2, vectors=True)
    want = _cond_reference(L, ref["evecs"], ref["spectrum"], ref["fermi"], wgrid, 0.2)
    assert np.abs(cond - want).max() < 1e-9 * max(1.0, np.abs(want).max())
    w = ref["spectrum"]
    gap = np.minimum(np.r_[np.inf, np.diff(w)], np.r_[np.diff(w), np.inf])
    iso = gap > 1e-6 * np.abs(w).max()
    assert np.abs(ipr - oracle.ipr(ref["evecs"]))[iso].max() < 1e-10
