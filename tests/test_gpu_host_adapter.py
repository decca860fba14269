"""Drop-in parity: the C++ host adapter (the reference's configuration_t,
move_*, mc_metropolis and measure_energy classes with calc_ed on the GPU)
against the oracle's restatement of the reference run, same seed.

The random streams are identical (std::mt19937 and the libstdc++
distributions in both), so the initial configuration, every site draw and
every uniform must match bit for bit, and every accept/reject decision must
match except near-ties |w - u| < 1e-12 (FP64 path) or 1e-8 (mixed path),
which are counted and excluded. Energies (measure_energy) to 1e-10 relative."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def host(cuda_ok, fkg_lib):
    from fk_mc_gb300 import host_lib
    host_lib.load()
    return host_lib


def _compare(r, g, tie):
    near = np.abs(np.abs(r["weight"]) - r["uniform"]) < tie
    mism = np.nonzero((r["accepted"] != g["accepted"]) & ~near)[0]
    assert mism.size == 0, f"decisions differ at proposals {mism[:10]}"
    return near.sum()


@pytest.mark.parametrize("precision,tie", [("f64", 1e-12), ("mixed", 1e-8)])
def test_single_chain_c1(host, oracle, precision, tie):
    # cubic2d L=8 (N=64), t=1, U=1, mu=U/2, beta=1, single-site flips, sweep_len=N
    kw = dict(kind="cubic2d", L=8, beta=1.0, U=1.0, mu_c=0.5, mu_f=0.5, seed=34788, nsweeps=60, sweep_len=64)
    g = host.run_chain(precision=precision, **kw)
    r = oracle.mc_run(**kw)
    assert np.array_equal(g["f_initial"], r["f_initial"])
    assert np.array_equal(g["uniform"], r["uniform"])
    _compare(r, g, tie)
    assert np.array_equal(g["f_final"], r["f_final"])
    assert np.allclose(g["energy"], r["energy"], rtol=1e-10, atol=0)
    assert np.allclose(g["d2energy"], r["d2energy"], rtol=1e-10, atol=0)


def test_all_three_moves(host, oracle):
    # move_flip, move_addremove and move_randomize registered together (include/fk_mc/fk_mc.hxx:67-78)
    kw = dict(kind="cubic2d", L=4, beta=2.0, U=2.0, mu_c=1.0, mu_f=1.0, seed=7, nsweeps=30, sweep_len=16,
              ntherm_sweeps=2, mc_flip=1.0, mc_add_remove=1.0, mc_reshuffle=0.3)
    g = host.run_chain(**kw)
    r = oracle.mc_run(**kw)
    assert np.array_equal(g["move_index"], r["move_index"])
    assert np.array_equal(g["uniform"], r["uniform"])
    _compare(r, g, 1e-12)
    assert np.array_equal(g["f_final"], r["f_final"])
    assert np.allclose(g["energy"], r["energy"], rtol=1e-10, atol=0)


def test_triangular_and_3d(host, oracle):
    for kind, L in (("triangular", 6), ("cubic3d", 3)):
        kw = dict(kind=kind, L=L, beta=3.0, U=1.5, mu_c=0.75, mu_f=0.75, seed=101, nsweeps=10, sweep_len=20)
        g = host.run_chain(**kw)
        r = oracle.mc_run(**kw)
        _compare(r, g, 1e-12)
        assert np.array_equal(g["f_final"], r["f_final"])


@pytest.mark.parametrize("precision,tie", [("f64", 1e-12), ("mixed", 1e-8)])
def test_batched_chains_are_independent_ranks(host, oracle, precision, tie):
    # chain c of the batch == a reference rank with seed SEED + c
    B, kw = 6, dict(kind="cubic2d", L=6, beta=2.0, U=2.0, mu_c=1.0, mu_f=1.0, nsweeps=20, sweep_len=36)
    g = host.run_batched(seed=500, batch=B, precision=precision, **kw)
    for c in range(B):
        r = oracle.mc_run(seed=500 + c, **kw)
        assert np.array_equal(g["f_initial"][c], r["f_initial"])
        near = np.abs(np.abs(r["weight"]) - r["uniform"]) < tie
        mism = np.nonzero((r["accepted"] != g["accepted"][c]) & ~near)[0]
        assert mism.size == 0, f"chain {c}: decisions differ at {mism[:10]}"
        assert np.array_equal(g["f_final"][c], r["f_final"])
        assert np.allclose(g["energy"][c], r["energy"], rtol=1e-10, atol=0)


def test_chain_series_and_histories(host, oracle):
    """measure_nf0pi, measure_spectrum_history and measure_focc of the adapter: n_f(q=0) and
    n_f(q=pi) from the recorded f history, and each recorded spectrum equal to the oracle's
    calc_ed of the recorded configuration."""
    L = 6
    kw = dict(kind="cubic2d", L=L, beta=2.0, U=2.0, mu_c=1.0, mu_f=1.0, seed=34789, nsweeps=12, sweep_len=36)
    g = host.run_chain(history=True, **kw)
    focc = g["focc_history"]                      # V x nsweeps
    x, y = np.divmod(np.arange(L * L), L)
    phase = np.where((x + y) % 2 == 0, 1, -1)
    assert np.array_equal(g["nf0"], focc.sum(axis=0).astype(float))
    assert np.array_equal(g["nfpi"], np.abs(phase @ focc).astype(float))
    assert np.array_equal(focc[:, -1], g["f_final"])
    for m in range(kw["nsweeps"]):
        r = oracle.calc_ed("cubic2d", L, focc[:, m], kw["beta"], kw["U"], kw["mu_c"])
        assert np.allclose(g["spectrum_history"][:, m], r["spectrum"], rtol=0, atol=1e-12)


def test_graph_lattice_chain_equals_hypercubic(host, oracle, tmp_path):
    """The same square lattice given as a graph lattice (coordinates + hopping rows in .npy files,
    src/lattice/graph.cpp:52-80) runs the same chain as the hypercubic builder's."""
    from fk_mc_gb300 import stats
    L = 6
    rowptr, col, val = oracle.lattice_csr("cubic2d", L, 1.0)
    rows = [(i, int(col[k]), float(val[k])) for i in range(L * L) for k in range(rowptr[i], rowptr[i + 1])]
    stats.write_graph_lattice(str(tmp_path), [L, L], 1, [(i // L, i % L) for i in range(L * L)], np.array(rows))
    kw = dict(beta=2.0, U=2.0, mu_c=1.0, mu_f=1.0, seed=34790, nsweeps=10, sweep_len=36)
    a = host.run_chain(kind="cubic2d", L=L, **kw)
    b = host.run_chain_graph(str(tmp_path), L * L, **kw)
    assert np.array_equal(a["f_initial"], b["f_initial"])
    assert np.array_equal(a["accepted"], b["accepted"])
    assert np.array_equal(a["f_final"], b["f_final"])
    assert np.allclose(a["energy"], b["energy"], rtol=1e-13, atol=0)
    assert np.array_equal(a["nfpi"], b["nfpi"])


def test_chain_to_saved_statistics(host, tmp_path):
    """A chain's series through the statistics stage: energy and cv binned, n_f statistics present."""
    from fk_mc_gb300 import stats
    kw = dict(kind="cubic2d", L=6, beta=2.0, U=2.0, mu_c=1.0, mu_f=1.0, seed=34791, nsweeps=64, sweep_len=36)
    g = host.run_chain(history=True, **kw)
    obs = {"energies": g["energy"], "d2energies": g["d2energy"], "c_energies": g["c_energy"], "nf0": g["nf0"],
           "nfpi": g["nfpi"], "spectrum_history": g["spectrum_history"],
           "focc_history": g["focc_history"].astype(float)}
    js = stats.save_stats(str(tmp_path), obs, kw["beta"], 36, dos_npts=24)
    for k in ("energy", "cv", "nf_0", "nf_pi", "fsusc_0", "binder_0", "dos0", "nc"):
        assert k in js, k
    assert abs(js["energy"]["mean"] - g["energy"].mean()) < 1e-12 * abs(g["energy"].mean()) + 1e-12
