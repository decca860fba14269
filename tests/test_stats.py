"""Statistics and output stage (binning, jackknife, save_all) and the
graph-lattice loader of the C++ host adapter, against the oracle restatement
(oracle/stats.py), which is itself pinned to the binning and jackknife known
answers of the reference's tests. CPU only."""
import json
import os

import numpy as np
import pytest

from oracle import stats as S

GOLD = os.path.join(os.path.dirname(__file__), "golden", "reference_kats.json")
KATS = json.load(open(GOLD))


@pytest.fixture(scope="module")
def st():
    from fk_mc_gb300 import stats
    stats._h()
    return stats


# ---- the oracle against the reference's own known answers ----

def test_oracle_binning_kats():
    k = KATS["binning"]
    rows = S.accumulate_binning(k["a"], k["max_depth"])
    for got, exp in zip(rows, k["stats"]):
        assert got[0] == exp[0]
        assert np.allclose(got[1:], exp[1:], atol=k["tol"], rtol=0)
    assert np.allclose(S.cor_length(rows), k["cor_lens"], atol=k["tol"], rtol=0)


def test_oracle_jackknife_kats():
    k = KATS["jackknife"]
    a, b = k["a"], k["b"]
    a2 = [x * x for x in a]
    for c in k["cases"]:
        if c["func"] == "mean":
            got = S.jack(S.FUNCS["mean"], [a], c["depth"])
        else:
            got = S.jack(S.cv_function(1.0, 1.0), [a, a2, b], c["depth"])
        assert got[0] == c["stats"][0]
        assert np.allclose(got[1:], c["stats"][1:], atol=k["tol"], rtol=0), c


# ---- the host adapter against the oracle ----

def test_binning_kats_through_host(st):
    k = KATS["binning"]
    rows = st.binning(k["a"], k["max_depth"])
    assert np.allclose(rows[:, :4], np.array(k["stats"]), atol=k["tol"], rtol=0)
    assert np.allclose(rows[:, 4], k["cor_lens"], atol=k["tol"], rtol=0)


def test_jackknife_kats_through_host(st):
    k = KATS["jackknife"]
    a = np.array(k["a"])
    b = np.array(k["b"])
    for c in k["cases"]:
        if c["func"] == "mean":
            rows = st.jackknife("mean", [a], c["depth"])
        else:
            rows = st.jackknife("cv", [a, a * a, b], c["depth"], fparams=[1.0, 1.0])
        assert np.allclose(rows[c["depth"]], c["stats"], atol=k["tol"], rtol=0), c


@pytest.mark.parametrize("n,depth,reverse", [(17, 3, False), (1000, 5, True), (4097, 11, False), (64, 6, True)])
def test_binning_matches_oracle(st, n, depth, reverse):
    rng = np.random.default_rng(n + depth)
    x = np.cumsum(rng.normal(size=n)) * 0.01 + rng.normal(size=n)   # correlated series
    rows = st.binning(x, depth, reverse=reverse)
    seq = list(x[::-1]) if reverse else list(x)
    ref = S.accumulate_binning(seq, depth)
    ref5 = np.array([list(r) + [c] for r, c in zip(ref, S.cor_length(ref))])
    if n >> depth == 1:      # one bin at the deepest level: variance 0/0
        assert np.isnan(rows[-1, 2]) and np.isnan(ref5[-1, 2])
        rows, ref5 = rows[:-1], ref5[:-1]
    assert np.array_equal(rows[:, 0], ref5[:, 0])
    assert np.allclose(rows, ref5, rtol=1e-13, atol=0)
    assert st.estimate_bin(rows) == S.estimate_bin(ref5)


@pytest.mark.parametrize("func,nser", [("mean", 1), ("disp", 2), ("binder", 2), ("cv", 3), ("linear", 4)])
def test_jackknife_matches_oracle(st, func, nser):
    rng = np.random.default_rng(7 + nser)
    n, depth = 300, 4
    base = rng.normal(loc=2.0, size=n)
    series = [base ** (k + 1) + 0.1 * rng.normal(size=n) for k in range(nser)]
    fp = {"cv": [4.0, 576.0], "linear": [1.0, -2.0, 0.5, 3.0]}.get(func)
    rows = st.jackknife(func, series, depth, fparams=fp)
    if func == "cv":
        F = S.cv_function(*fp)
    elif func == "linear":
        F = lambda x: sum(c * v for c, v in zip(fp, x))
    else:
        F = S.FUNCS[func]
    ref = np.array(S.accumulate_jackknife(F, [list(s) for s in series], depth))
    assert np.allclose(rows, ref, rtol=1e-11, atol=1e-14)
    rrows = st.jackknife(func, series, depth, reverse=True, fparams=fp)
    rref = np.array(S.accumulate_jackknife(F, [list(s[::-1]) for s in series], depth))
    assert np.allclose(rrows, rref, rtol=1e-11, atol=1e-14)


def test_errors_are_reported(st):
    from fk_mc_gb300._lib import FkgError
    with pytest.raises(FkgError, match="binning step"):
        st.binning(np.arange(8.0), 4)          # 16-sample bins of 8 samples
    with pytest.raises(FkgError, match="max_bin"):
        st.binning(np.arange(1 << 17, dtype=float), 16)
    with pytest.raises(FkgError, match="three series"):
        st.jackknife("cv", [np.ones(8), np.ones(8)], 1, fparams=[1.0, 1.0])
    with pytest.raises(FkgError):
        st.jackknife("mean", [np.ones(8), np.ones(7)], 1)


def _synthetic_run(rng, M, V, nw):
    e = np.cumsum(rng.normal(size=M)) * 0.02 - 0.5 * V
    obs = {"energies": e, "d2energies": np.abs(rng.normal(size=M)) + V * 0.1, "c_energies": e + 0.1,
           "nf0": rng.integers(V // 3, 2 * V // 3, M).astype(float),
           "nfpi": np.abs(rng.integers(-V // 4, V // 4, M)).astype(float),
           "stiffness": 0.3 + 0.01 * rng.normal(size=M)}
    spec = np.sort(rng.normal(scale=2.0, size=(M, V)), axis=1)
    obs["spectrum_history"] = spec.T.copy()
    obs["ipr_history"] = (0.2 + 0.05 * rng.random(size=(V, M)))
    obs["focc_history"] = rng.integers(0, 2, size=(V, M)).astype(float)
    w = np.linspace(-2.0, 2.0, nw) + 1e-3
    obs["cond_history"] = 0.1 * rng.normal(size=(nw, M)) + w[:, None]
    return obs, w


def test_save_stats_matches_oracle(st, tmp_path):
    rng = np.random.default_rng(34788)
    M, V, nw = 256, 16, 7
    obs, w = _synthetic_run(rng, M, V, nw)
    beta = 4.0
    js = st.save_stats(str(tmp_path), obs, beta, V, measure_history=True, measure_ipr=True, measure_stiffness=True,
                       dos_npts=40, wgrid_cond=w)
    ref = S.save_all({k: v.tolist() for k, v in obs.items()}, beta, V, dos_npts=40, measure_history=True,
                     measure_ipr=True, measure_stiffness=True, wgrid_cond=w.tolist())
    assert set(js) == set(ref["stats"])
    for name, (b, row) in ref["stats"].items():
        assert js[name]["bin"] == b, name
        got = [js[name]["size"], js[name]["mean"], js[name]["disp"], js[name]["error"]]
        assert np.allclose(got, row, rtol=1e-10, atol=1e-14), name
        npy = np.load(os.path.join(tmp_path, "stats", name + ".npy"))
        assert np.allclose(npy, row, rtol=1e-10, atol=1e-14), name
    for name, rows in ref["binning"].items():
        got = np.load(os.path.join(tmp_path, "binning", name + ".npy"))
        assert got.shape == (len(rows), 5), name
        assert np.allclose(got, np.array(rows), rtol=1e-10, atol=1e-14), name
    for name, rows in ref["tables"].items():
        got = np.load(os.path.join(tmp_path, "stats", name + ".npy"))
        assert np.allclose(got, np.array(rows), rtol=1e-10, atol=1e-14), name
    # the measured series are stored unchanged
    for k in ("energies", "d2energies", "nf0", "nfpi", "stiffness"):
        assert np.array_equal(np.load(os.path.join(tmp_path, "mc_data", k + ".npy")), obs[k])
    assert np.array_equal(np.load(os.path.join(tmp_path, "mc_data", "spectrum_history.npy")), obs["spectrum_history"])
    assert np.array_equal(np.load(os.path.join(tmp_path, "mc_data", "cond_history.npy")), obs["cond_history"])
    # default depth: the reference's rule on 256 measurements
    assert S.default_max_bin(M) == 3
    assert len(np.load(os.path.join(tmp_path, "binning", "energy.npy"))) == 4


def test_save_stats_parameters_and_minimal_input(st, tmp_path):
    from fk_mc_gb300 import host_lib
    P, _ = host_lib._params("cubic2d", 4, 2.0, 1.0, 0.5, 0.5, 34788, 64, 16, 0, 1.0, 1.0, 0.0, 1.0, 0.0, None, "f64")
    rng = np.random.default_rng(1)
    e = rng.normal(size=64)
    js = st.save_stats(str(tmp_path), {"energies": e, "d2energies": np.abs(e)}, 2.0, 16, params=P,
                       measure_history=False)
    assert set(js) == {"energy", "d2energy", "cv"}
    p = json.load(open(os.path.join(tmp_path, "parameters.json")))
    assert p["beta"] == 2.0 and p["L"] == 4 and p["random_seed"] == 34788 and p["dos_npts"] == 240


def test_graph_lattice_loader_matches_hypercubic(st, tmp_path):
    """A 4x5 periodic square lattice written as a graph (coordinates + hopping rows, real and complex
    storage) loads to the same CSR as the hypercubic builder's."""
    from oracle import oracle as O
    L = 4
    rowptr, col, val = O.lattice_csr("cubic2d", L, 1.0)
    n = L * L
    coords = [(i // L, i % L) for i in range(n)]
    rows = [(i, int(col[k]), float(val[k])) for i in range(n) for k in range(rowptr[i], rowptr[i + 1])]
    for dtype in (np.float64, np.complex128):
        d = os.path.join(tmp_path, str(np.dtype(dtype)))
        st.write_graph_lattice(d, [L, L], 1, coords, np.array(rows, dtype=dtype))
        r2, c2, v2 = st.graph_lattice_csr(d)
        assert np.array_equal(r2, rowptr) and np.array_equal(c2, col) and np.array_equal(v2, val)


def test_graph_lattice_rejects_bad_input(st, tmp_path):
    from fk_mc_gb300._lib import FkgError
    d = str(tmp_path)
    st.write_graph_lattice(d, [2], 1, [[0], [1]], np.array([[0, 1, -1.0 + 0.5j], [1, 0, -1.0 - 0.5j]]))
    with pytest.raises(FkgError, match="complex hopping"):
        st.graph_lattice_csr(d)
    st.write_graph_lattice(d, [2], 1, [[0], [1]], np.array([[0, 2, -1.0]]))
    with pytest.raises(FkgError, match="out of range"):
        st.graph_lattice_csr(d)
    st.write_graph_lattice(d, [3], 1, [[0], [1]], np.array([[0, 1, -1.0]]))
    with pytest.raises(FkgError, match="coordinates"):
        st.graph_lattice_csr(d)
