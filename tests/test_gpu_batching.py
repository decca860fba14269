"""The batching form: uneven batches (mixed lattices and sizes in one launch),
the persistent longest-first reduction, CUDA-graph replay of proposal steps,
and the autotuned panel widths. Graph replay and direct launches must give
identical decisions and logZ differences (the same kernels run on the same
data); panel widths only change rounding (|dlogZ| agreement 1e-9)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

C4 = [("cubic2d", 12), ("cubic2d", 16), ("cubic2d", 20), ("cubic2d", 24), ("cubic2d", 32), ("triangular", 12),
      ("triangular", 18), ("triangular", 24)]


def _setup(s, B, seed):
    rng = np.random.default_rng(seed)
    ns = [s.set_lattice(i, k, L) for i, (k, L) in enumerate(C4)]
    ids = np.array([c % 8 for c in range(B)], np.int32)
    U = rng.uniform(0.5, 4.0, B)
    beta = rng.uniform(1.0, 10.0, B)
    f = np.concatenate([rng.integers(0, 2, ns[i]) for i in ids]).astype(np.int32)
    sites = np.stack([[rng.integers(0, ns[i]) for i in ids] for _ in range(4)]).astype(np.int32)
    u = rng.uniform(0, 1, (4, B))
    return ids, U, beta, f, sites, u, ns


@pytest.mark.parametrize("precision", ["f64", "mixed"])
def test_graph_replay_equals_direct_launches(cuda_ok, fkg_lib, precision):
    import fk_mc_gb300
    s = fk_mc_gb300.Solver(max_n=1024, max_batch=64, precision=precision)
    ids, U, beta, f, sites, u, ns = _setup(s, 24, 1)
    res = []
    for graphs in (True, False):
        s.set_graphs(graphs)
        s.chains_init(ids, f, U, U / 2, U / 2, beta)
        acc, dl = s.propose_accept(sites, u)
        fend, logz, _ = s.chains_get()
        res.append((acc, dl, fend, logz))
    assert np.array_equal(res[0][0], res[1][0])
    assert np.array_equal(res[0][1], res[1][1])
    assert np.array_equal(res[0][2], res[1][2])
    s.close()


def test_graph_survives_growing_step_buffers(cuda_ok, fkg_lib):
    """fkg_propose_accept with more steps than before reallocates its step buffers; the captured
    step graph must follow them (a graph replayed on the freed buffers reads stale sites)."""
    import fk_mc_gb300
    L, B = 6, 8
    n = L * L
    rng = np.random.default_rng(3)
    f = rng.integers(0, 2, (B, n)).astype(np.int32)
    site = rng.integers(0, n, (13, B)).astype(np.int32)
    u = rng.random((13, B))
    outs = []
    for graphs in (True, False):
        s = fk_mc_gb300.Solver(max_n=64, max_batch=B)
        try:
            s.set_lattice(0, "cubic2d", L)
            s.set_graphs(graphs)
            s.chains_init(np.zeros(B, np.int32), f.ravel(), 2.0, 1.0, 1.0, 2.0)
            a1, d1 = s.propose_accept(site[:1], u[:1])
            a2, d2 = s.propose_accept(site[1:3], u[1:3])
            a3, d3 = s.propose_accept(site[3:], u[3:])
            outs.append((np.concatenate([a1, a2, a3]), np.concatenate([d1, d2, d3]), s.chains_get()[0]))
        finally:
            s.close()
    assert np.array_equal(outs[0][0], outs[1][0])
    assert np.array_equal(outs[0][1], outs[1][1])
    assert np.array_equal(outs[0][2], outs[1][2])


def test_uneven_c4_batch_against_oracle(cuda_ok, fkg_lib, oracle):
    # the C4 mix (N = 144..1024) in one persistent launch; a sample of chains replayed on the oracle
    import fk_mc_gb300
    s = fk_mc_gb300.Solver(max_n=1024, max_batch=64, precision="mixed")
    ids, U, beta, f, sites, u, ns = _setup(s, 16, 2)
    s.chains_init(ids, f, U, U / 2, U / 2, beta)
    acc, dl = s.propose_accept(sites[:1], u[:1])
    offs = np.concatenate([[0], np.cumsum([ns[i] for i in ids])])
    for c in (0, 3, 4, 6, 12):
        k, L = C4[ids[c]]
        fc = f[offs[c]:offs[c + 1]].copy()
        cur = oracle.calc_ed(k, L, fc, beta[c], U[c], U[c] / 2)
        fc[sites[0, c]] ^= 1
        new = oracle.calc_ed(k, L, fc, beta[c], U[c], U[c] / 2)
        assert abs(dl[0, c] - (new["logZ"] - cur["logZ"])) < 1e-8
    s.close()


def test_panel_width_variants_agree(cuda_ok, fkg_lib, oracle):
    import fk_mc_gb300
    for prec, nvar in (("mixed", 3), ("f64", 2)):
        s = fk_mc_gb300.Solver(max_n=576, max_batch=4, precision=prec, tuning=None)
        n = s.set_lattice(0, "cubic2d", 24)
        f = np.random.default_rng(3).integers(0, 2, (2, n))
        d = (-1.0 + 2.0 * f).ravel()
        ref = [oracle.calc_ed("cubic2d", 24, f[c], 4.0, 2.0, 1.0)["logZ"] for c in range(2)]
        for v in range(nvar):
            s.set_tuning(prec, n, v)
            out = s.eigh_logz([0, 0], d, 4.0)
            assert np.allclose(out["logz"], ref, rtol=1e-10, atol=0)
        s.close()


def test_autotune_table_applies(cuda_ok, fkg_lib, tmp_path):
    import json
    import fk_mc_gb300
    from fk_mc_gb300 import autotune
    p = tmp_path / "t.json"
    json.dump({"entries": [{"precision": "mixed", "n_max": 576, "variant": 2}]}, open(p, "w"))
    s = fk_mc_gb300.Solver(max_n=576, max_batch=2, precision="mixed", tuning=str(p))
    s.set_lattice(0, "cubic2d", 24)
    out = s.eigh_logz([0], np.zeros(576), 2.0)
    assert np.all(np.isfinite(out["evals"]))
    s.close()
