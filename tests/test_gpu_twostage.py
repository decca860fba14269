"""The two-stage reduction of the mixed path (twostage.cu; reduction variant 3):
dense -> band 16 by panel QR and tensor-core rank-2k updates, band ->
tridiagonal by bulge chasing, eigenvectors through both stages' reflectors,
refinement and compensated logZ as on the one-stage path. Against the FP64 CPU
oracle.

Tolerances (those of the mixed path): eigenvalues |dlambda| <= 1e-9 ||H||_2,
free energy F = -logZ/beta relative error < 1e-9, eigenvector residual
||H X - X Lambda|| <= 1e-5 ||H||, orthogonality |X^T X - I| <= 1e-3 (FP32
eigenvectors: members of near-clusters just above the cluster fix-up's
tolerance, 1e-5 ||T||, keep eps32 ||T|| / gap, seen up to 4e-4 at N = 1024),
dlogZ of a proposal to 1e-8 absolute; graph replays equal direct launches bit
for bit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
NDIM = {"cubic1d": 1, "cubic2d": 2, "cubic3d": 3, "triangular": 2}
TWO_STAGE = 3


def _two_stage(s):
    for n_max in range(64, 1025, 64):
        s.set_tuning("mixed", n_max, TWO_STAGE)


@pytest.fixture(scope="module")
def solver(cuda_ok, fkg_lib):
    import fk_mc_gb300
    s = fk_mc_gb300.Solver(max_n=1024, max_batch=16, precision="mixed")
    _two_stage(s)
    yield s
    s.close()


@pytest.mark.parametrize("kind,L,U,beta", [("cubic1d", 3, 1.0, 1.0), ("cubic2d", 4, 1.0, 1.0),
                                           ("cubic1d", 17, 2.0, 3.0), ("cubic1d", 19, 2.0, 3.0),
                                           ("cubic2d", 8, 1.0, 1.0), ("cubic2d", 16, 2.0, 5.0),
                                           ("triangular", 12, 3.0, 5.0), ("cubic2d", 24, 2.0, 4.0),
                                           ("cubic3d", 8, 2.0, 5.0), ("triangular", 18, 3.0, 10.0),
                                           ("cubic2d", 32, 0.5, 1.0)])
def test_two_stage_matches_oracle(solver, oracle, kind, L, U, beta):
    from fk_mc_gb300.lattice import dense
    solver.set_lattice(0, kind, L)
    n = L ** NDIM[kind]
    rng = np.random.default_rng(L + 7)
    B = 2
    f = rng.integers(0, 2, (B, n))
    out = solver.eigh_logz(np.zeros(B, np.int32), (-U / 2 + U * f).ravel(), beta, vectors=True)
    for c in range(B):
        ref = oracle.calc_ed(kind, L, f[c], beta, U, U / 2)
        w = out["evals"][c * n:(c + 1) * n]
        hn = np.abs(ref["spectrum"]).max()
        assert np.all(np.diff(w) >= 0)
        el = np.abs(w - ref["spectrum"]).max() / hn
        eF = abs(out["logz"][c] - ref["logZ"]) / abs(ref["logZ"])
        X = out["evecs"][c]
        H = dense(kind, L) + np.diag(-U / 2 + U * f[c])
        res = np.abs(H @ X - X * w).max() / hn
        orth = np.abs(X.T @ X - np.eye(n)).max()
        print(f"{kind} L={L} chain {c}: |dlambda|/||H|| {el:.2e}, |dF|/|F| {eF:.2e}, residual {res:.2e}, "
              f"orthogonality {orth:.2e}")
        assert el <= 1e-9 and eF < 1e-9
        assert res <= 1e-5 and orth <= 1e-3


def test_two_stage_uneven_batch(solver, oracle):
    lat = [("cubic2d", 12), ("cubic2d", 20), ("triangular", 12), ("triangular", 24), ("cubic1d", 10)]
    for i, (k, L) in enumerate(lat):
        solver.set_lattice(i, k, L)
    rng = np.random.default_rng(19)
    ids, diags, refs, betas = [], [], [], []
    for c in range(10):
        i = c % len(lat)
        k, L = lat[i]
        n = L ** NDIM[k]
        U, beta = rng.uniform(0.5, 4), rng.uniform(1, 10)
        f = rng.integers(0, 2, n)
        ids.append(i)
        betas.append(beta)
        diags.append(-U / 2 + U * f)
        refs.append(oracle.calc_ed(k, L, f, beta, U, U / 2))
    out = solver.eigh_logz(np.array(ids), np.concatenate(diags), np.array(betas))
    off = 0
    for c, ref in enumerate(refs):
        n = ref["spectrum"].size
        assert np.abs(out["evals"][off:off + n] - ref["spectrum"]).max() <= 1e-9 * np.abs(ref["spectrum"]).max()
        assert abs(out["logz"][c] - ref["logZ"]) < 1e-9 * abs(ref["logZ"])
        off += n


def test_two_stage_chain_decisions_and_graph_replay(cuda_ok, fkg_lib, oracle):
    import fk_mc_gb300
    L, n, B, steps, U, beta = 16, 256, 12, 3, 2.0, 5.0
    rng = np.random.default_rng(23)
    f0 = rng.integers(0, 2, (B, n)).astype(np.int32)
    site = rng.integers(0, n, (steps, B)).astype(np.int32)
    u = rng.uniform(0, 1, (steps, B))
    res = []
    for graphs in (True, False):
        s = fk_mc_gb300.Solver(max_n=n, max_batch=B, precision="mixed")
        try:
            _two_stage(s)
            s.set_lattice(0, "cubic2d", L)
            s.set_graphs(graphs)
            s.chains_init(np.zeros(B, np.int32), f0.ravel(), U, U / 2, U / 2, beta)
            acc, dl = s.propose_accept(site, u)
            fend, logz, _ = s.chains_get()
            res.append((acc, dl, fend, logz))
        finally:
            s.close()
    for a, b in zip(res[0], res[1]):
        assert np.array_equal(a, b), "graph replay differs from direct launches"
    acc, dl = res[0][0], res[0][1]
    for c in range(B):
        f = f0[c].copy()
        cur = oracle.calc_ed("cubic2d", L, f, beta, U, U / 2)
        for st in range(steps):
            fn = f.copy()
            fn[site[st, c]] ^= 1
            new = oracle.calc_ed("cubic2d", L, fn, beta, U, U / 2)
            dlog = new["logZ"] - cur["logZ"]
            assert abs(dl[st, c] - dlog) < 1e-8
            wgt = np.exp(dlog) * (np.exp(beta * U / 2) if fn[site[st, c]] else np.exp(-beta * U / 2))
            if abs(wgt - u[st, c]) <= 1e-8 * wgt:
                print(f"near-tie chain {c} step {st}: |w - u| = {abs(wgt - u[st, c]):.3e}")
            else:
                assert acc[st, c] == (wgt > u[st, c])
            if acc[st, c]:
                f, cur = fn, new


def test_default_table_takes_two_stage_only_for_uniform_batches(cuda_ok, fkg_lib):
    """With the shipped tuning table, the two-stage reduction runs for a batch whose every chain's size selects
    it, and a batch that also holds a smaller chain keeps the one-stage kernel: a two-stage solve launches two
    kernels more (dense -> band and band -> tridiagonal instead of one reduction, and the band stage's
    back-transformation)."""
    import json
    import fk_mc_gb300
    from fk_mc_gb300 import autotune
    table = json.load(open(autotune.DEFAULT_TABLE))
    two_stage_n = [e["n_max"] for e in table["entries"]
                   if e.get("precision") == "mixed" and e["variant"] == TWO_STAGE]
    if 1024 not in two_stage_n:
        pytest.skip("the shipped table does not select the two-stage reduction at n = 1024")
    s = fk_mc_gb300.Solver(max_n=1024, max_batch=2, precision="mixed")
    try:
        s.set_graphs(False)
        s.set_lattice(0, "cubic2d", 32)  # n = 1024
        s.set_lattice(1, "cubic2d", 12)  # n = 144
        rng = np.random.default_rng(5)
        launches = {}
        for name, ids in (("uniform", [0, 0]), ("mixed sizes", [0, 1])):
            diag = np.concatenate([rng.uniform(-1, 1, 1024 if i == 0 else 144) for i in ids])
            s.eigh_logz(np.array(ids, np.int32), diag, 4.0)  # warm
            n0 = s.launch_count()
            s.eigh_logz(np.array(ids, np.int32), diag, 4.0)
            launches[name] = s.launch_count() - n0
        assert launches["uniform"] == launches["mixed sizes"] + 2, launches
    finally:
        s.close()
