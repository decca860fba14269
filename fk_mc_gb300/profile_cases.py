"""Workloads for profiler captures (ncu) of the library's kernels.

    python -m fk_mc_gb300.profile_cases all [B]        every kernel family once, cubic2d L=24 (N=576), B chains
    python -m fk_mc_gb300.profile_cases reduce [B] [V] one mixed-path solve of B chains (two warm-up solves first)
                                                       with reduction variant V (0..2 panel widths, 3 two-stage)

`all` runs, in order: the plain FP64 solve with eigenvectors (reduction,
tridiagonal eigenvalues, inverse iteration, compact-WY factors,
back-transformation), the mixed-precision solve with eigenvectors, the
stiffness measure with a 64-point conductivity grid, the IPR measure, the
free-energy gradients with the full dF/dH, two proposal steps of
device-resident chains (the step graph, logZ fused with the decision), and the
two-stage mixed solve. Inputs are seeded Bernoulli(0.5) configurations at
U = 2, mu = 1, beta = 4 (the benchmark's physics). Nothing is checked here; the
tests check the results.
"""
import sys

import numpy as np

L, N = 24, 576


def _setup(B, precision):
    from .solver import Solver
    s = Solver(max_n=N, max_batch=B, precision=precision)
    s.set_lattice(0, "cubic2d", L)
    rng = np.random.default_rng(1)
    f = rng.integers(0, 2, (B, N)).astype(np.int32)
    diag = (-1.0 + 2.0 * f).ravel().astype(float)
    return s, rng, f, diag, np.zeros(B, np.int32)


def run_all(B=16):
    s, rng, f, diag, ids = _setup(B, "f64")
    s.set_stiffness_ops(0, "cubic2d", L, 1.0)
    s.eigh_logz(ids, diag, 4.0, vectors=True)
    s.set_precision("mixed")
    s.eigh_logz(ids, diag, 4.0, vectors=True)
    s.measure_stiffness(ids, diag, 4.0, np.linspace(-4, 4, 64), 0.05)
    s.measure_ipr(ids, diag, 4.0)
    s.free_energy_grad(ids, f.ravel(), 2.0, 1.0, 1.0, 4.0, rho=True)
    s.chains_init(ids, f.ravel(), 2.0, 1.0, 1.0, 4.0)
    s.propose_accept(rng.integers(0, N, (2, B)).astype(np.int32), rng.uniform(0, 1, (2, B)))
    for n_max in range(64, 1025, 64):
        s.set_tuning("mixed", n_max, 3)
    s.eigh_logz(ids, diag, 4.0, vectors=True)
    s.close()


def run_reduce(B=256, variant=1):
    s, _, _, diag, ids = _setup(B, "mixed")
    for n_max in range(64, 1025, 64):
        s.set_tuning("mixed", n_max, variant)
    for _ in range(3):
        s.eigh_logz(ids, diag, 4.0)
    s.close()


if __name__ == "__main__":
    what = sys.argv[1] if len(sys.argv) > 1 else "all"
    args = [int(a) for a in sys.argv[2:]]
    {"all": run_all, "reduce": run_reduce}[what](*args)
    print("ok")
