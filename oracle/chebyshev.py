"""Oracle (test infrastructure only): numpy restatement of the reference's
Chebyshev-expansion logZ, configuration_t::calc_chebyshev
(src/configuration.cpp:94-205), and of chebyshev::chebyshev_eval
(include/fk_mc/chebyshev.hpp:16-66), used to check the GPU path
(fk_mc_gb300/csrc/chebyshev.cu). Pinned against the moment_f known answers of
the reference's test/fast_update_test.cpp:62-65 (tests/golden/reference_kats.json)
and, for the moments, against the identity Tr T_m(x) = sum_k T_m(x_k) over the
eigenvalues of x.

The reference takes the spectral bounds from ARPACK's converged extreme
eigenvalues; here they are the extreme eigenvalues of numpy's dense eigvalsh.
"""
import math

import numpy as np


class ChebyshevEval:
    """include/fk_mc/chebyshev.hpp:16-66: Lobatto grid x_i = -cos(pi theta_i) on
    theta_i = i/(G-1), T_k(x_i) = cos(k acos(x_i)), moment() = trapezoid rule in
    theta of f(x) T_k(x)."""

    def __init__(self, max_moment, grid_size):
        self.M = max_moment + max_moment % 2
        self.G = grid_size
        step = 1.0 / (grid_size - 1)
        self.theta = [i * step for i in range(grid_size)]
        self.x = [-math.cos(math.pi * t) for t in self.theta]
        self.T = [[math.cos(k * math.acos(x)) for x in self.x] for k in range(self.M)]

    def moment(self, vals, order):
        s = 0.0
        for i in range(self.G - 1):
            s += (vals[i + 1] * self.T[order][i + 1] + vals[i] * self.T[order][i]) * (self.theta[i + 1] - self.theta[i])
        return s * 0.5

    def moment_f(self, f, order):
        return self.moment([f(x) for x in self.x], order)


def moments(x, M):
    """Tr T_m(x)/N for m < M in the reference's order (src/configuration.cpp:124-183):
    the recursion for m <= M/2 unless already set, T_{2m-1} and T_{2m} from the
    products T_{m-1} T_m and T_m^2 once 2m-1 >= M/2."""
    N = x.shape[0]
    mu = [None] * M
    mu[0] = 1.0
    c0 = np.eye(N)
    c1 = x.copy()
    mu[1] = np.trace(c1) / N
    trx = np.trace(x)
    for m in range(2, M // 2 + 1):
        c0, c1 = c1, 2.0 * x @ c1 - c0
        if mu[m] is None:
            mu[m] = np.trace(c1) / N
        k = 2 * m - 1
        if M // 2 <= k < M:
            mu[k] = (np.sum(c0 * c1) * 2. - trx) / N       # Tr(T_{m-1} T_m), both symmetric
            if k != M - 1:
                mu[k + 1] = np.sum(c1 * c1) / N * 2. - 1.0
    return np.array(mu, dtype=float)


def calc_chebyshev(H, beta, cheb_size, grid_size):
    """logZ of the dense symmetric H by the Chebyshev expansion: dict with
    logZ, e_min, e_max, a, b, moments."""
    ev = np.linalg.eigvalsh(H)
    e_min, e_max = float(ev[0]), float(ev[-1])
    a = (e_max - e_min) / 2.
    b = (e_max + e_min) / 2.
    N = H.shape[0]
    x = (H - b * np.eye(N)) / a
    ch = ChebyshevEval(cheb_size, grid_size)
    mu = moments(x, ch.M)
    f = lambda w: N * math.log(1. + math.exp(-beta * (a * w + b)))
    s = ch.moment_f(f, 0)
    for m in range(1, ch.M):
        s += 2. * ch.moment_f(f, m) * mu[m]
    return {"logZ": s, "e_min": e_min, "e_max": e_max, "a": a, "b": b, "moments": mu}


def dense_h(csr, f, U, mu_c):
    """H = hopping + diag(-mu_c + U f) from a CSR triple (src/configuration.cpp:79-91)."""
    rowptr, col, val = csr
    n = len(rowptr) - 1
    H = np.zeros((n, n))
    for i in range(n):
        for p in range(rowptr[i], rowptr[i + 1]):
            H[i, col[p]] += val[p]
    H[np.diag_indices(n)] += -mu_c + U * np.asarray(f, dtype=float)
    return H
