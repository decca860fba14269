"""measure_stiffness's operators (include/fk_mc/measures/stiffness.hpp:70-125)
as fk_mc_gb300.lattice.stiffness_ops builds them: Tm(i, left) = Tm(i, right)
= -t, Jm(i, left) = -1, Jm(i, right) = +1 along axis 0, periodic, duplicates
summed; Jm antisymmetric (the GPU measure relies on it)."""
import numpy as np
import pytest

from fk_mc_gb300.lattice import index_to_pos, pos_to_index, stiffness_ops


@pytest.mark.parametrize("kind,L,D", [("cubic2d", 5, 2), ("cubic2d", 2, 2), ("cubic3d", 3, 3), ("triangular", 4, 2)])
def test_stiffness_ops_match_reference_construction(kind, L, D):
    n = L ** D
    rp, c, tv, jv = stiffness_ops(kind, L, 1.0)
    T, J = np.zeros((n, n)), np.zeros((n, n))
    for i in range(n):
        for p in range(rp[i], rp[i + 1]):
            T[i, c[p]] += tv[p]
            J[i, c[p]] += jv[p]
    Tr, Jr = np.zeros((n, n)), np.zeros((n, n))
    for i in range(n):
        pos = index_to_pos(i, D, L)[0]
        pl, pr = pos.copy(), pos.copy()
        pl[0] = (pos[0] - 1 + L) % L
        pr[0] = (pos[0] + 1 + L) % L
        il, ir = pos_to_index(pl[None], L)[0], pos_to_index(pr[None], L)[0]
        Tr[i, il] += -1.0
        Tr[i, ir] += -1.0
        Jr[i, il] += -1.0
        Jr[i, ir] += 1.0
    assert np.array_equal(T, Tr) and np.array_equal(J, Jr)
    assert np.array_equal(J, -J.T)
