"""Lattice hopping matrices, as the reference's lattice classes build them.

hypercubic_lattice<D> numbers sites with the last coordinate fastest
(src/lattice/hypercubic.cpp:30-51); fill_nearest_neighbors puts -t on the two
periodic neighbours along every axis (src/lattice/hypercubic.cpp:115-131);
fill_triangular adds -tp on the (-1,-1) and (+1,+1) diagonal neighbours
(src/lattice/hypercubic.cpp:137-155). The result is returned as CSR with
sorted columns; entries that coincide (only possible for L <= 2) are summed.
"""
import numpy as np

KINDS = {"cubic1d": (1, False), "cubic2d": (2, False), "cubic3d": (3, False), "triangular": (2, True)}


def index_to_pos(index, D, L):
    pos = np.zeros((np.size(index), D), dtype=np.int64)
    idx = np.array(index, dtype=np.int64).reshape(-1)
    for i in range(D - 1, -1, -1):
        pos[:, i] = idx % L
        idx = idx // L
    return pos


def pos_to_index(pos, L):
    D = pos.shape[1]
    out = np.zeros(pos.shape[0], dtype=np.int64)
    mult = 1
    for i in range(D - 1, -1, -1):
        out += pos[:, i] * mult
        mult *= L
    return out


def hopping_csr(kind, L, t=1.0, tp=1.0):
    """(n, rowptr, col, val) of the hopping matrix of lattice `kind` with side L."""
    D, tri = KINDS[kind]
    V = L ** D
    sites = np.arange(V)
    pos = index_to_pos(sites, D, L)
    rows, cols, vals = [], [], []
    for n in range(D):
        for step in (-1, 1):
            p = pos.copy()
            p[:, n] = (p[:, n] + step) % L
            rows.append(sites)
            cols.append(pos_to_index(p, L))
            vals.append(np.full(V, -t))
    if tri:
        for step in (-1, 1):
            p = (pos + step) % L
            rows.append(sites)
            cols.append(pos_to_index(p, L))
            vals.append(np.full(V, -tp))
    r = np.concatenate(rows)
    c = np.concatenate(cols)
    v = np.concatenate(vals)
    key = r * V + c
    uk, inv = np.unique(key, return_inverse=True)
    sv = np.zeros(uk.size)
    np.add.at(sv, inv, v)
    ur, uc = uk // V, uk % V
    rowptr = np.zeros(V + 1, dtype=np.int32)
    np.add.at(rowptr, ur + 1, 1)
    rowptr = np.cumsum(rowptr).astype(np.int32)
    return V, rowptr, uc.astype(np.int32), sv


def stiffness_ops(kind, L, t=1.0):
    """(rowptr, col, tval, jval): measure_stiffness's kinetic and current
    operators along axis 0 (include/fk_mc/measures/stiffness.hpp:70-125):
    Tm(i, left) = Tm(i, right) = -t, Jm(i, left) = -1, Jm(i, right) = +1 for the
    periodic neighbours along the first axis; coinciding entries are summed."""
    D, _ = KINDS[kind]
    V = L ** D
    sites = np.arange(V)
    pos = index_to_pos(sites, D, L)
    rows, cols, tv, jv = [], [], [], []
    for step, jsign in ((-1, -1.0), (1, 1.0)):
        p = pos.copy()
        p[:, 0] = (p[:, 0] + step) % L
        rows.append(sites)
        cols.append(pos_to_index(p, L))
        tv.append(np.full(V, -t))
        jv.append(np.full(V, jsign))
    r = np.concatenate(rows)
    c = np.concatenate(cols)
    key = r * V + c
    uk, inv = np.unique(key, return_inverse=True)
    st, sj = np.zeros(uk.size), np.zeros(uk.size)
    np.add.at(st, inv, np.concatenate(tv))
    np.add.at(sj, inv, np.concatenate(jv))
    ur, uc = uk // V, uk % V
    rowptr = np.zeros(V + 1, dtype=np.int32)
    np.add.at(rowptr, ur + 1, 1)
    rowptr = np.cumsum(rowptr).astype(np.int32)
    return rowptr, uc.astype(np.int32), st, sj


def dense(kind, L, t=1.0, tp=1.0):
    n, rp, c, v = hopping_csr(kind, L, t, tp)
    H = np.zeros((n, n))
    for i in range(n):
        H[i, c[rp[i]:rp[i + 1]]] += v[rp[i]:rp[i + 1]]
    return H
