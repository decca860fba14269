"""ctypes wrapper around the CPU oracle (oracle/fk_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as the
checker, and by bench.py's CPU-baseline legs. The product package
(fk_mc_gb300) never imports this module.
"""
import ctypes
import os

import numpy as np

from . import build_oracle

_lib = None

KIND = {"cubic1d": 1, "cubic2d": 2, "cubic3d": 3, "triangular": 4}


class McParams(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int), ("L", ctypes.c_int),
        ("t", ctypes.c_double), ("tp", ctypes.c_double),
        ("beta", ctypes.c_double), ("U", ctypes.c_double),
        ("mu_c", ctypes.c_double), ("mu_f", ctypes.c_double),
        ("seed", ctypes.c_longlong),
        ("nsweeps", ctypes.c_int), ("sweep_len", ctypes.c_int), ("ntherm_sweeps", ctypes.c_int),
        ("mc_flip", ctypes.c_double), ("mc_add_remove", ctypes.c_double), ("mc_reshuffle", ctypes.c_double),
        ("nf_start", ctypes.c_int),
        ("f_init", ctypes.POINTER(ctypes.c_int)),
        ("cheb_moves", ctypes.c_int), ("cheb_prefactor", ctypes.c_double),
    ]


class McOut(ctypes.Structure):
    _fields_ = [
        ("move_index", ctypes.POINTER(ctypes.c_int)), ("accepted", ctypes.POINTER(ctypes.c_int)),
        ("site", ctypes.POINTER(ctypes.c_int)),
        ("weight", ctypes.POINTER(ctypes.c_double)), ("uniform", ctypes.POINTER(ctypes.c_double)),
        ("energy", ctypes.POINTER(ctypes.c_double)), ("d2energy", ctypes.POINTER(ctypes.c_double)),
        ("c_energy", ctypes.POINTER(ctypes.c_double)),
        ("f_final", ctypes.POINTER(ctypes.c_int)),
        ("f_initial", ctypes.POINTER(ctypes.c_int)),
        ("naccept", ctypes.c_longlong),
    ]


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = ctypes.CDLL(path)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        L.orc_lattice_csr.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ip, ip, ip, dp]
        L.orc_lattice_csr.restype = ctypes.c_int
        L.orc_eigh.argtypes = [ctypes.c_int, dp, dp, dp]
        L.orc_eigh.restype = ctypes.c_int
        L.orc_tridiag.argtypes = [ctypes.c_int, dp, dp, dp]
        L.orc_tridiag.restype = ctypes.c_int
        L.orc_calc_ed.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ip,
                                  ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                  dp, dp, dp, dp, dp]
        L.orc_calc_ed.restype = ctypes.c_int
        L.orc_logz_of_spectrum.argtypes = [ctypes.c_int, dp, ctypes.c_double]
        L.orc_logz_of_spectrum.restype = ctypes.c_double
        L.orc_stiffness.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, ip]
        L.orc_stiffness.restype = ctypes.c_double
        L.orc_ipr.argtypes = [ctypes.c_int, dp, dp]
        L.orc_ipr.restype = None
        L.orc_mc_run.argtypes = [ctypes.POINTER(McParams), ctypes.POINTER(McOut)]
        L.orc_mc_run.restype = ctypes.c_int
        L.orc_bench_proposals.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                          ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                          ctypes.c_longlong, ctypes.c_int, ctypes.c_double, ctypes.c_int, dp]
        L.orc_bench_proposals.restype = ctypes.c_longlong
        L.orc_bench_steps.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                      ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                      ctypes.c_longlong, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp]
        L.orc_bench_steps.restype = ctypes.c_longlong
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def lattice_csr(kind, L, t=1.0, tp=1.0):
    """Hopping matrix of fill_nearest_neighbors / fill_triangular as CSR."""
    k = KIND[kind] if isinstance(kind, str) else int(kind)
    n = ctypes.c_int(0)
    nnz = lib().orc_lattice_csr(k, L, t, tp, ctypes.byref(n), None, None, None)
    if nnz < 0:
        raise ValueError("bad lattice")
    rowptr = np.zeros(n.value + 1, np.int32)
    col = np.zeros(nnz, np.int32)
    val = np.zeros(nnz, np.float64)
    lib().orc_lattice_csr(k, L, t, tp, None, _ip(rowptr), _ip(col), _dp(val))
    return rowptr, col, val


def dense_hopping(kind, L, t=1.0, tp=1.0):
    rowptr, col, val = lattice_csr(kind, L, t, tp)
    n = len(rowptr) - 1
    H = np.zeros((n, n))
    for i in range(n):
        for p in range(rowptr[i], rowptr[i + 1]):
            H[i, col[p]] += val[p]
    return H


def eigh(A, vectors=False):
    A = np.asfortranarray(A, dtype=np.float64)
    n = A.shape[0]
    w = np.zeros(n)
    Z = np.zeros((n, n), order="F") if vectors else None
    rc = lib().orc_eigh(n, _dp(A), _dp(w), _dp(Z) if vectors else None)
    if rc:
        raise RuntimeError("oracle eigensolver failed")
    return (w, Z) if vectors else w


def tridiag(A):
    A = np.asfortranarray(A, dtype=np.float64)
    n = A.shape[0]
    d = np.zeros(n)
    e = np.zeros(max(n - 1, 1))
    lib().orc_tridiag(n, _dp(A), _dp(d), _dp(e))
    return d, e[: n - 1]


def calc_ed(kind, L, f, beta, U, mu_c, t=1.0, tp=1.0, vectors=False):
    """configuration_t::calc_hamiltonian + calc_ed; returns a dict of ed_cache fields."""
    k = KIND[kind] if isinstance(kind, str) else int(kind)
    f = np.ascontiguousarray(f, dtype=np.int32)
    n = f.size
    spec, ex, fe = np.zeros(n), np.zeros(n), np.zeros(n)
    Z = np.zeros((n, n), order="F") if vectors else None
    logz = ctypes.c_double(0)
    rc = lib().orc_calc_ed(k, L, t, tp, _ip(f), beta, U, mu_c, int(vectors), _dp(spec), _dp(ex), _dp(fe),
                           _dp(Z) if vectors else None, ctypes.byref(logz))
    if rc:
        raise RuntimeError("oracle calc_ed failed")
    out = {"spectrum": spec, "exp": ex, "fermi": fe, "logZ": logz.value}
    if vectors:
        out["evecs"] = Z
    return out


def logz_of_spectrum(spec, beta):
    spec = np.ascontiguousarray(spec, dtype=np.float64)
    return lib().orc_logz_of_spectrum(spec.size, _dp(spec), beta)


def stiffness(L, t, U, beta, f):
    f = np.ascontiguousarray(f, dtype=np.int32)
    return lib().orc_stiffness(L, t, U, beta, _ip(f))


def ipr(X):
    X = np.asfortranarray(X, dtype=np.float64)
    out = np.zeros(X.shape[1])
    lib().orc_ipr(X.shape[0], _dp(X), _dp(out))
    return out


def mc_run(kind, L, beta, U, mu_c, mu_f, seed, nsweeps, sweep_len, ntherm_sweeps=0, t=1.0, tp=1.0,
           mc_flip=0.0, mc_add_remove=1.0, mc_reshuffle=0.0, nf_start=None, f_init=None, cheb_moves=False,
           cheb_prefactor=2.2):
    """One chain driven like fk_mc::initialize + mcbase::run. Returns a dict of arrays. With
    cheb_moves the Chebyshev moves run (and, as in the reference, no energy is measured)."""
    k = KIND[kind] if isinstance(kind, str) else int(kind)
    n_sites = L ** (2 if k == 4 else k)
    nprop = (nsweeps + ntherm_sweeps) * sweep_len
    arrs = {
        "move_index": np.zeros(nprop, np.int32), "accepted": np.zeros(nprop, np.int32),
        "site": np.zeros(nprop, np.int32), "weight": np.zeros(nprop), "uniform": np.zeros(nprop),
        "energy": np.zeros(nsweeps), "d2energy": np.zeros(nsweeps), "c_energy": np.zeros(nsweeps),
        "f_final": np.zeros(n_sites, np.int32), "f_initial": np.zeros(n_sites, np.int32),
    }
    fi = None
    if f_init is not None:
        fi = np.ascontiguousarray(f_init, dtype=np.int32)
    P = McParams(k, L, t, tp, beta, U, mu_c, mu_f, seed, nsweeps, sweep_len, ntherm_sweeps,
                 mc_flip, mc_add_remove, mc_reshuffle,
                 -1 if f_init is not None else (n_sites // 2 if nf_start is None else nf_start),
                 _ip(fi) if fi is not None else None, int(bool(cheb_moves)), float(cheb_prefactor))
    O = McOut(*[(_ip(arrs[nm]) if arrs[nm].dtype == np.int32 else _dp(arrs[nm])) for nm in
                ["move_index", "accepted", "site", "weight", "uniform", "energy", "d2energy", "c_energy",
                 "f_final", "f_initial"]], 0)
    rc = lib().orc_mc_run(ctypes.byref(P), ctypes.byref(O))
    if rc:
        raise RuntimeError(f"oracle mc_run failed ({rc})")
    arrs["naccept"] = O.naccept
    return arrs


def bench_proposals(kind, L, beta, U, mu_c, mu_f, seed, threads, seconds, max_props_per_thread=1 << 30,
                    t=1.0, tp=1.0):
    k = KIND[kind] if isinstance(kind, str) else int(kind)
    el = ctypes.c_double(0)
    n = lib().orc_bench_proposals(k, L, t, tp, beta, U, mu_c, mu_f, seed, threads, seconds,
                                  max_props_per_thread, ctypes.byref(el))
    return n, el.value


def bench_steps(kind, L, beta, U, mu_c, mu_f, seed, threads, warmup, steps, t=1.0, tp=1.0):
    """Steady-state timing of `threads` running chains: `warmup` untimed
    proposals each (the first also solves the starting configuration), then
    `steps` timed proposals each from a common start line. Returns
    (timed proposals, seconds)."""
    k = KIND[kind] if isinstance(kind, str) else int(kind)
    el = ctypes.c_double(0)
    n = lib().orc_bench_steps(k, L, t, tp, beta, U, mu_c, mu_f, seed, threads, warmup, steps, ctypes.byref(el))
    return n, el.value
