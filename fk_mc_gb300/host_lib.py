"""ctypes binding of libfk_mc_host.so (include/fk_mc_host.h): whole Markov
chains run through the C++ host adapter, i.e. the reference's
configuration_t / move_* / mc_metropolis / measure_energy classes with calc_ed
on the GPU."""
import ctypes
import os

import numpy as np

from . import _lib

HOST_LIB_PATH = os.path.join(_lib.HERE, "_build", "libfk_mc_host.so")
KINDS = {"cubic1d": 1, "cubic2d": 2, "cubic3d": 3, "triangular": 4}
_host = None


class Params(ctypes.Structure):
    _fields_ = [("lattice_kind", ctypes.c_int), ("L", ctypes.c_int), ("t", ctypes.c_double),
                ("tp", ctypes.c_double), ("beta", ctypes.c_double), ("U", ctypes.c_double),
                ("mu_c", ctypes.c_double), ("mu_f", ctypes.c_double), ("seed", ctypes.c_longlong),
                ("nsweeps", ctypes.c_int), ("sweep_len", ctypes.c_int), ("ntherm_sweeps", ctypes.c_int),
                ("mc_flip", ctypes.c_double), ("mc_add_remove", ctypes.c_double), ("mc_reshuffle", ctypes.c_double),
                ("nf_start", ctypes.c_int), ("precision", ctypes.c_int), ("cheb_moves", ctypes.c_int),
                ("cheb_prefactor", ctypes.c_double), ("rank1_moves", ctypes.c_int)]


class Out(ctypes.Structure):
    _fields_ = [("move_index", ctypes.POINTER(ctypes.c_int32)), ("accepted", ctypes.POINTER(ctypes.c_int32)),
                ("weight", ctypes.POINTER(ctypes.c_double)), ("uniform", ctypes.POINTER(ctypes.c_double)),
                ("energy", ctypes.POINTER(ctypes.c_double)), ("d2energy", ctypes.POINTER(ctypes.c_double)),
                ("c_energy", ctypes.POINTER(ctypes.c_double)), ("f_initial", ctypes.POINTER(ctypes.c_int32)),
                ("f_final", ctypes.POINTER(ctypes.c_int32)), ("naccept", ctypes.c_longlong),
                ("nf0", ctypes.POINTER(ctypes.c_double)), ("nfpi", ctypes.POINTER(ctypes.c_double)),
                ("spectrum_history", ctypes.POINTER(ctypes.c_double)),
                ("focc_history", ctypes.POINTER(ctypes.c_int32))]


SIGNATURES = {
    "fkh_run_chain": ([ctypes.POINTER(Params), ctypes.POINTER(Out), ctypes.c_char_p, ctypes.c_int], ctypes.c_int),
    "fkh_run_batched": ([ctypes.POINTER(Params), ctypes.c_int, ctypes.POINTER(Out), ctypes.c_char_p, ctypes.c_int],
                        ctypes.c_int),
    "fkh_measure_eigen": ([ctypes.POINTER(Params), ctypes.POINTER(ctypes.c_int32), ctypes.c_int,
                           ctypes.POINTER(ctypes.c_double), ctypes.c_double, ctypes.POINTER(ctypes.c_double),
                           ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), ctypes.c_char_p,
                           ctypes.c_int], ctypes.c_int),
    "fkh_run_chain_graph": ([ctypes.c_char_p, ctypes.POINTER(Params), ctypes.POINTER(Out), ctypes.c_char_p,
                             ctypes.c_int], ctypes.c_int),
}


def load():
    global _host
    if _host is None:
        _lib.load()  # libfkg.so first
        if not os.path.exists(HOST_LIB_PATH):
            raise _lib.FkgError(f"{HOST_LIB_PATH} is missing: run __graft_entry__.build() first")
        h = ctypes.CDLL(HOST_LIB_PATH)
        for name, (args, res) in SIGNATURES.items():
            getattr(h, name).argtypes = args
            getattr(h, name).restype = res
        _host = h
    return _host


def _params(kind, L, beta, U, mu_c, mu_f, seed, nsweeps, sweep_len, ntherm_sweeps, t, tp, mc_flip, mc_add_remove,
            mc_reshuffle, nf_start, precision, cheb_moves=False, cheb_prefactor=2.2, rank1_moves=False):
    n = L ** {1: 1, 2: 2, 3: 3, 4: 2}[KINDS[kind]]
    return Params(KINDS[kind], L, t, tp, beta, U, mu_c, mu_f, seed, nsweeps, sweep_len, ntherm_sweeps, mc_flip,
                  mc_add_remove, mc_reshuffle, n // 2 if nf_start is None else nf_start, _lib.PREC[precision],
                  int(bool(cheb_moves)), float(cheb_prefactor), int(bool(rank1_moves))), n


def _chain_arrays(n, nprop, nsweeps, history):
    a = {"move_index": np.zeros(nprop, np.int32), "accepted": np.zeros(nprop, np.int32), "weight": np.zeros(nprop),
         "uniform": np.zeros(nprop), "energy": np.zeros(nsweeps), "d2energy": np.zeros(nsweeps),
         "c_energy": np.zeros(nsweeps), "f_initial": np.zeros(n, np.int32), "f_final": np.zeros(n, np.int32),
         "nf0": np.zeros(nsweeps), "nfpi": np.zeros(nsweeps)}
    if history:
        a["spectrum_history"] = np.zeros((n, nsweeps))
        a["focc_history"] = np.zeros((n, nsweeps), np.int32)
    ptr = lambda k: None if k not in a else (_lib.i32(a[k]) if a[k].dtype == np.int32 else _lib.f64(a[k]))
    O = Out(*[ptr(k) for k in ["move_index", "accepted", "weight", "uniform", "energy", "d2energy", "c_energy",
                               "f_initial", "f_final"]], 0,
            *[ptr(k) for k in ["nf0", "nfpi", "spectrum_history", "focc_history"]])
    return a, O


def run_chain(kind, L, beta, U, mu_c, mu_f, seed, nsweeps, sweep_len, ntherm_sweeps=0, t=1.0, tp=1.0,
              mc_flip=0.0, mc_add_remove=1.0, mc_reshuffle=0.0, nf_start=None, precision="f64", history=False,
              cheb_moves=False, cheb_prefactor=2.2, rank1_moves=False):
    """One chain through the adapter: per-proposal records, the energy, n_f(q=0) and n_f(q=pi) series and,
    with history=True, the eigenvalue and f histories (state-major, V x nsweeps). cheb_moves selects the
    Chebyshev moves (then no energy is measured)."""
    P, n = _params(kind, L, beta, U, mu_c, mu_f, seed, nsweeps, sweep_len, ntherm_sweeps, t, tp, mc_flip,
                   mc_add_remove, mc_reshuffle, nf_start, precision, cheb_moves, cheb_prefactor, rank1_moves)
    nprop = (nsweeps + ntherm_sweeps) * sweep_len
    a, O = _chain_arrays(n, nprop, nsweeps, history)
    err = ctypes.create_string_buffer(512)
    rc = load().fkh_run_chain(ctypes.byref(P), ctypes.byref(O), err, 512)
    if rc:
        raise _lib.FkgError(f"fkh_run_chain failed: {err.value.decode()}")
    a["naccept"] = O.naccept
    return a


def run_chain_graph(lattice_dir, n, beta, U, mu_c, mu_f, seed, nsweeps, sweep_len, ntherm_sweeps=0,
                    mc_flip=0.0, mc_add_remove=1.0, mc_reshuffle=0.0, nf_start=None, precision="f64", history=False):
    """run_chain on the graph lattice stored as .npy files in lattice_dir (n sites)."""
    P = Params(2, 0, 0.0, 0.0, beta, U, mu_c, mu_f, seed, nsweeps, sweep_len, ntherm_sweeps, mc_flip, mc_add_remove,
               mc_reshuffle, n // 2 if nf_start is None else nf_start, _lib.PREC[precision], 0, 2.2, 0)
    nprop = (nsweeps + ntherm_sweeps) * sweep_len
    a, O = _chain_arrays(n, nprop, nsweeps, history)
    err = ctypes.create_string_buffer(512)
    rc = load().fkh_run_chain_graph(os.fsencode(lattice_dir), ctypes.byref(P), ctypes.byref(O), err, 512)
    if rc:
        raise _lib.FkgError(f"fkh_run_chain_graph failed: {err.value.decode()}")
    a["naccept"] = O.naccept
    return a


def run_batched(kind, L, beta, U, mu_c, mu_f, seed, batch, nsweeps, sweep_len, ntherm_sweeps=0, t=1.0, tp=1.0,
                nf_start=None, precision="f64", cheb_moves=False, cheb_prefactor=2.2):
    P, n = _params(kind, L, beta, U, mu_c, mu_f, seed, nsweeps, sweep_len, ntherm_sweeps, t, tp, 0.0, 1.0, 0.0,
                   nf_start, precision, cheb_moves, cheb_prefactor)
    nprop = (nsweeps + ntherm_sweeps) * sweep_len
    a = {"accepted": np.zeros((batch, nprop), np.int32), "energy": np.zeros((batch, nsweeps)),
         "d2energy": np.zeros((batch, nsweeps)), "c_energy": np.zeros((batch, nsweeps)),
         "f_initial": np.zeros((batch, n), np.int32), "f_final": np.zeros((batch, n), np.int32)}
    O = Out(None, _lib.i32(a["accepted"]), None, None, _lib.f64(a["energy"]), _lib.f64(a["d2energy"]),
            _lib.f64(a["c_energy"]), _lib.i32(a["f_initial"]), _lib.i32(a["f_final"]), 0, None, None, None, None)
    err = ctypes.create_string_buffer(512)
    rc = load().fkh_run_batched(ctypes.byref(P), batch, ctypes.byref(O), err, 512)
    if rc:
        raise _lib.FkgError(f"fkh_run_batched failed: {err.value.decode()}")
    a["naccept"] = O.naccept
    return a


def measure_eigen(kind, L, f, beta, U, mu_c, wgrid=(), eta=0.1, t=1.0, tp=1.0, precision="f64"):
    """measure_stiffness and measure_ipr of the adapter for configuration f: (stiffness, cond, ipr)."""
    P, n = _params(kind, L, beta, U, mu_c, mu_c, 0, 0, 1, 0, t, tp, 0.0, 1.0, 0.0, None, precision)
    f = _lib.as_i32(f)
    w = _lib.as_f64(wgrid)
    cond = np.zeros(w.size)
    ipr = np.zeros(n)
    st = ctypes.c_double(0)
    err = ctypes.create_string_buffer(512)
    rc = load().fkh_measure_eigen(ctypes.byref(P), _lib.i32(f), w.size, _lib.f64(w) if w.size else None, float(eta),
                                  ctypes.byref(st), _lib.f64(cond) if w.size else None, _lib.f64(ipr), err, 512)
    if rc:
        raise _lib.FkgError(f"fkh_measure_eigen failed: {err.value.decode()}")
    return st.value, cond, ipr
