"""Statistics and output stage of a run through the C++ host adapter
(libfk_mc_host.so, include/fk_mc_host.h): binning and jackknife
(include/fk_mc/binning.hpp, jackknife.hpp of the reference), estimate_bin and
save_all (prog/data_save.hpp, prog/data_save.hxx) writing .npy files in place of
the reference's HDF5 datasets, and the graph-lattice loader
(src/lattice/graph.cpp:52-80) reading .npy files. Nothing here touches the GPU.
"""
import ctypes
import os

import numpy as np

from . import _lib
from . import host_lib

JACK = {"mean": 0, "cv": 1, "disp": 2, "binder": 3, "linear": 4}
_dp = ctypes.POINTER(ctypes.c_double)


class Observables(ctypes.Structure):
    _fields_ = [("n_meas", ctypes.c_longlong), ("volume", ctypes.c_int), ("energies", _dp), ("d2energies", _dp),
                ("c_energies", _dp), ("nf0", _dp), ("nfpi", _dp), ("stiffness", _dp), ("spectrum", _dp),
                ("n_spectrum", ctypes.c_longlong), ("spectrum_history", _dp), ("ipr_history", _dp),
                ("focc_history", _dp), ("cond_history", _dp), ("nw", ctypes.c_int), ("wgrid_cond", _dp)]


class SaveOptions(ctypes.Structure):
    _fields_ = [("beta", ctypes.c_double), ("measure_history", ctypes.c_int), ("measure_ipr", ctypes.c_int),
                ("measure_stiffness", ctypes.c_int), ("dos_npts", ctypes.c_int), ("dos_width", ctypes.c_double),
                ("dos_offset", ctypes.c_double), ("max_bin", ctypes.c_int)]


SIGNATURES = {
    "fkh_binning": ([_dp, ctypes.c_longlong, ctypes.c_int, ctypes.c_int, _dp, ctypes.c_char_p, ctypes.c_int],
                    ctypes.c_int),
    "fkh_estimate_bin": ([_dp, ctypes.c_int, ctypes.c_int], ctypes.c_int),
    "fkh_jackknife": ([ctypes.c_int, ctypes.c_int, ctypes.POINTER(_dp), ctypes.c_longlong, ctypes.c_int, ctypes.c_int,
                       _dp, _dp, ctypes.c_char_p, ctypes.c_int], ctypes.c_int),
    "fkh_save_stats": ([ctypes.c_char_p, ctypes.POINTER(host_lib.Params), ctypes.POINTER(Observables),
                        ctypes.POINTER(SaveOptions), ctypes.c_char_p, ctypes.c_int], ctypes.c_int),
    "fkh_graph_lattice_csr": ([ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                               ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int32),
                               ctypes.POINTER(ctypes.c_int32), _dp, ctypes.c_char_p, ctypes.c_int], ctypes.c_int),
}
_bound = False


def _h():
    global _bound
    h = host_lib.load()
    if not _bound:
        for name, (args, res) in SIGNATURES.items():
            getattr(h, name).argtypes = args
            getattr(h, name).restype = res
        _bound = True
    return h


def _check(rc, err, name):
    if rc < 0:
        raise _lib.FkgError(f"{name} failed: {err.value.decode()}")


def binning(x, max_bin, reverse=False):
    """Rows (number of bins, mean, variance, error, correlation length) for depths 0..max_bin."""
    x = _lib.as_f64(x)
    rows = np.zeros((max_bin + 1, 5))
    err = ctypes.create_string_buffer(512)
    _check(_h().fkh_binning(_lib.f64(x), x.size, int(bool(reverse)), int(max_bin), _lib.f64(rows), err, 512), err,
           "fkh_binning")
    return rows


def estimate_bin(rows):
    """Depth at which the error (column 3) of a binning saturates."""
    r = np.ascontiguousarray(rows, dtype=np.float64)
    return _h().fkh_estimate_bin(_lib.f64(r), r.shape[0], r.shape[1])


def jackknife(func, series, max_bin, reverse=False, fparams=None):
    """Rows (number of bins, estimate, variance, error) of a jackknife of `func`
    ("mean", "cv", "disp", "binder", "linear") over equal-length series, for depths 0..max_bin."""
    ss = [_lib.as_f64(s) for s in series]
    n = ss[0].size
    if any(s.size != n for s in ss):
        raise _lib.FkgError("series of different lengths")
    arr = (_dp * len(ss))(*[_lib.f64(s) for s in ss])
    fp = _lib.as_f64(fparams) if fparams is not None else None
    rows = np.zeros((max_bin + 1, 4))
    err = ctypes.create_string_buffer(512)
    _check(_h().fkh_jackknife(JACK[func], len(ss), arr, n, int(bool(reverse)), int(max_bin),
                              _lib.f64(fp) if fp is not None else None, _lib.f64(rows), err, 512), err,
           "fkh_jackknife")
    return rows


def save_stats(directory, observables, beta, volume, params=None, measure_history=True, measure_ipr=False,
               measure_stiffness=False, dos_npts=240, dos_width=6.0, dos_offset=0.05, max_bin=-1, wgrid_cond=None):
    """Write the reference's output (binning, jackknife, derived quantities) under `directory`.

    observables: dict with any of energies, d2energies, c_energies, nf0, nfpi, stiffness (one value per
    measurement), spectrum, and the state-major histories spectrum_history, ipr_history, focc_history
    (volume x measurements) and cond_history (frequencies x measurements). params: a host_lib.Params or None.
    Returns the parsed stats.json."""
    keep = {}

    def arr(name, shape=None):
        if name not in observables or observables[name] is None:
            return None
        a = np.ascontiguousarray(observables[name], dtype=np.float64)
        if shape is not None and a.shape != shape:
            raise _lib.FkgError(f"{name} has shape {a.shape}, expected {shape}")
        keep[name] = a
        return _lib.f64(a)

    series = [k for k in ("energies", "d2energies", "c_energies", "nf0", "nfpi", "stiffness") if k in observables]
    M = len(observables[series[0]]) if series else 0
    O = Observables()
    O.n_meas, O.volume = M, int(volume)
    for k in ("energies", "d2energies", "c_energies", "nf0", "nfpi", "stiffness"):
        setattr(O, k, arr(k, (M,)))
    O.spectrum = arr("spectrum")
    O.n_spectrum = keep["spectrum"].size if "spectrum" in keep else 0
    for k in ("spectrum_history", "ipr_history", "focc_history"):
        setattr(O, k, arr(k, (int(volume), M)))
    w = _lib.as_f64(wgrid_cond) if wgrid_cond is not None else np.zeros(0)
    O.cond_history = arr("cond_history", (w.size, M))
    O.nw = w.size
    O.wgrid_cond = _lib.f64(w) if w.size else None
    opt = SaveOptions(float(beta), int(measure_history), int(measure_ipr), int(measure_stiffness), int(dos_npts),
                      float(dos_width), float(dos_offset), int(max_bin))
    err = ctypes.create_string_buffer(512)
    os.makedirs(directory, exist_ok=True)
    _check(_h().fkh_save_stats(os.fsencode(directory), ctypes.byref(params) if params is not None else None,
                               ctypes.byref(O), ctypes.byref(opt), err, 512), err, "fkh_save_stats")
    import json
    with open(os.path.join(directory, "stats.json")) as fh:
        return json.load(fh)


def write_graph_lattice(directory, dims, norbitals, coordinates, hopping):
    """Store a graph lattice as the .npy datasets read_lattice_npy reads: dims, norbitals,
    coordinates (sites x ndim), hopping (rows p1, p2, m)."""
    os.makedirs(directory, exist_ok=True)
    np.save(os.path.join(directory, "dims.npy"), np.asarray(dims, dtype=np.int64))
    np.save(os.path.join(directory, "norbitals.npy"), np.asarray(norbitals, dtype=np.int64))
    np.save(os.path.join(directory, "coordinates.npy"), np.asarray(coordinates, dtype=np.int64))
    np.save(os.path.join(directory, "hopping.npy"), np.asarray(hopping))


def graph_lattice_csr(directory):
    """The hopping matrix of a stored graph lattice as CSR (rowptr, col, val), built by the adapter's loader."""
    n, nnz = ctypes.c_int(0), ctypes.c_int(0)
    err = ctypes.create_string_buffer(512)
    h = _h()
    rc = h.fkh_graph_lattice_csr(os.fsencode(directory), 0, 0, ctypes.byref(n), ctypes.byref(nnz), None, None, None,
                                 err, 512)
    _check(rc, err, "fkh_graph_lattice_csr")
    rowptr = np.zeros(n.value + 1, np.int32)
    col = np.zeros(nnz.value, np.int32)
    val = np.zeros(nnz.value)
    rc = h.fkh_graph_lattice_csr(os.fsencode(directory), rowptr.size, col.size, ctypes.byref(n), ctypes.byref(nnz),
                                 _lib.i32(rowptr), _lib.i32(col), _lib.f64(val), err, 512)
    _check(rc, err, "fkh_graph_lattice_csr")
    return rowptr, col, val
