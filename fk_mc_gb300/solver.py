"""Python handle on a libfkg context (include/fkg.h).

`Solver` mirrors the entry points one to one: `eigh_logz` is the batched
configuration_t::calc_ed (src/configuration.cpp:208-246); `chains_init`,
`propose_accept` and `chains_get` run move_addremove proposals and the
Metropolis test of mc_metropolis::update (src/moves.cpp:52-67,
src/mc_metropolis.cpp:34-52) on device-resident chains.
"""
import ctypes

import numpy as np

from . import _lib
from .lattice import hopping_csr


class Solver:
    def __init__(self, max_n=1024, max_batch=256, precision="f64", tuning="default"):
        self.lib = _lib.load()
        self.ctx = self.lib.fkg_create(int(max_n), int(max_batch), 0)
        if not self.ctx:
            raise _lib.FkgError("fkg_create failed (no CUDA device or out of memory)")
        self.sizes = {}
        self.set_precision(precision)
        if tuning:
            from . import autotune
            autotune.apply(self, autotune.DEFAULT_TABLE if tuning == "default" else tuning)

    def close(self):
        if getattr(self, "ctx", None):
            self.lib.fkg_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        _lib.check(self.ctx, rc, what)

    def set_precision(self, precision):
        self._check(self.lib.fkg_set_precision(self.ctx, _lib.PREC[precision]), "fkg_set_precision")
        self.precision = precision

    def set_hopping(self, lattice_id, rowptr, col, val):
        rowptr, col, val = _lib.as_i32(rowptr), _lib.as_i32(col), _lib.as_f64(val)
        n = rowptr.size - 1
        self._check(self.lib.fkg_set_hopping(self.ctx, int(lattice_id), n, _lib.i32(rowptr), _lib.i32(col),
                                             _lib.f64(val)), "fkg_set_hopping")
        self.sizes[int(lattice_id)] = n

    def set_lattice(self, lattice_id, kind, L, t=1.0, tp=1.0):
        n, rp, c, v = hopping_csr(kind, L, t, tp)
        self.set_hopping(lattice_id, rp, c, v)
        return n

    def eigh_logz(self, lattice_ids, diag, beta, exp_fermi=False, vectors=False):
        ids = _lib.as_i32(lattice_ids)
        ns = [self.sizes[int(i)] for i in ids]
        tot = int(sum(ns))
        diag = _lib.as_f64(diag)
        beta = _lib.as_f64(np.broadcast_to(beta, ids.shape))
        if diag.size != tot:
            raise ValueError("diag must hold sum(n_c) entries")
        w = np.zeros(tot)
        ex = np.zeros(tot) if exp_fermi else None
        fe = np.zeros(tot) if exp_fermi else None
        Z = np.zeros(int(sum(n * n for n in ns))) if vectors else None
        logz = np.zeros(ids.size)
        self._check(self.lib.fkg_eigh_logz(self.ctx, ids.size, _lib.i32(ids), _lib.f64(diag), _lib.f64(beta),
                                           _lib.f64(w), _lib.f64(ex), _lib.f64(fe), _lib.f64(Z), _lib.f64(logz)),
                    "fkg_eigh_logz")
        out = {"evals": w, "logz": logz, "n": ns}
        if exp_fermi:
            out["exp"] = ex
            out["fermi"] = fe
        if vectors:
            mats, off = [], 0
            for n in ns:  # column k = eigenvector k (column-major storage)
                mats.append(Z[off:off + n * n].reshape(n, n).T)
                off += n * n
            out["evecs"] = mats
        return out

    def set_chebyshev(self, cheb_size, grid_size):
        """Moments and Lobatto grid points of the Chebyshev-expansion logZ."""
        self._check(self.lib.fkg_set_chebyshev(self.ctx, int(cheb_size), int(grid_size)), "fkg_set_chebyshev")
        self._cheb_m = int(cheb_size) + int(cheb_size) % 2

    def set_method(self, method):
        """"ed" (eigen-solve) or "chebyshev" for device-resident chains."""
        self._check(self.lib.fkg_set_method(self.ctx, _lib.METHOD[method]), "fkg_set_method")

    def chebyshev_logz(self, lattice_ids, diag, beta, moments=False):
        """logZ by the Chebyshev expansion (calc_chebyshev) with the spectral bounds and, optionally, the moments."""
        ids = _lib.as_i32(lattice_ids)
        ns = [self.sizes[int(i)] for i in ids]
        diag = _lib.as_f64(diag)
        beta = _lib.as_f64(np.broadcast_to(beta, ids.shape))
        if diag.size != int(sum(ns)):
            raise ValueError("diag must hold sum(n_c) entries")
        logz, emin, emax = np.zeros(ids.size), np.zeros(ids.size), np.zeros(ids.size)
        steps = np.zeros(ids.size, np.int32)
        mu = None
        if moments:
            mu = np.zeros((ids.size, self._cheb_m)) if getattr(self, "_cheb_m", 0) else None
        self._check(self.lib.fkg_chebyshev_logz(self.ctx, ids.size, _lib.i32(ids), _lib.f64(diag), _lib.f64(beta),
                                                _lib.f64(logz), _lib.f64(emin), _lib.f64(emax),
                                                _lib.f64(mu) if mu is not None else None, _lib.i32(steps)),
                    "fkg_chebyshev_logz")
        out = {"logz": logz, "e_min": emin, "e_max": emax, "lanczos_steps": steps}
        if mu is not None:
            out["moments"] = mu
        return out

    def rank1_logz(self, evals, z, rho, beta, evals_new=False):
        """Proposal logZ by the rank-one update: evals (batch, n) ascending, z (batch, n) rows of the
        eigenvector matrices, rho (batch,) diagonal changes, beta (batch,)."""
        ev = _lib.as_f64(evals)
        zz = _lib.as_f64(z)
        B, n = ev.shape
        r = _lib.as_f64(np.broadcast_to(rho, (B,)))
        b = _lib.as_f64(np.broadcast_to(beta, (B,)))
        logz = np.zeros(B)
        out = np.zeros((B, n)) if evals_new else None
        self._check(self.lib.fkg_rank1_logz(self.ctx, B, n, _lib.f64(ev), _lib.f64(zz), _lib.f64(r), _lib.f64(b),
                                            _lib.f64(logz), _lib.f64(out) if out is not None else None),
                    "fkg_rank1_logz")
        return (logz, out) if evals_new else logz

    def rank1_logz_device(self, batch, n, d_evals, d_z, d_rho, d_beta, d_logz, d_evals_new=0):
        """Device-pointer variant (integers holding CUDA device addresses)."""
        self._check(self.lib.fkg_rank1_logz_device(self.ctx, int(batch), int(n), ctypes.c_void_p(d_evals),
                                                   ctypes.c_void_p(d_z), ctypes.c_void_p(d_rho),
                                                   ctypes.c_void_p(d_beta), ctypes.c_void_p(d_logz),
                                                   ctypes.c_void_p(d_evals_new) if d_evals_new else None),
                    "fkg_rank1_logz_device")

    def free_energy_grad(self, lattice_ids, f, U, mu_c, t, beta, rho=False):
        """F = -logZ/beta per configuration and dF/dU, dF/dt, dF/dmu, dF/dbeta (and rho = dF/dH)."""
        ids = _lib.as_i32(lattice_ids)
        B = ids.size
        bc = lambda x: _lib.as_f64(np.broadcast_to(np.asarray(x, dtype=np.float64), (B,)))
        ns = [self.sizes[int(i)] for i in ids]
        f = _lib.as_i32(f)
        out = {k: np.zeros(B) for k in ("F", "dU", "dt", "dmu", "dbeta")}
        R = np.zeros(int(sum(n * n for n in ns))) if rho else None
        self._check(self.lib.fkg_free_energy_grad(self.ctx, B, _lib.i32(ids), _lib.i32(f), _lib.f64(bc(U)),
                                                  _lib.f64(bc(mu_c)), _lib.f64(bc(t)), _lib.f64(bc(beta)),
                                                  _lib.f64(out["F"]), _lib.f64(out["dU"]), _lib.f64(out["dt"]),
                                                  _lib.f64(out["dmu"]), _lib.f64(out["dbeta"]), _lib.f64(R)),
                    "fkg_free_energy_grad")
        if rho:
            mats, off = [], 0
            for n in ns:
                mats.append(R[off:off + n * n].reshape(n, n).T)
                off += n * n
            out["rho"] = mats
        return out

    def set_stiffness_ops(self, lattice_id, kind, L, t=1.0):
        """Register measure_stiffness's operators for lattice `lattice_id` (after set_lattice)."""
        from .lattice import stiffness_ops
        rp, c, tv, jv = stiffness_ops(kind, L, t)
        rp, c, tv, jv = _lib.as_i32(rp), _lib.as_i32(c), _lib.as_f64(tv), _lib.as_f64(jv)
        self._check(self.lib.fkg_set_stiffness_ops(self.ctx, int(lattice_id), rp.size - 1, _lib.i32(rp), _lib.i32(c),
                                                   _lib.f64(tv), _lib.f64(jv)), "fkg_set_stiffness_ops")

    def measure_ipr(self, lattice_ids, diag, beta):
        """measure_ipr on the GPU: ||x_k||_4 / ||x_k||_2^2 per eigenvector (ascending), one array per chain."""
        ids = _lib.as_i32(lattice_ids)
        ns = [self.sizes[int(i)] for i in ids]
        out = np.zeros(int(sum(ns)))
        self._check(self.lib.fkg_measure_ipr(self.ctx, ids.size, _lib.i32(ids), _lib.f64(_lib.as_f64(diag)),
                                             _lib.f64(_lib.as_f64(np.broadcast_to(beta, ids.shape))), _lib.f64(out)),
                    "fkg_measure_ipr")
        return np.split(out, np.cumsum(ns)[:-1])

    def measure_stiffness(self, lattice_ids, diag, beta, wgrid=None, eta=0.0):
        """measure_stiffness on the GPU: the Drude stiffness per chain, and with a
        frequency grid also the resonant-term sums (batch x len(wgrid))."""
        ids = _lib.as_i32(lattice_ids)
        out = np.zeros(ids.size)
        w = _lib.as_f64(wgrid) if wgrid is not None else None
        nw = 0 if w is None else w.size
        cond = np.zeros((ids.size, nw)) if nw else None
        self._check(self.lib.fkg_measure_stiffness(self.ctx, ids.size, _lib.i32(ids), _lib.f64(_lib.as_f64(diag)),
                                                   _lib.f64(_lib.as_f64(np.broadcast_to(beta, ids.shape))),
                                                   _lib.f64(out), nw, _lib.f64(w), float(eta), _lib.f64(cond)),
                    "fkg_measure_stiffness")
        return (out, cond) if nw else out

    def chains_init(self, lattice_ids, f, U, mu_c, mu_f, beta):
        ids = _lib.as_i32(lattice_ids)
        B = ids.size
        bc = lambda x: _lib.as_f64(np.broadcast_to(np.asarray(x, dtype=np.float64), (B,)))
        f = _lib.as_i32(f)
        self._chain_n = [self.sizes[int(i)] for i in ids]
        self._check(self.lib.fkg_chains_init(self.ctx, B, _lib.i32(ids), _lib.i32(f), _lib.f64(bc(U)),
                                             _lib.f64(bc(mu_c)), _lib.f64(bc(mu_f)), _lib.f64(bc(beta))),
                    "fkg_chains_init")
        self.batch = B

    def propose_accept(self, site, u):
        site = _lib.as_i32(site)
        u = _lib.as_f64(u)
        nsteps = site.size // self.batch
        acc = np.zeros(site.size, np.int32)
        dl = np.zeros(site.size)
        self._check(self.lib.fkg_propose_accept(self.ctx, nsteps, _lib.i32(site), _lib.f64(u), _lib.i32(acc),
                                                _lib.f64(dl)), "fkg_propose_accept")
        return acc.reshape(nsteps, self.batch), dl.reshape(nsteps, self.batch)

    def propose_accept_device(self, nsteps, d_site, d_u, d_acc, d_dlogz):
        """Device-pointer variant (integers holding CUDA device addresses)."""
        self._check(self.lib.fkg_propose_accept_device(self.ctx, int(nsteps), ctypes.c_void_p(d_site),
                                                       ctypes.c_void_p(d_u), ctypes.c_void_p(d_acc),
                                                       ctypes.c_void_p(d_dlogz)), "fkg_propose_accept_device")

    def chains_get(self):
        tot = int(sum(self._chain_n))
        f = np.zeros(tot, np.int32)
        w = np.zeros(tot)
        logz = np.zeros(self.batch)
        self._check(self.lib.fkg_chains_get(self.ctx, _lib.i32(f), _lib.f64(logz), _lib.f64(w)), "fkg_chains_get")
        return f, logz, w

    def launch_count(self):
        return int(self.lib.fkg_launch_count(self.ctx))

    def set_stream(self, stream_handle):
        """Enqueue on a caller-owned cudaStream_t (int handle, e.g. torch.cuda.Stream.cuda_stream)."""
        self._check(self.lib.fkg_set_stream(self.ctx, ctypes.c_void_p(stream_handle or None)), "fkg_set_stream")

    def set_tuning(self, precision, n_max, variant):
        self._check(self.lib.fkg_set_tuning(self.ctx, _lib.PREC[precision], int(n_max), int(variant)), "fkg_set_tuning")

    def set_tuning_back(self, n_max, variant):
        """Back-transformation kernel of the mixed path for orders up to n_max: 0 mma.sync, 1 tcgen05, -1 default."""
        self._check(self.lib.fkg_set_tuning_back(self.ctx, int(n_max), int(variant)), "fkg_set_tuning_back")

    def set_wait_limit(self, iters=-1):
        """Checks before a tcgen05 main-loop mbarrier wait gives up (-1: the default; 0: at once)."""
        self._check(self.lib.fkg_set_wait_limit(self.ctx, int(iters)), "fkg_set_wait_limit")

    def set_graphs(self, enable=True):
        self._check(self.lib.fkg_set_graphs(self.ctx, int(enable)), "fkg_set_graphs")

    def profile(self, enable=True):
        self._check(self.lib.fkg_profile(self.ctx, int(enable)), "fkg_profile")

    def stage_time(self, stage):
        ms = ctypes.c_double(0)
        n = ctypes.c_longlong(0)
        self._check(self.lib.fkg_stage_time(self.ctx, _lib.STAGES[stage], ctypes.byref(ms), ctypes.byref(n)),
                    "fkg_stage_time")
        return ms.value, n.value
