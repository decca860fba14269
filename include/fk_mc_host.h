/*
 * fk_mc_host.h — C entry points of the C++ host adapter (libfk_mc_host.so):
 * whole Markov-chain runs through the reference's classes, as the reference's
 * driver runs them (fk_mc<L>::initialize, include/fk_mc/fk_mc.hxx:35-125, and
 * mc.run, prog/fk_mc_exec.cpp:151), with every calc_ed on the GPU. They exist
 * so that non-C++ callers (and the tests) can drive the adapter.
 */
#ifndef FK_MC_HOST_H
#define FK_MC_HOST_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Model and Monte Carlo parameters (fk_mc::define_parameters,
 * include/fk_mc/fk_mc.hxx:177-207; mc_metropolis::define_parameters,
 * src/mc_metropolis.cpp:11-19). lattice_kind: 1,2,3 = cubic1d/2d/3d,
 * 4 = triangular (t, tp as fill_nearest_neighbors / fill_triangular). */
typedef struct fkh_params {
    int lattice_kind, L;
    double t, tp;
    double beta, U, mu_c, mu_f;
    long long seed;
    int nsweeps, sweep_len, ntherm_sweeps;
    double mc_flip, mc_add_remove, mc_reshuffle;
    int nf_start;
    int precision; /* FKG_PREC_F64 or FKG_PREC_MIXED */
    /* the Chebyshev moves (include/fk_mc/fk_mc.hxx:55-78): logZ by the
     * Chebyshev expansion with cheb_size = int(log(V) * cheb_prefactor)
     * (even) moments on max(2 cheb_size, 10) grid points; no energy is then
     * measured, as in the reference (fk_mc.hxx:94-114). */
    int cheb_moves;
    double cheb_prefactor;
    /* add/remove proposals by the rank-one update of the current
     * eigen-decomposition (move_addremove_rank1; FP64 eigenvectors):
     * fkh_run_chain only. */
    int rank1_moves;
} fkh_params;

/* Outputs (caller-sized; any pointer may be NULL): per proposal
 * (nsweeps+ntherm)*sweep_len entries of move index (0 flip, 1 add/remove,
 * 2 reshuffle), accepted flag, weight and uniform; per measurement nsweeps
 * entries of the measure_energy estimators and of n_f(q=0), n_f(q=pi)
 * (measure_nf0pi, include/fk_mc/measures/fsusc0pi.hpp:35-44); f_initial and
 * f_final of V entries; the histories of the eigenvalues
 * (measure_spectrum_history) and of f (measure_focc), V*nsweeps entries
 * state-major ([i*nsweeps + m]) as the reference stores them. */
typedef struct fkh_out {
    int32_t* move_index;
    int32_t* accepted;
    double* weight;
    double* uniform;
    double* energy;
    double* d2energy;
    double* c_energy;
    int32_t* f_initial;
    int32_t* f_final;
    long long naccept;
    double* nf0;
    double* nfpi;
    double* spectrum_history;
    int32_t* focc_history;
} fkh_out;

/* One chain through configuration_t / move_* / mc_metropolis / measure_energy
 * with calc_ed on the GPU (fkg_eigh_logz). Returns 0 or a negative error;
 * errbuf (may be NULL) receives the exception text. */
int fkh_run_chain(const fkh_params* p, fkh_out* out, char* errbuf, int errlen);

/* `batch` chains with seeds p->seed + c (one reference rank each), only
 * single-site-flip moves, through the batched device path (batched_mc).
 * Arrays are chain-major: accepted[c*nprop + k], energy[c*nsweeps + m],
 * f_initial / f_final [c*V + i]; move_index, weight and uniform are unused. */
int fkh_run_batched(const fkh_params* p, int batch, fkh_out* out, char* errbuf, int errlen);

/* measure_stiffness and measure_ipr (include/fk_mc/measures/stiffness.hpp,
 * ipr.hpp) through the adapter's classes for one configuration f (V entries)
 * of the lattice in p (lattice_kind, L, t, tp; beta, U, mu_c; precision):
 * one accumulate() each. Outputs: *stiffness, cond[nw] (the resonant terms on
 * wgrid with width eta; may be NULL when nw = 0) and ipr[V] (may be NULL). */
int fkh_measure_eigen(const fkh_params* p, const int32_t* f, int nw, const double* wgrid, double eta,
                      double* stiffness, double* cond, double* ipr, char* errbuf, int errlen);

/* fkh_run_chain on a graph lattice read from the .npy files in lattice_dir
 * (dims, norbitals, coordinates, hopping: the datasets of the reference's
 * read_lattice_hdf5, src/lattice/graph.cpp:52-80). p->lattice_kind, L, t and
 * tp are ignored. */
int fkh_run_chain_graph(const char* lattice_dir, const fkh_params* p, fkh_out* out, char* errbuf, int errlen);

/* The hopping matrix of the graph lattice in lattice_dir as CSR (rows sorted
 * by column): *n rows, *nnz elements; rowptr[n+1], col[nnz], val[nnz] are
 * written when their capacities (cap_n >= n+1, cap_nnz >= nnz) suffice,
 * otherwise only *n and *nnz are (and the call returns 1). */
int fkh_graph_lattice_csr(const char* lattice_dir, int cap_n, int cap_nnz, int* n, int* nnz, int32_t* rowptr,
                          int32_t* col, double* val, char* errbuf, int errlen);

/* ---- statistics (include/fk_mc/binning.hpp, jackknife.hpp,
 *      prog/data_save.hpp, prog/data_save.hxx) ---- */

/* Binning analysis of x[0..n) read backwards when `reverse` is non-zero (the
 * reference bins its energy series from the end, data_save.hxx:171): for
 * every depth 0..max_bin one row (number of bins, mean, variance, error of
 * the mean, correlation length) in rows[5*depth .. 5*depth+4]. max_bin <= 15
 * and 2^max_bin <= n, else an error. */
int fkh_binning(const double* x, long long n, int reverse, int max_bin, double* rows, char* errbuf, int errlen);

/* The depth at which the error bar of a binning saturates (estimate_bin,
 * prog/data_save.hpp:108-122), from nrows rows of `stride` doubles whose
 * column 3 is the error. */
int fkh_estimate_bin(const double* rows, int nrows, int stride);

/* Jackknife functions of the reference's statistics stage:
 *   FKH_JACK_MEAN   F(x) = x0;
 *   FKH_JACK_CV     F(e, e2, d2e) = beta^2 (e2 - d2e - e^2) / volume, fparams = {beta, volume}
 *                   (data_save.hxx:187);
 *   FKH_JACK_DISP   F(x, x2) = x2 - x^2 (data_save.hxx:212);
 *   FKH_JACK_BINDER F(x2, x4) = 1 - x4 / (3 x2^2) (data_save.hxx:229);
 *   FKH_JACK_LINEAR F(x) = sum_i fparams[i] x_i. */
enum { FKH_JACK_MEAN = 0, FKH_JACK_CV = 1, FKH_JACK_DISP = 2, FKH_JACK_BINDER = 3, FKH_JACK_LINEAR = 4 };

/* Jackknife of `func` over nseries series of n samples each (series[i],
 * read backwards when `reverse`), binned at every depth 0..max_bin: rows of
 * (number of bins, estimate, variance, error) in rows[4*depth ..]. */
int fkh_jackknife(int func, int nseries, const double* const* series, long long n, int reverse, int max_bin,
                  const double* fparams, double* rows, char* errbuf, int errlen);

/* The measured series of a run, as the reference's observables_t holds them
 * (include/fk_mc/fk_mc.hpp:13-34). Every pointer may be NULL. Per
 * measurement n_meas entries: energies, d2energies, c_energies, nf0, nfpi,
 * stiffness; spectrum: n_spectrum entries; histories state-major
 * [i*n_meas + m]: spectrum_history, ipr_history and focc_history with
 * `volume` states, cond_history with nw frequencies. */
typedef struct fkh_observables {
    long long n_meas;
    int volume;
    const double* energies;
    const double* d2energies;
    const double* c_energies;
    const double* nf0;
    const double* nfpi;
    const double* stiffness;
    const double* spectrum;
    long long n_spectrum;
    const double* spectrum_history;
    const double* ipr_history;
    const double* focc_history;
    const double* cond_history;
    int nw;
    const double* wgrid_cond;
} fkh_observables;

/* Output options (prog/fk_mc_exec.cpp:202-207, include/fk_mc/fk_mc.hxx:160-201).
 * max_bin < 0 takes the reference's rule min(15, max(int(log2(n/16) - 1), 1)). */
typedef struct fkh_save_options {
    double beta;
    int measure_history, measure_ipr, measure_stiffness;
    int dos_npts;
    double dos_width, dos_offset;
    int max_bin;
} fkh_save_options;

/* The reference's save_all (prog/data_save.hxx:32-95): binning, jackknife
 * and derived quantities of the observables, written under the directory
 * `dir` with one .npy file per HDF5 dataset of the reference's output
 * (mc_data/, binning/, stats/), parameters.json (the fields of p, may be
 * NULL) and stats.json (every /stats entry with its bin depth). */
int fkh_save_stats(const char* dir, const fkh_params* p, const fkh_observables* obs, const fkh_save_options* opt,
                   char* errbuf, int errlen);

#ifdef __cplusplus
}
#endif

#endif /* FK_MC_HOST_H */
