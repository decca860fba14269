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
} fkh_params;

/* Outputs (caller-sized): per proposal (nsweeps+ntherm)*sweep_len entries of
 * move index (0 flip, 1 add/remove, 2 reshuffle), accepted flag, weight and
 * uniform; per measurement nsweeps entries of the measure_energy estimators;
 * f_initial and f_final of V entries. */
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

#ifdef __cplusplus
}
#endif

#endif /* FK_MC_HOST_H */
