/*
 * fkg.h — C ABI of the GB300 (sm_103a) exact-diagonalisation solver for the
 * Falicov–Kimball Metropolis path of aeantipov/fk_mc.
 *
 * The reference does this work inside configuration_t::calc_ed
 * (include/fk_mc/configuration.hpp:71, src/configuration.cpp:208-246): it
 * builds H = hopping + diag(-mu_c + U f) (src/configuration.cpp:79-91),
 * copies it to a dense matrix (:212), diagonalises it with
 * Eigen::SelfAdjointEigenSolver (:213) and forms logZ, exp(beta eps) and the
 * Fermi factors (:224-245). move_addremove::attempt (src/moves.cpp:52-67) and
 * mc_metropolis::update (src/mc_metropolis.cpp:34-52) then turn logZ into an
 * accept/reject decision. The entry points below replace those steps; the
 * C++ host adapter in fk_mc_gb300/host keeps the reference's classes and
 * calls these functions.
 *
 * Conventions
 *   - All functions return 0 (FKG_OK) on success and a negative FKG_ERR_* code
 *     on failure; fkg_last_error() then describes the failure. Nothing throws
 *     across this boundary (the reference throws std::logic_error through
 *     FKMC_ERROR, include/fk_mc/common.hpp:49-59; the C++ adapter turns a
 *     negative return code back into that exception).
 *   - Host pointers are owned by the caller and only read/written during the
 *     call. The context owns every device buffer and its CUDA stream.
 *   - One context per host thread; a context is not thread-safe.
 *   - Matrices are column-major; eigenvalues are ascending; eigenvector k is
 *     column k (as Eigen returns them).
 *   - Per-chain vectors are packed back to back: chain c's n_c entries start
 *     after the entries of chains 0..c-1 (n_c is the size of its lattice).
 */
#ifndef FKG_H
#define FKG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fkg_ctx fkg_ctx;

#define FKG_OK 0
#define FKG_ERR_ARG (-1)      /* bad argument (size, id, null pointer) */
#define FKG_ERR_CUDA (-2)     /* a CUDA runtime call failed */
#define FKG_ERR_ALLOC (-3)    /* device or pinned allocation failed */
#define FKG_ERR_STATE (-4)    /* call out of order (e.g. no chains set up) */
#define FKG_ERR_TIMEOUT (-5)  /* a bounded device wait ran out */
#define FKG_ERR_NUMERIC (-6)  /* NaN/Inf or a non-converged iteration */

#define FKG_PREC_F64 0   /* plain FP64 path (the drop-in) */
#define FKG_PREC_MIXED 1 /* FP32 reduction + FP64 eigen-solve/refinement */

/* Create a context for matrices up to max_n and batches up to max_batch
 * (both are hints for pre-allocation; larger calls grow the buffers).
 * flags: reserved, pass 0. Returns NULL on failure. */
fkg_ctx* fkg_create(int max_n, int max_batch, unsigned flags);

/* Destroy a context and release its device memory and stream. */
void fkg_destroy(fkg_ctx* ctx);

/* Text of the last error on this context ("" when none). */
const char* fkg_last_error(const fkg_ctx* ctx);

/* Select FKG_PREC_F64 or FKG_PREC_MIXED for subsequent calls. */
int fkg_set_precision(fkg_ctx* ctx, int precision);

/* Register the hopping matrix of a lattice (abstract_lattice::hopping_m,
 * include/fk_mc/lattice.hpp:12-46, filled by fill_nearest_neighbors /
 * fill_triangular, src/lattice/hypercubic.cpp:115-155) as symmetric CSR
 * (rowptr[n+1], col[nnz], val[nnz]), including any on-site (diagonal)
 * entries; every col must lie in [0, n). lattice_id in [0, 64). */
int fkg_set_hopping(fkg_ctx* ctx, int lattice_id, int n, const int32_t* rowptr, const int32_t* col,
                    const double* val);

/* Batched configuration_t::calc_ed (src/configuration.cpp:208-246) for
 * `batch` independent Hamiltonians H_c = hopping(lattice_id[c]) + diag(diag_c).
 *   diag   : packed per-chain diagonals  -mu_c + U f_i  (input): what
 *            calc_hamiltonian adds to the hopping's diagonal, NOT the
 *            diagonal of the whole H (on-site hopping entries registered by
 *            fkg_set_hopping are added by the solver)
 *   beta   : [batch] inverse temperatures
 *   evals  : packed ascending spectra (ed_cache::cached_spectrum)
 *   exp_e  : packed exp(beta eps) (ed_cache::cached_exp), may be NULL
 *   fermi  : packed 1/(1+exp(beta eps)) (ed_cache::cached_fermi), may be NULL
 *   evecs  : packed n_c x n_c column-major eigenvectors (ed_cache::cached_evecs,
 *            the calc_evecs = true branch, :216-219), may be NULL
 *   logz   : [batch] ed_cache::logZ
 * All pointers are host memory. */
int fkg_eigh_logz(fkg_ctx* ctx, int batch, const int32_t* lattice_id, const double* diag, const double* beta,
                  double* evals, double* exp_e, double* fermi, double* evecs, double* logz);

/* Set up `batch` Markov chains resident on the device, one per
 * configuration_t + move_addremove pair (src/moves.cpp:52-67,
 * include/fk_mc/moves.hpp:41-47): packed f-occupations f (0/1), and per chain
 * U, mu_c, mu_f, beta. Computes and caches each chain's current spectrum and
 * logZ (the ed_cache of the current configuration). Host pointers. */
int fkg_chains_init(fkg_ctx* ctx, int batch, const int32_t* lattice_id, const int32_t* f, const double* U,
                    const double* mu_c, const double* mu_f, const double* beta);

/* Run `nsteps` proposal steps on all chains: step s proposes, for chain c, the
 * flip of site[s*batch + c] (move_addremove::attempt, src/moves.cpp:57-58),
 * diagonalises the proposed Hamiltonian, forms
 *   w = exp(logZ_new - logZ_cur) * (f_new ? e^{beta mu_f} : e^{-beta mu_f})
 * (src/moves.cpp:64-65) and accepts iff |w| > u[s*batch + c]
 * (src/mc_metropolis.cpp:43); an accepted chain takes the proposed f, logZ
 * and spectrum (move_flip::accept, src/moves.cpp:23-28).
 * Outputs accepted[s*batch+c] (0/1) and dlogz = logZ_new - logZ_cur, both may
 * be NULL. Host pointers; the copies to and from the device are part of the
 * call. */
int fkg_propose_accept(fkg_ctx* ctx, int nsteps, const int32_t* site, const double* u, int32_t* accepted,
                       double* dlogz);

/* Same as fkg_propose_accept with DEVICE pointers (inputs already resident
 * in HBM). Enqueued on the context's stream; synchronises before returning
 * so that the status word can be checked. */
int fkg_propose_accept_device(fkg_ctx* ctx, int nsteps, const int32_t* d_site, const double* d_u,
                              int32_t* d_accepted, double* d_dlogz);

/* Free energy F = -logZ/beta of `batch` configurations and its derivatives
 * (no counterpart in the reference, which only uses logZ: the
 * differentiation form of the path). H_c = hopping(lattice_id[c]) +
 * diag(-mu_c[c] + U[c] f_i); the hopping matrix is taken as linear in t[c]
 * (fill_nearest_neighbors stores -t per bond, src/lattice/hypercubic.cpp:115-131);
 * for lattices with several hopping amplitudes (fill_triangular's t and tp)
 * dF/dt is the derivative for a uniform scale of all of them.
 *   dF/dH = rho = V diag(fermi) V^T (optional output rho: packed n x n
 *   column-major per chain), dF/dU = sum_i f_i rho_ii, dF/dmu = -tr rho,
 *   dF/dt = tr(rho hopping)/t, dF/dbeta = (E_c - F)/beta with
 *   E_c = sum_k eps_k fermi_k (the c-energy of measure_energy,
 *   src/measures/energy.cpp:15-18).
 * Uses the context's precision (FKG_PREC_MIXED: FP32 eigenvectors, FP64
 * refined eigenvalues). Any output pointer may be NULL. Host pointers. */
int fkg_free_energy_grad(fkg_ctx* ctx, int batch, const int32_t* lattice_id, const int32_t* f, const double* U,
                         const double* mu_c, const double* t, const double* beta, double* F, double* dF_dU,
                         double* dF_dt, double* dF_dmu, double* dF_dbeta, double* rho);

/* The kinetic and current operators of measure_stiffness along the first
 * axis of lattice `lattice_id` (include/fk_mc/measures/stiffness.hpp:70-125:
 * Tm(i, left) = Tm(i, right) = -t, Jm(i, left) = -1, Jm(i, right) = +1, with
 * left/right the periodic neighbours along axis 0), as CSR with one pattern:
 * tval holds Tm, jval holds Jm. Required before fkg_measure_stiffness. */
int fkg_set_stiffness_ops(fkg_ctx* ctx, int lattice_id, int n, const int32_t* rowptr, const int32_t* col,
                          const double* tval, const double* jval);

/* measure_ipr::accumulate (include/fk_mc/measures/ipr.hpp:39-56) for a batch:
 * calc_ed(true) of each configuration (diag and beta as fkg_eigh_logz), then
 * ipr[k] = ||x_k||_4 / ||x_k||_2^2 for every eigenvector, in ascending
 * eigenvalue order (packed per chain like evals). Host pointers. */
int fkg_measure_ipr(fkg_ctx* ctx, int batch, const int32_t* lattice_id, const double* diag, const double* beta,
                    double* ipr);

/* measure_stiffness::accumulate (include/fk_mc/measures/stiffness.hpp:129-187)
 * for a batch: calc_ed(true), T = -pi sum_k fermi_k x_k^T Tm x_k,
 * mJ = X^T Jm X, V = sum_{i>j, |e_i-e_j| > 1e-12, |sigma| > 1e-13}
 * 2 sigma / (e_i - e_j) with sigma = pi (fermi_j - fermi_i) mJ(j,i) mJ(i,j):
 * stiffness[c] = (V + T)/n. With nw > 0, also the value of the
 * configuration's resonant terms on the frequency grid wgrid (width eta, the
 * measure's offset): cond[c*nw + q] = sum over the same pairs of
 * sigma (L(w_q + e_j - e_i) - L(w_q + e_i - e_j)), L(x) = eta/pi/(x^2+eta^2)
 * (one cond_history entry per frequency). The operators come from
 * fkg_set_stiffness_ops of each chain's lattice. Host pointers; wgrid and
 * cond may be NULL when nw = 0. */
int fkg_measure_stiffness(fkg_ctx* ctx, int batch, const int32_t* lattice_id, const double* diag,
                          const double* beta, double* stiffness, int nw, const double* wgrid, double eta,
                          double* cond);

/* ---- Chebyshev-expansion logZ (the reference's large-N method,
 *      configuration_t::calc_chebyshev, src/configuration.cpp:94-205;
 *      chebyshev::chebyshev_eval, include/fk_mc/chebyshev.hpp) ---- */

/* Number of Chebyshev moments (odd values are rounded up to even, as
 * chebyshev_eval does) and points of the Lobatto grid the coefficients are
 * integrated on: the reference's move set uses
 * cheb_size = int(log(V) * cheb_prefactor) and grid_size = max(2 cheb_size, 10)
 * (include/fk_mc/fk_mc.hxx:60-64). cheb_size in [2, 1024], grid_size in
 * [2, 4096]. Existing device-resident chains must be set up again. */
int fkg_set_chebyshev(fkg_ctx* ctx, int cheb_size, int grid_size);

/* logZ of each chain by the Chebyshev expansion, the counterpart of
 * fkg_eigh_logz for calc_chebyshev: spectral bounds of H by Lanczos (the
 * reference uses ARPACK), exact moments Tr T_m(x)/n of x = (H - b)/a, and
 * logZ = sum_m (2 - [m = 0]) c_m mu_m with c_m the trapezoid-rule Chebyshev
 * coefficients of n log(1 + exp(-beta (a x + b))). Inputs as fkg_eigh_logz.
 * Outputs (any may be NULL except logz): logz[batch], e_min[batch],
 * e_max[batch], moments[batch * cheb_size], lanczos_steps[batch] (the Lanczos
 * steps each chain's bounds took). Needs fkg_set_chebyshev. */
int fkg_chebyshev_logz(fkg_ctx* ctx, int batch, const int32_t* lattice_id, const double* diag, const double* beta,
                       double* logz, double* e_min, double* e_max, double* moments, int32_t* lanczos_steps);

/* How device-resident chains (fkg_chains_init / fkg_propose_accept*) get
 * logZ: FKG_METHOD_ED (the eigen-solve, default) or FKG_METHOD_CHEBYSHEV
 * (the expansion above; the chains then keep no spectrum). Existing chains
 * must be set up again. */
#define FKG_METHOD_ED 0
#define FKG_METHOD_CHEBYSHEV 1
int fkg_set_method(fkg_ctx* ctx, int method);

/* ---- single-site-flip proposals by the rank-one update (no counterpart in
 *      the reference: a shortcut for move_addremove, src/moves.cpp:52-67) ---- */

/* Flipping f_s changes H by rho e_s e_s^T (rho = +U for 0 -> 1, -U for
 * 1 -> 0). Given the current eigenvalues (ascending) and z = row s of the
 * current eigenvector matrix, the proposal's eigenvalues are the roots of the
 * secular equation 1 + rho sum_k z_k^2 / (l_k - x) = 0 after deflation: O(n^2)
 * per proposal, no re-solve. batch proposals of order n each: evals[batch*n],
 * z[batch*n], rho[batch], beta[batch] in; logz[batch] and (may be NULL)
 * evals_new[batch*n] ascending out. The eigenvectors must be accurate to
 * FP64 (the FP64 path's fkg_eigh_logz with evecs): the new eigenvalues are
 * as accurate as z. */
int fkg_rank1_logz(fkg_ctx* ctx, int batch, int n, const double* evals, const double* z, const double* rho,
                   const double* beta, double* logz, double* evals_new);
/* The same on device pointers (asynchronous up to the status check). */
int fkg_rank1_logz_device(fkg_ctx* ctx, int batch, int n, const double* d_evals, const double* d_z,
                          const double* d_rho, const double* d_beta, double* d_logz, double* d_evals_new);

/* Copy the chains' current state to the host: packed f, [batch] logZ and
 * packed ascending spectra (zeros under FKG_METHOD_CHEBYSHEV). Any pointer
 * may be NULL. */
int fkg_chains_get(fkg_ctx* ctx, int32_t* f, double* logz, double* evals);

/* Number of kernel launches this context has issued since creation. */
long long fkg_launch_count(const fkg_ctx* ctx);

/* Run the context's work on `cuda_stream` (a cudaStream_t owned by the
 * caller, e.g. a torch stream); NULL returns to the context's own stream. */
int fkg_set_stream(fkg_ctx* ctx, void* cuda_stream);

/* Panel width of the Householder reduction for matrices of order up to n_max
 * (size buckets of 64): variant indexes the compiled widths {4, 8, 16}
 * (FKG_PREC_MIXED) or {2, 4} (FKG_PREC_F64); -1 restores the default.
 * Written by the autotuner (fk_mc_gb300/autotune.py) from measured times. */
int fkg_set_tuning(fkg_ctx* ctx, int precision, int n_max, int variant);

/* Back-transformation kernel of the mixed path for matrices of order up to
 * n_max (size buckets of 64): 0 = mma.sync 3xTF32 with the column block of Z
 * in shared memory (the default), 1 = tcgen05 3xTF32 with tensor-memory
 * accumulators; -1 restores the default. Written by the autotuner. */
int fkg_set_tuning_back(fkg_ctx* ctx, int n_max, int variant);

/* Iteration limit of the bounded mbarrier waits in the main loops of the
 * tcgen05 kernels (the mixed path's tcgen05 back-transformation): a wait
 * that has not seen its MMAs complete after `iters` checks gives up, the
 * kernel waits for the MMAs it has issued, frees its tensor memory and
 * returns, and the call fails with FKG_ERR_TIMEOUT; the context stays usable.
 * iters < 0 restores the default (2^24 checks); 0 makes every such wait give
 * up without checking (tests of the timeout path). No counterpart in the
 * reference. */
int fkg_set_wait_limit(fkg_ctx* ctx, long long iters);

/* Replay one captured CUDA graph per proposal step in fkg_propose_accept*
 * (enable = 1, the default; profiling timers force direct launches). */
int fkg_set_graphs(fkg_ctx* ctx, int enable);

/* Per-stage CUDA-event timers. With enable != 0 every launch of a stage is
 * bracketed by events on the context's stream; fkg_stage_time() returns the
 * summed device time in ms and the launch count of stage `stage`
 * (FKG_STAGE_*) since the last fkg_profile(ctx, 1). */
#define FKG_STAGE_REDUCE 0  /* Householder tridiagonalisation (FP64 or FP32) */
#define FKG_STAGE_TRIEIG 1  /* tridiagonal eigenvalues (and vectors) */
#define FKG_STAGE_BACK 2    /* back-transformation of eigenvectors */
#define FKG_STAGE_REFINE 3  /* FP64 Rayleigh-quotient refinement */
#define FKG_STAGE_LOGZ 4    /* free energy, acceptance, proposal set-up */
#define FKG_NUM_STAGES 5
int fkg_profile(fkg_ctx* ctx, int enable);
int fkg_stage_time(fkg_ctx* ctx, int stage, double* total_ms, long long* launches);

/* Limits of fkg_eigh_logz_noalloc (its scratch is a fixed-size device array
 * of about 1.1 MB that every GPU loading this library keeps until exit). */
#define FKG_NOALLOC_MAX_N 128
#define FKG_NOALLOC_MAX_BATCH 8

/* Batched FP64 eigen-solve + logZ that allocates nothing: no cudaMalloc, no
 * cudaFree, no allocating library routine. No counterpart in the reference;
 * it exists for callers that cannot allocate device memory (e.g. a rank whose
 * device memory is already reserved by a host application's pool allocator,
 * or a step in which a synchronising device allocation is not allowed).
 *   batch Hamiltonians of order n share one hopping matrix, given as device
 *   CSR (d_rowptr[n+1], d_col, d_val): rowptr non-decreasing from 0, every
 *   col in [0, n) (a column outside it is skipped and the call returns
 *   FKG_ERR_ARG; rowptr itself is not checked); d_diag holds batch*n diagonals
 *   (-mu_c + U f_i), d_beta batch inverse temperatures; outputs d_evals
 *   (batch*n ascending spectra) and d_logz (batch). All pointers are device
 *   memory owned by the caller; work is enqueued on `stream` (NULL = default
 *   stream) and the call synchronises that stream before returning.
 * Scratch lives in a file-scope device array shared by every call. The
 * first call on each device looks up the array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture.
 * Calls that overlap on the GPU race on the shared scratch: serialise them.
 * Returns FKG_ERR_ARG for batch > FKG_NOALLOC_MAX_BATCH or
 * n > FKG_NOALLOC_MAX_N; on failure a message is written to errbuf
 * (errlen bytes, may be NULL). */
int fkg_eigh_logz_noalloc(int batch, int n, const int32_t* d_rowptr, const int32_t* d_col, const double* d_val,
                          const double* d_diag, const double* d_beta, double* d_evals, double* d_logz,
                          void* stream, char* errbuf, int errlen);

#ifdef __cplusplus
}
#endif

#endif /* FKG_H */
