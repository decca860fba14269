// fkg_internal.h — host-side definition of the fkg_ctx context.
#pragma once
#include <cmath>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/fkg.h"
#include "fkg_common.cuh"

namespace fkg {

constexpr int kMaxLattices = 64;
constexpr int kMaxN = 1024;  // largest matrix order the kernels are built for
// reduction variants of the mixed path (fkg_set_tuning): 0..2 the one-stage
// kernel's panel widths (kSytrdF32Nb), kTwoStageVariant the two-stage reduction
constexpr int kTwoStageVariant = 3;
constexpr int kMixedVariants = 4;

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

struct LatticeDev {
    int n = 0, nnz = 0;
    int32_t* rowptr = nullptr;
    int32_t* col = nullptr;
    double* val = nullptr;
    float2* valf = nullptr;  // val as FP32 pairs hi + lo
    // measure_stiffness operators along axis 0 (fkg_set_stiffness_ops)
    int snnz = -1;
    int32_t* srow = nullptr;
    int32_t* scol = nullptr;
    double* stval = nullptr;
    double* sjval = nullptr;
    // host copy of the hopping (the Chebyshev balls are built from it)
    std::vector<int32_t> h_rowptr, h_col;
    std::vector<double> h_val;
    // Chebyshev balls of radius kpm_R around every site (-1: not built), see KpmDesc
    int kpm_R = -1, kpm_bmax = 0;
    int32_t* kpm_bptr = nullptr;
    int32_t* kpm_bsite = nullptr;
    int32_t* kpm_bcnt = nullptr;
    int32_t* kpm_blrp = nullptr;
    int32_t* kpm_blcol = nullptr;
    double* kpm_blval = nullptr;
    float2* kpm_blv2 = nullptr;
    double* kpm_hdiag = nullptr;
    void free_kpm() {
        for (void* q : {(void*)kpm_bptr, (void*)kpm_bsite, (void*)kpm_bcnt, (void*)kpm_blrp, (void*)kpm_blcol,
                        (void*)kpm_blval, (void*)kpm_blv2, (void*)kpm_hdiag})
            if (q) cudaFree(q);
        kpm_bptr = kpm_bsite = kpm_bcnt = kpm_blrp = kpm_blcol = nullptr;
        kpm_blval = kpm_hdiag = nullptr;
        kpm_blv2 = nullptr;
        kpm_R = -1;
        kpm_bmax = 0;
    }
    void free_all() {
        for (void* q : {(void*)rowptr, (void*)col, (void*)val, (void*)valf, (void*)srow, (void*)scol, (void*)stval,
                        (void*)sjval})
            if (q) cudaFree(q);
        free_kpm();
    }
};

// Host copy of a batch layout.
struct Layout {
    int batch = 0, max_n = 0, max_ld = 0, min_n = 0;
    long long n_total = 0, v_total = 0, a_total = 0;
    std::vector<ChainDesc> desc;
    std::vector<int> order;  // chain indices by decreasing n (work list of the persistent reduction)
};

// Device buffers of one batched eigen-solve.
struct Workspace {
    DevBuf desc, A, diag, d, e, tau, w, beta, logz, exp_e, fermi;
    // mixed-precision path
    DevBuf A32, aux32, aux64, Z, Tf;
    DevBuf perm;  // sorted-eigenvalue -> eigenvector-column map (mixed path)
    DevBuf VT;    // V_p T_p and V_p of every panel, split hi/lo for 3xTF32: 4 planes (mixed path)
    DevBuf zsc;   // 1/||z_j|| of the twisted-factorisation vectors (mixed path)
    DevBuf ctol;  // per-chain cluster tolerance of the eigenvector kernels (mixed path)
    DevBuf Q2;    // two-stage reduction: the band stage's reflectors and their tau (mixed path)
    DevBuf S1;    // two-stage reduction: per-chain operand tiles of the first stage's tensor-core pass
    DevBuf TM;    // two-stage reduction: one TMA tensor map per chain over its A32 matrix
    std::vector<unsigned char> tm_host;  // ... their host copy (the source of the upload)
    std::vector<long long> tm_key;       // A32 address, then (a_off, ld) per chain, of the maps in TM
    // eigenvectors and gradients
    DevBuf Z64, stein, Tf64, fint, gout, fermiw, rho, Ulist, mulist, tlist;
    DevBuf order, counter;  // persistent-reduction work list and its counter
    DevBuf mout, ef, mscr, sops, mcond;  // measures: output, (eps, fermi) per column, partial sums, operators, grid + cond
    DevBuf kdesc, ksteps, kab, kpart, kmu;  // Chebyshev logZ: descriptors, Lanczos steps, bounds, column sums, moments
    int kpm_batch = 0;                    // chains the uploaded Chebyshev descriptors describe
};

}  // namespace fkg

namespace fkg {
// CUDA-event pairs bracketing every launch of one stage (fkg_profile).
struct StageTimer {
    std::vector<cudaEvent_t> ev;
    size_t used = 0;
    double acc_ms = 0.0;
    long long launches = 0;
};
}  // namespace fkg

struct fkg_ctx {
    int max_n = 0, max_batch = 0;
    unsigned flags = 0;
    int precision = FKG_PREC_F64;
    int method = FKG_METHOD_ED;  // how device-resident chains get logZ
    int kpm_M = 0, kpm_G = 0;    // Chebyshev moments (even) and grid points; 0 = not set
    int device = 0;
    int num_sms = 0;
    cudaStream_t st = nullptr;      // stream all work is enqueued on
    cudaStream_t own_st = nullptr;  // the context's own stream
    // second and third streams for independent kernels of one mixed solve
    cudaStream_t aux_st = nullptr, aux2_st = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_red = nullptr, ev_larft = nullptr;
    bool profiling = false;
    long long wait_iters = fkg::kDefaultWaitIters;  // main-loop limit of the bounded mbarrier waits
    fkg::StageTimer timers[FKG_NUM_STAGES];
    std::string err;
    long long launches = 0;
    fkg::LatticeDev lat[fkg::kMaxLattices];
    fkg::DevBuf status;
    // one-off solves (fkg_eigh_logz)
    fkg::Layout solve_layout;
    fkg::Workspace solve;
    // device-resident chains (fkg_chains_init / fkg_propose_accept)
    bool chains_ready = false;
    fkg::Layout chain_layout;
    fkg::Workspace chain;
    fkg::DevBuf ch_f, ch_U, ch_mu_c, ch_ebmf, ch_logz_cur, ch_w_cur;
    fkg::DevBuf st_site, st_u, st_acc, st_dlogz;
    // pinned host staging
    void* pin = nullptr;
    size_t pin_bytes = 0;
    // tuning: panel-width variant of the reduction per matrix-size bucket
    // (bucket b covers n in (64 (b-1), 64 b]); -1 = default
    int tune_f32[17], tune_f64[17];
    int tune_bt[17];  // back-transformation kernel of the mixed path per size bucket (-1: default)
    // CUDA graph of one proposal step (fkg_propose_accept*), replayed per step
    bool use_graphs = true;
    int graph_kernels = 0;  // kernel launches in one replay of the step graph
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    fkg::DevBuf d_step;
    fkg_ctx() {
        for (int i = 0; i < 17; ++i) tune_f32[i] = tune_f64[i] = tune_bt[i] = -1;
    }
    void drop_graph() {
        if (graph_exec) cudaGraphExecDestroy(graph_exec);
        if (graph) cudaGraphDestroy(graph);
        graph_exec = nullptr;
        graph = nullptr;
    }

    std::vector<fkg::DevBuf*> all_buffers() {
        std::vector<fkg::DevBuf*> v = {&status, &d_step, &ch_f, &ch_U, &ch_mu_c, &ch_ebmf, &ch_logz_cur, &ch_w_cur,
                                       &st_site, &st_u, &st_acc, &st_dlogz};
        for (fkg::Workspace* w : {&solve, &chain})
            for (fkg::DevBuf* b : {&w->desc, &w->A, &w->diag, &w->d, &w->e, &w->tau, &w->w, &w->beta, &w->logz,
                                   &w->exp_e, &w->fermi, &w->A32, &w->aux32, &w->aux64, &w->Z, &w->Tf, &w->perm, &w->VT, &w->zsc, &w->ctol, &w->Q2, &w->S1, &w->TM, &w->Z64,
                                   &w->stein, &w->Tf64, &w->fint, &w->gout, &w->fermiw, &w->rho, &w->Ulist,
                                   &w->mulist, &w->tlist, &w->order, &w->counter, &w->mout, &w->ef, &w->mscr, &w->sops, &w->mcond,
                                   &w->kdesc, &w->ksteps, &w->kab, &w->kpart, &w->kmu})
                v.push_back(b);
        return v;
    }
};

namespace fkg {
int ensure_dev(fkg_ctx* ctx, DevBuf& b, size_t bytes);
int ensure_pinned(fkg_ctx* ctx, size_t bytes);
int make_layout(fkg_ctx* ctx, int batch, const int32_t* lattice_id, Layout& L);
int upload_layout(fkg_ctx* ctx, Workspace& ws, const Layout& L);
int ensure_solve_ws(fkg_ctx* ctx, Workspace& ws, const Layout& L, bool need_vecs);
// The per-step inputs and outputs of a proposal step on the device-resident
// chains (device pointers; step: the device step index of a graph replay, or
// null). Given to enqueue_solve, the logZ kernel also takes each chain's
// Metropolis decision.
struct StepIO {
    const int32_t* site;
    const double* u;
    int32_t* acc;
    double* dl;
    const int* step;
};
int enqueue_solve(fkg_ctx* ctx, Workspace& ws, const Layout& L, bool want_exp, const StepIO* io = nullptr);
int enqueue_steps(fkg_ctx* ctx, int nsteps, const int32_t* d_site, const double* d_u, int32_t* d_acc,
                  double* d_dlogz);
int check_status(fkg_ctx* ctx);
int eigh_vectors(fkg_ctx* ctx, int batch, const int32_t* lattice_id, const double* diag, const double* beta,
                 double* evals, double* exp_e, double* fermi, double* evecs, double* logz);
int enqueue_vectors(fkg_ctx* ctx, Workspace& ws, const Layout& L);
void stage_begin(fkg_ctx* ctx, int stage);
// Chebyshev logZ: prepare_kpm builds the balls of the layout's lattices and
// uploads the chain descriptors and scratch (allocates; not inside a graph
// capture); enqueue_kpm launches the kernels on ws.diag / ws.beta -> ws.logz.
int prepare_kpm(fkg_ctx* ctx, Workspace& ws, const Layout& L);
int enqueue_kpm(fkg_ctx* ctx, Workspace& ws, const Layout& L, double* d_mu);
void stage_end(fkg_ctx* ctx, int stage);
}  // namespace fkg
