// logz_accept.cu — the free energy, the proposal set-up and the Metropolis
// decision.
//
//  * logz: the loop of src/configuration.cpp:224-245. logZ =
//    sum_k log(1 + exp(-beta eps_k)) evaluated in the overflow-free form
//    max(0, -beta eps) + log1p(exp(-|beta eps|)) with Neumaier compensated
//    summation in FP64; cached_exp = exp(beta eps) and cached_fermi =
//    1/(1 + cached_exp) exactly as the reference writes them.
//  * accept: move_addremove::attempt's weight (src/moves.cpp:60-66) and the
//    test |w| > u of mc_metropolis::update (src/mc_metropolis.cpp:43), with the
//    accepted state kept on the device (move_flip::accept, src/moves.cpp:23-28).
//  * logz_accept: both in one launch per proposal step of the eigen-solve
//    path: the block that sums a chain's logZ takes the decision and updates
//    the chain's state (same sums in the same order, so the results equal the
//    two-kernel sequence bit for bit).
#include <cfloat>

#include "fkg_common.cuh"

namespace fkg {
namespace {

constexpr int kEigThreads = 128;

// The Metropolis decision of one chain (thread 0): move_addremove's weight
// exp(logZ_new - logZ_cur) e^{+-beta mu_f} against u; an accepted chain takes
// the flipped f and the new logZ. Returns the decision (0 for a bad site, which
// also flags the call).
__device__ __forceinline__ int decide(const ChainDesc& D, int c, int s, double u, double lz_new,
                                      const double* __restrict__ ebmf, int32_t* __restrict__ f,
                                      double* __restrict__ logz_cur, int32_t* __restrict__ accepted,
                                      double* __restrict__ dlogz, int* __restrict__ status) {
    if (s < 0 || s >= D.n) {  // reject the proposal and flag the call as failed
        atomicOr(status, kStatusBadArg);
        accepted[c] = 0;
        dlogz[c] = 0.0;
        return 0;
    }
    const double dl = lz_new - logz_cur[c];
    const double ratio = exp(dl);
    const int fnew = 1 - f[D.v_off + s];
    const double wgt = fnew ? ratio * ebmf[c] : ratio / ebmf[c];
    const int acc = fabs(wgt) > u;
    accepted[c] = acc;
    dlogz[c] = dl;
    if (acc) {
        f[D.v_off + s] = fnew;
        logz_cur[c] = lz_new;
    }
    return acc;
}

// Inputs of the fused decision (logz_kernel with acc.f != null): the step's
// site and uniform per chain (offset by the device step index when `step` is
// set), e^{beta mu_f}, the chains' f, current logZ and spectrum, and the
// step's outputs.
struct AcceptArgs {
    const int32_t* site;
    const double* u;
    const double* ebmf;
    int32_t* f;
    double* logz_cur;
    double* w_cur;
    int32_t* accepted;
    double* dlogz;
    const int* step;
};

__global__ void __launch_bounds__(kEigThreads)
logz_kernel(const ChainDesc* __restrict__ descs, const double* __restrict__ ww, const double* __restrict__ beta,
            double* __restrict__ logz, double* __restrict__ exp_out, double* __restrict__ fermi_out,
            int* __restrict__ status, AcceptArgs acc) {
    const ChainDesc D = descs[blockIdx.x];
    const int n = D.n;
    const double b = beta[blockIdx.x];
    double s = 0.0, c = 0.0;  // Neumaier running sum and compensation
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double e = ww[D.v_off + i];
        const double x = -b * e;
        const double term = fmax(x, 0.0) + log1p(exp(-fabs(x)));
        const double t = s + term;
        c += fabs(s) >= fabs(term) ? (s - t) + term : (term - t) + s;
        s = t;
        if (exp_out) {
            const double ex = exp(b * e);
            exp_out[D.v_off + i] = ex;
            fermi_out[D.v_off + i] = 1.0 / (1.0 + ex);
        }
    }
    __shared__ double ps[kEigThreads], pc[kEigThreads];
    ps[threadIdx.x] = s;
    pc[threadIdx.x] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        double S = 0.0, C = 0.0;
        for (int q = 0; q < (int)blockDim.x; ++q) {
            C += pc[q];
            const double t = S + ps[q];
            C += fabs(S) >= fabs(ps[q]) ? (S - t) + ps[q] : (ps[q] - t) + S;
            S = t;
        }
        const double r = S + C;
        logz[blockIdx.x] = r;
        if (!isfinite(r)) atomicOr(status, kStatusNaN);
        if (acc.f) {
            const size_t off = acc.step ? (size_t)(*acc.step) * gridDim.x : 0;
            const int ch = blockIdx.x;
            pc[0] = (double)decide(D, ch, acc.site[off + ch], acc.u[off + ch], r, acc.ebmf, acc.f, acc.logz_cur,
                                   acc.accepted + off, acc.dlogz + off, status);
        }
    }
    if (acc.f && acc.w_cur) {  // an accepted chain keeps the proposal's spectrum
        __syncthreads();
        if (pc[0] != 0.0)
            for (int i = threadIdx.x; i < n; i += blockDim.x) acc.w_cur[D.v_off + i] = ww[D.v_off + i];
    }
}

// site == null: the current configuration (no flip). step (may be null):
// device step index s, the proposal's site is site[s * gridDim.x + chain]
// (one captured CUDA-graph step replays every step).
__global__ void proposal_diag_kernel(const ChainDesc* __restrict__ descs, const int32_t* __restrict__ f,
                                     const int32_t* __restrict__ site, const double* __restrict__ U,
                                     const double* __restrict__ mu_c, double* __restrict__ diag,
                                     int* __restrict__ status, const int* __restrict__ step) {
    const ChainDesc D = descs[blockIdx.x];
    if (site && step) site += (size_t)(*step) * gridDim.x;
    int s = site ? site[blockIdx.x] : -1;
    if (site && (s < 0 || s >= D.n)) {  // device-side check: the pointer variant is not validated on the host
        if (threadIdx.x == 0) atomicOr(status, kStatusBadArg);
        s = -1;
    }
    const double u = U[blockIdx.x], mu = mu_c[blockIdx.x];
    for (int i = threadIdx.x; i < D.n; i += blockDim.x) {
        int fi = f[D.v_off + i];
        if (i == s) fi = 1 - fi;
        diag[D.v_off + i] = -mu + u * fi;
    }
}

__global__ void accept_kernel(const ChainDesc* __restrict__ descs, const int32_t* __restrict__ site,
                              const double* __restrict__ uu, const double* __restrict__ logz_new,
                              const double* __restrict__ w_new, const double* __restrict__ ebmf,
                              int32_t* __restrict__ f, double* __restrict__ logz_cur, double* __restrict__ w_cur,
                              int32_t* __restrict__ accepted, double* __restrict__ dlogz,
                              int* __restrict__ status, const int* __restrict__ step) {
    const ChainDesc D = descs[blockIdx.x];
    const int c = blockIdx.x;
    if (step) {
        const size_t off = (size_t)(*step) * gridDim.x;
        site += off; uu += off; accepted += off; dlogz += off;
    }
    __shared__ int acc;
    if (threadIdx.x == 0)
        acc = decide(D, c, site[c], uu[c], logz_new[c], ebmf, f, logz_cur, accepted, dlogz, status);
    __syncthreads();
    if (acc && w_cur)
        for (int i = threadIdx.x; i < D.n; i += blockDim.x) w_cur[D.v_off + i] = w_new[D.v_off + i];
}

}  // namespace

cudaError_t launch_logz(const ChainDesc* d_desc, int batch, int max_n, const double* d_w, const double* d_beta,
                        double* d_logz, double* d_exp, double* d_fermi, int* d_status, cudaStream_t st) {
    if (batch <= 0) return cudaSuccess;
    logz_kernel<<<batch, kEigThreads, 0, st>>>(d_desc, d_w, d_beta, d_logz, d_exp, d_fermi, d_status, AcceptArgs{});
    return cudaGetLastError();
}

cudaError_t launch_logz_accept(const ChainDesc* d_desc, int batch, const double* d_w, const double* d_beta,
                               double* d_logz, const int32_t* d_site, const double* d_u, const double* d_ebmf,
                               int32_t* d_f, double* d_logz_cur, double* d_w_cur, int32_t* d_accepted,
                               double* d_dlogz, int* d_status, cudaStream_t st, const int* d_step) {
    if (batch <= 0) return cudaSuccess;
    const AcceptArgs a{d_site, d_u, d_ebmf, d_f, d_logz_cur, d_w_cur, d_accepted, d_dlogz, d_step};
    logz_kernel<<<batch, kEigThreads, 0, st>>>(d_desc, d_w, d_beta, d_logz, nullptr, nullptr, d_status, a);
    return cudaGetLastError();
}

cudaError_t launch_proposal_diag(const ChainDesc* d_desc, int batch, int max_n, const int32_t* d_f,
                                 const int32_t* d_site, const double* d_U, const double* d_mu_c, double* d_diag,
                                 int* d_status, cudaStream_t st, const int* d_step) {
    if (batch <= 0) return cudaSuccess;
    proposal_diag_kernel<<<batch, 128, 0, st>>>(d_desc, d_f, d_site, d_U, d_mu_c, d_diag, d_status, d_step);
    return cudaGetLastError();
}

cudaError_t launch_accept(const ChainDesc* d_desc, int batch, int max_n, const int32_t* d_site, const double* d_u,
                          const double* d_logz_new, const double* d_w_new, const double* d_ebmf, int32_t* d_f,
                          double* d_logz_cur, double* d_w_cur, int32_t* d_accepted, double* d_dlogz,
                          int* d_status, cudaStream_t st, const int* d_step) {
    if (batch <= 0) return cudaSuccess;
    accept_kernel<<<batch, 128, 0, st>>>(d_desc, d_site, d_u, d_logz_new, d_w_new, d_ebmf, d_f, d_logz_cur,
                                         d_w_cur, d_accepted, d_dlogz, d_status, d_step);
    return cudaGetLastError();
}

__global__ void step_inc_kernel(int* step) { *step += 1; }

cudaError_t launch_step_inc(int* d_step, cudaStream_t st) {
    step_inc_kernel<<<1, 1, 0, st>>>(d_step);
    return cudaGetLastError();
}

}  // namespace fkg
