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
#include <cfloat>

#include "fkg_common.cuh"

namespace fkg {
namespace {

constexpr int kEigThreads = 128;

__global__ void __launch_bounds__(kEigThreads)
logz_kernel(const ChainDesc* __restrict__ descs, const double* __restrict__ ww, const double* __restrict__ beta,
            double* __restrict__ logz, double* __restrict__ exp_out, double* __restrict__ fermi_out,
            int* __restrict__ status) {
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
    if (threadIdx.x == 0) {
        const int s = site[c];
        if (s < 0 || s >= D.n) {  // reject the proposal and flag the call as failed
            atomicOr(status, kStatusBadArg);
            acc = 0;
            accepted[c] = 0;
            dlogz[c] = 0.0;
        } else {
        const double dl = logz_new[c] - logz_cur[c];
        const double ratio = exp(dl);
        const int fnew = 1 - f[D.v_off + s];
        const double wgt = fnew ? ratio * ebmf[c] : ratio / ebmf[c];
        acc = fabs(wgt) > uu[c];
        accepted[c] = acc;
        dlogz[c] = dl;
        if (acc) {
            f[D.v_off + s] = fnew;
            logz_cur[c] = logz_new[c];
        }
        }
    }
    __syncthreads();
    if (acc && w_cur)
        for (int i = threadIdx.x; i < D.n; i += blockDim.x) w_cur[D.v_off + i] = w_new[D.v_off + i];
}

}  // namespace

cudaError_t launch_logz(const ChainDesc* d_desc, int batch, int max_n, const double* d_w, const double* d_beta,
                        double* d_logz, double* d_exp, double* d_fermi, int* d_status, cudaStream_t st) {
    if (batch <= 0) return cudaSuccess;
    logz_kernel<<<batch, kEigThreads, 0, st>>>(d_desc, d_w, d_beta, d_logz, d_exp, d_fermi, d_status);
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
