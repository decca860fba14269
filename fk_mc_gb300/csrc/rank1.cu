// rank1.cu — single-site-flip proposals by the rank-one update of a known
// eigen-decomposition (no counterpart in the reference; an algorithmic
// shortcut for move_addremove, src/moves.cpp:52-67). Flipping f_s changes
// H by rho e_s e_s^T, rho = +U (0 -> 1) or -U (1 -> 0). With H = Q diag(l) Q^T
// the new eigenvalues are those of diag(l) + rho z z^T, z = Q^T e_s = row s
// of Q: the roots of the secular equation
//     f(x) = 1 + rho sum_k z_k^2 / (l_k - x) = 0,
// one in each gap between consecutive poles (and one beyond the last), after
// deflation of negligible weights and of (nearly) equal poles (Golub, "Some
// modified matrix eigenvalue problems", SIAM Review 15, 1973; the deflation
// by Givens rotation of Bunch, Nielsen and Sorensen, Numer. Math. 31, 1978).
// O(n^2) per proposal instead of the O(n^3) re-solve.
//
// One CTA per proposal. Every root is found in two phases:
//   1. FP32: safeguarded iteration inside its gap, each step the root of the
//      model c + s/(p - x) that matches f and f' at the iterate (p the nearer
//      pole; a Newton step on the pole's hyperbola), the pole differences
//      formed from double-float (hi, lo) copies of the poles so that they keep
//      their relative accuracy in small gaps;
//   2. double-float / FP64: the same steps from the FP32 root with the origin at the nearer
//      pole (the root = pole + tau, tau carried separately), safeguarded by
//      the gap: one step when it moves tau by less than 1e-6 (the convergence
//      is quadratic, so that leaves an FP64-rounding error), else until the
//      step is below 2 ulps of tau.
// Both phases run on GB300's wide FP32 pipe (phase 2 in double-float, ~48
// bits, with the step itself in FP64); the narrow FP64 pipe only sees O(n)
// work per proposal. logZ of the new spectrum uses the logz_kernel form
// (overflow-free term, Neumaier sum).
#include <cfloat>
#include <cstring>
#include <string>
#include <vector>

#include "fkg_internal.h"

namespace fkg {
namespace {

constexpr int kR1Threads = 256;

__device__ __forceinline__ void neumaier(double& s, double& c, double term) {
    const double t = s + term;
    c += fabs(s) >= fabs(term) ? (s - t) + term : (term - t) + s;
    s = t;
}

// n eigenvalues per proposal (ascending), z: n weights (row `site` of the
// eigenvector matrix), rho: the diagonal change, beta. Outputs logz and,
// when ev_out is not null, the new eigenvalues ascending.
__global__ void __launch_bounds__(kR1Threads)
rank1_kernel(int n, const double* __restrict__ evals, const double* __restrict__ zrow, const double* __restrict__ rho_c,
             const double* __restrict__ beta_c, double* __restrict__ logz, double* __restrict__ ev_out,
             int* __restrict__ status) {
    extern __shared__ __align__(16) double rsm[];
    double* d = rsm;           // poles, sign-adjusted ascending (then the kept ones, compacted)
    double* w = d + n;         // weights z_k^2 (compacted with d)
    double* fixed = w + n;     // deflated eigenvalues (sign-adjusted, ascending)
    double* root = fixed + n;  // roots (sign-adjusted, ascending)
    float2* dhl = (float2*)(root + n);  // poles as FP32 pairs hi + lo
    float2* whl = dhl + n;              // weights as FP32 pairs hi + lo
    __shared__ int sh_m, sh_nf;
    __shared__ double sh_tol;
    __shared__ double ps[kR1Threads], pc[kR1Threads];
    const int c = blockIdx.x, tid = threadIdx.x;
    const double* lam = evals + (size_t)c * n;
    const double* z = zrow + (size_t)c * n;
    const double rho_s = rho_c[c], beta = beta_c[c];
    const double sg = rho_s < 0.0 ? -1.0 : 1.0, rho = fabs(rho_s);
    // poles of the problem with rho >= 0: diag(sg l) + rho z z^T, reordered ascending
    for (int k = tid; k < n; k += blockDim.x) {
        const int src = sg > 0 ? k : n - 1 - k;
        d[k] = sg * lam[src];
        w[k] = z[src];  // z for now; squared below
    }
    __syncthreads();
    if (tid == 0) {
        // deflation, in pole order: merge (nearly) equal poles by a Givens
        // rotation of their z components, drop negligible weights
        double dmax = 0.0, zz = 0.0;
        for (int k = 0; k < n; ++k) {
            dmax = fmax(dmax, fabs(d[k]));
            zz += w[k] * w[k];
        }
        const double tol = 8.0 * DBL_EPSILON * fmax(dmax, rho * zz);
        int m = 0, nf = 0;
        double cd = d[0], cz = w[0];
        for (int k = 1; k <= n; ++k) {
            if (k < n && d[k] - cd <= tol) {
                const double r = hypot(cz, w[k]);
                if (r == 0.0) {
                    fixed[nf++] = d[k];
                    continue;
                }
                const double cs = cz / r, sn = w[k] / r;
                fixed[nf++] = sn * sn * cd + cs * cs * d[k];
                cd = cs * cs * cd + sn * sn * d[k];
                cz = r;
                continue;
            }
            if (rho * cz * cz <= tol) {
                fixed[nf++] = cd;
            } else {
                d[m] = cd;   // m <= k - 1: never overwrites an unread pole
                w[m] = cz * cz;
                ++m;
            }
            if (k < n) {
                cd = d[k];
                cz = w[k];
            }
        }
        // the fixed values are produced in pole order but a merged pole can
        // sit a rounding above the next one: insertion sort (nearly sorted)
        for (int a = 1; a < nf; ++a) {
            const double v = fixed[a];
            int b = a - 1;
            while (b >= 0 && fixed[b] > v) { fixed[b + 1] = fixed[b]; --b; }
            fixed[b + 1] = v;
        }
        sh_m = m;
        sh_nf = nf;
        sh_tol = tol;
    }
    __syncthreads();
    const int m = sh_m, nf = sh_nf;
    const double tol = sh_tol;
    double wsum_l = 0.0;
    for (int k = tid; k < m; k += blockDim.x) {
        const float hi = (float)d[k];
        dhl[k] = make_float2(hi, (float)(d[k] - (double)hi));
        const float wh = (float)w[k];
        whl[k] = make_float2(wh, (float)(w[k] - (double)wh));
        wsum_l += w[k];
    }
    // total weight (for the last root's bracket): a fixed-order block sum
    ps[tid] = wsum_l;
    __syncthreads();
    if (tid == 0) {
        double s = 0.0;
        for (int q = 0; q < (int)blockDim.x; ++q) s += ps[q];
        pc[0] = s;
    }
    __syncthreads();
    const double wsum = pc[0];
    __syncthreads();
    const float rhof = (float)rho;
    int bad = 0;
    for (int i = tid; i < m; i += blockDim.x) {
        const bool last = i == m - 1;
        const double gap = last ? rho * wsum : d[i + 1] - d[i];
        // phase 1 (FP32): tau in (0, gap) measured from pole i
        const float2 oi = dhl[i];
        // the bracket in the same FP32 differences the iteration uses
        const float gap32 = last ? (float)gap : (dhl[i + 1].x - oi.x) + (dhl[i + 1].y - oi.y);
        float lo = 0.0f, hi = gap32, tau = 0.5f * gap32;
        for (int it = 0; it < 64; ++it) {
            float f = 0.0f, fp = 0.0f;
            for (int k = 0; k < m; ++k) {
                const float2 q = dhl[k];
                const float den = ((q.x - oi.x) + (q.y - oi.y)) - tau;
                const float r = __fdividef(1.0f, den);
                const float wk = whl[k].x, wr = wk * r;
                f = fmaf(wk, r, f);
                fp = fmaf(wr, r, fp);
            }
            f = fmaf(rhof, f, 1.0f);
            fp *= rhof;
            if (f > 0.0f) hi = tau; else lo = tau;
            // step: the root of the model c + s / (p - x) matched to f and f' at
            // tau, p the nearer pole of the gap (exact when the other terms are
            // constant; converges fast for roots that hug a pole, where plain
            // Newton crawls)
            const float po = (last || tau < 0.5f * gap32) ? 0.0f : gap32;
            const float dd = po - tau, sm = fp * dd * dd, cm = f - sm / dd;
            float tn = cm != 0.0f ? po + sm / cm : tau - f / fp;
            // a Newton step below a few ulps ends the search (it may round onto
            // the bracket end it just moved); otherwise stay inside the bracket
            if (fabsf(tn - tau) <= 4.0f * FLT_EPSILON * fabsf(tau)) break;
            if (!(tn > lo && tn < hi)) tn = 0.5f * (lo + hi);
            const bool conv = hi - lo <= 4.0f * FLT_EPSILON * fmaxf(fabsf(lo), fabsf(hi));
            tau = tn;
            if (conv) break;
        }
        // phase 2 (double-float sums, FP64 steps): origin at the nearer pole
        const int org = (!last && (double)tau > 0.5 * gap) ? i + 1 : i;
        double t = org == i ? (double)tau : (double)tau - gap;
        double blo = org == i ? 0.0 : -gap, bhi = org == i ? gap : 0.0;
        // the FP32 root may sit a rounding outside the FP64 gap: pull it inside
        const double margin = 4.0 * DBL_EPSILON * gap;
        t = fmin(fmax(t, blo + margin), bhi - margin);
        const double dorg = d[org];
        const float2 og = dhl[org];
        bool conv = false;
        for (int it = 0; it < 40 && !conv; ++it) {
            // f and f' in double-float: den = (d_k - d_org) - t, r = 1/den
            const dfl nt = df_of(-t);
            dfl F = {0.0f, 0.0f}, FP = {0.0f, 0.0f};
            float mag = 0.0f;  // sum of |w_k / den_k|: the scale of f's rounding
            for (int k = 0; k < m; ++k) {
                const float2 q = dhl[k], wq = whl[k];
                const dfl den = df_add(df_add({q.x, q.y}, {-og.x, -og.y}), nt);
                const dfl r = df_rcp(den);
                const dfl wr = df_mul({wq.x, wq.y}, r);
                F = df_add(F, wr);
                FP = df_add(FP, df_mul(wr, r));
                mag += fabsf(wr.hi);
            }
            double f = df_val(F), fp = df_val(FP);
            // a step the double-float rounding of f could cause is not a step
            const double noise = 1e-13 * (1.0 + rho * (double)mag) / (rho * fp);
            f = fma(rho, f, 1.0);
            fp *= rho;
            if (f > 0.0) bhi = t; else if (f < 0.0) blo = t; else { conv = true; break; }
            // the pole model of phase 1 about the origin pole (at t = 0)
            const double sm = fp * t * t, cm = f + sm / t;
            double tn = cm != 0.0 ? sm / cm : t - f / fp;
            // the steps converge quadratically: a first step below 1e-6 of tau from
            // the FP32 root leaves an error near FP64 rounding, no second pass
            if (it == 0 && fabs(tn - t) <= 1e-6 * fabs(t) && tn > blo && tn < bhi) {
                t = tn;
                conv = true;
                break;
            }
            // converged at the double-float resolution: keep t or the step
            if (fabs(tn - t) <= fmax(64.0 * DBL_EPSILON * fabs(t), noise)) {
                if (tn > blo && tn < bhi) t = tn;
                conv = true;
                break;
            }
            if (!(tn > blo && tn < bhi)) tn = 0.5 * (blo + bhi);
            conv = bhi - blo <= 64.0 * DBL_EPSILON * fmax(fabs(blo), fabs(bhi));
            t = tn;
        }
        // a gap of a few deflation tolerances places the root to within the gap
        // whether or not the iteration settled
        if (!conv && gap > 1024.0 * tol) bad = 1;
        root[i] = dorg + t;
    }
    if (bad) atomicOr(status, kStatusNoConverge);
    __syncthreads();
    // logZ over roots and fixed values (sign back), logz_kernel's form
    double s = 0.0, cc = 0.0;
    for (int k = tid; k < m + nf; k += blockDim.x) {
        const double e = sg * (k < m ? root[k] : fixed[k - m]);
        const double x = -beta * e;
        neumaier(s, cc, fmax(x, 0.0) + log1p(exp(-fabs(x))));
    }
    ps[tid] = s;
    pc[tid] = cc;
    __syncthreads();
    if (tid == 0) {
        double S = 0.0, C = 0.0;
        for (int q = 0; q < (int)blockDim.x; ++q) {
            C += pc[q];
            neumaier(S, C, ps[q]);
        }
        const double r = S + C;
        logz[c] = r;
        if (!isfinite(r)) atomicOr(status, kStatusNaN);
        if (ev_out) {  // merge roots and fixed values, back to the original sign, ascending
            double* out = ev_out + (size_t)c * n;
            int a = 0, b = 0;
            for (int k = 0; k < n; ++k) {
                double v;
                if (b >= nf || (a < m && root[a] <= fixed[b])) v = root[a++];
                else v = fixed[b++];
                if (sg > 0) out[k] = v; else out[n - 1 - k] = -v;
            }
        }
    }
}

}  // namespace

size_t rank1_smem_bytes(int n) { return (size_t)n * (4 * sizeof(double) + 2 * sizeof(float2)); }

cudaError_t launch_rank1(int batch, int n, const double* d_evals, const double* d_z, const double* d_rho,
                         const double* d_beta, double* d_logz, double* d_ev_out, int* d_status, cudaStream_t st) {
    if (batch <= 0) return cudaSuccess;
    const size_t sm = rank1_smem_bytes(n);
    cudaError_t e = cudaFuncSetAttribute(rank1_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    rank1_kernel<<<batch, kR1Threads, sm, st>>>(n, d_evals, d_z, d_rho, d_beta, d_logz, d_ev_out, d_status);
    return cudaGetLastError();
}

}  // namespace fkg

using namespace fkg;

namespace {

int r1_err(fkg_ctx* ctx, int code, const std::string& msg) {
    ctx->err = msg;
    return code;
}

}  // namespace

extern "C" {

int fkg_rank1_logz_device(fkg_ctx* ctx, int batch, int n, const double* d_evals, const double* d_z,
                          const double* d_rho, const double* d_beta, double* d_logz, double* d_evals_new) {
    if (!ctx) return FKG_ERR_ARG;
    if (batch < 1 || n < 1 || n > kMaxN) return r1_err(ctx, FKG_ERR_ARG, "batch or n out of range");
    if (!d_evals || !d_z || !d_rho || !d_beta || !d_logz) return r1_err(ctx, FKG_ERR_ARG, "null device pointer");
    cudaError_t e = cudaMemsetAsync(ctx->status.p, 0, sizeof(int), ctx->st);
    if (e == cudaSuccess) e = launch_rank1(batch, n, d_evals, d_z, d_rho, d_beta, d_logz, d_evals_new, (int*)ctx->status.p, ctx->st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return r1_err(ctx, FKG_ERR_CUDA, std::string("rank-one update: ") + cudaGetErrorString(e));
    }
    ctx->launches++;
    return check_status(ctx);
}

int fkg_rank1_logz(fkg_ctx* ctx, int batch, int n, const double* evals, const double* z, const double* rho,
                   const double* beta, double* logz, double* evals_new) {
    if (!ctx) return FKG_ERR_ARG;
    if (batch < 1 || n < 1 || n > kMaxN) return r1_err(ctx, FKG_ERR_ARG, "batch or n out of range");
    if (!evals || !z || !rho || !beta || !logz) return r1_err(ctx, FKG_ERR_ARG, "null argument");
    const size_t V = (size_t)batch * n;
    for (int c = 0; c < batch; ++c) {
        if (!(beta[c] > 0.0) || beta[c] - beta[c] != 0.0) return r1_err(ctx, FKG_ERR_ARG, "beta must be finite and > 0");
        if (rho[c] - rho[c] != 0.0) return r1_err(ctx, FKG_ERR_ARG, "rho must be finite");
        for (int k = 1; k < n; ++k)
            if (!(evals[(size_t)c * n + k] >= evals[(size_t)c * n + k - 1]))
                return r1_err(ctx, FKG_ERR_ARG, "eigenvalues must be finite and ascending");
    }
    Workspace& ws = ctx->solve;
    int rc;
    // scratch: evals, z, new evals (V each) + rho, beta, logz (batch each)
    if ((rc = ensure_dev(ctx, ws.mscr, sizeof(double) * (3 * V + 3 * (size_t)batch)))) return rc;
    if ((rc = ensure_pinned(ctx, sizeof(double) * (3 * V + 3 * (size_t)batch)))) return rc;
    double* dev = (double*)ws.mscr.p;
    double *d_ev = dev, *d_z = dev + V, *d_evn = dev + 2 * V, *d_rho = dev + 3 * V, *d_beta = d_rho + batch,
           *d_lz = d_beta + batch;
    double* h = (double*)ctx->pin;
    std::memcpy(h, evals, sizeof(double) * V);
    std::memcpy(h + V, z, sizeof(double) * V);
    std::memcpy(h + 3 * V, rho, sizeof(double) * batch);
    std::memcpy(h + 3 * V + batch, beta, sizeof(double) * batch);
    cudaStream_t st = ctx->st;
    cudaError_t e = cudaMemcpyAsync(dev, h, sizeof(double) * 2 * V, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_rho, h + 3 * V, sizeof(double) * 2 * batch, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return r1_err(ctx, FKG_ERR_CUDA, std::string("rank-one upload: ") + cudaGetErrorString(e));
    }
    if ((rc = fkg_rank1_logz_device(ctx, batch, n, d_ev, d_z, d_rho, d_beta, d_lz, evals_new ? d_evn : nullptr)))
        return rc;
    e = cudaMemcpyAsync(h + 3 * V + 2 * batch, d_lz, sizeof(double) * batch, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && evals_new) e = cudaMemcpyAsync(h + 2 * V, d_evn, sizeof(double) * V, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return r1_err(ctx, FKG_ERR_CUDA, std::string("rank-one download: ") + cudaGetErrorString(e));
    }
    std::memcpy(logz, h + 3 * V + 2 * batch, sizeof(double) * batch);
    if (evals_new) std::memcpy(evals_new, h + 2 * V, sizeof(double) * V);
    return FKG_OK;
}

}  // extern "C"
