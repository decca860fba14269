// chebyshev.cu — the Chebyshev-expansion logZ of the reference's large-N
// method, configuration_t::calc_chebyshev (src/configuration.cpp:94-205) with
// the coefficients of chebyshev::chebyshev_eval
// (include/fk_mc/chebyshev.hpp:16-66), for a batch of chains:
//
//   1. spectral bounds e_min, e_max of H (the reference asks ARPACK for the
//      smallest and largest eigenvalue): Lanczos on the sparse H, one CTA per
//      chain, until the extreme Ritz values stop moving;
//   2. the exact moments mu_m = Tr T_m(x) / N of x = (H - b) / a,
//      a = (e_max - e_min)/2, b = (e_max + e_min)/2, for m < M: the reference
//      forms the matrices T_m(x) for m <= M/2 by the three-term recursion and
//      the rest from Tr(T_{m-1} T_m) and Tr(T_m^2). Here every column j of
//      T_m(x) is built on its own by one warp, T_m(x) e_j = 2 x T_{m-1}(x) e_j
//      - T_{m-2}(x) e_j. That column vanishes outside the sites within m hops
//      of j, so the warp works on the ball of radius M/2 around j only (sites
//      in hop order, the ball's own CSR), in shared memory; it adds its
//      column's diagonal entry to Tr T_m and its dot products to Tr(T_{m-1}T_m)
//      and Tr(T_m^2);
//   3. per chain: the column sums in a fixed order, the moments assembled in
//      the reference's order, the coefficients c_m = moment_f(logz_f, m) by the
//      trapezoid rule on the Lobatto grid, logZ = c_0 + sum_m 2 c_m mu_m.
// Everything is FP64; every reduction has a fixed order.
#include "fkg_common.cuh"

namespace fkg {
namespace {

constexpr int kKpmThreads = 256;

// Eigenvalues of the k x k tridiagonal (al, b2 = squared off-diagonal) below
// x: the sign changes of the leading principal minors p_i of T - x, p_0 = 1,
// p_i = (al_i - x) p_{i-1} - b2_{i-1} p_{i-2} (Sylvester's inertia: the
// pivots p_i / p_{i-1} of the LDL^T factorisation of T - x). The minors are
// rescaled by a common power of two when they leave [2^-600, 2^600]; an exact
// zero counts as a tiny pivot of the opposite sign. No division on the chain
// of dependent operations (FP64 division is long on this part).
__device__ __forceinline__ int sturm_count(const double* al, const double* b2, int k, double x) {
    double pm = 1.0, p = al[0] - x;
    if (p == 0.0) p = -1e-300;
    int cnt = p < 0.0;
    for (int i = 1; i < k; ++i) {
        double q = fma(al[i] - x, p, -b2[i - 1] * pm);
        if (q == 0.0) q = p > 0.0 ? -1e-300 * fabs(p) : 1e-300 * fabs(p);
        cnt += (q < 0.0) != (p < 0.0);
        pm = p;
        p = q;
        const double ap = fabs(p);
        if (ap > 0x1p600 || ap < 0x1p-600) {
            const double sc = ap > 0x1p600 ? 0x1p-600 : 0x1p600;
            p *= sc;
            pm *= sc;
        }
    }
    return cnt;
}

// Smallest (largest = false) or largest eigenvalue of the tridiagonal in
// the bracket [lo, hi] by multisection on one warp: every round each lane
// counts at one of 32 interior points and the bracket shrinks to one
// sub-interval (5 bits a round), until it is a few ulps wide.
__device__ double warp_extreme(const double* al, const double* b2, int k, double lo, double hi, bool largest) {
    const int lane = threadIdx.x & 31;
    for (int round = 0; round < 48; ++round) {
        const double w = hi - lo;
        if (!(w > 4.5e-16 * fmax(fabs(lo), fabs(hi)))) break;
        const double x = lo + w * (double)(lane + 1) / 33.0;
        const int c = sturm_count(al, b2, k, x);
        const unsigned mask = __ballot_sync(0xffffffffu, c >= (largest ? k : 1));
        const int t = mask ? __ffs(mask) - 1 : 32;
        const double nlo = t == 0 ? lo : lo + w * (double)t / 33.0;
        const double nhi = t == 32 ? hi : lo + w * (double)(t + 1) / 33.0;
        lo = nlo;
        hi = nhi;
    }
    return 0.5 * (lo + hi);
}

// Block-wide FP64 sum with the cross-warp step done once (thread 0) and
// broadcast: on this part every warp-wide FP64 instruction occupies the
// narrow FP64 pipe, so the fewer the better. `red` needs blockDim/32 + 1 slots.
__device__ __forceinline__ double block_sum1(double x, double* red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    x = warp_sum(x);
    if (lane == 0) red[wid] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = red[0];
        for (int i = 1; i < nw; ++i) s += red[i];
        red[nw] = s;
    }
    __syncthreads();
    const double r = red[nw];
    __syncthreads();  // red is reused by the next call
    return r;
}

// Extreme eigenvalue of the tridiagonal, searched first in the narrow
// bracket prev +- span around the previous Ritz value (Sturm counts at its ends
// confirm that it holds the extreme eigenvalue), else in the Gershgorin bracket.
__device__ double ritz_extreme(const double* al, const double* b2, int k, double glo, double ghi, double prev,
                               double span, bool have_prev, bool largest) {
    if (have_prev) {
        const double lo = prev - span, hi = prev + span;
        const int lane = threadIdx.x & 31;
        int c = 0;
        if (lane < 2) c = sturm_count(al, b2, k, lane == 0 ? lo : hi);
        const int clo = __shfl_sync(0xffffffffu, c, 0), chi = __shfl_sync(0xffffffffu, c, 1);
        const bool holds = largest ? (clo <= k - 1 && chi >= k) : (clo == 0 && chi >= 1);
        if (holds) return warp_extreme(al, b2, k, lo, hi, largest);
    }
    return warp_extreme(al, b2, k, glo, ghi, largest);
}

// Lanczos on H = hopping + diag(d) from a fixed start vector, no
// re-orthogonalisation (the extreme Ritz values converge regardless); the
// three Lanczos vectors live in shared memory. Every 16 steps warp 0 and
// warp 1 compute the smallest and largest eigenvalue of the Lanczos
// tridiagonal; the run stops when both moved less than 1e-14 of the spectral
// width in two consecutive checks, when the Krylov space is exhausted, or at
// kmax (then kStatusNoConverge). Writes (e_min, e_max, a, b) and the number
// of Lanczos steps.
__global__ void __launch_bounds__(kKpmThreads)
kpm_bounds_kernel(const KpmDesc* __restrict__ descs, const double* __restrict__ diag, int kmax,
                  double4* __restrict__ ab, int* __restrict__ steps, int* __restrict__ status) {
    extern __shared__ __align__(16) double ksm[];
    const KpmDesc D = descs[blockIdx.x];
    const int n = D.n, tid = threadIdx.x;
    double* al = ksm;
    double* b2 = al + kmax;
    double* V0 = b2 + kmax;  // three vectors of spacing ld
    double* V1 = V0 + D.ld;
    double* V2 = V1 + D.ld;
    __shared__ double red[kKpmThreads / 32 + 1];
    __shared__ double ext[2];
    const double* dg = diag + D.v_off;
    double s2 = 0.0;
    for (int i = tid; i < n; i += blockDim.x) {
        const double x = (double)i * 0.6180339887498949;
        const double v = 0.5 + (x - floor(x));
        V1[i] = v;
        V0[i] = 0.0;
        s2 += v * v;
    }
    const double inv = 1.0 / sqrt(block_sum1(s2, red));
    for (int i = tid; i < n; i += blockDim.x) V1[i] *= inv;
    __syncthreads();
    double bprev = 0.0, hnorm = 0.0, tmin = 0.0, tmax = 0.0, dmin = 0.0, dmax = 0.0;
    int stable = 0, kdim = 0;
    bool have_prev = false, done = false;
    for (int k = 0; k < kmax && !done; ++k) {
        double dot = 0.0;
        for (int i = tid; i < n; i += blockDim.x) {
            double s = dg[i] * V1[i];
            for (int p = D.rowptr[i]; p < D.rowptr[i + 1]; ++p) s += D.val[p] * V1[D.col[p]];
            const double w = s - bprev * V0[i];
            V2[i] = w;
            dot += w * V1[i];
        }
        const double alpha = block_sum1(dot, red);
        double nn = 0.0;
        for (int i = tid; i < n; i += blockDim.x) {
            const double w = V2[i] - alpha * V1[i];
            V2[i] = w;
            nn += w * w;
        }
        const double beta = sqrt(block_sum1(nn, red));
        if (tid == 0) {
            al[k] = alpha;
            b2[k] = beta * beta;
        }
        hnorm = fmax(hnorm, fabs(alpha) + beta + bprev);
        kdim = k + 1;
        const bool exhausted = !(beta > 1e-12 * hnorm);
        if (!exhausted) {
            const double ib = 1.0 / beta;
            for (int i = tid; i < n; i += blockDim.x) V2[i] *= ib;
        }
        __syncthreads();  // al/b2 and the new vector visible to all
        double* t = V0;
        V0 = V1;
        V1 = V2;
        V2 = t;
        bprev = beta;
        if (exhausted || (kdim >= 32 && kdim % 16 == 0) || kdim == kmax) {
            // Gershgorin bracket of the kdim x kdim tridiagonal (its last
            // off-diagonal b2[kdim-1] is the residual, not part of it)
            double lo = 1e300, hi = -1e300;
            for (int i = tid; i < kdim; i += blockDim.x) {
                const double r = (i > 0 ? sqrt(b2[i - 1]) : 0.0) + (i + 1 < kdim ? sqrt(b2[i]) : 0.0);
                lo = fmin(lo, al[i] - r);
                hi = fmax(hi, al[i] + r);
            }
            lo = block_min(lo, red);
            hi = block_max(hi, red);
            const double width = hi - lo;
            lo -= 1e-14 * width + 1e-300;
            hi += 1e-14 * width + 1e-300;
            const int wid = tid >> 5;
            if (wid < 2) {
                const bool largest = wid == 1;
                const double prev = largest ? tmax : tmin;
                const double span = fmax(4.0 * (largest ? dmax : dmin), 1e-12 * width);
                const double e = ritz_extreme(al, b2, kdim, lo, hi, prev, span, have_prev, largest);
                if ((tid & 31) == 0) ext[wid] = e;
            }
            __syncthreads();
            const double nmin = ext[0], nmax = ext[1];
            __syncthreads();
            if (exhausted) {
                tmin = nmin;
                tmax = nmax;
                break;
            }
            const double tol = 1e-14 * fmax(nmax - nmin, fmax(fabs(nmin), fabs(nmax)));
            dmin = fabs(nmin - tmin);
            dmax = fabs(nmax - tmax);
            if (have_prev && dmin <= tol && dmax <= tol) {
                if (++stable >= 2) done = true;
            } else {
                stable = 0;
            }
            tmin = nmin;
            tmax = nmax;
            have_prev = true;
            if (!done && kdim == kmax && tid == 0) atomicOr(status, kStatusNoConverge);
        }
    }
    if (tid == 0) {
        if (!(tmax - tmin == tmax - tmin)) atomicOr(status, kStatusNaN);
        ab[blockIdx.x] = make_double4(tmin, tmax, (tmax - tmin) / 2., (tmax + tmin) / 2.);
        if (steps) steps[blockIdx.x] = kdim;
    }
}

// One warp per column j of T_m(x), m = 0..R, on the ball of radius R around
// j (local row 0 is j; rows in hop order, cnt[d] = rows within d hops).
// Writes, per column, tr[m] = (T_m(x))_jj, p1[m] = T_{m-1}(x)e_j . T_m(x)e_j and
// p2[m] = |T_m(x) e_j|^2 for m = 1..R at part[(v_off + j) * 3R + ...].
__global__ void kpm_moments_kernel(const KpmDesc* __restrict__ descs, const double* __restrict__ diag,
                                   const double4* __restrict__ ab, double* __restrict__ part, int wpc) {
    extern __shared__ __align__(16) double ksm[];
    const int c = blockIdx.y, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const KpmDesc D = descs[c];
    const int j = blockIdx.x * wpc + warp;
    if (j >= D.n) return;  // whole warps only; no block-wide barrier below
    const int R = D.R, nq = 3 * R;
    const int base = D.bptr[j], size = D.bptr[j + 1] - base;
    const int* cnt = D.bcnt + (size_t)j * (R + 1);
    double* vp = ksm + (size_t)warp * 3 * D.bmax;
    double* vc = vp + D.bmax;
    double* xd = vc + D.bmax;  // diagonal of x on the ball's rows
    const double4 s = ab[c];
    const double b = s.w, inv_a = 1.0 / s.z;
    const double* dg = diag + D.v_off;
    double* out = part + (size_t)(D.v_off + j) * nq;
    for (int r = lane; r < size; r += 32) {
        const int site = D.bsite[base + r];
        xd[r] = ((D.hdiag[site] + dg[site]) + -b) * inv_a;
        vp[r] = r == 0 ? 1.0 : 0.0;
        vc[r] = 0.0;
    }
    __syncwarp();
    // x restricted to local row r: diagonal (H_ss - b)/a, off-diagonal H/a
    // (the off-diagonal sum is scaled by 1/a once)
    auto xrow = [&](int r, const double* v) {
        const int g = base + r;
        double off = 0.0;
        for (int p = D.blrp[g]; p < D.blrp[g + 1]; ++p) off += D.blval[p] * v[D.blcol[p]];
        return fma(off, inv_a, xd[r] * v[r]);
    };
    // T_1(x) e_j = x e_j on the rows within one hop
    double d2 = 0.0;
    for (int r = lane; r < cnt[1]; r += 32) {
        const double v = xrow(r, vp);
        vc[r] = v;
        d2 += v * v;
    }
    __syncwarp();
    d2 = warp_sum(d2);
    if (lane == 0) {
        out[0] = vc[0];          // tr[1]
        out[R] = vc[0];          // p1[1] = e_j . x e_j
        out[2 * R] = d2;         // p2[1]
    }
    for (int m = 1; m < R; ++m) {
        // T_{m+1} e_j = 2 x T_m e_j - T_{m-1} e_j, written over T_{m-1} e_j
        const int rows = cnt[m + 1];
        for (int r = lane; r < rows; r += 32) vp[r] = 2.0 * xrow(r, vc) - vp[r];
        __syncwarp();
        double* t = vp;
        vp = vc;
        vc = t;
        double q1 = 0.0, q2 = 0.0;
        for (int r = lane; r < rows; r += 32) {
            q1 += vp[r] * vc[r];
            q2 += vc[r] * vc[r];
        }
        q1 = warp_sum(q1);
        q2 = warp_sum(q2);
        if (lane == 0) {
            out[m] = vc[0];
            out[R + m] = q1;
            out[2 * R + m] = q2;
        }
        __syncwarp();
    }
}

// Per chain: column sums, moments in the reference's order, coefficients,
// logZ. M moments (even), G grid points.
__global__ void __launch_bounds__(kKpmThreads)
kpm_final_kernel(const KpmDesc* __restrict__ descs, const double* __restrict__ part, const double4* __restrict__ ab,
                 const double* __restrict__ beta_c, int M, int G, double* __restrict__ mu_out,
                 double* __restrict__ logz, int* __restrict__ status) {
    extern __shared__ __align__(16) double ksm[];
    __shared__ double red[kKpmThreads / 32];
    const KpmDesc D = descs[blockIdx.x];
    const int R = D.R, nq = 3 * R, n = D.n, tid = threadIdx.x;
    double* sums = ksm;          // nq
    double* mu = sums + nq;      // M
    double* fg = mu + M;         // G: logz_f on the grid
    double* cm = fg + G;         // M: coefficients
    for (int q = 0; q < nq; ++q) {
        double s = 0.0;
        for (int j = tid; j < n; j += blockDim.x) s += part[(size_t)(D.v_off + j) * nq + q];
        s = block_sum(s, red);
        if (tid == 0) sums[q] = s;
    }
    const double4 st = ab[blockIdx.x];
    const double a = st.z, b = st.w, beta = beta_c[blockIdx.x], N = (double)n;
    const double step = 1.0 / (double)(G - 1);
    for (int i = tid; i < G; i += blockDim.x) {
        const double x = -cos(M_PI * ((double)i * step));
        fg[i] = N * log(1. + exp(-beta * (a * x + b)));
    }
    __syncthreads();
    if (tid == 0) {
        // src/configuration.cpp:124-183: mu_1 from Tr x, mu_m (m <= M/2) from
        // the recursion unless set before, mu_{2m-1}, mu_{2m} from products
        // once 2m-1 >= M/2
        const double trx = sums[0];
        for (int m = 0; m < M; ++m) mu[m] = nan("");
        mu[0] = 1.0;
        if (M > 1) mu[1] = trx / N;
        for (int m = 2; m <= M / 2; ++m) {
            if (mu[m] != mu[m]) mu[m] = sums[m - 1] / N;
            int k = 2 * m - 1;
            if (k < M && k >= M / 2) {
                mu[k] = (sums[R + m - 1] * 2. - trx) / N;
                if (k != M - 1) {
                    ++k;
                    mu[k] = sums[2 * R + m - 1] / N * 2. - 1.0;
                }
            }
        }
    }
    // c_m = moment_f(logz_f, m): trapezoid in the angle (include/fk_mc/chebyshev.hpp:38-56)
    for (int m = tid; m < M; m += blockDim.x) {
        double s = 0.0;
        for (int i = 0; i + 1 < G; ++i) {
            const double xi = -cos(M_PI * ((double)i * step)), xi1 = -cos(M_PI * ((double)(i + 1) * step));
            const double ti = cos((double)m * acos(xi)), ti1 = cos((double)m * acos(xi1));
            s += (fg[i + 1] * ti1 + fg[i] * ti) * ((double)(i + 1) * step - (double)i * step);
        }
        cm[m] = s * 0.5;
    }
    __syncthreads();
    if (tid == 0) {
        double s = cm[0];
        for (int m = 1; m < M; ++m) s += 2. * cm[m] * mu[m];
        logz[blockIdx.x] = s;
        if (!(s - s == 0.0)) atomicOr(status, kStatusNaN);
        if (mu_out)
            for (int m = 0; m < M; ++m) mu_out[(size_t)blockIdx.x * M + m] = mu[m];
    }
}

}  // namespace

size_t kpm_moment_smem_bytes(int bmax, int wpc) { return sizeof(double) * 3 * (size_t)bmax * wpc; }

int kpm_warps_per_cta(int bmax) {
    const size_t per = sizeof(double) * 3 * (size_t)bmax;
    int w = (int)((96 * 1024) / per);
    return w < 1 ? 1 : (w > 8 ? 8 : w);
}

cudaError_t launch_kpm(const KpmDesc* d_kdesc, int batch, int max_n, int max_ld, int max_bmax, int R, int M, int G,
                       int kmax, const double* d_diag, const double* d_beta, double4* d_ab, int* d_steps,
                       double* d_part, double* d_mu, double* d_logz, int* d_status, cudaStream_t st) {
    if (batch <= 0) return cudaSuccess;
    if (batch > 65535) return cudaErrorInvalidValue;  // grid y limit of the moment kernel
    cudaError_t err;
    const size_t sm_b = sizeof(double) * (2 * (size_t)kmax + 3 * (size_t)max_ld);
    if ((err = cudaFuncSetAttribute(kpm_bounds_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_b))) return err;
    kpm_bounds_kernel<<<batch, kKpmThreads, sm_b, st>>>(d_kdesc, d_diag, kmax, d_ab, d_steps, d_status);
    if ((err = cudaGetLastError())) return err;
    const int wpc = kpm_warps_per_cta(max_bmax);
    const size_t sm_m = kpm_moment_smem_bytes(max_bmax, wpc);
    if ((err = cudaFuncSetAttribute(kpm_moments_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_m))) return err;
    kpm_moments_kernel<<<dim3((max_n + wpc - 1) / wpc, batch), 32 * wpc, sm_m, st>>>(d_kdesc, d_diag, d_ab, d_part,
                                                                                      wpc);
    if ((err = cudaGetLastError())) return err;
    const size_t sm_f = sizeof(double) * (3 * (size_t)R + 2 * (size_t)M + (size_t)G);
    if ((err = cudaFuncSetAttribute(kpm_final_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_f))) return err;
    kpm_final_kernel<<<batch, kKpmThreads, sm_f, st>>>(d_kdesc, d_part, d_ab, d_beta, M, G, d_mu, d_logz, d_status);
    return cudaGetLastError();
}

}  // namespace fkg
