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

// Eigenvalues of the k x k tridiagonal (al, b2 = squared off-diagonal) below x.
__device__ __forceinline__ int sturm_count(const double* al, const double* b2, int k, double x, double pivmin) {
    double d = al[0] - x;
    if (fabs(d) < pivmin) d = -pivmin;
    int cnt = d < 0.0;
    for (int i = 1; i < k; ++i) {
        d = (al[i] - x) - b2[i - 1] / d;
        if (fabs(d) < pivmin) d = -pivmin;
        cnt += d < 0.0;
    }
    return cnt;
}

// Smallest (largest = false) or largest eigenvalue of the tridiagonal inside
// [lo, hi] by multisection: every round each thread counts at one of
// blockDim.x interior points and the bracket shrinks to one sub-interval.
__device__ double tri_extreme(const double* al, const double* b2, int k, double lo, double hi, double pivmin,
                              bool largest, int* sh_t) {
    const int B = blockDim.x;
    for (int round = 0; round < 12; ++round) {
        const double w = hi - lo;
        if (!(w > 4.5e-16 * fmax(fabs(lo), fabs(hi)))) break;
        const double x = lo + w * (double)(threadIdx.x + 1) / (double)(B + 1);
        const int c = sturm_count(al, b2, k, x, pivmin);
        if (threadIdx.x == 0) *sh_t = B;
        __syncthreads();
        if (c >= (largest ? k : 1)) atomicMin(sh_t, (int)threadIdx.x);
        __syncthreads();
        const int t = *sh_t;
        __syncthreads();
        const double nlo = t == 0 ? lo : lo + w * (double)t / (double)(B + 1);
        const double nhi = t == B ? hi : lo + w * (double)(t + 1) / (double)(B + 1);
        lo = nlo;
        hi = nhi;
    }
    return 0.5 * (lo + hi);
}

// Lanczos on H = hopping + diag(d) from a fixed start vector, no
// re-orthogonalisation (the extreme Ritz values converge regardless). Every
// 32 steps the extreme eigenvalues of the Lanczos tridiagonal are computed;
// the run stops when both moved less than 1e-14 of the spectral width in two
// consecutive checks, when the Krylov space is exhausted, or at kmax (then
// kStatusNoConverge). Writes (e_min, e_max, a, b).
__global__ void __launch_bounds__(kKpmThreads)
kpm_bounds_kernel(const KpmDesc* __restrict__ descs, const double* __restrict__ diag, double* __restrict__ vec,
                  int kmax, double4* __restrict__ ab, int* __restrict__ status) {
    extern __shared__ __align__(16) double ksm[];
    double* al = ksm;
    double* b2 = al + kmax;
    __shared__ double red[kKpmThreads / 32];
    __shared__ int sh_t;
    const KpmDesc D = descs[blockIdx.x];
    const int n = D.n, tid = threadIdx.x;
    const double* dg = diag + D.v_off;
    double* V0 = vec + 3 * D.v_off;  // 3 vectors of spacing ld per chain
    double* V1 = V0 + D.ld;
    double* V2 = V1 + D.ld;
    double s2 = 0.0;
    for (int i = tid; i < n; i += blockDim.x) {
        const double x = (double)i * 0.6180339887498949;
        const double v = 0.5 + (x - floor(x));
        V1[i] = v;
        V0[i] = 0.0;
        s2 += v * v;
    }
    const double inv = 1.0 / sqrt(block_sum(s2, red));
    for (int i = tid; i < n; i += blockDim.x) V1[i] *= inv;
    __syncthreads();
    double bprev = 0.0, hnorm = 0.0, tmin = 0.0, tmax = 0.0, pmin = 0.0, pmax = 0.0;
    int stable = 0, kdim = 0, have_prev = 0;
    bool done = false;
    for (int k = 0; k < kmax && !done; ++k) {
        double dot = 0.0;
        for (int i = tid; i < n; i += blockDim.x) {
            double s = dg[i] * V1[i];
            for (int p = D.rowptr[i]; p < D.rowptr[i + 1]; ++p) s += D.val[p] * V1[D.col[p]];
            const double w = s - bprev * V0[i];
            V2[i] = w;
            dot += w * V1[i];
        }
        const double alpha = block_sum(dot, red);
        double nn = 0.0;
        for (int i = tid; i < n; i += blockDim.x) {
            const double w = V2[i] - alpha * V1[i];
            V2[i] = w;
            nn += w * w;
        }
        const double beta = sqrt(block_sum(nn, red));
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
        if (exhausted || kdim % 32 == 0 || kdim == kmax) {
            // Gershgorin bracket of the kdim x kdim tridiagonal (its last
            // off-diagonal b2[kdim-1] is the residual, not part of it)
            double lo = 1e300, hi = -1e300, bmax2 = 0.0;
            for (int i = tid; i < kdim; i += blockDim.x) {
                const double r = (i > 0 ? sqrt(b2[i - 1]) : 0.0) + (i + 1 < kdim ? sqrt(b2[i]) : 0.0);
                lo = fmin(lo, al[i] - r);
                hi = fmax(hi, al[i] + r);
                if (i + 1 < kdim) bmax2 = fmax(bmax2, b2[i]);
            }
            lo = block_min(lo, red);
            hi = block_max(hi, red);
            bmax2 = block_max(bmax2, red);
            const double width = hi - lo;
            lo -= 1e-14 * width + 1e-300;
            hi += 1e-14 * width + 1e-300;
            const double pivmin = 1e-300 * fmax(1.0, bmax2);
            tmin = tri_extreme(al, b2, kdim, lo, hi, pivmin, false, &sh_t);
            tmax = tri_extreme(al, b2, kdim, lo, hi, pivmin, true, &sh_t);
            if (exhausted) break;
            const double tol = 1e-14 * fmax(tmax - tmin, fmax(fabs(tmin), fabs(tmax)));
            if (have_prev && fabs(tmin - pmin) <= tol && fabs(tmax - pmax) <= tol) {
                if (++stable >= 2) done = true;
            } else {
                stable = 0;
            }
            pmin = tmin;
            pmax = tmax;
            have_prev = 1;
            if (!done && kdim == kmax && tid == 0) atomicOr(status, kStatusNoConverge);
        }
    }
    if (tid == 0) {
        if (!(tmax - tmin == tmax - tmin)) atomicOr(status, kStatusNaN);
        ab[blockIdx.x] = make_double4(tmin, tmax, (tmax - tmin) / 2., (tmax + tmin) / 2.);
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
    double* vp = ksm + (size_t)warp * 2 * D.bmax;
    double* vc = vp + D.bmax;
    const double4 s = ab[c];
    const double a = s.z, b = s.w;
    const double* dg = diag + D.v_off;
    double* out = part + (size_t)(D.v_off + j) * nq;
    for (int r = lane; r < size; r += 32) {
        vp[r] = r == 0 ? 1.0 : 0.0;
        vc[r] = 0.0;
    }
    __syncwarp();
    // x restricted to local row r: diagonal (H_ss - b)/a, off-diagonal H/a
    auto xrow = [&](int r, const double* v) {
        const int g = base + r, site = D.bsite[g];
        double acc = ((D.hdiag[site] + dg[site]) + -b) / a * v[r];
        for (int p = D.blrp[g]; p < D.blrp[g + 1]; ++p) acc += (D.blval[p] / a) * v[D.blcol[p]];
        return acc;
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

size_t kpm_moment_smem_bytes(int bmax, int wpc) { return sizeof(double) * 2 * (size_t)bmax * wpc; }

int kpm_warps_per_cta(int bmax) {
    const size_t per = sizeof(double) * 2 * (size_t)bmax;
    int w = (int)((96 * 1024) / per);
    return w < 1 ? 1 : (w > 8 ? 8 : w);
}

cudaError_t launch_kpm(const KpmDesc* d_kdesc, int batch, int max_n, int max_bmax, int R, int M, int G, int kmax,
                       const double* d_diag, const double* d_beta, double* d_vec, double4* d_ab, double* d_part,
                       double* d_mu, double* d_logz, int* d_status, cudaStream_t st) {
    if (batch <= 0) return cudaSuccess;
    if (batch > 65535) return cudaErrorInvalidValue;  // grid y limit of the moment kernel
    cudaError_t err;
    const size_t sm_b = sizeof(double) * 2 * (size_t)kmax;
    if ((err = cudaFuncSetAttribute(kpm_bounds_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_b))) return err;
    kpm_bounds_kernel<<<batch, kKpmThreads, sm_b, st>>>(d_kdesc, d_diag, d_vec, kmax, d_ab, d_status);
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
