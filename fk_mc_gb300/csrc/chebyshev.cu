// chebyshev.cu — the Chebyshev-expansion logZ of the reference's large-N
// method, configuration_t::calc_chebyshev (src/configuration.cpp:94-205) with
// the coefficients of chebyshev::chebyshev_eval
// (include/fk_mc/chebyshev.hpp:16-66), for a batch of chains:
//
//   1. spectral bounds e_min, e_max of H (the reference asks ARPACK for the
//      smallest and largest eigenvalue): Lanczos on the sparse H, one CTA per
//      chain, in double-float, until the extreme Ritz values stop moving;
//   2. the exact moments mu_m = Tr T_m(x) / N of x = (H - b) / a,
//      a = (e_max - e_min)/2, b = (e_max + e_min)/2, for m < M: the reference
//      forms the matrices T_m(x) for m <= M/2 by the three-term recursion and
//      the rest from Tr(T_{m-1} T_m) and Tr(T_m^2). Here every column j of
//      T_m(x) is built on its own by one warp, T_m(x) e_j = 2 x T_{m-1}(x) e_j
//      - T_{m-2}(x) e_j. That column vanishes outside the sites within m hops
//      of j, so the warp works on the ball of radius M/2 around j only (sites
//      in hop order, the ball's own CSR), in shared memory, in double-float
//      (FP32 pairs: GB300's FP32 pipe is ~60x its FP64 pipe); it adds its
//      column's diagonal entry to Tr T_m and its dot products to Tr(T_{m-1}T_m)
//      and Tr(T_m^2);
//   3. per chain: the column sums in a fixed order, the moments assembled in
//      the reference's order, the coefficients c_m = moment_f(logz_f, m) by the
//      trapezoid rule on the Lobatto grid, logZ = c_0 + sum_m 2 c_m mu_m.
// The Lanczos vectors and the column recursion are double-float (FP32 pairs,
// ~48 bits), the final step FP64; every reduction has a fixed order.
#include "fkg_common.cuh"

namespace fkg {
namespace {

constexpr int kKpmThreads = 256;

// Eigenvalues of the k x k tridiagonal (al, b2 = squared off-diagonal, as
// FP32 pairs) below x: the sign changes of the leading principal minors p_i
// of T - x, p_0 = 1, p_i = (al_i - x) p_{i-1} - b2_{i-1} p_{i-2} (Sylvester's
// inertia: the pivots p_i / p_{i-1} of the LDL^T factorisation of T - x), in
// double-float. The minors are rescaled by a common power of two when they
// leave [2^-60, 2^60]; an exact zero counts as a tiny pivot of the opposite
// sign. No division, no FP64: GB300's FP64 pipe is ~60x narrower than FP32.
__device__ __forceinline__ int sturm_count(const dfl* al, const dfl* b2, int k, dfl x) {
    const dfl nx = {-x.hi, -x.lo};
    dfl pm = {1.0f, 0.0f}, p = df_add(al[0], nx);
    if (p.hi == 0.0f) p = {-1e-30f, 0.0f};
    int cnt = p.hi < 0.0f;
    for (int i = 1; i < k; ++i) {
        const dfl u = df_mul(df_add(al[i], nx), p), v = df_mul(b2[i - 1], pm);
        dfl q = df_add(u, {-v.hi, -v.lo});
        if (q.hi == 0.0f) q = {p.hi > 0.0f ? -1e-30f * fabsf(p.hi) : 1e-30f * fabsf(p.hi), 0.0f};
        cnt += (q.hi < 0.0f) != (p.hi < 0.0f);
        pm = p;
        p = q;
        const float ap = fabsf(p.hi);
        if (ap > 0x1p60f || ap < 0x1p-60f) {
            const float sc = ap > 0x1p60f ? 0x1p-60f : 0x1p60f;
            p = {p.hi * sc, p.lo * sc};
            pm = {pm.hi * sc, pm.lo * sc};
        }
    }
    return cnt;
}

// Smallest (largest = false) or largest eigenvalue of the tridiagonal in
// the bracket [lo, hi] by multisection on one warp: every round each lane
// counts at one of 32 interior points and the bracket shrinks to one
// sub-interval (5 bits a round), until it is as narrow as the double-float
// counts resolve (4e-14 relative).
__device__ double warp_extreme(const dfl* al, const dfl* b2, int k, double lo, double hi, bool largest) {
    const int lane = threadIdx.x & 31;
    for (int round = 0; round < 40; ++round) {
        const double w = hi - lo;
        if (!(w > 4e-14 * fmax(fabs(lo), fabs(hi)))) break;
        const double x = lo + w * (double)(lane + 1) / 33.0;
        const int c = sturm_count(al, b2, k, df_of(x));
        const unsigned mask = __ballot_sync(0xffffffffu, c >= (largest ? k : 1));
        const int t = mask ? __ffs(mask) - 1 : 32;
        const double nlo = t == 0 ? lo : lo + w * (double)t / 33.0;
        const double nhi = t == 32 ? hi : lo + w * (double)(t + 1) / 33.0;
        lo = nlo;
        hi = nhi;
    }
    return 0.5 * (lo + hi);
}

// Extreme eigenvalue of the tridiagonal, searched first in the narrow
// bracket prev +- span around the previous Ritz value (Sturm counts at its ends
// confirm that it holds the extreme eigenvalue), else in the Gershgorin bracket.
__device__ double ritz_extreme(const dfl* al, const dfl* b2, int k, double glo, double ghi, double prev,
                               double span, bool have_prev, bool largest) {
    if (have_prev) {
        const double lo = prev - span, hi = prev + span;
        const int lane = threadIdx.x & 31;
        int c = 0;
        if (lane < 2) c = sturm_count(al, b2, k, df_of(lane == 0 ? lo : hi));
        const int clo = __shfl_sync(0xffffffffu, c, 0), chi = __shfl_sync(0xffffffffu, c, 1);
        const bool holds = largest ? (clo <= k - 1 && chi >= k) : (clo == 0 && chi >= 1);
        if (holds) return warp_extreme(al, b2, k, lo, hi, largest);
    }
    return warp_extreme(al, b2, k, glo, ghi, largest);
}

// Block-wide double-float sum, returned as FP64 to every thread; the
// cross-warp step is done once (thread 0). `red` needs blockDim/32 + 1 slots.
__device__ __forceinline__ double block_sum_df(dfl x, float2* red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    x = warp_sum_df(x);
    if (lane == 0) red[wid] = make_float2(x.hi, x.lo);
    __syncthreads();
    if (threadIdx.x == 0) {
        dfl s = {red[0].x, red[0].y};
        for (int i = 1; i < nw; ++i) s = df_add(s, {red[i].x, red[i].y});
        red[nw] = make_float2(s.hi, s.lo);
    }
    __syncthreads();
    const double r = (double)red[nw].x + (double)red[nw].y;
    __syncthreads();  // red is reused by the next call
    return r;
}

// Lanczos on H = hopping + diag(d) from a fixed start vector, no
// re-orthogonalisation (the extreme Ritz values converge regardless), in
// double-float with the three Lanczos vectors in shared memory. Every 16
// steps warp 0 and warp 1 compute the smallest and largest eigenvalue of the
// Lanczos tridiagonal; the run stops when both moved less than 1e-13 of the
// spectral width in two consecutive checks, when the Krylov space is
// exhausted, or at kmax (then kStatusNoConverge). Writes (e_min, e_max, a, b)
// and the number of Lanczos steps.
__global__ void __launch_bounds__(kKpmThreads)
kpm_bounds_kernel(const KpmDesc* __restrict__ descs, const double* __restrict__ diag, int kmax,
                  KpmAB* __restrict__ ab, int* __restrict__ steps, int* __restrict__ status) {
    extern __shared__ __align__(16) double ksm[];
    const KpmDesc D = descs[blockIdx.x];
    const int n = D.n, tid = threadIdx.x;
    dfl* al = reinterpret_cast<dfl*>(ksm);
    dfl* b2 = al + kmax;
    dfl* V0 = b2 + kmax;  // three vectors and the diagonal, spacing ld
    dfl* V1 = V0 + D.ld;
    dfl* V2 = V1 + D.ld;
    dfl* dgd = V2 + D.ld;
    __shared__ float2 red[kKpmThreads / 32 + 1];
    __shared__ double redd[kKpmThreads / 32];
    __shared__ double ext[2];
    const double* dg = diag + D.v_off;
    dfl s2 = {0.0f, 0.0f};
    for (int i = tid; i < n; i += blockDim.x) {
        const double x = (double)i * 0.6180339887498949;
        const dfl v = df_of(0.5 + (x - floor(x)));
        V1[i] = v;
        V0[i] = {0.0f, 0.0f};
        dgd[i] = df_of(dg[i]);
        s2 = df_add(s2, df_mul(v, v));
    }
    const dfl inv = df_of(1.0 / sqrt(block_sum_df(s2, red)));
    for (int i = tid; i < n; i += blockDim.x) V1[i] = df_mul(V1[i], inv);
    __syncthreads();
    double bprev = 0.0, hnorm = 0.0, tmin = 0.0, tmax = 0.0, dmin = 0.0, dmax = 0.0;
    int stable = 0, kdim = 0;
    bool have_prev = false, done = false;
    for (int k = 0; k < kmax && !done; ++k) {
        const dfl nb = df_of(-bprev);
        dfl dot = {0.0f, 0.0f};
        for (int i = tid; i < n; i += blockDim.x) {
            dfl sacc = df_mul(dgd[i], V1[i]);
            for (int p = D.rowptr[i]; p < D.rowptr[i + 1]; ++p) {
                const float2 h = D.valf[p];
                sacc = df_add(sacc, df_mul({h.x, h.y}, V1[D.col[p]]));
            }
            const dfl w = df_add(sacc, df_mul(nb, V0[i]));
            V2[i] = w;
            dot = df_add(dot, df_mul(w, V1[i]));
        }
        const double alpha = block_sum_df(dot, red);
        const dfl na = df_of(-alpha);
        dfl nn = {0.0f, 0.0f};
        for (int i = tid; i < n; i += blockDim.x) {
            const dfl w = df_add(V2[i], df_mul(na, V1[i]));
            V2[i] = w;
            nn = df_add(nn, df_mul(w, w));
        }
        const double beta = sqrt(block_sum_df(nn, red));
        if (tid == 0) {
            al[k] = df_of(alpha);
            b2[k] = df_of(beta * beta);
        }
        hnorm = fmax(hnorm, fabs(alpha) + beta + bprev);
        kdim = k + 1;
        const bool exhausted = !(beta > 1e-11 * hnorm);
        if (!exhausted) {
            const dfl ib = df_of(1.0 / beta);
            for (int i = tid; i < n; i += blockDim.x) V2[i] = df_mul(V2[i], ib);
        }
        __syncthreads();  // al/b2 and the new vector visible to all
        dfl* t = V0;
        V0 = V1;
        V1 = V2;
        V2 = t;
        bprev = beta;
        if (exhausted || (kdim >= 32 && kdim % 16 == 0) || kdim == kmax) {
            // Gershgorin bracket of the kdim x kdim tridiagonal (its last
            // off-diagonal b2[kdim-1] is the residual, not part of it)
            double lo = 1e300, hi = -1e300;
            for (int i = tid; i < kdim; i += blockDim.x) {
                const double r = (i > 0 ? sqrt(df_val(b2[i - 1])) : 0.0) + (i + 1 < kdim ? sqrt(df_val(b2[i])) : 0.0);
                const double a = df_val(al[i]);
                lo = fmin(lo, a - r);
                hi = fmax(hi, a + r);
            }
            lo = block_min(lo, redd);
            hi = block_max(hi, redd);
            const double width = hi - lo;
            lo -= 1e-12 * width + 1e-300;
            hi += 1e-12 * width + 1e-300;
            const int wid = tid >> 5;
            if (wid < 2) {
                const bool largest = wid == 1;
                const double prev = largest ? tmax : tmin;
                const double span = fmax(4.0 * (largest ? dmax : dmin), 1e-11 * width);
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
            const double tol = 1e-13 * fmax(nmax - nmin, fmax(fabs(nmin), fabs(nmax)));
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
        ab[blockIdx.x] = KpmAB{tmin, tmax, (tmax - tmin) / 2., (tmax + tmin) / 2.};
        if (steps) steps[blockIdx.x] = kdim;
    }
}

// One warp per column j of T_m(x), m = 0..R, on the ball of radius R around
// j (local row 0 is j; rows in hop order, cnt[d] = rows within d hops).
// Writes, per column, tr[m] = (T_m(x))_jj, p1[m] = T_{m-1}(x)e_j . T_m(x)e_j and
// p2[m] = |T_m(x) e_j|^2 for m = 1..R at part[(v_off + j) * 3R + ...].
__global__ void kpm_moments_kernel(const KpmDesc* __restrict__ descs, const double* __restrict__ diag,
                                   const KpmAB* __restrict__ ab, double* __restrict__ part, int wpc) {
    extern __shared__ __align__(16) double ksm[];
    const int c = blockIdx.y, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const KpmDesc D = descs[c];
    const int j = blockIdx.x * wpc + warp;
    if (j >= D.n) return;  // whole warps only; no block-wide barrier below
    const int R = D.R, nq = 3 * R;
    const int base = D.bptr[j], size = D.bptr[j + 1] - base;
    const int* cnt = D.bcnt + (size_t)j * (R + 1);
    // column vectors and the diagonal of x on the ball's rows, as FP32 pairs
    dfl* vp = reinterpret_cast<dfl*>(ksm) + (size_t)warp * 3 * D.bmax;
    dfl* vc = vp + D.bmax;
    dfl* xd = vc + D.bmax;
    const KpmAB s = ab[c];
    const double b = s.b, inv_a = 1.0 / s.a;
    const dfl ia = df_of(inv_a);
    const double* dg = diag + D.v_off;
    double* out = part + (size_t)(D.v_off + j) * nq;
    for (int r = lane; r < size; r += 32) {
        const int site = D.bsite[base + r];
        xd[r] = df_of(((D.hdiag[site] + dg[site]) + -b) * inv_a);
        vp[r] = {r == 0 ? 1.0f : 0.0f, 0.0f};
        vc[r] = {0.0f, 0.0f};
    }
    __syncwarp();
    // x restricted to local row r: diagonal (H_ss - b)/a, off-diagonal H/a
    // (the off-diagonal sum is scaled by 1/a once), in double-float
    auto xrow = [&](int r, const dfl* v) {
        const int g = base + r;
        dfl off = {0.0f, 0.0f};
        for (int p = D.blrp[g]; p < D.blrp[g + 1]; ++p) {
            const float2 h = D.blv2[p];
            off = df_add(off, df_mul({h.x, h.y}, v[D.blcol[p]]));
        }
        return df_add(df_mul(off, ia), df_mul(xd[r], v[r]));
    };
    // T_1(x) e_j = x e_j on the rows within one hop
    dfl d2 = {0.0f, 0.0f};
    for (int r = lane; r < cnt[1]; r += 32) {
        const dfl v = xrow(r, vp);
        vc[r] = v;
        d2 = df_add(d2, df_mul(v, v));
    }
    __syncwarp();
    d2 = warp_sum_df(d2);
    if (lane == 0) {
        const double t1 = df_val(vc[0]);
        out[0] = t1;             // tr[1]
        out[R] = t1;             // p1[1] = e_j . x e_j
        out[2 * R] = df_val(d2); // p2[1]
    }
    for (int m = 1; m < R; ++m) {
        // T_{m+1} e_j = 2 x T_m e_j - T_{m-1} e_j, written over T_{m-1} e_j
        const int rows = cnt[m + 1];
        for (int r = lane; r < rows; r += 32) {
            const dfl x = xrow(r, vc), o = vp[r];
            vp[r] = df_add({2.0f * x.hi, 2.0f * x.lo}, {-o.hi, -o.lo});
        }
        __syncwarp();
        dfl* t = vp;
        vp = vc;
        vc = t;
        dfl q1 = {0.0f, 0.0f}, q2 = {0.0f, 0.0f};
        for (int r = lane; r < rows; r += 32) {
            q1 = df_add(q1, df_mul(vp[r], vc[r]));
            q2 = df_add(q2, df_mul(vc[r], vc[r]));
        }
        q1 = warp_sum_df(q1);
        q2 = warp_sum_df(q2);
        if (lane == 0) {
            out[m] = df_val(vc[0]);
            out[R + m] = df_val(q1);
            out[2 * R + m] = df_val(q2);
        }
        __syncwarp();
    }
}

// Per chain: column sums, moments in the reference's order, coefficients,
// logZ. M moments (even), G grid points.
__global__ void __launch_bounds__(kKpmThreads)
kpm_final_kernel(const KpmDesc* __restrict__ descs, const double* __restrict__ part, const KpmAB* __restrict__ ab,
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
    const KpmAB st = ab[blockIdx.x];
    const double a = st.a, b = st.b, beta = beta_c[blockIdx.x], N = (double)n;
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
                       int kmax, const double* d_diag, const double* d_beta, KpmAB* d_ab, int* d_steps,
                       double* d_part, double* d_mu, double* d_logz, int* d_status, cudaStream_t st) {
    if (batch <= 0) return cudaSuccess;
    if (batch > 65535) return cudaErrorInvalidValue;  // grid y limit of the moment kernel
    cudaError_t err;
    const size_t sm_b = sizeof(dfl) * (2 * (size_t)kmax + 4 * (size_t)max_ld);
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
