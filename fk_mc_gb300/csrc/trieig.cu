// trieig.cu — eigenvalues (and, for the mixed path and calc_ed(true),
// eigenvectors) of the symmetric tridiagonal T = tridiag(e, d, e).
//
// Replaces the tridiagonal QR half of Eigen::SelfAdjointEigenSolver used at
// src/configuration.cpp:213. The eigenvalues are computed in FP64 and come
// out ascending (src/measures/spectrum.cpp:13-21 relies on the order).
//
// GB300's FP64 pipe runs at about 1/58 of its FP32 pipe, so the eigenvalue
// search spends as little FP64 work as possible while staying FP64-accurate:
//   1. FP32 bisection on Sturm counts of the FP32-rounded T isolates each
//      eigenvalue to an interval of width ~ 4 eps32 ||T||.  Kahan's analysis
//      of the Sturm recurrence makes each FP32 count exact for a matrix
//      within a few eps32 ||T|| of T, so widening by 16 eps32 ||T|| gives a
//      bracket of the FP64 eigenvalue;
//   2. where the widened brackets of the neighbouring indices j-1 and j+1
//      stay clear of it, that bracket holds exactly lambda_j; elsewhere (block
//      edges, eigenvalues closer than the FP32 resolution) two FP64 Sturm
//      counts verify it (a failed check falls back to the Gershgorin
//      interval);
//   3. if the bracket holds exactly one eigenvalue, a safeguarded Newton
//      iteration on the characteristic polynomial p_n(x) = det(T - x I)
//      (three-term recurrence for p and p', rescaled by powers of two, no
//      divisions) converges quadratically to full FP64 accuracy; the sign of
//      p_n at the bracket ends is (-1)^count, so every iterate keeps a valid
//      bracket and falls back to bisection when Newton leaves it;
//   4. otherwise (eigenvalues closer than the FP32 resolution) FP64 bisection
//      on Sturm counts finishes the job.
// One thread per eigenvalue index; d and e of the chain sit in shared memory.
#include <cfloat>

#include "fkg_common.cuh"

namespace fkg {
namespace {

constexpr int kEigThreads = 128;

__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// FP32 Sturm count: eigenvalues of T below x, from q_0 = d_0 - x,
// q_k = (d_k - x) - e_{k-1}^2 / q_{k-1}, counting the q_k with the sign bit
// set. de[k] = (d_k, e_{k-1}^2). The approximate reciprocal perturbs each
// e^2 by a relative 2^-22 at most. A zero q_k makes q_{k+1} an infinity of
// the opposite sign and q_{k+2} = d_{k+2} - x again (IEEE arithmetic; e^2 is
// floored at FLT_MIN so that 0 x inf cannot occur), which counts exactly one
// negative between them for either sign of the zero.
__device__ __forceinline__ int count32(const float2* __restrict__ de, int n, float x) {
    float q = de[0].x - x;
    int c = __float_as_uint(q) >> 31;
    for (int i = 1; i < n; ++i) {
        const float2 v = de[i];
        q = fmaf(-v.y, rcp_approx(q), v.x - x);
        c += __float_as_uint(q) >> 31;
    }
    return c;
}

// Number of eigenvalues below x: sign changes of the Sturm sequence
// p_0 = 1, p_k = (d_k - x) p_{k-1} - e_{k-1}^2 p_{k-2} (division-free
// projective form of q_k = p_k / p_{k-1}; rescaled by powers of two, which
// keeps every sign). A zero p_k is replaced by -pivmin p_{k-1}, i.e.
// q_k = -pivmin, the usual pivot floor of Sturm counting.
__device__ __forceinline__ int count64(const double* __restrict__ d, const double* __restrict__ e2, int n, double x,
                                       double pivmin) {
    double p0 = 1.0;
    double p1 = d[0] - x;
    if (p1 == 0.0) p1 = -pivmin;
    int c = p1 < 0.0;
    for (int i = 1; i < n; ++i) {
        double p2 = fma(d[i] - x, p1, -e2[i - 1] * p0);
        if (p2 == 0.0) p2 = -pivmin * p1;
        c += (__double2hiint(p2) ^ __double2hiint(p1)) < 0;
        p0 = p1;
        p1 = p2;
        if ((i & 7) == 0) {
            const double m = fmax(fabs(p0), fabs(p1));
            if (m > 0x1p400) { p0 *= 0x1p-400; p1 *= 0x1p-400; }
            else if (m < 0x1p-400) { p0 *= 0x1p400; p1 *= 0x1p400; }
        }
    }
    return c;
}

// p_n(x) and p_n'(x) up to a common positive power-of-two scale.
__device__ __forceinline__ void charpoly(const double* __restrict__ d, const double* __restrict__ e2, int n,
                                         double x, double& p, double& dp) {
    double p0 = 1.0, dp0 = 0.0;          // p_{k-1}, p'_{k-1}
    double p1 = d[0] - x, dp1 = -1.0;    // p_k, p'_k
    for (int i = 1; i < n; ++i) {
        const double t = d[i] - x, b = e2[i - 1];
        const double p2 = fma(t, p1, -b * p0);
        const double dp2 = fma(t, dp1, fma(-b, dp0, -p1));
        p0 = p1; dp0 = dp1; p1 = p2; dp1 = dp2;
        if ((i & 7) == 0) {
            const double m = fmax(fabs(p1), fabs(dp1));
            if (m > 0x1p400) { p0 *= 0x1p-400; dp0 *= 0x1p-400; p1 *= 0x1p-400; dp1 *= 0x1p-400; }
            else if (m < 0x1p-400 && m > 0.0) { p0 *= 0x1p400; dp0 *= 0x1p400; p1 *= 0x1p400; dp1 *= 0x1p400; }
        }
    }
    p = p1;
    dp = dp1;
}

struct TriShared {
    double* d;
    double* e2;
    float* d32;
    float* e232;  // e_i^2 in FP32, floored at FLT_MIN (i < n - 1)
    float2* de;   // (d_i, e_{i-1}^2) for the FP32 counts
};

// shared-memory layout of one chain's tridiagonal; `extra` floats follow
__device__ __forceinline__ TriShared tri_shared(double* sm, int ld) {
    float* f = (float*)(sm + 2 * ld);
    return TriShared{sm, sm + ld, f, f + ld, (float2*)(f + 2 * ld)};
}

// Loads d, e^2 (FP64 and FP32 copies) of chain D into shared memory and
// returns the Gershgorin interval, max e^2 and the norm estimate.
__device__ void load_tridiag(const ChainDesc& D, const double* __restrict__ dd, const double* __restrict__ ee,
                             TriShared S, double& gl, double& gu, double& emax2) {
    const int n = D.n;
    __shared__ double red[3][kEigThreads / 32];
    gl = DBL_MAX; gu = -DBL_MAX; emax2 = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double di = dd[D.v_off + i];
        const double el = i > 0 ? fabs(ee[D.v_off + i - 1]) : 0.0;
        const double er = i + 1 < n ? fabs(ee[D.v_off + i]) : 0.0;
        S.d[i] = di;
        S.e2[i] = er * er;
        S.d32[i] = (float)di;
        S.e232[i] = i + 1 < n ? fmaxf((float)(er * er), FLT_MIN) : 0.f;
        S.de[i] = make_float2((float)di, i > 0 ? fmaxf((float)(el * el), FLT_MIN) : 0.f);
        gl = fmin(gl, di - el - er);
        gu = fmax(gu, di + el + er);
        emax2 = fmax(emax2, er * er);
    }
    gl = warp_min(gl);
    gu = warp_max(gu);
    emax2 = warp_max(emax2);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { red[0][wid] = gl; red[1][wid] = gu; red[2][wid] = emax2; }
    __syncthreads();
    gl = red[0][0]; gu = red[1][0]; emax2 = red[2][0];
    for (int q = 1; q < (int)(blockDim.x / 32); ++q) {
        gl = fmin(gl, red[0][q]); gu = fmax(gu, red[1][q]); emax2 = fmax(emax2, red[2][q]);
    }
}

// Derived bounds of one chain's tridiagonal: the norm estimate, the pivot
// floor and the Gershgorin interval widened by the rounding of the counts.
struct TriBounds {
    double gl, gu, tnorm, pivmin;
};

__device__ __forceinline__ TriBounds tri_bounds(int n, double gl, double gu, double emax2) {
    TriBounds B;
    B.tnorm = fmax(fabs(gl), fabs(gu));
    B.pivmin = DBL_MIN * fmax(1.0, emax2);
    B.gl = gl - (2.0 * DBL_EPSILON * B.tnorm * n + 4.0 * B.pivmin);
    B.gu = gu + (2.0 * DBL_EPSILON * B.tnorm * n + 4.0 * B.pivmin);
    return B;
}

// Step 1: FP32 brackets [lo, hi] of the block's eigenvalues j (all threads
// of the block call this). Two rounds of multisection narrow the start: the
// block's threads count at 128 evenly spaced points, first over the
// Gershgorin interval, then over the span of the block's own eigenvalues,
// and each thread takes the pair of neighbouring points whose counts enclose
// its index (a binary search for the first count above j, which keeps
// count(lo) <= j < count(hi) whether or not the FP32 counts are monotone);
// bisection finishes.
__device__ void block_brackets(const TriShared& S, int n, int j, bool active, const TriBounds& B, float& lo,
                               float& hi) {
    __shared__ int cs[kEigThreads];
    __shared__ float span[2];
    const int t = threadIdx.x, T = blockDim.x;
    const float t32 = (float)B.tnorm;
    const float L0 = fminf((float)B.gl, (float)B.gl - 4.f * FLT_EPSILON * t32);
    const float R0 = fmaxf((float)B.gu, (float)B.gu + 4.f * FLT_EPSILON * t32);
    float L = L0, R = R0;
    lo = L0;
    hi = R0;
    const int jfirst = blockIdx.y * T, jlast = min(n - 1, jfirst + T - 1);
    for (int round = 0; round < 2; ++round) {
        const float h = (R - L) / (float)T;
        cs[t] = count32(S.de, n, t + 1 < T ? L + (float)(t + 1) * h : R);
        __syncthreads();
        if (active) {
            int a = 0, b = T;  // first index with cs > j
            while (a < b) {
                const int m = (a + b) >> 1;
                if (cs[m] > j) b = m; else a = m + 1;
            }
            if (a < T) {
                const float nlo = a == 0 ? L : L + (float)a * h;
                const float nhi = a + 1 < T ? L + (float)(a + 1) * h : R;
                if (nlo < nhi) { lo = nlo; hi = nhi; }
            }
            if (j == jfirst) span[0] = lo;
            if (j == jlast) span[1] = hi;
        }
        __syncthreads();
        L = span[0];
        R = span[1];
        if (!(L < R)) break;  // uniform: every thread read the same span
    }
    if (!active) return;
    for (int it = 0; it < 64; ++it) {
        const float mid = 0.5f * (lo + hi);
        if (hi - lo <= 4.f * FLT_EPSILON * fmaxf(fabsf(lo), fabsf(hi)) + FLT_EPSILON * t32 || mid <= lo || mid >= hi) break;
        if (count32(S.de, n, mid) > j) hi = mid;
        else lo = mid;
    }
}

// Half-width of the band around an FP32 bracket that is sure to hold the
// eigenvalue: Kahan's analysis makes each FP32 count exact for a matrix
// within a few eps32 ||T|| of T.
__device__ __forceinline__ double bracket_slack(const TriBounds& B) { return 16.0 * FLT_EPSILON * B.tnorm; }

// Steps 2-4: FP64 eigenvalue j from its FP32 bracket. isolated: the widened
// brackets of j-1 and j+1 stay clear of this one, so it holds exactly
// lambda_j and the FP64 Sturm counts that would verify it are skipped.
__device__ double refine64(TriShared S, int n, int j, const TriBounds& B, float lo, float hi, bool isolated,
                           int* status) {
    const double eps = DBL_EPSILON;
    const double tnorm = B.tnorm, pivmin = B.pivmin;
    const double delta = bracket_slack(B);
    double a = fmax((double)lo - delta, B.gl), b = fmin((double)hi + delta, B.gu);
    int ca = j, cb = j + 1;
    if (!isolated) {
        ca = count64(S.d, S.e2, n, a, pivmin);
        cb = count64(S.d, S.e2, n, b, pivmin);
        if (!(ca <= j && j < cb)) {
            a = B.gl; b = B.gu; ca = 0; cb = n;
        }
    }
    if (ca == j && cb == j + 1) {
        // ---- 3. safeguarded Newton on p_n; sign(p_n(x)) = (-1)^count(x) ----
        // Converged when the step falls below 4 eps max(|x|, ||T||), i.e. at
        // the accuracy of the Sturm recurrence itself; from the FP32 bracket
        // that takes 3-5 evaluations, the cap of 12 only stops rounding-level
        // oscillation.
        // A Newton step s_k after s_{k-1} leaves an error of about
        // |s_k|^2 |p''/2p'| ~ |s_k|^3 / s_{k-1}^2 (quadratic convergence);
        // when that is 4x below the tolerance the step is the last one, which
        // from an FP32 bracket usually saves the third evaluation.
        const double sa = (ca & 1) ? -1.0 : 1.0;  // sign of p_n at a
        double x = 0.5 * (a + b), dxold = b - a, dx = dxold, prev = 0.0;
        for (int it = 0; it < 12; ++it) {
            double p, dp;
            charpoly(S.d, S.e2, n, x, p, dp);
            if (p == 0.0) { a = b = x; break; }
            if ((p > 0.0) == (sa > 0.0)) a = x; else b = x;
            const double step = p / dp;
            const double tol = 4.0 * eps * fmax(fabs(x), tnorm);
            // converged: the Newton correction is at the rounding level of p_n,
            // or the one after it would be
            if (dp != 0.0 && (fabs(step) <= tol || (prev > 0.0 && fabs(step) * step * step <= 0.25 * tol * prev * prev)) &&
                x - step >= a && x - step <= b) {
                x -= step;
                break;
            }
            double xn = x - step;
            if (!(dp != 0.0) || !(xn > a && xn < b) || fabs(2.0 * (xn - x)) > fabs(dxold)) {
                dxold = dx;
                xn = 0.5 * (a + b);
                dx = xn - x;
                prev = 0.0;
            } else {
                dxold = dx;
                dx = xn - x;
                prev = fabs(step);
            }
            x = xn;
            if (fabs(dx) <= 4.0 * eps * fmax(fabs(x), tnorm) || b - a <= 4.0 * eps * fmax(fabs(x), tnorm)) break;
        }
        return fmin(fmax(x, a), b);
    }
    // ---- 4. FP64 bisection inside the bracket ----
    for (int it = 0; it < 128; ++it) {
        const double mid = 0.5 * (a + b);
        if (b - a <= 2.0 * eps * fmax(fabs(a), fabs(b)) + 0.5 * eps * tnorm || mid <= a || mid >= b) break;
        if (count64(S.d, S.e2, n, mid, pivmin) > j) b = mid;
        else a = mid;
        if (it == 127) atomicOr(status, kStatusNoConverge);
    }
    return 0.5 * (a + b);
}

// Gaps between the widened FP32 bracket of this thread's eigenvalue and its
// neighbours' (same block; +inf at the ends of the spectrum, -1 where the
// neighbour belongs to another block). br: 2 floats per thread, shared.
__device__ __forceinline__ void neighbour_gaps(float* br, int n, int j, bool active, float lo, float hi,
                                               double delta, double& gl_gap, double& gr_gap) {
    const int t = threadIdx.x;
    br[2 * t] = lo;
    br[2 * t + 1] = hi;
    __syncthreads();
    gl_gap = -1.0;
    gr_gap = -1.0;
    if (!active) return;
    if (j == 0) gl_gap = DBL_MAX;
    else if (t > 0) gl_gap = ((double)lo - delta) - ((double)br[2 * (t - 1) + 1] + delta);
    if (j == n - 1) gr_gap = DBL_MAX;
    else if (t + 1 < (int)blockDim.x) gr_gap = ((double)br[2 * (t + 1)] - delta) - ((double)hi + delta);
}

// One thread per eigenvalue index, FP64 result for every index.
__global__ void __launch_bounds__(kEigThreads)
trieig_values_kernel(const ChainDesc* __restrict__ descs, const double* __restrict__ dd,
                     const double* __restrict__ ee, double* __restrict__ ww, int* __restrict__ status) {
    extern __shared__ double sm[];
    const ChainDesc D = descs[blockIdx.x];
    const int n = D.n;
    if ((int)(blockIdx.y * blockDim.x) >= n) return;
    const TriShared S = tri_shared(sm, D.ld);
    double gl, gu, emax2;
    load_tridiag(D, dd, ee, S, gl, gu, emax2);
    const TriBounds B = tri_bounds(n, gl, gu, emax2);
    __shared__ float br[2 * kEigThreads];
    const int j = blockIdx.y * blockDim.x + threadIdx.x;
    const bool active = j < n;
    float lo = 0.f, hi = 0.f;
    block_brackets(S, n, j, active, B, lo, hi);
    double lgap, rgap;
    const double delta = bracket_slack(B);
    neighbour_gaps(br, n, j, active, lo, hi, delta, lgap, rgap);
    if (!active) return;
    const double lam = refine64(S, n, j, B, lo, hi, lgap > 2.0 * delta && rgap > 2.0 * delta, status);
    ww[D.v_off + j] = lam;
    if (!isfinite(lam)) atomicOr(status, kStatusNaN);
}

// ---- mixed path: the eigenvalues of T only serve as shifts of the FP32
// twisted factorisation (the final eigenvalues are FP64 Rayleigh quotients
// with H). T comes from the FP32 reduction, so d_i and e_i are FP32 numbers
// and e_i^2 is exactly the FP32 pair e2h + e2l. The shifts are refined in
// double-float arithmetic (an unevaluated FP32 pair, ~48 significant bits),
// which GB300 runs about ten times faster than FP64: the FP32 bracket, then
// safeguarded Newton on p_n in double-float (p_n'(x) in FP32 is accurate
// enough for the step); converged at 1e-13 ||T||, far below what the FP32
// twisted factorisation can resolve. FP64 (refine64) remains only for the
// rare brackets the double-float Sturm counts cannot confirm.

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float v = s - a;
    e = (a - (s - v)) + (b - v);
}
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    e = b - (s - a);
}

// One step of p_k = (d_k - x) p_{k-1} - e_{k-1}^2 p_{k-2} in double-float.
struct DfRow {
    float th, tl;  // d_k - x as a pair
};
__device__ __forceinline__ DfRow df_shift(float dk, float xh, float xl) {
    DfRow r;
    float e;
    two_sum(dk, -xh, r.th, e);
    r.tl = e - xl;
    return r;
}
__device__ __forceinline__ void df_step(const DfRow& t, float bh, float bl, float p1h, float p1l, float p0h,
                                        float p0l, float& p2h, float& p2l) {
    const float ah = t.th * p1h;
    const float al = fmaf(t.th, p1l, fmaf(t.tl, p1h, fmaf(t.th, p1h, -ah)));
    const float ch = bh * p0h;
    const float cl = fmaf(bh, p0l, fmaf(bl, p0h, fmaf(bh, p0h, -ch)));
    float sh, se;
    two_sum(ah, -ch, sh, se);
    fast_two_sum(sh, se + (al - cl), p2h, p2l);
}
// power-of-two rescaling of the recurrence state (keeps every sign and ratio)
__device__ __forceinline__ float df_scale(float m) {
    return m > 0x1p50f ? 0x1p-50f : (m < 0x1p-50f && m > 0.f ? 0x1p50f : 1.f);
}

// p_n(x) (pair, up to a positive power-of-two scale) and p_n'(x) (FP32, same scale)
__device__ void charpoly_df(const float* __restrict__ d, const float* __restrict__ e2h,
                            const float* __restrict__ e2l, int n, float xh, float xl, float& ph, float& pl,
                            float& dp) {
    float p0h = 1.f, p0l = 0.f, dp0 = 0.f;
    DfRow t = df_shift(d[0], xh, xl);
    float p1h, p1l;
    fast_two_sum(t.th, t.tl, p1h, p1l);
    float dp1 = -1.f;
    for (int i = 1; i < n; ++i) {
        t = df_shift(d[i], xh, xl);
        float p2h, p2l;
        df_step(t, e2h[i - 1], e2l[i - 1], p1h, p1l, p0h, p0l, p2h, p2l);
        const float dp2 = fmaf(t.th, dp1, -fmaf(e2h[i - 1], dp0, p1h));
        p0h = p1h; p0l = p1l; dp0 = dp1;
        p1h = p2h; p1l = p2l; dp1 = dp2;
        if ((i & 3) == 0) {
            const float sc = df_scale(fmaxf(fabsf(p1h), fabsf(dp1)));
            p0h *= sc; p0l *= sc; dp0 *= sc; p1h *= sc; p1l *= sc; dp1 *= sc;
        }
    }
    ph = p1h;
    pl = p1l;
    dp = dp1;
}

// Sturm count at x in double-float: sign changes of p_0 = 1, p_1, ..., p_n (a
// zero p_k counts as the sign opposite to p_{k-1}, i.e. as negative for q_k).
__device__ int count_df(const float* __restrict__ d, const float* __restrict__ e2h, const float* __restrict__ e2l,
                        int n, float xh, float xl) {
    float p0h = 1.f, p0l = 0.f;
    DfRow t = df_shift(d[0], xh, xl);
    float p1h, p1l;
    fast_two_sum(t.th, t.tl, p1h, p1l);
    int c = !(p1h > 0.f);
    for (int i = 1; i < n; ++i) {
        t = df_shift(d[i], xh, xl);
        float p2h, p2l;
        df_step(t, e2h[i - 1], e2l[i - 1], p1h, p1l, p0h, p0l, p2h, p2l);
        const bool neg = p2h == 0.f ? (p1h > 0.f) : ((p2h > 0.f) != (p1h > 0.f));
        c += neg;
        if (p2h == 0.f) p2h = p1h > 0.f ? -0x1p-100f : 0x1p-100f;  // sign opposite to p_{k-1}
        p0h = p1h; p0l = p1l;
        p1h = p2h; p1l = p2l;
        if ((i & 3) == 0) {
            const float sc = df_scale(fabsf(p1h) + fabsf(p0h));
            p0h *= sc; p0l *= sc; p1h *= sc; p1l *= sc;
        }
    }
    return c;
}

constexpr int kDfIters = 6;

// Shift j from its FP32 bracket in double-float; false when the bracket or the
// iteration cannot be trusted (then FP64 decides).
__device__ bool shift_df(const float* d, const float* e2h, const float* e2l, int n, int j, const TriBounds& B,
                         float lo, float hi, bool isolated, double& out) {
    const double delta = bracket_slack(B);
    const double a0 = fmax((double)lo - delta, B.gl), b0 = fmin((double)hi + delta, B.gu);
    double a = a0, b = b0;
    int ca = j;
    if (!isolated) {
        const float ah = (float)a, al = (float)(a - (double)ah), bh = (float)b, bl = (float)(b - (double)bh);
        ca = count_df(d, e2h, e2l, n, ah, al);
        const int cb = count_df(d, e2h, e2l, n, bh, bl);
        if (!(ca == j && cb == j + 1)) return false;
    }
    const bool neg_at_a = ca & 1;  // sign of p_n at a is (-1)^count
    const double tol = 1e-13 * B.tnorm;
    float xh = 0.5f * (lo + hi), xl = 0.5f * (lo + hi) - xh;
    xl = (float)(0.5 * ((double)lo + (double)hi) - (double)xh);
    float prev = 0.f;
    for (int it = 0; it < kDfIters; ++it) {
        float ph, pl, dp;
        charpoly_df(d, e2h, e2l, n, xh, xl, ph, pl, dp);
        const double x = (double)xh + (double)xl;
        const float p = ph + pl;
        if (p == 0.f) { out = x; return true; }
        if ((p < 0.f) == neg_at_a) a = x; else b = x;
        if (!(dp != 0.f) || !isfinite(p / dp)) return false;
        const float step = p / dp;
        float sh, se;
        two_sum(xh, -step, sh, se);
        float nh, nl;
        fast_two_sum(sh, se + xl, nh, nl);
        const double xn = (double)nh + (double)nl;
        if (!(xn >= a0 && xn <= b0)) return false;
        const float as = fabsf(step);
        if ((double)as <= tol || (prev > 0.f && (double)as * as * as <= 0.25 * tol * (double)prev * prev)) {
            out = xn;
            return true;
        }
        prev = as;
        xh = nh;
        xl = nl;
    }
    return false;
}

__global__ void __launch_bounds__(kEigThreads)
trieig_shift_kernel(const ChainDesc* __restrict__ descs, const double* __restrict__ dd,
                    const double* __restrict__ ee, double* __restrict__ ww, double* __restrict__ ctol,
                    int* __restrict__ status) {
    extern __shared__ double sm[];
    const ChainDesc D = descs[blockIdx.x];
    const int n = D.n;
    if ((int)(blockIdx.y * blockDim.x) >= n) return;
    const TriShared S = tri_shared(sm, D.ld);
    float* e2l = (float*)(S.de + D.ld);
    __shared__ float br[2 * kEigThreads];
    __shared__ int list[kEigThreads];
    __shared__ float lbr[2 * kEigThreads];
    __shared__ int cnt;
    double gl, gu, emax2;
    load_tridiag(D, dd, ee, S, gl, gu, emax2);
    for (int i = threadIdx.x; i < n; i += blockDim.x) e2l[i] = (float)(S.e2[i] - (double)S.e232[i]);
    if (threadIdx.x == 0) cnt = 0;
    __syncthreads();
    const TriBounds B = tri_bounds(n, gl, gu, emax2);
    // the cluster tolerance of the eigenvector kernels (twisted factorisation
    // and cluster fix-up decide membership from the same number)
    if (blockIdx.y == 0 && threadIdx.x == 0) ctol[blockIdx.x] = kClusterTol * B.tnorm;
    const int j = blockIdx.y * blockDim.x + threadIdx.x;
    const bool active = j < n;
    float lo = 0.f, hi = 0.f;
    block_brackets(S, n, j, active, B, lo, hi);
    double lgap, rgap;
    const double delta = bracket_slack(B);
    neighbour_gaps(br, n, j, active, lo, hi, delta, lgap, rgap);
    if (active) {
        double x;
        if (shift_df(S.d32, S.e232, e2l, n, j, B, lo, hi, lgap > 2.0 * delta && rgap > 2.0 * delta, x)) {
            ww[D.v_off + j] = x;
        } else {
            const int q = atomicAdd(&cnt, 1);
            list[q] = j;
            lbr[2 * q] = lo;
            lbr[2 * q + 1] = hi;
        }
    }
    __syncthreads();
    // the rest in FP64, packed onto the first threads
    const int k = cnt;
    if ((int)threadIdx.x < k) {
        const int jj = list[threadIdx.x];
        const double lam = refine64(S, n, jj, B, lbr[2 * threadIdx.x], lbr[2 * threadIdx.x + 1], false, status);
        ww[D.v_off + jj] = lam;
        if (!isfinite(lam)) atomicOr(status, kStatusNaN);
    }
}

}  // namespace

size_t trieig_smem_bytes(int max_ld) {
    return (size_t)max_ld * (2 * sizeof(double) + 2 * sizeof(float) + sizeof(float2));
}


cudaError_t launch_trieig_shifts(const ChainDesc* d_desc, int batch, int max_n, int max_ld, const double* d_d,
                                 const double* d_e, double* d_w, double* d_ctol, int* d_status, cudaStream_t st) {
    if (batch <= 0) return cudaSuccess;
    const size_t smem = trieig_smem_bytes(max_ld) + sizeof(float) * (size_t)max_ld;
    cudaError_t err = cudaFuncSetAttribute(trieig_shift_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    dim3 grid(batch, (max_n + kEigThreads - 1) / kEigThreads);
    trieig_shift_kernel<<<grid, kEigThreads, smem, st>>>(d_desc, d_d, d_e, d_w, d_ctol, d_status);
    return cudaGetLastError();
}

cudaError_t launch_trieig_values(const ChainDesc* d_desc, int batch, int max_n, int max_ld, const double* d_d,
                                 const double* d_e, double* d_w, int* d_status, cudaStream_t st) {
    if (batch <= 0) return cudaSuccess;
    const size_t smem = trieig_smem_bytes(max_ld);
    cudaError_t err = cudaFuncSetAttribute(trieig_values_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    dim3 grid(batch, (max_n + kEigThreads - 1) / kEigThreads);
    trieig_values_kernel<<<grid, kEigThreads, smem, st>>>(d_desc, d_d, d_e, d_w, d_status);
    return cudaGetLastError();
}

}  // namespace fkg
