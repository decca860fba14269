// mixed.cu — the mixed-precision eigen-solve: FP32 reduction, FP64 accuracy.
//
// After the FP32 Householder reduction (sytrd_v3.cu) and the tridiagonal
// eigenvalues (trieig.cu) the eigenvalues carry the FP32 reduction's error,
// about eps32 ||H||. One step of eigenvalue refinement wins the accuracy back:
//   1. larft: the compact-WY factor T_p of every panel of 32 reflectors,
//      H_{k0} ... H_{k0+31} = I - V_p T_p V_p^T, and V_p T_p (on its own
//      stream, concurrent with the shifts and step 2; the cluster fix-up of
//      vectors64.cu runs on a third, beside step 2);
//   2. eigenvectors z_j of the tridiagonal by a twisted factorisation of
//      T - lambda_j I (one thread per eigenvalue, FP32 recurrences; the
//      shifted diagonal d_i - lambda_j is rounded once to FP32 with FP32
//      arithmetic), stored row-major Z[i*ld + j] unnormalised, with the
//      scale 1/||z_j|| beside it;
//   3. back-transformation X = Q Z = Q_0 Q_1 ... Q_{P-1} Z, panel by panel
//      from the last one, on the tensor cores (backtransform_tc.cu);
//   4. Rayleigh quotients theta_j = x_j^T H x_j / x_j^T x_j with the exact
//      sparse H (hopping CSR + FP64 diagonal), summed in double-float, which
//      are accurate to second order in the eigenvector error; then an
//      ascending sort.
// Work per chain: 4/3 n^3 FP32 (reduction) + 2 n^3 FP32 (back-transformation)
// + O(n^2) double-float; the FP64 pipe never sees an O(n^3) loop.
#include <cfloat>

#include "fkg_common.cuh"

namespace fkg {
namespace {

constexpr int kNb = 32;        // reflectors per panel
constexpr int kChunk = 128;    // rows of V staged per pass
constexpr int kBtThreads = 256;
constexpr int kTwBatch = 16;   // twisted factorisation: stored values read per batch

template <typename T>
__device__ __forceinline__ T vref(const T* __restrict__ A, int ld, int n, int k, int i, int shift = 1) {
    // element i of Householder vector k (v_k(k+shift) = 1, zero above; shift 1
    // for the one-stage reduction, the band width for the two-stage one)
    if (i == k + shift) return T(1);
    if (i > k + shift && i < n) return A[(size_t)k * ld + i];
    return T(0);
}

// ---- 1. compact-WY factors, one CTA per (chain, panel) ----
// With VT (mixed path) the CTA also writes, for the panel's rows k0 .. ld-1
// and columns k0 .. k0+31 (the reduced matrix's layout), V_p T_p and V_p
// itself (unit element and zeros above it included) split for the 3xTF32
// products: four planes `plane` floats apart, tf32(x) and tf32(x - tf32(x))
// of V_p T_p, then of V_p. The back-transformation applies Q_p as
// Z - (V_p T_p)(V_p^T Z) from these planes without splitting anything of V
// itself (every column block of a chain would otherwise split the same V).
// FP32: 64 registers (no spills) so that four CTAs share an SM and hide the
// latency of the V loads
template <typename T>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 2)
larft_kernel(const ChainDesc* __restrict__ descs, const T* __restrict__ A32, const T* __restrict__ tau,
             T* __restrict__ Tf, T* __restrict__ VT, long long plane, int shift) {
    const ChainDesc D = descs[blockIdx.x];
    const int n = D.n, ld = D.ld, p = blockIdx.y;
    const int nrefl = n - 1 - shift;  // reflector k has its unit at row k + shift
    const int npanel = (nrefl + kNb - 1) / kNb;
    if (nrefl <= 0 || p >= npanel) return;
    const int k0 = p * kNb, kb = min(kNb, nrefl - k0), r0 = k0 + shift;
    const T* A = A32 + D.a_off;
    __shared__ T Vc[kChunk][kNb + 1];
    __shared__ T G[kNb][kNb + 1];
    __shared__ T Ts[kNb][kNb + 1];
    const int t = threadIdx.x, c = t & 31, g = t >> 5;
    T acc[4] = {T(0), T(0), T(0), T(0)};  // G[g + 8q][c]
    for (int i0 = r0; i0 < n; i0 += kChunk) {
        for (int q = 0; q < kChunk * kNb / 256; ++q) {
            const int idx = t + 256 * q, kk = idx / kChunk, ii = idx % kChunk;
            Vc[ii][kk] = (kk < kb) ? vref(A, ld, n, k0 + kk, i0 + ii, shift) : T(0);
        }
        __syncthreads();
        const int rows = min(kChunk, n - i0);
        for (int ii = 0; ii < rows; ++ii) {
            const T vc = Vc[ii][c];
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[q] = fma(Vc[ii][g + 8 * q], vc, acc[q]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) G[g + 8 * q][c] = acc[q];
    for (int q = 0; q < 4; ++q) Ts[g + 8 * q][c] = T(0);
    __syncthreads();
    // T from its inverse, T^-1 = diag(1/tau) + triu(G, 1) (Puglisi 1992;
    // Joffrain, Low, Quintana-Orti, van de Geijn, Van Zee 2006): lane j of warp
    // 0 solves T^-1 t = e_j by back substitution, t_j = tau_j and
    // t_r = -tau_r sum_{q > r} G(r, q) t_q, which needs no division and gives
    // zero rows and columns for tau = 0 (an identity reflector) by itself.
    // The 32 columns are independent: one pass of 528 FMAs per lane instead
    // of 32 dependent triangular products.
    if (g == 0) {
        const T* tp = tau + D.v_off + k0;
        const int j = c;
        T t[kNb];
#pragma unroll
        for (int r = kNb - 1; r >= 0; --r) {
            const T tr = r < kb ? tp[r] : T(0);
            T s0 = T(0), s1 = T(0), s2 = T(0), s3 = T(0);
#pragma unroll
            for (int q = r + 1; q < kNb; ++q) {
                const T gq = G[r][q] * t[q];  // t_q = 0 for q > j
                if ((q & 3) == 0) s0 += gq;
                else if ((q & 3) == 1) s1 += gq;
                else if ((q & 3) == 2) s2 += gq;
                else s3 += gq;
            }
            t[r] = r > j ? T(0) : (r == j ? tr : -tr * ((s0 + s1) + (s2 + s3)));
        }
#pragma unroll
        for (int r = 0; r < kNb; ++r) Ts[r][j] = t[r];
    }
    __syncthreads();
    T* out = Tf + (D.v_off / kNb + p) * (size_t)(kNb * kNb);
    for (int q = 0; q < 4; ++q) out[(g + 8 * q) * kNb + c] = Ts[g + 8 * q][c];
    if constexpr (sizeof(T) == 4) {
        if (VT == nullptr) return;
        // VT(i, kk) = sum_l V(i, l) T(l, kk), T upper triangular: l <= kk
        T* vth = VT + D.a_off;
        T* vtl = vth + plane;
        T* vh = vtl + plane;
        T* vl = vh + plane;
        for (int i = k0 + t; i < ld; i += blockDim.x) {
            T vrow[kNb];
#pragma unroll
            for (int l = 0; l < kNb; ++l) vrow[l] = (l < kb) ? vref(A, ld, n, k0 + l, i, shift) : T(0);
#pragma unroll 4
            for (int kk = 0; kk < kNb; ++kk) {
                T s = T(0);
#pragma unroll
                for (int l = 0; l < kNb; ++l)
                    if (l <= kk) s = fma(vrow[l], Ts[l][kk], s);
                unsigned hi, lo;
                split_tf32(s, hi, lo);
                const size_t o = (size_t)(k0 + kk) * ld + i;
                vth[o] = __uint_as_float(hi);
                vtl[o] = __uint_as_float(lo);
                split_tf32(vrow[kk], hi, lo);
                vh[o] = __uint_as_float(hi);
                vl[o] = __uint_as_float(lo);
            }
        }
    }
}

// ---- 2. tridiagonal eigenvectors by twisted factorisation ----
__global__ void __launch_bounds__(128)
twisted_kernel(const ChainDesc* __restrict__ descs, const double* __restrict__ dd, const double* __restrict__ ee,
               const double* __restrict__ ww, const double* __restrict__ ctol, float* __restrict__ Zws,
               float* __restrict__ zscale) {
    extern __shared__ double smt[];
    const ChainDesc D = descs[blockIdx.x];
    const int n = D.n, ld = D.ld;
    if ((int)(blockIdx.y * blockDim.x) >= n) return;
    float* d = (float*)smt;  // the FP32 reduction's diagonal: exact in FP32
    float* e = d + ld;
    float* e2 = e + ld;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        d[i] = (float)dd[D.v_off + i];
        const float ei = i + 1 < n ? (float)ee[D.v_off + i] : 0.f;
        e[i] = ei;
        e2[i] = ei * ei;
    }
    __syncthreads();
    const int j = blockIdx.y * blockDim.x + threadIdx.x;
    if (j >= n) return;
    {  // members of a cluster are left to cluster_fix_kernel (same tolerance)
        const double tol = ctol[blockIdx.x], wj = ww[D.v_off + j];
        if ((j > 0 && wj - ww[D.v_off + j - 1] <= tol) || (j + 1 < n && ww[D.v_off + j + 1] - wj <= tol)) return;
    }
    float* Z = Zws + D.a_off;
    // d_i - lambda_j rounded once to FP32, in FP32 arithmetic: lambda_j as the
    // pair lh + ll, d_i - lh split exactly by Knuth's TwoSum, then
    // s + (err - ll) (the FP64 difference rounded to FP32 in all but ties)
    const double lam = ww[D.v_off + j];
    const float lh = (float)lam, ll = (float)(lam - (double)lh);
    auto shift = [&](int i) {
        const float a = d[i];
        const float s = a - lh;
        const float bb = s - a;
        const float err = (a - (s - bb)) + (-lh - bb);
        return s + (err - ll);
    };
    const float pivmin = 1e-30f;
    auto guard = [&](float x) { return fabsf(x) < pivmin ? (x < 0.f ? -pivmin : pivmin) : x; };
    // forward: D+_0 = d_0 - lam, D+_{i+1} = (d_{i+1} - lam) - e_i^2 / D+_i
    float dp = guard(shift(0));
    Z[j] = dp;
    for (int i = 0; i + 1 < n; ++i) {
        dp = guard(shift(i + 1) - __fdividef(e2[i], dp));
        Z[(size_t)(i + 1) * ld + j] = dp;
    }
    // backward: D-_{n-1} = d_{n-1} - lam, D-_i = (d_i - lam) - e_i^2 / D-_{i+1};
    // gamma_i = D+_i + D-_i - (d_i - lam); twist index r = argmin |gamma|
    float dm = 0.f, best = FLT_MAX;
    int r = n - 1;
    for (int i0 = n - 1; i0 >= 0; i0 -= kTwBatch) {
        float dpv[kTwBatch];
#pragma unroll
        for (int u = 0; u < kTwBatch; ++u) dpv[u] = (i0 - u >= 0) ? Z[(size_t)(i0 - u) * ld + j] : 0.f;
#pragma unroll
        for (int u = 0; u < kTwBatch; ++u) {
            const int i = i0 - u;
            if (i >= 0) {
                const float s = shift(i);
                dm = (i == n - 1) ? guard(s) : guard(s - __fdividef(e2[i], dm));
                const float gam = fabsf(dpv[u] + dm - s);
                if (gam < best) { best = gam; r = i; }
            }
        }
    }
    // D-_i for i > r into Z (overwrites D+_i, no longer needed there)
    dm = 0.f;
    for (int i = n - 1; i > r; --i) {
        const float s = shift(i);
        dm = (i == n - 1) ? guard(s) : guard(s - __fdividef(e2[i], dm));
        Z[(size_t)i * ld + j] = dm;
    }
    // z_r = 1; z_{i+1} = -(e_i / D-_{i+1}) z_i (i >= r); z_i = -(e_i / D+_i) z_{i+1} (i < r)
    // The stored D values are read kTwBatch at a time, ahead of the stores
    // that overwrite them, so one memory latency covers kTwBatch steps.
    float nrm = 1.f, zi = 1.f;
    Z[(size_t)r * ld + j] = 1.f;
    for (int i0 = r; i0 + 1 < n; i0 += kTwBatch) {
        float dv[kTwBatch];
#pragma unroll
        for (int u = 0; u < kTwBatch; ++u) dv[u] = (i0 + 1 + u < n) ? Z[(size_t)(i0 + 1 + u) * ld + j] : 1.f;
#pragma unroll
        for (int u = 0; u < kTwBatch; ++u) {
            const int i = i0 + u;
            if (i + 1 < n) {
                zi = -__fdividef(e[i], dv[u]) * zi;
                Z[(size_t)(i + 1) * ld + j] = zi;
                nrm = fmaf(zi, zi, nrm);
            }
        }
    }
    zi = 1.f;
    for (int i0 = r - 1; i0 >= 0; i0 -= kTwBatch) {
        float dv[kTwBatch];
#pragma unroll
        for (int u = 0; u < kTwBatch; ++u) dv[u] = (i0 - u >= 0) ? Z[(size_t)(i0 - u) * ld + j] : 1.f;
#pragma unroll
        for (int u = 0; u < kTwBatch; ++u) {
            const int i = i0 - u;
            if (i >= 0) {
                zi = -__fdividef(e[i], dv[u]) * zi;
                Z[(size_t)i * ld + j] = zi;
                nrm = fmaf(zi, zi, nrm);
            }
        }
    }
    zscale[D.v_off + j] = rsqrtf(nrm);  // applied when the back-transformation loads Z
}

// ---- 3. back-transformation X = Q Z, one CTA per (chain, 32-column block) ----
// The 32-column block of Z stays in shared memory for all panels. Per panel:
//   W = V^T Zb (32 x 32): every warp takes a slice of the rows, each lane one
//       column c with 32 register accumulators; the V row (32 values) is read
//       with 128-bit broadcast loads from a staged chunk; the 8 partial W are
//       summed through shared memory;
//   W2 = T W, kept per lane as one column (32 registers);
//   Zb -= V W2 with the same row split and broadcast loads.
constexpr int kVs = kNb + 4;  // staged V row stride (elements): 16-byte aligned rows
constexpr int kBtChunk = 64;   // rows of V staged per step of the back-transformation
constexpr int kStageRegs = kBtChunk * kNb / kBtThreads;  // V values staged per thread per chunk

// V(i0 + ii, k0 + kk) for this thread's share of a chunk (lane-contiguous rows:
// coalesced global reads), into registers, so the next chunk's loads overlap
// the current chunk's arithmetic.
template <typename T>
__device__ __forceinline__ void load_v(const T* __restrict__ A, int ld, int n, int k0, int kb, int i0,
                                       T (&r)[kStageRegs]) {
#pragma unroll
    for (int q = 0; q < kStageRegs; ++q) {
        const int idx = threadIdx.x + kBtThreads * q, kk = idx / kBtChunk, ii = idx % kBtChunk;
        r[q] = (kk < kb) ? vref(A, ld, n, k0 + kk, i0 + ii) : T(0);
    }
}
template <typename T>
__device__ __forceinline__ void store_v(const T (&r)[kStageRegs], T* __restrict__ Vs) {
#pragma unroll
    for (int q = 0; q < kStageRegs; ++q) {
        const int idx = threadIdx.x + kBtThreads * q, kk = idx / kBtChunk, ii = idx % kBtChunk;
        Vs[ii * kVs + kk] = r[q];
    }
}

// The column block lives in shared memory for FP32 (ZB_SMEM) and stays in
// global memory for FP64 (a 32-column FP64 block of a 1024-row matrix would
// not fit); its row stride is zs.
// four contiguous values from 16-byte-aligned shared memory
__device__ __forceinline__ void load4(const double* p, double (&o)[4]) {
    const double2 a = *reinterpret_cast<const double2*>(p), b = *reinterpret_cast<const double2*>(p + 2);
    o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y;
}

template <typename T, bool ZB_SMEM>
__global__ void __launch_bounds__(kBtThreads, 2)
backtransform_kernel(const ChainDesc* __restrict__ descs, const T* __restrict__ A32, const T* __restrict__ Tf,
                     T* __restrict__ Zws) {
    extern __shared__ __align__(16) unsigned char smb_raw[];
    T* smb = reinterpret_cast<T*>(smb_raw);
    // one chain's column blocks are adjacent in launch order (blockIdx.x), so
    // its reflector panels are read from DRAM once and from L2 afterwards
    const ChainDesc D = descs[blockIdx.y];
    const int n = D.n, ld = D.ld, j0 = blockIdx.x * 32;
    if (j0 >= n) return;
    const T* A = A32 + D.a_off;
    T* Z = Zws + D.a_off;
    const int zs = ZB_SMEM ? 32 : ld;
    T* Zb = ZB_SMEM ? smb : Z + j0;                           // row i, column c at Zb[i * zs + c]
    T* Vs = ZB_SMEM ? smb + (size_t)ld * 32 : smb;          // [kBtChunk][kVs]
    T* Ws = Vs + kBtChunk * kVs;                              // [4][32 kk][32 c] partial sums
    T* Ts = Ws + 4 * kNb * 32;                                // [32][33]
    const int t = threadIdx.x, c = t & 31, g = t >> 5;
    if (ZB_SMEM)
        for (int i = g; i < n; i += kBtThreads / 32) Zb[i * 32 + c] = Z[(size_t)i * ld + j0 + c];
    const int nrefl = n - 2;
    const int npanel = nrefl > 0 ? (nrefl + kNb - 1) / kNb : 0;
    const T* Tbase = Tf + (D.v_off / kNb) * (size_t)(kNb * kNb);
    T stage[kStageRegs];
    for (int p = npanel - 1; p >= 0; --p) {
        const int k0 = p * kNb, kb = min(kNb, nrefl - k0), r0 = k0 + 1;
        for (int q = t; q < kNb * kNb; q += kBtThreads) Ts[(q / kNb) * (kNb + 1) + q % kNb] = Tbase[(size_t)p * kNb * kNb + q];
        T acc[kNb];
#pragma unroll
        for (int kk = 0; kk < kNb; ++kk) acc[kk] = T(0);
        load_v(A, ld, n, k0, kb, r0, stage);
        for (int i0 = r0; i0 < n; i0 += kBtChunk) {
            __syncthreads();
            store_v(stage, Vs);
            __syncthreads();
            if (i0 + kBtChunk < n) load_v(A, ld, n, k0, kb, i0 + kBtChunk, stage);
            const int rows = min(kBtChunk, n - i0);
            for (int ii = g; ii < rows; ii += kBtThreads / 32) {
                const T z = (j0 + c < ld) ? Zb[(size_t)(i0 + ii) * zs + c] : T(0);
                const T* vr = Vs + ii * kVs;
#pragma unroll
                for (int q = 0; q < kNb; q += 4) {
                    T v4[4];
                    load4(vr + q, v4);
#pragma unroll
                    for (int u = 0; u < 4; ++u) acc[q + u] = fma(v4[u], z, acc[q + u]);
                }
            }
        }
        // W(kk, c) = sum of the 8 warps' partial sums, in a fixed order (a
        // three-level tree through Ws), so the result is bit-reproducible
#pragma unroll
        for (int half = 4; half >= 1; half >>= 1) {
            if (g >= half && g < 2 * half)
#pragma unroll
                for (int kk = 0; kk < kNb; ++kk) Ws[((g - half) * kNb + kk) * 32 + c] = acc[kk];
            __syncthreads();
            if (g < half)
#pragma unroll
                for (int kk = 0; kk < kNb; ++kk) acc[kk] += Ws[(g * kNb + kk) * 32 + c];
            __syncthreads();
        }
        if (g == 0)
#pragma unroll
            for (int kk = 0; kk < kNb; ++kk) Ws[kk * 32 + c] = acc[kk];
        __syncthreads();
        T w2[kNb];
#pragma unroll
        for (int kk = 0; kk < kNb; ++kk) {
            T s = T(0);
#pragma unroll
            for (int l = 0; l < kNb; ++l) s = fma(Ts[kk * (kNb + 1) + l], Ws[l * 32 + c], s);  // T upper triangular
            w2[kk] = s;
        }
        // Zb(i, c) -= sum_kk V(i, kk) W2(kk, c), rows i in [r0, n)
        load_v(A, ld, n, k0, kb, r0, stage);
        for (int i0 = r0; i0 < n; i0 += kBtChunk) {
            __syncthreads();
            store_v(stage, Vs);
            __syncthreads();
            if (i0 + kBtChunk < n) load_v(A, ld, n, k0, kb, i0 + kBtChunk, stage);
            const int rows = min(kBtChunk, n - i0);
            for (int ii = g; ii < rows; ii += kBtThreads / 32) {
                if (!ZB_SMEM && j0 + c >= n) continue;
                T z0 = Zb[(size_t)(i0 + ii) * zs + c], z1 = T(0);
                const T* vr = Vs + ii * kVs;
#pragma unroll
                for (int q = 0; q < kNb; q += 4) {
                    T v4[4];
                    load4(vr + q, v4);
                    z0 = fma(-v4[0], w2[q], z0);
                    z1 = fma(-v4[1], w2[q + 1], z1);
                    z0 = fma(-v4[2], w2[q + 2], z0);
                    z1 = fma(-v4[3], w2[q + 3], z1);
                }
                Zb[(size_t)(i0 + ii) * zs + c] = z0 + z1;
            }
        }
        __syncthreads();
    }
    if (ZB_SMEM && j0 + c < n)
        for (int i = g; i < n; i += kBtThreads / 32) Z[(size_t)i * ld + j0 + c] = Zb[i * 32 + c];
}

// ---- 4. Rayleigh quotients with the exact sparse H ----
// theta_k = x_k^T H x_k / x_k^T x_k for the FP32 vector x_k, summed in
// double-float (unevaluated FP32 pairs, ~48 significant bits): the diagonal
// and hopping values enter as pairs hi + lo, every product of a pair with an
// FP32 number is formed exactly up to the pair's own rounding, and the sums
// are pair additions. The result's rounding error (~1e-13 ||H||) is far below
// the second-order error of the quotient itself, and GB300 runs this about
// ten times faster than the same sums in FP64.
__device__ __forceinline__ void df_fast_two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    e = b - (s - a);
}
__device__ __forceinline__ void df_mul_f(float ah, float al, float b, float& ph, float& pl) {
    const float p = ah * b;
    df_fast_two_sum(p, fmaf(al, b, fmaf(ah, b, -p)), ph, pl);
}
__device__ __forceinline__ void df_add(float ah, float al, float bh, float bl, float& sh, float& sl) {
    const float s = ah + bh;
    const float v = s - ah;
    const float e = ((ah - (s - v)) + (bh - v)) + (al + bl);
    df_fast_two_sum(s, e, sh, sl);
}

// Rayleigh quotient of eigenvector k: thread (k, seg) of a 32 x 4 block sums
// rows seg*ceil(n/4) ... of x^T H x and x^T x in double-float; the four
// segments' sums are added in order (shorter dependent chains and four times
// the warps of one thread per vector: the row loop is bound by the latency of
// its CSR gathers).
constexpr int kRfSeg = 4;
__global__ void __launch_bounds__(32 * kRfSeg)
refine_kernel(const ChainDesc* __restrict__ descs, const float* __restrict__ Xws, const double* __restrict__ diag,
              double* __restrict__ theta) {
    extern __shared__ float2 dgs[];  // the chain's diagonal as pairs
    __shared__ float4 part[kRfSeg][32];
    const ChainDesc D = descs[blockIdx.x];
    const int n = D.n, ld = D.ld;
    if ((int)(blockIdx.y * 32) >= n) return;
    const int tid = threadIdx.x, lane = tid & 31, seg = tid >> 5;
    for (int i = tid; i < n; i += blockDim.x) {
        const double v = diag[D.v_off + i];
        const float h = (float)v;
        dgs[i] = make_float2(h, (float)(v - (double)h));
    }
    __syncthreads();
    const int k = blockIdx.y * 32 + lane;
    const float* X = Xws + D.a_off;
    float nh = 0.f, nl = 0.f, sh = 0.f, sl = 0.f;
    const int rows = (n + kRfSeg - 1) / kRfSeg, i0 = seg * rows, i1 = min(n, i0 + rows);
    if (k < n)
        for (int i = i0; i < i1; ++i) {
            const float xi = X[(size_t)i * ld + k];
            const float2 dg = dgs[i];
            float yh, yl;
            df_mul_f(dg.x, dg.y, xi, yh, yl);
            for (int p = D.rowptr[i]; p < D.rowptr[i + 1]; ++p) {
                const float2 v = D.valf[p];
                float th, tl;
                df_mul_f(v.x, v.y, X[(size_t)D.col[p] * ld + k], th, tl);
                df_add(yh, yl, th, tl, yh, yl);
            }
            float ph, pl;
            df_mul_f(yh, yl, xi, ph, pl);
            df_add(nh, nl, ph, pl, nh, nl);
            const float sq = xi * xi;
            df_add(sh, sl, sq, fmaf(xi, xi, -sq), sh, sl);
        }
    part[seg][lane] = make_float4(nh, nl, sh, sl);
    __syncthreads();
    if (seg == 0 && k < n) {
        for (int q = 1; q < kRfSeg; ++q) {
            const float4 o = part[q][lane];
            df_add(nh, nl, o.x, o.y, nh, nl);
            df_add(sh, sl, o.z, o.w, sh, sl);
        }
        theta[D.v_off + k] = ((double)nh + (double)nl) / ((double)sh + (double)sl);
    }
}

// ascending insertion sort of the (nearly sorted) Rayleigh quotients; perm[i]
// is the eigenvector column that belongs to the i-th sorted eigenvalue
__global__ void sort_kernel(const ChainDesc* __restrict__ descs, const double* __restrict__ theta,
                            double* __restrict__ w, int* __restrict__ perm, int* __restrict__ status) {
    extern __shared__ double sms[];
    const ChainDesc D = descs[blockIdx.x];
    const int n = D.n;
    int* idx = reinterpret_cast<int*>(sms + D.ld);
    for (int i = threadIdx.x; i < n; i += blockDim.x) { sms[i] = theta[D.v_off + i]; idx[i] = i; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 1; i < n; ++i) {
            const double x = sms[i];
            const int xi = idx[i];
            int q = i - 1;
            while (q >= 0 && sms[q] > x) { sms[q + 1] = sms[q]; idx[q + 1] = idx[q]; --q; }
            sms[q + 1] = x;
            idx[q + 1] = xi;
            if (!isfinite(x)) atomicOr(status, kStatusNaN);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        w[D.v_off + i] = sms[i];
        if (perm) perm[D.v_off + i] = idx[i];
    }
}

}  // namespace

template <typename T, bool ZB_SMEM>
size_t backtransform_smem_bytes(int max_ld) {
    return sizeof(T) * ((ZB_SMEM ? (size_t)max_ld * 32 : 0) + kBtChunk * kVs + 4 * kNb * 32 + kNb * (kNb + 1));
}

// larft (+ V T): needs only the reduction; enqueued on its own stream right
// after it, so that it overlaps the shift and eigenvector kernels.
cudaError_t launch_larft_vt(const ChainDesc* d_desc, int batch, int max_n, const float* d_A32, const float* d_tau32,
                            float* d_Tf, float* d_VT, long long plane, int shift, cudaStream_t st) {
    if (batch <= 0) return cudaSuccess;
    const int npanel = (max_n + kNb - 1) / kNb;
    larft_kernel<float><<<dim3(batch, npanel), 256, 0, st>>>(d_desc, d_A32, d_tau32, d_Tf, d_VT, plane, shift);
    return cudaGetLastError();
}

// The eigenvectors and the refinement. On entry the shifts are on `st` and
// larft on the stream that recorded ev_larft. The cluster fix-up runs on
// `aux` beside the twisted factorisation of all other eigenvectors; both and
// larft are joined before the back-transformation.
cudaError_t launch_mixed_refine(const ChainDesc* d_desc, int batch, int max_n, int max_ld, const double* d_diag,
                                const float* d_A32, const float* d_VT, long long vt_plane, const double* d_d,
                                const double* d_e,
                                double* d_w, const double* d_ctol, float* d_Z, float* d_zscale, double* d_theta,
                                int* d_perm, double* d_scratch, int* d_status, cudaStream_t st, cudaStream_t aux,
                                cudaEvent_t ev_fork, cudaEvent_t ev_join, cudaEvent_t ev_larft, int bt_variant,
                                long long wait_iters, int shift, const float* d_Q2, long long q2t_off,
                                void (*stage)(void*, int, int), void* sctx) {
    if (batch <= 0) return cudaSuccess;
    cudaError_t err;
    if ((err = cudaEventRecord(ev_fork, st)) != cudaSuccess) return err;
    if ((err = cudaStreamWaitEvent(aux, ev_fork, 0)) != cudaSuccess) return err;
    if ((err = launch_cluster_fix_f32(d_desc, batch, max_ld, d_d, d_e, d_w, d_ctol, d_Z, d_zscale, d_scratch, aux)) !=
        cudaSuccess)
        return err;
    if ((err = cudaEventRecord(ev_join, aux)) != cudaSuccess) return err;
    stage(sctx, 1, 0);
    const size_t sm_tw = (size_t)max_ld * 3 * sizeof(float);
    if ((err = cudaFuncSetAttribute(twisted_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_tw))) return err;
    twisted_kernel<<<dim3(batch, (max_n + 127) / 128), 128, sm_tw, st>>>(d_desc, d_d, d_e, d_w, d_ctol, d_Z, d_zscale);
    if ((err = cudaGetLastError()) != cudaSuccess) return err;
    stage(sctx, 1, 1);
    if ((err = cudaStreamWaitEvent(st, ev_join, 0)) != cudaSuccess) return err;
    if ((err = cudaStreamWaitEvent(st, ev_larft, 0)) != cudaSuccess) return err;
    stage(sctx, 2, 0);
    // two-stage reduction: the band stage's reflectors first (Z <- Q2 Z), then Q1 as below
    if (d_Q2 && (err = launch_q2_apply(d_desc, batch, max_n, d_Q2, q2t_off, d_Z, st)) != cudaSuccess) return err;
    err = bt_variant == 1 ? launch_backtransform_tc5(d_desc, batch, max_n, d_VT, vt_plane, d_Z, d_zscale, d_status,
                                                     wait_iters, shift, st)
                          : launch_backtransform_tc(d_desc, batch, max_n, max_ld, d_VT, vt_plane, d_Z, d_zscale, shift,
                                                    st);
    if (err != cudaSuccess) return err;
    stage(sctx, 2, 1);
    stage(sctx, 3, 0);
    refine_kernel<<<dim3(batch, (max_n + 31) / 32), 32 * kRfSeg, sizeof(float2) * (size_t)max_ld, st>>>(
        d_desc, d_Z, d_diag, d_theta);
    if ((err = cudaGetLastError()) != cudaSuccess) return err;
    const size_t sm_s = (sizeof(double) + sizeof(int)) * max_ld;
    if ((err = cudaFuncSetAttribute(sort_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_s))) return err;
    sort_kernel<<<batch, 128, sm_s, st>>>(d_desc, d_theta, d_w, d_perm, d_status);
    if ((err = cudaGetLastError()) != cudaSuccess) return err;
    stage(sctx, 3, 1);
    return cudaSuccess;
}

// FP64 compact-WY factors and back-transformation (X = Q Z with Z row-major in
// global memory) for the plain path's eigenvectors.
cudaError_t launch_backtransform_f64(const ChainDesc* d_desc, int batch, int max_n, int max_ld, const double* d_A,
                                     const double* d_tau, double* d_Tf, double* d_Z, cudaStream_t st) {
    if (batch <= 0) return cudaSuccess;
    cudaError_t err;
    const int npanel = (max_n + kNb - 1) / kNb;
    larft_kernel<double><<<dim3(batch, npanel), 256, 0, st>>>(d_desc, d_A, d_tau, d_Tf, nullptr, 0, 1);
    if ((err = cudaGetLastError()) != cudaSuccess) return err;
    const size_t sm_bt = backtransform_smem_bytes<double, false>(max_ld);
    if ((err = cudaFuncSetAttribute(backtransform_kernel<double, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_bt))) return err;
    if (batch > 65535) return cudaErrorInvalidValue;  // grid y limit
    backtransform_kernel<double, false><<<dim3((max_n + 31) / 32, batch), kBtThreads, sm_bt, st>>>(d_desc, d_A, d_Tf, d_Z);
    return cudaGetLastError();
}

}  // namespace fkg
