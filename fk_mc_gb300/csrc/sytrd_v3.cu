// sytrd_v3.cu — blocked Householder tridiagonalisation, one CTA per chain,
// FP64 (plain path) or FP32 (mixed path).
//
// Replaces the first half of Eigen::SelfAdjointEigenSolver at
// src/configuration.cpp:213; the Hamiltonian build (src/configuration.cpp:79-91)
// and the dense copy (:212) are fused into the matrix load.
//
// Algorithm (panel of NB reflectors, deferred symmetric rank-2k update):
//   for each column k of a panel:
//     (1) apply the panel's pending updates to column k;
//     (2) Householder reflector of A(k+1:, k) (v, tau, beta);
//     (3) p = A22 v with the STALE trailing matrix, corrected:
//         p -= V (W^T v) + W (V^T v);  w = tau p - (tau/2)(tau p . v) v;
//   after the panel: A22 -= V W^T + W V^T on the lower triangle.
// The trailing matrix is read once per column (the matrix-vector product) and
// read+written once per panel (the rank-2k update).
//
// The design aims at a low instruction count per matrix element, which is
// what bounds this kernel on GB300 (the FP32 version is issue bound, the FP64
// version bound by the narrow FP64 pipe):
//   * the padding rows/columns and the upper part of every 32x32 diagonal
//     tile are zeroed once, so interior tiles load with no per-element masks
//     (entries outside the active window multiply a zero of v);
//   * the panel's V and W live in shared memory as rows of NB contiguous
//     values (VpT[i][l]), read with vector loads by the corrections and the
//     rank-2k update; W never touches global memory;
//   * matrix-vector tiles issue their 32 column loads before using them;
//     column sums go through a padded per-warp shared-memory transpose;
//   * 8 warps per CTA; FP32 at N <= 576 fits two CTAs per SM.
#include "fkg_common.cuh"

namespace fkg {
namespace {

constexpr int kPad = kTile + 1;
constexpr int kWarps = 8;
constexpr int kThreads = kWarps * 32;
constexpr int kColRegs = 4;                    // column entries per thread kept in registers
constexpr int kColCache = kColRegs * kThreads; // rows of the current column cached in registers

// Sums of V values over the 32 lanes of a warp by recursive halving: at the
// stage with offset o a lane keeps the half of its values that (lane & o)
// selects and adds the partner's copy of it; once one value is left the
// remaining lane bits are summed by a butterfly. Returns the total of value
// `idx` (every lane of a group of 32/V lanes holds the same one). V is a
// power of two <= 32; V - 1 + log2(32/V) shuffles instead of 5 V.
template <int V, typename T>
__device__ __forceinline__ T warp_reduce_scatter(T (&x)[V], int lane, int& idx) {
    int base = 0;
#pragma unroll
    for (int half = V / 2, o = 16; half >= 1; half >>= 1, o >>= 1) {
        const bool up = lane & o;
#pragma unroll
        for (int m = 0; m < half; ++m) {
            const T send = up ? x[m] : x[m + half];
            const T keep = up ? x[m + half] : x[m];
            x[m] = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
        if (up) base += half;
    }
    T t = x[0];
#pragma unroll
    for (int o = 16 / V; o >= 1; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    idx = base;
    return t;
}

// c - a b - d e. FP64: as two fused multiply-adds (written out, `c -= a * b +
// d * e` compiles to a multiply, a fused multiply-add and an add: three issues
// of the narrow FP64 pipe for two multiply-adds of work). FP32 keeps the
// written-out form and its rounding (that kernel is not bound by its pipe).
__device__ __forceinline__ double fnma2(double a, double b, double d, double e, double c) {
    return fma(-d, e, fma(-a, b, c));
}
__device__ __forceinline__ float fnma2(float a, float b, float d, float e, float c) { return c - (a * b + d * e); }

// four contiguous values from 16-byte-aligned shared memory (vector loads)
__device__ __forceinline__ void load4(const float* p, float (&o)[4]) {
    const float4 x = *reinterpret_cast<const float4*>(p);
    o[0] = x.x; o[1] = x.y; o[2] = x.z; o[3] = x.w;
}
__device__ __forceinline__ void load4(const double* p, double (&o)[4]) {
    const double2 x = *reinterpret_cast<const double2*>(p), y = *reinterpret_cast<const double2*>(p + 2);
    o[0] = x.x; o[1] = x.y; o[2] = y.x; o[3] = y.y;
}

// One CTA reduces one chain at a time. Without a work list (order == null)
// CTA b takes chain b; with one, the CTAs are persistent: each takes the next
// entry of `order` (chains sorted by decreasing n, longest first) from the
// counter until the list is used up, which balances uneven batches.
template <typename T, int NB>
__global__ void __launch_bounds__(kThreads, sizeof(T) == 4 ? 2 : 1)
sytrd_v3_kernel(const ChainDesc* __restrict__ descs, const double* __restrict__ diag, T* __restrict__ Aws,
                double* __restrict__ dout, double* __restrict__ eout, T* __restrict__ tauout,
                const int* __restrict__ order, int norder, int* __restrict__ counter, int* __restrict__ status) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_item;
    for (int item = blockIdx.x;;) {
    if (order) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
        __syncthreads();
        item = s_item;
        if (item >= norder) return;
    }
    const ChainDesc D = descs[order ? order[item] : item];
    const int n = D.n, ld = D.ld;
    T* __restrict__ A = Aws + D.a_off;
    T* VpT = reinterpret_cast<T*>(smem_raw);     // [ld][NB]
    T* WpT = VpT + (size_t)ld * NB;              // [ld][NB]
    T* pw = WpT + (size_t)ld * NB;               // [kWarps][ld]
    T* tile = pw + (size_t)kWarps * ld;          // [kWarps][32][kPad]
    T* v = tile + (size_t)kWarps * kTile * kPad; // [ld]
    T* p = v + ld;                               // [ld]
    T* c1 = p + ld;                              // [NB]  W^T v
    T* c2 = c1 + NB;                             // [NB]  V^T v
    T* red = c2 + NB;                            // [kWarps]
    T* red2 = red + kWarps;                      // [kWarps][2*NB]
    T* colk_s = red2 + kWarps * 2 * NB;          // [2]  A(s, k), A(k, k)
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    T* mytile = tile + (size_t)warp * kTile * kPad;
    T* mypw = pw + (size_t)warp * ld;

    // ---- build: zero the lower triangle (with padding) and the upper part of
    //      the diagonal tiles, then scatter H = hopping + diag(-mu_c + U f) ----
    for (int j = warp; j < ld; j += kWarps)
        for (int i = (j & ~31) + lane; i < ld; i += 32) A[(size_t)j * ld + i] = T(0);
    for (int t = tid; t < 2 * NB * ld; t += kThreads) VpT[t] = T(0);  // VpT and WpT
    for (int i = tid; i < ld; i += kThreads) { v[i] = T(0); p[i] = T(0); }
    __syncthreads();
    for (int i = tid; i < n; i += kThreads) {
        for (int q = D.rowptr[i]; q < D.rowptr[i + 1]; ++q) {
            const int j = D.col[q];
            if ((unsigned)j >= (unsigned)n) {  // a column outside [0, n): skipped, the call fails
                if (status) atomicOr(status, kStatusBadArg);
                continue;
            }
            if (j <= i) A[(size_t)j * ld + i] += T(D.val[q]);
        }
        A[(size_t)i * ld + i] += T(diag[D.v_off + i]);
    }
    __syncthreads();

    const int nt = ld / kTile;
    for (int k0 = 0; k0 < n - 2; k0 += NB) {
        const int nbk = min(NB, n - 2 - k0);
        for (int j = 0; j < nbk; ++j) {
            const int k = k0 + j, s = k + 1;
            T* colk = A + (size_t)k * ld;
            // ---- (1) pending updates of this panel on column k (rows k..n-1),
            //      kept in registers (row tid + kThreads q) for (2) ----
            T cv[kColRegs];
#pragma unroll
            for (int q = 0; q < kColRegs; ++q) {
                const int i = tid + kThreads * q;
                cv[q] = (i >= k && i < n) ? colk[i] : T(0);
            }
            if (j > 0) {
                T vk[NB], wk[NB];
#pragma unroll
                for (int l = 0; l < NB; ++l) { vk[l] = VpT[(size_t)k * NB + l]; wk[l] = WpT[(size_t)k * NB + l]; }
#pragma unroll
                for (int q = 0; q < kColRegs; ++q) {
                    const int i = tid + kThreads * q;
                    if (i >= k && i < n) {
                        T a = cv[q];
#pragma unroll
                        for (int l = 0; l < NB; ++l) a = fnma2(VpT[(size_t)i * NB + l], wk[l], WpT[(size_t)i * NB + l], vk[l], a);
                        cv[q] = a;
                    }
                }
                // rows beyond the register cache (ld > kColCache) go through global memory
                for (int i = tid + kColCache; i < n; i += kThreads) {
                    T a = colk[i];
#pragma unroll
                    for (int l = 0; l < NB; ++l) a = fnma2(VpT[(size_t)i * NB + l], wk[l], WpT[(size_t)i * NB + l], vk[l], a);
                    colk[i] = a;
                }
            }
            // ---- (2) reflector from A(s:, k) ----
            T part = T(0);
#pragma unroll
            for (int q = 0; q < kColRegs; ++q) {
                const int i = tid + kThreads * q;
                if (i > s && i < n) part += cv[q] * cv[q];
                if (i == s) colk_s[0] = cv[q];
                if (i == k) colk_s[1] = cv[q];
            }
            for (int i = tid + kColCache; i < n; i += kThreads) {
                const T x = colk[i];
                if (i > s) part += x * x;
                if (i == s) colk_s[0] = x;
                if (i == k) colk_s[1] = x;
            }
            const T sigma = block_sum(part, red);
            const T alpha = colk_s[0];
            T tau = T(0), beta = alpha, scale = T(0);
            if (sigma != T(0)) {
                const T xnorm = sqrt(alpha * alpha + sigma);
                beta = alpha >= T(0) ? -xnorm : xnorm;
                tau = (beta - alpha) / beta;
                scale = T(1) / (alpha - beta);
            }
            if (tid == 0) {
                eout[D.v_off + k] = (double)beta;
                dout[D.v_off + k] = (double)colk_s[1];
                tauout[D.v_off + k] = tau;
            }
#pragma unroll
            for (int q = 0; q < kColRegs; ++q) {
                const int i = tid + kThreads * q;
                if (i < ld) {
                    T vi = T(0);
                    if (i == s) vi = T(1);
                    else if (i > s && i < n) { vi = cv[q] * scale; colk[i] = vi; }
                    v[i] = vi;
                    VpT[(size_t)i * NB + j] = vi;
                }
            }
            for (int i = tid + kColCache; i < ld; i += kThreads) {
                T vi = T(0);
                if (i == s) vi = T(1);
                else if (i > s && i < n) { vi = colk[i] * scale; colk[i] = vi; }
                v[i] = vi;
                VpT[(size_t)i * NB + j] = vi;
            }
            for (int t = tid; t < kWarps * ld; t += kThreads) pw[t] = T(0);
            __syncthreads();
            if (tau == T(0)) {
                for (int i = tid; i < ld; i += kThreads) WpT[(size_t)i * NB + j] = T(0);
                __syncthreads();
                continue;
            }
            // ---- (3a) p = A22 v, stale trailing matrix, lower tiles, no masks ----
            // Warp w takes tiles w, w + kWarps, ... of the lower tiles (I, J),
            // I0 <= J <= I, in row order; the column sums go through a
            // shared-memory transpose of the tile. FP32 keeps two tiles in
            // registers: the next tile's 32 loads are in flight while the
            // current one is used.
            {
                const int I0 = s >> 5;
                const int ntr = nt - I0;
                const int total = ntr * (ntr + 1) / 2;
                auto advance = [&](int& I, int& J, int by) {
                    J += by;
                    while (J > I) { J -= I - I0 + 1; ++I; }
                };
                auto load = [&](int I, int J, T (&a)[kTile]) {
                    const T* At = A + (size_t)(J * kTile) * ld + I * kTile + lane;
#pragma unroll
                    for (int c = 0; c < kTile; ++c) a[c] = At[(size_t)c * ld];
                };
                auto use = [&](int I, int J, const T (&a)[kTile]) {
                    const int i = I * kTile + lane;
                    const T* vJ = v + J * kTile;
                    T r0 = T(0), r1 = T(0), r2 = T(0), r3 = T(0);
#pragma unroll
                    for (int c = 0; c < kTile; c += 4) {
                        T x[4];
                        load4(vJ + c, x);  // broadcast, 16-byte aligned
                        r0 += a[c] * x[0];
                        r1 += a[c + 1] * x[1];
                        r2 += a[c + 2] * x[2];
                        r3 += a[c + 3] * x[3];
                    }
#pragma unroll
                    for (int c = 0; c < kTile; ++c) mytile[c * kPad + lane] = a[c];
                    if (I == J) mytile[lane * kPad + lane] = T(0);  // diagonal counted once, in the row sums
                    __syncwarp();
                    const T* vI = v + I * kTile;
                    T q0 = T(0), q1 = T(0), q2 = T(0), q3 = T(0);
#pragma unroll
                    for (int r = 0; r < kTile; r += 4) {
                        T x[4];
                        load4(vI + r, x);
                        q0 += mytile[lane * kPad + r] * x[0];
                        q1 += mytile[lane * kPad + r + 1] * x[1];
                        q2 += mytile[lane * kPad + r + 2] * x[2];
                        q3 += mytile[lane * kPad + r + 3] * x[3];
                    }
                    mypw[i] += (r0 + r1) + (r2 + r3);
                    mypw[J * kTile + lane] += (q0 + q1) + (q2 + q3);
                    __syncwarp();
                };
                int I = I0, J = I0;
                advance(I, J, warp);
                if constexpr (sizeof(T) == 4) {
                    T a0[kTile], a1[kTile];
                    int t = warp;
                    if (t < total) load(I, J, a0);
                    while (t < total) {
                        int I1 = I, J1 = J;
                        advance(I1, J1, kWarps);
                        const bool h1 = t + kWarps < total;
                        if (h1) load(I1, J1, a1);
                        use(I, J, a0);
                        if (!h1) break;
                        int I2 = I1, J2 = J1;
                        advance(I2, J2, kWarps);
                        const bool h2 = t + 2 * kWarps < total;
                        if (h2) load(I2, J2, a0);
                        use(I1, J1, a1);
                        t += 2 * kWarps;
                        I = I2;
                        J = J2;
                    }
                } else {
                    T a[kTile];
                    for (int t = warp; t < total; t += kWarps) {
                        load(I, J, a);
                        use(I, J, a);
                        advance(I, J, kWarps);
                    }
                }
            }
            // ---- (3b) c1 = W^T v, c2 = V^T v over the panel's earlier reflectors ----
            if (j > 0) {
                T s1[NB], s2[NB];
#pragma unroll
                for (int l = 0; l < NB; ++l) { s1[l] = T(0); s2[l] = T(0); }
                for (int i = s + tid; i < n; i += kThreads) {
                    const T vi = v[i];
#pragma unroll
                    for (int l = 0; l < NB; ++l) {
                        s1[l] += WpT[(size_t)i * NB + l] * vi;
                        s2[l] += VpT[(size_t)i * NB + l] * vi;
                    }
                }
                T x[2 * NB];
#pragma unroll
                for (int l = 0; l < NB; ++l) { x[l] = s1[l]; x[NB + l] = s2[l]; }
                int idx;
                const T tot = warp_reduce_scatter<2 * NB>(x, lane, idx);
                if ((lane & (32 / (2 * NB) - 1)) == 0) red2[warp * 2 * NB + idx] = tot;
            }
            __syncthreads();
            if (j > 0 && tid < 2 * NB) {
                T acc = T(0);
                for (int w8 = 0; w8 < kWarps; ++w8) acc += red2[w8 * 2 * NB + tid];
                c1[tid] = acc;  // c1[0..NB) then c2[0..NB) (contiguous)
            }
            __syncthreads();
            // ---- (3c)+(4) p corrected, scaled; w = p - K v into WpT(:, j) ----
            part = T(0);
            for (int i = s + tid; i < n; i += kThreads) {
                T q = T(0);
#pragma unroll
                for (int w8 = 0; w8 < kWarps; ++w8) q += pw[(size_t)w8 * ld + i];
                if (j > 0)
#pragma unroll
                    for (int l = 0; l < NB; ++l) q = fnma2(VpT[(size_t)i * NB + l], c1[l], WpT[(size_t)i * NB + l], c2[l], q);
                q *= tau;
                p[i] = q;
                part += q * v[i];
            }
            const T pv = block_sum(part, red);
            const T K = T(0.5) * tau * pv;
            for (int i = tid; i < ld; i += kThreads)
                WpT[(size_t)i * NB + j] = (i >= s && i < n) ? p[i] - K * v[i] : T(0);
            __syncthreads();
        }
        // ---- (5) A(tb:, tb:) -= V W^T + W V^T (lower tiles) ----
        // FP32: on the tensor cores. Per 32 x 32 tile, u = [V_I W_I] [W_J V_J]^T
        // (K = 2 NB) as mma.sync m16n8k8 3xTF32 from zero, then A -= u with
        // round-to-nearest FP32 (the tensor core's own accumulation truncates);
        // the tile (in accumulator layout) is loaded before u is formed.
        // FP64 (bound by its FP64 pipe, not by latency): four columns at a
        // time with fewer live registers.
        if constexpr (sizeof(T) == 4) {
            const int tb = k0 + nbk;
            const int I0 = tb >> 5;
            const int ntr = nt - I0;
            const int total = ntr * (ntr + 1) / 2;
            constexpr int KS = (2 * NB + 7) / 8;  // k-steps of 8
            const int g = lane >> 2, t4 = lane & 3;
            auto advance = [&](int& I, int& J, int by) {
                J += by;
                while (J > I) { J -= I - I0 + 1; ++I; }
            };
            // element (row, k) of [V W] and (col, k) of [W V]: k < NB from the
            // first panel, else from the second
            auto aval = [&](int row, int k, bool first) {
                return first ? VpT[(size_t)row * NB + k] : WpT[(size_t)row * NB + k - NB];
            };
            auto bval = [&](int col, int k, bool first) {
                return first ? WpT[(size_t)col * NB + k] : VpT[(size_t)col * NB + k - NB];
            };
            int I = I0, J = I0;
            advance(I, J, warp);
            for (int tt = warp; tt < total; tt += kWarps) {
                float c[8][4];
#pragma unroll
                for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                    for (int nt8 = 0; nt8 < 4; ++nt8) {
                        const int row = I * kTile + mt * 16 + g, col = J * kTile + nt8 * 8 + 2 * t4;
                        c[mt * 4 + nt8][0] = A[(size_t)col * ld + row];
                        c[mt * 4 + nt8][1] = A[(size_t)(col + 1) * ld + row];
                        c[mt * 4 + nt8][2] = A[(size_t)col * ld + row + 8];
                        c[mt * 4 + nt8][3] = A[(size_t)(col + 1) * ld + row + 8];
                    }
                float u[8][4];
#pragma unroll
                for (int q = 0; q < 8; ++q) u[q][0] = u[q][1] = u[q][2] = u[q][3] = 0.f;
#pragma unroll
                for (int ks = 0; ks < KS; ++ks) {
                    const int k0a = ks * 8 + t4, k0b = k0a + 4;
                    const bool fa = ks * 8 < NB, fb = ks * 8 + 4 < NB;  // NB is a multiple of 4
                    unsigned ah[2][4], al[2][4];
#pragma unroll
                    for (int mt = 0; mt < 2; ++mt) {
                        const int row = I * kTile + mt * 16 + g;
                        split_tf32(aval(row, k0a, fa), ah[mt][0], al[mt][0]);
                        split_tf32(aval(row + 8, k0a, fa), ah[mt][1], al[mt][1]);
                        split_tf32(aval(row, k0b, fb), ah[mt][2], al[mt][2]);
                        split_tf32(aval(row + 8, k0b, fb), ah[mt][3], al[mt][3]);
                    }
#pragma unroll
                    for (int nt8 = 0; nt8 < 4; ++nt8) {
                        const int col = J * kTile + nt8 * 8 + g;
                        unsigned bh[2], bl[2];
                        split_tf32(bval(col, k0a, fa), bh[0], bl[0]);
                        split_tf32(bval(col, k0b, fb), bh[1], bl[1]);
#pragma unroll
                        for (int mt = 0; mt < 2; ++mt) {
                            mma_tf32(u[mt * 4 + nt8], al[mt], bh);
                            mma_tf32(u[mt * 4 + nt8], ah[mt], bl);
                            mma_tf32(u[mt * 4 + nt8], ah[mt], bh);
                        }
                    }
                }
                const bool edge = (J == I0) || (I == J);  // holds columns < tb or the diagonal
#pragma unroll
                for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                    for (int nt8 = 0; nt8 < 4; ++nt8)
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            const int row = I * kTile + mt * 16 + g + (q >> 1) * 8;
                            const int col = J * kTile + nt8 * 8 + 2 * t4 + (q & 1);
                            const float x = c[mt * 4 + nt8][q] - u[mt * 4 + nt8][q];
                            if (!edge || (col >= tb && row >= col)) A[(size_t)col * ld + row] = x;
                        }
                advance(I, J, kWarps);
            }
        } else {
        const int tb = k0 + nbk;
        const int I0 = tb >> 5;
        int cnt = 0;
        for (int I = I0; I < nt; ++I) {
            for (int J = I0; J <= I; ++J, ++cnt) {
                if ((cnt & (kWarps - 1)) != warp) continue;
                const int i = I * kTile + lane;
                T VI[NB], WI[NB];
#pragma unroll
                for (int l = 0; l < NB; ++l) { VI[l] = VpT[(size_t)i * NB + l]; WI[l] = WpT[(size_t)i * NB + l]; }
                T* At = A + (size_t)(J * kTile) * ld + i;
                const bool edge = (J == I0) || (I == J);
                if (!edge) {
                    for (int c = 0; c < kTile; c += 4) {
                        T acc[4];
#pragma unroll
                        for (int q = 0; q < 4; ++q) acc[q] = At[(size_t)(c + q) * ld];
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            const T* vj = VpT + (size_t)(J * kTile + c + q) * NB;
                            const T* wj = WpT + (size_t)(J * kTile + c + q) * NB;
#pragma unroll
                            for (int l = 0; l < NB; ++l) acc[q] = fnma2(VI[l], wj[l], WI[l], vj[l], acc[q]);
                        }
#pragma unroll
                        for (int q = 0; q < 4; ++q) At[(size_t)(c + q) * ld] = acc[q];
                    }
                } else {
                    for (int c = 0; c < kTile; ++c) {
                        const int jc = J * kTile + c;
                        if (jc < tb || i < jc) continue;
                        const T* vj = VpT + (size_t)jc * NB;
                        const T* wj = WpT + (size_t)jc * NB;
                        T a = At[(size_t)c * ld];
#pragma unroll
                        for (int l = 0; l < NB; ++l) a = fnma2(VI[l], wj[l], WI[l], vj[l], a);
                        At[(size_t)c * ld] = a;
                    }
                }
            }
        }
        }
        __syncthreads();
        for (int t = tid; t < 2 * NB * ld; t += kThreads) VpT[t] = T(0);
        __syncthreads();
    }
    // ---- the trailing 2 x 2 block ----
    if (tid == 0 && n >= 2) {
        dout[D.v_off + n - 2] = (double)A[(size_t)(n - 2) * ld + n - 2];
        eout[D.v_off + n - 2] = (double)A[(size_t)(n - 2) * ld + n - 1];
        tauout[D.v_off + n - 2] = T(0);
    }
    if (tid == 0) dout[D.v_off + n - 1] = (double)A[(size_t)(n - 1) * ld + n - 1];
    if (!order) return;
    }
}

template <typename T, int NB>
size_t v3_smem(int max_ld) {
    return sizeof(T) * ((size_t)(2 * NB + kWarps + 2) * max_ld + (size_t)kWarps * kTile * kPad + 2 * NB + kWarps +
                        (size_t)kWarps * 2 * NB + 2);
}

template <typename T, int NB>
cudaError_t launch_v3(const ChainDesc* d_desc, int batch, int max_ld, const double* d_diag, T* d_A, double* d_d,
                      double* d_e, T* d_tau, const int* d_order, int* d_counter, int num_sms, cudaStream_t st,
                      int* d_status) {
    if (batch <= 0) return cudaSuccess;
    const size_t smem = v3_smem<T, NB>(max_ld);
    cudaError_t err = cudaFuncSetAttribute(sytrd_v3_kernel<T, NB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    int grid = batch;
    if (d_order) {  // persistent: as many CTAs as fit on the GPU at once
        int per_sm = 0;
        if ((err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sytrd_v3_kernel<T, NB>, kThreads, smem))) return err;
        grid = max(1, min(batch, per_sm * num_sms));
        if ((err = cudaMemsetAsync(d_counter, 0, sizeof(int), st))) return err;
    }
    sytrd_v3_kernel<T, NB><<<grid, kThreads, smem, st>>>(d_desc, d_diag, d_A, d_d, d_e, d_tau, d_order, batch,
                                                         d_counter, d_status);
    return cudaGetLastError();
}

}  // namespace

// Panel widths compiled per precision; `variant` picks one (the autotuner's choice).
const int kSytrdF32Nb[3] = {4, 8, 16};
const int kSytrdF64Nb[2] = {2, 4};

cudaError_t launch_sytrd_v3_f64(const ChainDesc* d_desc, int batch, int max_ld, const double* d_diag, double* d_A,
                                double* d_d, double* d_e, double* d_tau, cudaStream_t st, int variant,
                                const int* d_order, int* d_counter, int num_sms, int* d_status) {
    if (variant == 0)
        return launch_v3<double, 2>(d_desc, batch, max_ld, d_diag, d_A, d_d, d_e, d_tau, d_order, d_counter, num_sms, st, d_status);
    return launch_v3<double, 4>(d_desc, batch, max_ld, d_diag, d_A, d_d, d_e, d_tau, d_order, d_counter, num_sms, st, d_status);
}

cudaError_t launch_sytrd_v3_f32(const ChainDesc* d_desc, int batch, int max_ld, const double* d_diag, float* d_A,
                                double* d_d, double* d_e, float* d_tau, cudaStream_t st, int variant,
                                const int* d_order, int* d_counter, int num_sms, int* d_status) {
    if (variant == 0)
        return launch_v3<float, 4>(d_desc, batch, max_ld, d_diag, d_A, d_d, d_e, d_tau, d_order, d_counter, num_sms, st, d_status);
    if (variant == 2)
        return launch_v3<float, 16>(d_desc, batch, max_ld, d_diag, d_A, d_d, d_e, d_tau, d_order, d_counter, num_sms, st, d_status);
    return launch_v3<float, 8>(d_desc, batch, max_ld, d_diag, d_A, d_d, d_e, d_tau, d_order, d_counter, num_sms, st, d_status);
}

}  // namespace fkg
