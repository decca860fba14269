// twostage.cu — two-stage tridiagonalisation of the mixed path (FP32):
// dense -> band (bandwidth kBand) -> tridiagonal, and the band stage's part of
// the back-transformation.
//
// Replaces, like sytrd_v3.cu, the first half of Eigen::SelfAdjointEigenSolver
// at src/configuration.cpp:213 (the Hamiltonian build of
// src/configuration.cpp:79-91 and the dense copy of :212 are fused into the
// matrix load). The one-stage reduction reads the whole trailing matrix for
// every column (a matrix-vector product per reflector); here the trailing
// matrix is read and written three times per panel of kBand columns:
//
// Stage 1 (sy2sb_kernel), one CTA per chain, panels of kBand columns:
//   (a) QR of the panel A(k0+b : n, k0 : k0+b) in shared memory (Householder,
//       one column at a time): reflector j has its unit at row k0+b+j and is
//       stored below the band in column k0+j; R stays in the band;
//   (b) the compact-WY factor T of the panel, T^-1 = diag(1/tau) + triu(V^T V, 1);
//   (c) X = A22 (V T) over the full symmetric trailing matrix A22 (m x m);
//   (d) W = X - 1/2 V (T^T (V^T X));
//   (e) A22 -= V W^T + W V^T (both triangles: the next panels read rows).
// Stage 2 (sb2st_kernel), one CTA per chain, the band in shared memory:
//   bulge chasing with one column per sweep (Schwarz; Bischof, Lang and Sun's
//   successive band reduction with Householder reflectors): task (s, k) of
//   sweep s builds a reflector of length <= b from column c0 (= s for k = 0,
//   else the previous block's first column) on rows p = s + 1 + k b ..,
//   applies it to the block on the left (rows p.., columns c0 .. p-1), to the
//   diagonal block from both sides and to the block below from the right,
//   which leaves the next bulge in that block's first column. Sweep s + 1's
//   task k touches no element that sweep s's task k + 3 touches, so step t
//   runs every task (s, t - 3 s) at once, one warp each, with one barrier per
//   step (3 n steps). Band storage: column c holds A(c + d, c), d < 2 b (the
//   bulge reaches 2 b - 1 below the diagonal).
// Back-transformation of stage 2 (q2_apply_kernel): Z <- Q2 Z, sweeps in
//   reverse order, the reflectors of one sweep (disjoint rows) at once; the
//   stage-1 part uses the compact-WY back-transformation of the one-stage path
//   with the reflectors' unit row at k + b instead of k + 1.
#include "fkg_common.cuh"

namespace fkg {
namespace {

constexpr int kB = kBand;          // bandwidth between the stages
constexpr int kLdb = 2 * kB + 2;   // band storage per column (even: conflict-free rows)
constexpr int kS1Threads = 256;
constexpr int kS1Warps = kS1Threads / 32;
constexpr int kS2Warps = 16;
constexpr int kQ2Cols = 32;        // columns of Z per CTA of the stage-2 back-transformation
constexpr int kQ2Warps = 16;

// ---------------------------------------------------------------- stage 1

// Sum over the CTA of NV values per thread; every thread gets all NV sums in
// out[] (shared memory, NV floats). red: kS1Warps * NV floats of scratch.
template <int NV>
__device__ __forceinline__ void block_sums(float (&x)[NV], float* red, float* out) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        float v = x[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        x[q] = v;
    }
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < NV; ++q) red[warp * NV + q] = x[q];
    __syncthreads();
    if ((int)threadIdx.x < NV) {
        float s = 0.f;
        for (int w = 0; w < kS1Warps; ++w) s += red[w * NV + threadIdx.x];
        out[threadIdx.x] = s;
    }
    __syncthreads();
}

// One CTA per chain (persistent over the longest-first work list when given).
// Shared memory: the panel [kB][max_ld + 1] (column-major, V after the QR), V T
// and W [max_ld][kB] (row-major), T [kB][kB + 1], reductions: 113 KB at
// max_ld = 576, two CTAs per SM.
__global__ void __launch_bounds__(kS1Threads, 2)
sy2sb_kernel(const ChainDesc* __restrict__ descs, const double* __restrict__ diag, float* __restrict__ Aws,
             float* __restrict__ tauout, const int* __restrict__ order, int norder, int* __restrict__ counter,
             int* __restrict__ status, int max_ld) {
    extern __shared__ __align__(16) float s1[];
    const int pst = max_ld + 1;                      // panel column stride (conflict-free V^T V)
    float* P = s1;                                   // [kB][pst]: panel column j at P + j * pst
    float* VT = P + (size_t)kB * pst;                // [max_ld][kB]
    float* W = VT + (size_t)kB * max_ld;             // [max_ld][kB]: X, then W
    float* Ts = W + (size_t)kB * max_ld;             // [kB][kB + 1]
    float* G = Ts + kB * (kB + 1);                   // [kB][kB + 1]: V^T V, then V^T X, then T^T V^T X
    float* red = G + kB * (kB + 1);                  // [kS1Warps][kB]
    float* sums = red + kS1Warps * kB;               // [kB + 2]
    float* taus = sums + kB + 2;                     // [kB]
    __shared__ int s_item;
    const int tid = threadIdx.x;
    for (int item = blockIdx.x;;) {
        if (order) {
            __syncthreads();
            if (tid == 0) s_item = atomicAdd(counter, 1);
            __syncthreads();
            item = s_item;
            if (item >= norder) return;
        }
        const ChainDesc D = descs[order ? order[item] : item];
        const int n = D.n, ld = D.ld;
        float* __restrict__ A = Aws + D.a_off;

        // ---- build the full symmetric H = hopping + diag(-mu_c + U f) ----
        for (size_t t = tid; t < (size_t)ld * ld; t += kS1Threads) A[t] = 0.f;
        __syncthreads();
        for (int i = tid; i < n; i += kS1Threads) {
            for (int q = D.rowptr[i]; q < D.rowptr[i + 1]; ++q) {
                const int j = D.col[q];
                if ((unsigned)j >= (unsigned)n) {  // a column outside [0, n): skipped, the call fails
                    if (status) atomicOr(status, kStatusBadArg);
                    continue;
                }
                A[(size_t)j * ld + i] += (float)D.val[q];  // row i of the symmetric CSR: column i of A
            }
            A[(size_t)i * ld + i] += (float)diag[D.v_off + i];
        }
        __syncthreads();

        for (int k0 = 0; k0 + kB <= n - 2; k0 += kB) {
            const int r0 = k0 + kB, m = n - r0, kb = min(kB, m - 1);
            // ---- (a) the panel A(r0:n, k0:k0+kB) into shared memory ----
            for (int t = tid; t < kB * m; t += kS1Threads) {
                const int j = t / m, i = t - j * m;
                P[(size_t)j * pst + i] = A[(size_t)(k0 + j) * ld + r0 + i];
            }
            __syncthreads();
            // ---- QR, one column at a time ----
            for (int j = 0; j < kb; ++j) {
                float* pj = P + (size_t)j * pst;
                float part[1] = {0.f};
                for (int i = j + 1 + tid; i < m; i += kS1Threads) part[0] += pj[i] * pj[i];
                block_sums<1>(part, red, sums);
                const float sigma = sums[0], alpha = pj[j];
                float tau = 0.f, beta = alpha, scale = 0.f;
                if (sigma != 0.f) {
                    beta = -copysignf(sqrtf(alpha * alpha + sigma), alpha);
                    tau = (beta - alpha) / beta;
                    scale = 1.f / (alpha - beta);
                }
                for (int i = j + 1 + tid; i < m; i += kS1Threads) pj[i] *= scale;
                __syncthreads();
                if (tid == 0) {
                    pj[j] = beta;
                    taus[j] = tau;
                    tauout[D.v_off + k0 + j] = tau;
                }
                // apply H_j to the panel's later columns: w_l = v^T P(:, l), P(:, l) -= tau v w_l
                float w[kB];
#pragma unroll
                for (int l = 0; l < kB; ++l) w[l] = 0.f;
                for (int i = j + tid; i < m; i += kS1Threads) {
                    const float vi = i == j ? 1.f : pj[i];
#pragma unroll
                    for (int l = 0; l < kB; ++l)
                        if (l > j) w[l] += vi * P[(size_t)l * pst + i];
                }
                block_sums<kB>(w, red, sums);
                for (int i = j + tid; i < m; i += kS1Threads) {
                    const float vi = i == j ? 1.f : pj[i];
#pragma unroll
                    for (int l = 0; l < kB; ++l)
                        if (l > j) P[(size_t)l * pst + i] -= tau * vi * sums[l];
                }
                __syncthreads();
            }
            if (tid < kB - kb) taus[kb + tid] = 0.f;
            // the panel back: R in the band, V below it
            for (int t = tid; t < kB * m; t += kS1Threads) {
                const int j = t / m, i = t - j * m;
                A[(size_t)(k0 + j) * ld + r0 + i] = P[(size_t)j * pst + i];
            }
            // ---- (b) G = V^T V, then T from its inverse ----
            // (V: unit at row j of column j, zero above; columns j >= kb are zero)
            auto vget = [&](int i, int j) -> float {
                return j >= kb ? 0.f : (i == j ? 1.f : (i > j ? P[(size_t)j * pst + i] : 0.f));
            };
            {
                const int c = tid & (kB - 1), g = tid / kB;  // 16 x 16 entries over 256 threads
                float acc = 0.f;
                for (int i = 0; i < m; ++i) acc += vget(i, g) * vget(i, c);
                G[g * (kB + 1) + c] = acc;
            }
            __syncthreads();
            if (tid < kB) {  // lane j: column j of T by back substitution on T^-1 = diag(1/tau) + triu(G, 1)
                const int j = tid;
                float t[kB];
#pragma unroll
                for (int r = kB - 1; r >= 0; --r) {
                    float s = 0.f;
#pragma unroll
                    for (int q = r + 1; q < kB; ++q) s += G[r * (kB + 1) + q] * t[q];
                    t[r] = r > j ? 0.f : (r == j ? taus[r] : -taus[r] * s);
                }
#pragma unroll
                for (int r = 0; r < kB; ++r) Ts[r * (kB + 1) + j] = t[r];
            }
            __syncthreads();
            // ---- V T, row by row ----
            for (int i = tid; i < m; i += kS1Threads) {
                float vr[kB];
#pragma unroll
                for (int l = 0; l < kB; ++l) vr[l] = vget(i, l);
#pragma unroll
                for (int c = 0; c < kB; ++c) {
                    float s = 0.f;
#pragma unroll
                    for (int l = 0; l < kB; ++l)
                        if (l <= c) s += vr[l] * Ts[l * (kB + 1) + c];
                    VT[(size_t)i * kB + c] = s;
                }
            }
            __syncthreads();
            // ---- (c) X = A22 (V T): lanes take consecutive rows i, so every column q
            //      of A22 is read coalesced ----
            const float* A22 = A + (size_t)r0 * ld + r0;
            for (int i = tid; i < m; i += kS1Threads) {
                float x[kB];
#pragma unroll
                for (int c = 0; c < kB; ++c) x[c] = 0.f;
                int q = 0;
                for (; q + 4 <= m; q += 4) {
                    float av[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) av[u] = A22[(size_t)(q + u) * ld + i];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const float4* vt = reinterpret_cast<const float4*>(VT + (size_t)(q + u) * kB);
#pragma unroll
                        for (int c4 = 0; c4 < kB / 4; ++c4) {
                            const float4 b = vt[c4];
                            x[4 * c4] += av[u] * b.x;
                            x[4 * c4 + 1] += av[u] * b.y;
                            x[4 * c4 + 2] += av[u] * b.z;
                            x[4 * c4 + 3] += av[u] * b.w;
                        }
                    }
                }
                for (; q < m; ++q) {
                    const float a = A22[(size_t)q * ld + i];
#pragma unroll
                    for (int c = 0; c < kB; ++c) x[c] += a * VT[(size_t)q * kB + c];
                }
#pragma unroll
                for (int c = 0; c < kB; ++c) W[(size_t)i * kB + c] = x[c];
            }
            __syncthreads();
            // ---- (d) W = X - 1/2 V (T^T (V^T X)) ----
            {
                const int c = tid & (kB - 1), g = tid / kB;
                float acc = 0.f;  // (V^T X)(g, c)
                for (int i = 0; i < m; ++i) acc += vget(i, g) * W[(size_t)i * kB + c];
                G[g * (kB + 1) + c] = acc;
            }
            __syncthreads();
            float mtc = 0.f;
            {
                const int c = tid & (kB - 1), g = tid / kB;  // (T^T (V^T X))(g, c) = sum_l T(l, g) (V^T X)(l, c)
                for (int l = 0; l <= g; ++l) mtc += Ts[l * (kB + 1) + g] * G[l * (kB + 1) + c];
            }
            __syncthreads();
            G[(tid / kB) * (kB + 1) + (tid & (kB - 1))] = mtc;
            __syncthreads();
            for (int i = tid; i < m; i += kS1Threads) {
                float vr[kB];
#pragma unroll
                for (int l = 0; l < kB; ++l) vr[l] = vget(i, l);
#pragma unroll
                for (int c = 0; c < kB; ++c) {
                    float s = 0.f;
#pragma unroll
                    for (int l = 0; l < kB; ++l) s += vr[l] * G[l * (kB + 1) + c];
                    W[(size_t)i * kB + c] -= 0.5f * s;
                }
            }
            // V as rows (into VT's place: V T is no longer needed)
            __syncthreads();
            for (int i = tid; i < m; i += kS1Threads)
#pragma unroll
                for (int l = 0; l < kB; ++l) VT[(size_t)i * kB + l] = vget(i, l);
            __syncthreads();
            // ---- (e) A22 -= V W^T + W V^T, both triangles; thread: row i of one column at a time ----
            float* A22w = A + (size_t)r0 * ld + r0;
            for (int i = tid; i < m; i += kS1Threads) {
                float vi[kB], wi[kB];
#pragma unroll
                for (int l = 0; l < kB; ++l) { vi[l] = VT[(size_t)i * kB + l]; wi[l] = W[(size_t)i * kB + l]; }
                for (int c = 0; c < m; ++c) {
                    const float4* vc = reinterpret_cast<const float4*>(VT + (size_t)c * kB);
                    const float4* wc = reinterpret_cast<const float4*>(W + (size_t)c * kB);
                    float s = 0.f;
#pragma unroll
                    for (int l4 = 0; l4 < kB / 4; ++l4) {
                        const float4 a = vc[l4], b = wc[l4];
                        s += vi[4 * l4] * b.x + wi[4 * l4] * a.x;
                        s += vi[4 * l4 + 1] * b.y + wi[4 * l4 + 1] * a.y;
                        s += vi[4 * l4 + 2] * b.z + wi[4 * l4 + 2] * a.z;
                        s += vi[4 * l4 + 3] * b.w + wi[4 * l4 + 3] * a.w;
                    }
                    A22w[(size_t)c * ld + i] -= s;
                }
            }
            __syncthreads();
        }
        if (!order) return;
    }
}

// ---------------------------------------------------------------- stage 2

// One task (s, k) of the bulge chase on the band held in shared memory
// (band[c * kLdb + d] = A(c + d, c)), by one warp. Lanes: r = lane & 15 is a
// row (or column) of the 16 x 16 blocks, h = lane >> 4 picks which half of the
// other index a lane sums over; the halves are added with one shuffle. vw: 32
// floats of this warp's scratch (v, then w). All shuffles run on the full warp.
__device__ __forceinline__ void sb_task(float* __restrict__ band, int n, int s, int k, float* __restrict__ q2v,
                                        float* __restrict__ q2t, int ld, float* __restrict__ vw) {
    const int lane = threadIdx.x & 31, r = lane & 15, h = lane >> 4;
    const int p = s + 1 + k * kB;
    const int ln = min(kB, n - p);
    const int c0 = k == 0 ? s : p - kB;
    // (1) reflector from A(p .. p+ln-1, c0): (I - tau v v^T) x = beta e_0
    const float x = r < ln ? band[c0 * kLdb + (p + r - c0)] : 0.f;
    float sq = (r > 0) ? x * x : 0.f;
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
    const float alpha = __shfl_sync(0xffffffffu, x, 0);
    float tau = 0.f, beta = alpha, scale = 0.f;
    if (sq != 0.f) {
        beta = -copysignf(sqrtf(alpha * alpha + sq), alpha);
        tau = (beta - alpha) / beta;
        scale = 1.f / (alpha - beta);
    }
    const float v = r == 0 ? 1.f : (r < ln ? x * scale : 0.f);
    if (h == 0) {
        if (r < ln) {
            band[c0 * kLdb + (p + r - c0)] = r == 0 ? beta : 0.f;
            q2v[(size_t)s * ld + p + r] = v;
        }
        vw[r] = v;
    }
    if (lane == 0) q2t[(size_t)s * (ld / kB) + k] = tau;
    __syncwarp();
    if (tau == 0.f) return;  // identity reflector (the same in every lane)
    // (2) the block on the left, columns c0+1 .. p-1 (k > 0): lane column j = c0 + r, rows 8h .. 8h+7
    if (k > 0) {
        const int j = c0 + r;
        float* colj = band + j * kLdb + (p - j);  // colj[i] = A(p + i, j)
        float w = 0.f;
        if (r > 0)
#pragma unroll
            for (int i = 8 * h; i < 8 * h + 8; ++i)
                if (i < ln) w += vw[i] * colj[i];
        w += __shfl_xor_sync(0xffffffffu, w, 16);
        if (r > 0)
#pragma unroll
            for (int i = 8 * h; i < 8 * h + 8; ++i)
                if (i < ln) colj[i] -= tau * vw[i] * w;
    }
    // (3) the diagonal block from both sides: y = D v (lane row r, columns 8h .. 8h+7)
    float y = 0.f;
    if (r < ln)
#pragma unroll
        for (int j = 8 * h; j < 8 * h + 8; ++j)
            if (j < ln) {
                const float d = r >= j ? band[(p + j) * kLdb + (r - j)] : band[(p + r) * kLdb + (j - r)];
                y += d * vw[j];
            }
    y += __shfl_xor_sync(0xffffffffu, y, 16);
    float w = tau * y;  // rows r >= ln: y = 0
    float dot = h == 0 ? w * vw[r] : 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, o);
    w += -0.5f * tau * dot * vw[r];
    __syncwarp();  // every lane has read D and vw before the updates
    if (h == 0) vw[16 + r] = w;
    __syncwarp();
    if (r < ln)
#pragma unroll
        for (int j = 8 * h; j < 8 * h + 8; ++j)
            if (j <= r) band[(p + j) * kLdb + (r - j)] -= vw[r] * vw[16 + j] + vw[16 + r] * vw[j];
    // (4) the block below from the right: rows p+ln+q (lane row q = r), columns p+i (i in half h)
    const int nr = min(kB, n - p - ln);
    float z = 0.f;
    if (r < nr)
#pragma unroll
        for (int i = 8 * h; i < 8 * h + 8; ++i)
            if (i < ln) z += band[(p + i) * kLdb + (ln + r - i)] * vw[i];
    z += __shfl_xor_sync(0xffffffffu, z, 16);
    if (r < nr)
#pragma unroll
        for (int i = 8 * h; i < 8 * h + 8; ++i)
            if (i < ln) band[(p + i) * kLdb + (ln + r - i)] -= tau * z * vw[i];
    __syncwarp();
}

// One CTA per chain: the band of the stage-1 matrix into shared memory, the
// wavefront of tasks (one barrier per step), then d and e. Q2: the reflectors
// of sweep s at q2v[s * ld + row] (unit first element stored) and their tau at
// q2t[s * (ld / kB) + k].
__global__ void __launch_bounds__(kS2Warps * 32, 2)
sb2st_kernel(const ChainDesc* __restrict__ descs, const float* __restrict__ Aws, double* __restrict__ dout,
             double* __restrict__ eout, float* __restrict__ Q2, long long q2t_off) {
    extern __shared__ __align__(16) float band[];  // [n][kLdb]
    __shared__ float vw_all[kS2Warps][32];
    const ChainDesc D = descs[blockIdx.x];
    const int n = D.n, ld = D.ld;
    const float* A = Aws + D.a_off;
    float* q2v = Q2 + D.a_off;
    float* q2t = Q2 + q2t_off + D.a_off / kB;
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int t = tid; t < n * kLdb; t += blockDim.x) {
        const int c = t / kLdb, d = t - c * kLdb;
        band[t] = (d <= kB && c + d < n) ? A[(size_t)c * ld + c + d] : 0.f;
    }
    __syncthreads();
    const int last = 3 * (n - 3);
    for (int t = 0; t <= last; ++t) {
        // sweeps with a task at step t: k = t - 3 s >= 0 and p = s + 1 + k b <= n - 2
        const int shi = min(t / 3, n - 3);
        const int num = t * kB + 3 - n;
        const int slo = num <= 0 ? 0 : (num + 3 * kB - 2) / (3 * kB - 1);
        for (int s = slo + warp; s <= shi; s += kS2Warps) {
            const int k = t - 3 * s;
            if (s + 1 + k * kB <= n - 2) sb_task(band, n, s, k, q2v, q2t, ld, vw_all[warp]);
        }
        __syncthreads();
    }
    for (int i = tid; i < n; i += blockDim.x) {
        dout[D.v_off + i] = (double)band[i * kLdb];
        eout[D.v_off + i] = i + 1 < n ? (double)band[i * kLdb + 1] : 0.0;
    }
}

// Z <- Q2 Z for the columns j0 .. j0+31 of one chain (Z row-major, Z[i * ld + j]),
// held in shared memory: sweeps from the last to the first; within a sweep the
// reflectors act on disjoint rows, one warp each, lane = column.
__global__ void __launch_bounds__(kQ2Warps * 32)
q2_apply_kernel(const ChainDesc* __restrict__ descs, const float* __restrict__ Q2, long long q2t_off,
                float* __restrict__ Zws) {
    extern __shared__ __align__(16) float zs[];  // [n][kQ2Cols]
    const ChainDesc D = descs[blockIdx.y];
    const int n = D.n, ld = D.ld, j0 = blockIdx.x * kQ2Cols;
    if (j0 >= n) return;
    const float* q2v = Q2 + D.a_off;
    const float* q2t = Q2 + q2t_off + D.a_off / kB;
    float* Z = Zws + D.a_off;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const bool colok = j0 + lane < n;
    for (int i = warp; i < n; i += kQ2Warps) zs[i * kQ2Cols + lane] = colok ? Z[(size_t)i * ld + j0 + lane] : 0.f;
    __syncthreads();
    for (int s = n - 3; s >= 0; --s) {
        const int nk = (n - 2 - (s + 1)) / kB + 1;  // blocks k with s + 1 + k b <= n - 2
        for (int k = warp; k < nk; k += kQ2Warps) {
            const int p = s + 1 + k * kB, ln = min(kB, n - p);
            const float tau = q2t[(size_t)s * (ld / kB) + k];
            if (tau == 0.f) continue;
            const float* v = q2v + (size_t)s * ld + p;
            float* zc = zs + p * kQ2Cols + lane;
            float vv[kB];
            float dot = 0.f;
#pragma unroll
            for (int i = 0; i < kB; ++i) {
                vv[i] = i < ln ? v[i] : 0.f;
                if (i < ln) dot += vv[i] * zc[i * kQ2Cols];
            }
            dot *= tau;
#pragma unroll
            for (int i = 0; i < kB; ++i)
                if (i < ln) zc[i * kQ2Cols] -= dot * vv[i];
        }
        __syncthreads();
    }
    if (colok)
        for (int i = warp; i < n; i += kQ2Warps) Z[(size_t)i * ld + j0 + lane] = zs[i * kQ2Cols + lane];
}

}  // namespace

size_t sy2sb_smem_bytes(int max_ld) {
    return sizeof(float) * ((size_t)kB * (max_ld + 1) + (size_t)2 * kB * max_ld + 2 * kB * (kB + 1) + kS1Warps * kB +
                            2 * kB + 2);
}

cudaError_t launch_sy2sb(const ChainDesc* d_desc, int batch, int max_ld, const double* d_diag, float* d_A,
                         float* d_tau, const int* d_order, int* d_counter, int num_sms, int* d_status,
                         cudaStream_t st) {
    if (batch <= 0) return cudaSuccess;
    const size_t smem = sy2sb_smem_bytes(max_ld);
    cudaError_t err = cudaFuncSetAttribute(sy2sb_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    int grid = batch;
    if (d_order) {
        int per_sm = 0;
        if ((err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sy2sb_kernel, kS1Threads, smem))) return err;
        grid = max(1, min(batch, per_sm * num_sms));
        if ((err = cudaMemsetAsync(d_counter, 0, sizeof(int), st))) return err;
    }
    sy2sb_kernel<<<grid, kS1Threads, smem, st>>>(d_desc, d_diag, d_A, d_tau, d_order, batch, d_counter, d_status,
                                                 max_ld);
    return cudaGetLastError();
}

cudaError_t launch_sb2st(const ChainDesc* d_desc, int batch, int max_n, const float* d_A, double* d_d, double* d_e,
                         float* d_Q2, long long q2t_off, cudaStream_t st) {
    if (batch <= 0) return cudaSuccess;
    const size_t smem = sizeof(float) * (size_t)max_n * kLdb;
    cudaError_t err = cudaFuncSetAttribute(sb2st_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    sb2st_kernel<<<batch, kS2Warps * 32, smem, st>>>(d_desc, d_A, d_d, d_e, d_Q2, q2t_off);
    return cudaGetLastError();
}

cudaError_t launch_q2_apply(const ChainDesc* d_desc, int batch, int max_n, const float* d_Q2, long long q2t_off,
                            float* d_Z, cudaStream_t st) {
    if (batch <= 0) return cudaSuccess;
    if (batch > 65535) return cudaErrorInvalidValue;  // grid y limit
    const size_t smem = sizeof(float) * (size_t)max_n * kQ2Cols;
    cudaError_t err = cudaFuncSetAttribute(q2_apply_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    q2_apply_kernel<<<dim3((max_n + kQ2Cols - 1) / kQ2Cols, batch), kQ2Warps * 32, smem, st>>>(d_desc, d_Q2, q2t_off,
                                                                                             d_Z);
    return cudaGetLastError();
}

}  // namespace fkg
