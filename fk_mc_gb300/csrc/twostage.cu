// twostage.cu — two-stage tridiagonalisation of the mixed path (FP32):
// dense -> band (bandwidth kBand) -> tridiagonal, and the band stage's part of
// the back-transformation.
//
// Replaces, like sytrd_v3.cu, the first half of Eigen::SelfAdjointEigenSolver
// at src/configuration.cpp:213 (the Hamiltonian build of
// src/configuration.cpp:79-91 and the dense copy of :212 are fused into the
// matrix load). The one-stage reduction reads the whole trailing matrix for
// every column (a matrix-vector product per reflector); here the trailing
// matrix is read once and read + written once per panel of kBand columns, as
// tensor-core GEMMs:
//
// Stage 1 (sy2sb_kernel), one CTA per chain, panels of kBand columns:
//   (a) QR of the panel A(k0+b : n, k0 : k0+b) in shared memory (Householder,
//       one column at a time): reflector j has its unit at row k0+b+j and is
//       stored below the band in column k0+j; R stays in the band;
//   (b) the compact-WY factor T of the panel, T^-1 = diag(1/tau) + triu(V^T V, 1);
//   (c) X = A22 (V T) over the full symmetric trailing matrix A22 (m x m);
//   (d) W = X - 1/2 V (T^T (V^T X));
//   (e) A22 -= V W^T + W V^T (both triangles: the next panels read rows).
//   (c) and (e) run on tcgen05 (see sy2sb_kernel).
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
//   step (3 n steps; measured faster than a progress counter per sweep, whose
//   spinning warps take issue slots from the working ones). Band storage:
//   column c holds A(c + d, c), d < 2 b (the bulge reaches 2 b - 1 below the
//   diagonal).
// Back-transformation of stage 2 (q2_apply_kernel): Z <- Q2 Z by groups of b
//   sweeps, each a product of b-reflector blocks on 31-row windows applied to
//   register-resident columns; the stage-1 part uses the compact-WY
//   back-transformation of the one-stage path with the reflectors' unit row at
//   k + b instead of k + 1.
#include "fkg_common.cuh"
#include "tcgen05.cuh"

namespace fkg {
namespace {

constexpr int kB = kBand;          // bandwidth between the stages
constexpr int kLdb = 2 * kB + 2;   // band storage per column (even: conflict-free rows)
constexpr int kS1Threads = 256;
constexpr int kS1Warps = kS1Threads / 32;
constexpr int kS2Warps = 16;       // tasks of one wavefront step run at once (about n / (3 b))
constexpr int kQ2Thr = 32;         // threads per CTA of the stage-2 back-transformation
constexpr int kQ2Cols = 2 * kQ2Thr;  // columns of Z per CTA (two per thread)

// ---------------------------------------------------------------- stage 1

// Sums over the CTA of kB values per thread (x) and of one more (y); every
// thread then reads them from out[0 .. kB] (shared memory). Within a warp the
// kB values are summed by recursive halving (each lane keeps half of its
// values and adds its partner's copy of the same half: kB - 1 + log2(32 / kB)
// shuffles instead of 5 kB), the extra value by a butterfly. red: kS1Warps *
// (kB + 1) floats of scratch.
__device__ __forceinline__ void block_sums16(float (&x)[kB], float y, float* red, float* out) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int base = 0;
#pragma unroll
    for (int half = kB / 2, o = 16; half >= 1; half >>= 1, o >>= 1) {
        const bool up = lane & o;
#pragma unroll
        for (int q = 0; q < half; ++q) {
            const float send = up ? x[q] : x[q + half];
            const float keep = up ? x[q + half] : x[q];
            x[q] = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
        if (up) base += half;
    }
    float t = x[0];
    t += __shfl_xor_sync(0xffffffffu, t, 1);  // 32 / kB = 2 lanes hold each value
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) y += __shfl_xor_sync(0xffffffffu, y, o);
    if ((lane & 1) == 0) red[warp * (kB + 1) + base] = t;
    if (lane == 0) red[warp * (kB + 1) + kB] = y;
    __syncthreads();
    if ((int)threadIdx.x <= kB) {
        float sum = 0.f;
        for (int w = 0; w < kS1Warps; ++w) sum += red[w * (kB + 1) + threadIdx.x];
        out[threadIdx.x] = sum;
    }
    __syncthreads();
}

// G(g, c) = sum_i a(i, g) b(i, c) over rows i < m for kB x kB results, the rows
// spread over the CTA: lane c (= lane & 15) of half h of warp w takes rows
// i = 2 w + h (mod 16) and gets a(i, g) from the lanes of its half by
// shuffles; the 16 partial results per entry are summed through `part`
// (kS1Warps * kB * kB floats of shared memory). Writes G with row stride kB + 1.
template <typename FA, typename FB>
__device__ __forceinline__ void gram16(int m, FA a, FB b, float* part, float* G) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, c = lane & 15, h = lane >> 4;
    float acc[kB];
#pragma unroll
    for (int g = 0; g < kB; ++g) acc[g] = 0.f;
    for (int i0 = 2 * warp; i0 < m; i0 += 2 * kS1Warps) {  // the trip count is the same in both halves
        const int i = i0 + h;
        const bool ok = i < m;
        const float ai = ok ? a(i, c) : 0.f, bi = ok ? b(i, c) : 0.f;
#pragma unroll
        for (int g = 0; g < kB; ++g) acc[g] += __shfl_sync(0xffffffffu, ai, g + 16 * h) * bi;
    }
#pragma unroll
    for (int g = 0; g < kB; ++g) acc[g] += __shfl_xor_sync(0xffffffffu, acc[g], 16);
    if (h == 0)
#pragma unroll
        for (int g = 0; g < kB; ++g) part[(warp * kB + g) * kB + c] = acc[g];
    __syncthreads();
    {
        const int g = threadIdx.x / kB, cc = threadIdx.x & (kB - 1);
        float sum = 0.f;
        for (int w = 0; w < kS1Warps; ++w) sum += part[(w * kB + g) * kB + cc];
        G[g * (kB + 1) + cc] = sum;
    }
    __syncthreads();
}

// Stage 1 on the tensor cores. One CTA per chain (persistent over the
// longest-first work list when given), 256 threads, 256 tensor-memory columns.
// Per panel of kB columns:
//   QR and T on the CUDA cores in shared memory (P, Ts);
//   V T, split hi/lo, into the chain's scratch in the canonical operand layout
//     (one 16 x 32 tile per 32 rows);
//   X = A22 (V T) with tcgen05.mma kind::tf32 (M = 128 rows of A22, N = 16,
//     K = 32 rows per step): the threads load a 128 x 32 tile of A22 (coalesced;
//     the next tile and the next V T tile prefetched into registers) and split
//     it into hi/lo operand tiles; 3xTF32 (hi hi + hi lo + lo hi); the hi hi
//     products go into a fresh accumulator per K step and are added in FP32
//     registers (the tensor memory accumulates with truncation), the small
//     cross products accumulate in tensor memory;
//   W = X - 1/2 V (T^T (V^T X)) on the CUDA cores;
//   [V W], split hi/lo, into the scratch as 128 x 32 operand tiles (32 KB);
//   A22 -= [V W] [W V]^T: tiles of 128 x 128 (K = 32) with the operand tiles
//     moved into shared memory by TMA bulk copies (one 32 KB copy per tile,
//     completing on an mbarrier; the next row block's copy overlaps the current
//     tile's epilogue); [W V] is the [V W] tile read with its two K halves
//     swapped (descriptor offsets), so one tile serves as A and B; the epilogue
//     reads both accumulators and updates A22 in global memory (coalesced).
// Shared memory: the panel P [kB][max_ld + 1] and two X staging buffers (A tile
// hi/lo, B tile hi/lo; X itself goes to the scratch); the update's three 32 KB
// tiles reuse that space (112 KB at max_ld = 576: two CTAs per SM). Every mbarrier wait is bounded
// (wait_iters checks); a wait that gives up sets kStatusTimeout, the CTA stops,
// waits for what it has issued and frees its tensor memory.
constexpr int kTileF = 128 * 32;          // floats of one 128 x 32 operand tile (hi or lo)
constexpr int kBtileF = 16 * 32;          // floats of one 16 x 32 operand tile (hi or lo)
constexpr uint32_t kS1TmemCols = 256;
constexpr uint32_t kIdX = tc::idesc_tf32(16);
constexpr uint32_t kIdU = tc::idesc_tf32(128);

__host__ __device__ inline int s1_nblk(int ld) { return (ld + 127) / 128; }
// per-chain scratch (floats): [V W] tiles (hi, lo) per 128-row block, then V T tiles per 32 rows
__host__ __device__ inline long long s1_scratch_floats(int max_ld) {
    return (long long)s1_nblk(max_ld) * 2 * kTileF + (long long)(max_ld / 32) * 2 * kBtileF + (long long)max_ld * kB;
}
// floats of the shared-memory region that the QR / X phase and the update share
__host__ __device__ inline size_t s1_region_floats(int max_ld) {
    const size_t big = (size_t)kB * (max_ld + 1) + 32 + 2 * (2 * kTileF + 2 * kBtileF);
    return big > (size_t)6 * kTileF ? big : (size_t)6 * kTileF;
}

__global__ void __launch_bounds__(kS1Threads, 2)
sy2sb_kernel(const ChainDesc* __restrict__ descs, const double* __restrict__ diag, float* __restrict__ Aws,
             float* __restrict__ tauout, const int* __restrict__ order, int norder, int* __restrict__ counter,
             int* __restrict__ status, int max_ld, float* __restrict__ scratch, long long wait_iters) {
    extern __shared__ __align__(1024) float s1[];
    const int pst = max_ld + 1;                      // panel column stride (conflict-free V^T V)
    float* P = s1;                                   // [kB][pst]
    float* XS = P + (size_t)kB * pst;                // X staging, two buffers of A hi, A lo, B hi, B lo
    XS += (32 - ((XS - s1) & 31)) & 31;              // 128-byte aligned operand tiles
    float* U = s1;                                   // update staging (reuses the space): B, A[0], A[1]
    float* Ts = s1 + s1_region_floats(max_ld);       // [kB][kB + 1]
    float* G = Ts + kB * (kB + 1);                   // [kB][kB + 1]
    float* red = G + kB * (kB + 1);                  // [kS1Warps][kB + 1]
    float* sums = red + kS1Warps * (kB + 1);         // [kB + 2]
    float* taus = sums + kB + 2;                     // [kB]
    float* wl = taus + kB;                           // [kB]
    // [6]: update MMAs, B copy, A copies (2), X MMAs (2)
    uint64_t* bars = reinterpret_cast<uint64_t*>(wl + kB + ((wl + kB - s1) & 1));
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 6);
    int& s_item = *reinterpret_cast<int*>(tslot + 1);  // no static shared memory: two CTAs per SM at N = 576
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (tid == 0) {
        for (int b = 0; b < 6; ++b) tc::mbar_init(&bars[b], 1);
        tc::mbar_fence_init();
    }
    if (warp == 0) tc::tmem_alloc(tslot, kS1TmemCols);
    tc::before_sync();
    __syncthreads();
    tc::after_sync();
    const uint32_t tm = *tslot;
    // this thread's accumulator row (tensor-memory lane) and column half
    const int trow = (warp & 3) * 32 + lane, chalf = warp >> 2;
    const uint32_t tlane = tm + ((uint32_t)((warp & 3) * 32) << 16);
    uint32_t done[6] = {0u, 0u, 0u, 0u, 0u, 0u};    // completed phases per barrier (all threads)
    uint32_t issued[6] = {0u, 0u, 0u, 0u, 0u, 0u};  // arrivals issued per barrier (thread 0)
    bool ok = true;
    auto wait_bar = [&](int b) {
        ok = ok && tc::mbar_wait(&bars[b], done[b] & 1u, wait_iters);
        if (ok) ++done[b];
    };

    for (int item = blockIdx.x; ok;) {
        if (order) {
            __syncthreads();
            if (tid == 0) s_item = atomicAdd(counter, 1);
            __syncthreads();
            item = s_item;
            if (item >= norder) break;
        }
        const int ci = order ? order[item] : item;
        const ChainDesc D = descs[ci];
        const int n = D.n, ld = D.ld;
        float* __restrict__ A = Aws + D.a_off;
        float* VWc = scratch + (size_t)ci * s1_scratch_floats(max_ld);
        float* VTc = VWc + (size_t)s1_nblk(max_ld) * 2 * kTileF;
        float* Xg = VTc + (size_t)(max_ld / 32) * 2 * kBtileF;  // X = A22 V T, [m][kB]

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

        for (int k0 = 0; ok && k0 + kB <= n - 2; k0 += kB) {
            const int r0 = k0 + kB, m = n - r0, kb = min(kB, m - 1);
            const int nmb = (m + 127) / 128, nq = (m + 31) / 32;
            float* A22 = A + (size_t)r0 * ld + r0;
            // ---- the panel A(r0:n, k0:k0+kB) into shared memory ----
            for (int t = tid; t < kB * m; t += kS1Threads) {
                const int j = t / m, i = t - j * m;
                P[(size_t)j * pst + i] = A[(size_t)(k0 + j) * ld + r0 + i];
            }
            __syncthreads();
            // ---- QR, one column at a time; one block reduction per column gives both
            //      sigma = |x_{j+1..}|^2 and d_l = x_{j+1..}^T P(j+1.., l), from which
            //      w_l = v^T P(:, l) = P(j, l) + scale d_l (v = [1; scale x]) ----
            for (int j = 0; j < kb; ++j) {
                float* pj = P + (size_t)j * pst;
                float part[kB], sq = 0.f;
#pragma unroll
                for (int l = 0; l < kB; ++l) part[l] = 0.f;
                for (int i = j + 1 + tid; i < m; i += kS1Threads) {
                    const float xi = pj[i];
                    sq += xi * xi;
#pragma unroll
                    for (int l = 0; l < kB; ++l)
                        if (l > j) part[l] += xi * P[(size_t)l * pst + i];
                }
                block_sums16(part, sq, red, sums);
                const float sigma = sums[kB], alpha = pj[j];
                float tau = 0.f, beta = alpha, scale = 0.f;
                if (sigma != 0.f) {
                    beta = -copysignf(sqrtf(alpha * alpha + sigma), alpha);
                    tau = (beta - alpha) / beta;
                    scale = 1.f / (alpha - beta);
                }
                if (tid < kB) wl[tid] = tid > j ? tau * (P[(size_t)tid * pst + j] + scale * sums[tid]) : 0.f;
                if (tid == 0) {
                    taus[j] = tau;
                    tauout[D.v_off + k0 + j] = tau;
                }
                __syncthreads();
                for (int i = j + tid; i < m; i += kS1Threads) {
                    const float vi = i == j ? 1.f : pj[i] * scale;
#pragma unroll
                    for (int l = 0; l < kB; ++l)
                        if (l > j) P[(size_t)l * pst + i] -= vi * wl[l];
                    pj[i] = i == j ? beta : vi;
                }
                __syncthreads();
            }
            if (tid < kB - kb) taus[kb + tid] = 0.f;
            // the panel back: R in the band, V below it
            for (int t = tid; t < kB * m; t += kS1Threads) {
                const int j = t / m, i = t - j * m;
                A[(size_t)(k0 + j) * ld + r0 + i] = P[(size_t)j * pst + i];
            }
            auto vget = [&](int i, int j) -> float {
                return j >= kb ? 0.f : (i == j ? 1.f : (i > j ? P[(size_t)j * pst + i] : 0.f));
            };
            // ---- G = V^T V, then T from its inverse T^-1 = diag(1/tau) + triu(G, 1) ----
            gram16(m, vget, vget, XS, G);
            if (tid < kB) {
                const int j = tid;
                float t[kB];
#pragma unroll
                for (int r = kB - 1; r >= 0; --r) {
                    float sacc = 0.f;
#pragma unroll
                    for (int q = r + 1; q < kB; ++q) sacc += G[r * (kB + 1) + q] * t[q];
                    t[r] = r > j ? 0.f : (r == j ? taus[r] : -taus[r] * sacc);
                }
#pragma unroll
                for (int r = 0; r < kB; ++r) Ts[r * (kB + 1) + j] = t[r];
            }
            __syncthreads();
            // ---- V T into the scratch as B tiles: tile q / 32, element (column c, K = row & 31) ----
            for (int i = tid; i < 32 * nq; i += kS1Threads) {
                float vt[kB];
                if (i < m) {
                    float vr[kB];
#pragma unroll
                    for (int l = 0; l < kB; ++l) vr[l] = vget(i, l);
#pragma unroll
                    for (int c = 0; c < kB; ++c) {
                        float sacc = 0.f;
#pragma unroll
                        for (int l = 0; l < kB; ++l)
                            if (l <= c) sacc += vr[l] * Ts[l * (kB + 1) + c];
                        vt[c] = sacc;
                    }
                } else {
#pragma unroll
                    for (int c = 0; c < kB; ++c) vt[c] = 0.f;
                }
                float* tile = VTc + (size_t)(i >> 5) * 2 * kBtileF;
#pragma unroll
                for (int c = 0; c < kB; ++c) {
                    unsigned hi, lo;
                    split_tf32(vt[c], hi, lo);
                    tile[tc::kofs(c, i & 31)] = __uint_as_float(hi);
                    tile[kBtileF + tc::kofs(c, i & 31)] = __uint_as_float(lo);
                }
            }
            __syncthreads();
            // ---- X = A22 (V T) on the tensor cores: two staging buffers, chunk qc + 1
            //      staged while the MMAs of chunk qc run ----
            const int ra = tid & 127, kh = tid >> 7;  // staging: row ra of the A tile, K half kh
            for (int mb = 0; ok && mb < nmb; ++mb) {
                const int rowg = mb * 128 + ra;       // row of A22 this thread stages
                float av[16];
                float4 bv;
                auto load_ab = [&](int qc) {
#pragma unroll
                    for (int u = 0; u < 16; ++u) {
                        const int q = qc * 32 + 16 * kh + u;
                        av[u] = (rowg < m && q < m) ? A22[(size_t)q * ld + rowg] : 0.f;
                    }
                    bv = reinterpret_cast<const float4*>(VTc + (size_t)qc * 2 * kBtileF)[tid];
                };
                auto add_hh = [&](int b, float (&xacc)[8]) {  // chunk's hi hi products into registers
                    wait_bar(4 + b);
                    tc::after_sync();
                    if (ok) {
                        float v[8];
                        tc::tmem_ld8(tlane + 16 * b + 8 * chalf, v);
#pragma unroll
                        for (int e = 0; e < 8; ++e) xacc[e] += v[e];
                    }
                };
                load_ab(0);
                float xacc[8];
#pragma unroll
                for (int e = 0; e < 8; ++e) xacc[e] = 0.f;
                for (int qc = 0; qc < nq; ++qc) {
                    const int b = qc & 1;
                    float* Ah = XS + b * (2 * kTileF + 2 * kBtileF);
                    float* Al = Ah + kTileF;
                    float* Bh = Al + kTileF;
                    // stage: A tile (hi, lo) and B tile (V T hi, lo) from registers; the MMAs that
                    // read this buffer (chunk qc - 2) were waited for one iteration ago
#pragma unroll
                    for (int v4 = 0; v4 < 4; ++v4) {
                        const float x4[4] = {av[4 * v4], av[4 * v4 + 1], av[4 * v4 + 2], av[4 * v4 + 3]};
                        float4 lo;
                        const float4 hi = tc::split4(x4, lo);
                        const int o = tc::kofs(ra, 16 * kh + 4 * v4);
                        *reinterpret_cast<float4*>(Ah + o) = hi;
                        *reinterpret_cast<float4*>(Al + o) = lo;
                    }
                    reinterpret_cast<float4*>(Bh)[tid] = bv;
                    tc::fence_async_smem();
                    tc::before_sync();
                    ok = __syncthreads_and(ok);
                    if (!ok) break;
                    if (tid == 0) {
                        tc::after_sync();
                        const uint64_t a = tc::sdesc(tc::smem_addr(Ah)), al = a + (kTileF * 4 >> 4);
                        const uint64_t bd = tc::sdesc(tc::smem_addr(Bh)), bl = bd + (kBtileF * 4 >> 4);
#pragma unroll
                        for (int sk = 0; sk < 4; ++sk) {
                            const uint64_t o = 16 * sk;  // 256 B per K step
                            tc::umma<kIdX>(tm + 16 * b, a + o, bd + o, sk > 0);
                            tc::umma<kIdX>(tm + 32, a + o, bl + o, (qc > 0 || sk > 0));
                            tc::umma<kIdX>(tm + 32, al + o, bd + o, 1);
                        }
                        tc::umma_commit(&bars[4 + b]);
                        ++issued[4 + b];
                    }
                    if (qc + 1 < nq) load_ab(qc + 1);
                    if (qc > 0) add_hh(b ^ 1, xacc);  // chunk qc - 1
                }
                if (ok) add_hh((nq - 1) & 1, xacc);  // the last chunk (all MMAs complete with it)
                tc::before_sync();
                ok = __syncthreads_and(ok);
                if (!ok) break;
                tc::after_sync();
                {
                    float v[8];
                    tc::tmem_ld8(tlane + 32 + 8 * chalf, v);
                    const int row = mb * 128 + trow;
                    if (row < m)
#pragma unroll
                        for (int e = 0; e < 8; ++e) Xg[(size_t)row * kB + 8 * chalf + e] = xacc[e] + v[e];
                }
                tc::before_sync();
                __syncthreads();
            }
            if (!ok) break;
            // ---- W = X - 1/2 V (T^T (V^T X)) ----
            gram16(m, vget, [&](int i, int c) { return Xg[(size_t)i * kB + c]; }, XS, G);  // (V^T X)(g, c)
            float mtc = 0.f;
            {
                const int c = tid & (kB - 1), g = tid / kB;  // (T^T (V^T X))(g, c)
                for (int l = 0; l <= g; ++l) mtc += Ts[l * (kB + 1) + g] * G[l * (kB + 1) + c];
            }
            __syncthreads();
            G[(tid / kB) * (kB + 1) + (tid & (kB - 1))] = mtc;
            __syncthreads();
            // W rows, then [V W] (hi, lo) into the scratch as 128 x 32 operand tiles
            for (int i = tid; i < 128 * nmb; i += kS1Threads) {
                float vw[2 * kB];
                if (i < m) {
#pragma unroll
                    for (int l = 0; l < kB; ++l) vw[l] = vget(i, l);
#pragma unroll
                    for (int c = 0; c < kB; ++c) {
                        float sacc = 0.f;
#pragma unroll
                        for (int l = 0; l < kB; ++l) sacc += vw[l] * G[l * (kB + 1) + c];
                        vw[kB + c] = Xg[(size_t)i * kB + c] - 0.5f * sacc;
                    }
                } else {
#pragma unroll
                    for (int c = 0; c < 2 * kB; ++c) vw[c] = 0.f;
                }
                float* tile = VWc + (size_t)(i >> 7) * 2 * kTileF;
#pragma unroll
                for (int v4 = 0; v4 < 8; ++v4) {
                    const float x4[4] = {vw[4 * v4], vw[4 * v4 + 1], vw[4 * v4 + 2], vw[4 * v4 + 3]};
                    float4 lo;
                    const float4 hi = tc::split4(x4, lo);
                    const int o = tc::kofs(i & 127, 4 * v4);
                    *reinterpret_cast<float4*>(tile + o) = hi;
                    *reinterpret_cast<float4*>(tile + kTileF + o) = lo;
                }
            }
            tc::fence_async_global();  // the bulk copies below read these tiles
            tc::before_sync();
            __syncthreads();
            // ---- A22 -= [V W] [W V]^T, 128 x 128 tiles; operand tiles by TMA bulk copies ----
            float* Bt = U;
            float* At[2] = {U + 2 * kTileF, U + 4 * kTileF};
            const uint32_t tbytes = 2 * kTileF * 4;
            int ia = 0;  // A-tile copies consumed in this panel (buffer ia & 1)
            if (tid == 0) {
                tc::bulk_g2s(At[0], VWc, tbytes, &bars[2]);
                ++issued[2];
            }
            for (int J = 0; ok && J < nmb; ++J) {
                if (tid == 0) {
                    tc::bulk_g2s(Bt, VWc + (size_t)J * 2 * kTileF, tbytes, &bars[1]);
                    ++issued[1];
                }
                wait_bar(1);
                ok = __syncthreads_and(ok);
                if (!ok) break;
                for (int I = 0; ok && I < nmb; ++I, ++ia) {
                    const int ab = ia & 1;
                    wait_bar(2 + ab);
                    // prefetch this thread's 64 entries of the A22 tile
                    const int row = I * 128 + trow, c0 = J * 128 + 64 * chalf;
                    float a22[64];
#pragma unroll
                    for (int c = 0; c < 64; ++c)
                        a22[c] = (row < m && c0 + c < m) ? A22[(size_t)(c0 + c) * ld + row] : 0.f;
                    tc::before_sync();
                    ok = __syncthreads_and(ok);
                    if (!ok) break;
                    if (tid == 0) {
                        tc::after_sync();
                        const uint64_t a = tc::sdesc(tc::smem_addr(At[ab])), al = a + (kTileF * 4 >> 4);
                        const uint64_t b = tc::sdesc(tc::smem_addr(Bt)), bl = b + (kTileF * 4 >> 4);
#pragma unroll
                        for (int sk = 0; sk < 4; ++sk) {
                            const uint64_t oa = 16 * sk, ob = 16 * ((sk + 2) & 3);  // [W V] = [V W], halves swapped
                            tc::umma<kIdU>(tm + 0, a + oa, b + ob, sk > 0);
                            tc::umma<kIdU>(tm + 128, a + oa, bl + ob, sk > 0);
                            tc::umma<kIdU>(tm + 128, al + oa, b + ob, 1);
                        }
                        tc::umma_commit(&bars[0]);
                        ++issued[0];
                        // the next A tile (the MMAs above read the other buffer)
                        const bool last = I + 1 == nmb && J + 1 == nmb;
                        if (!last) {
                            const int In = I + 1 < nmb ? I + 1 : 0;
                            tc::bulk_g2s(At[ab ^ 1], VWc + (size_t)In * 2 * kTileF, tbytes, &bars[2 + (ab ^ 1)]);
                            ++issued[2 + (ab ^ 1)];
                        }
                    }
                    wait_bar(0);
                    tc::after_sync();
                    if (ok) {
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            float h[16], x[16];
                            tc::tmem_ld16(tlane + 64 * chalf + 16 * u, h);
                            tc::tmem_ld16(tlane + 128 + 64 * chalf + 16 * u, x);
#pragma unroll
                            for (int e = 0; e < 16; ++e) {
                                const int c = c0 + 16 * u + e;
                                if (row < m && c < m) A22[(size_t)c * ld + row] = a22[16 * u + e] - (h[e] + x[e]);
                            }
                        }
                    }
                    tc::before_sync();
                    ok = __syncthreads_and(ok);  // accumulators free for the next tile
                }
            }
        }
        if (!order) break;
    }
    if (!ok && tid == 0) {
        atomicOr(status, kStatusTimeout);
        // every MMA group and bulk copy this CTA started completes before the
        // tensor memory is freed and the CTA exits
        for (int b = 0; b < 6; ++b)
            while (done[b] < issued[b] && tc::mbar_wait(&bars[b], done[b] & 1u, kDefaultWaitIters)) ++done[b];
    }
    tc::before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tm, kS1TmemCols);
}

// ---------------------------------------------------------------- stage 2

// One task (s, k) of the bulge chase on the band held in shared memory
// (band[c * kLdb + d] = A(c + d, c)), by one warp. Lane (r, h) = (lane & 15,
// lane >> 4). Both halves build the reflector (lane r holds element r); then
// each application (the diagonal block from both sides, the block on the
// left, the block below) runs on all 32 lanes: half h takes 8 of the 16 rows
// or columns of the reflector's range and one shuffle joins the halves' sums.
// A step of the wavefront waits for its slowest task, so both the task's
// dependent chain and its instruction count matter (two CTAs share an SM).
// The band holds zeros below the last row and kB zero columns after the last
// one, so a short last reflector (fewer than kB rows) needs no masks: its
// missing elements are zeros, and the updates that reach them subtract zero.
// vw: the warp's 32 floats of scratch (v, then w), 16-byte aligned.
__device__ __forceinline__ void sb_task(float* __restrict__ band, int n, int s, int k, float* __restrict__ q2v,
                                        float* __restrict__ q2t, int ld, float* __restrict__ vw) {
    const int lane = threadIdx.x & 31, r = lane & 15, h8 = (lane >> 4) * 8;
    const int p = s + 1 + k * kB;
    const int c0 = k == 0 ? s : p - kB;
    // (1) reflector from A(p .. p+15, c0): (I - tau v v^T) x = beta e_0
    float* xcol = band + c0 * kLdb + (p - c0);  // xcol[r] = A(p + r, c0)
    const float x = xcol[r];
    float sq = r > 0 ? x * x : 0.f;
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
    const float alpha = __shfl_sync(0xffffffffu, x, 0, 16);
    float tau = 0.f, beta = alpha, scale = 0.f;
    if (sq != 0.f) {
        beta = -copysignf(sqrtf(alpha * alpha + sq), alpha);
        tau = (beta - alpha) / beta;
        scale = 1.f / (alpha - beta);
    }
    const float v = r == 0 ? 1.f : x * scale;  // zero below the matrix's last row
    if (lane < 16) {
        xcol[r] = r == 0 ? beta : 0.f;
        q2v[((size_t)s * (ld / kB) + k) * kB + r] = v;
        vw[r] = v;
    }
    if (lane == 0) q2t[(size_t)s * (ld / kB) + k] = tau;
    __syncwarp();
    if (tau == 0.f) return;  // identity reflector (the same in every lane)
    float vh[8];             // v over this half's 8 rows / columns
    {
        const float4 a = *reinterpret_cast<const float4*>(vw + h8), b = *reinterpret_cast<const float4*>(vw + h8 + 4);
        vh[0] = a.x; vh[1] = a.y; vh[2] = a.z; vh[3] = a.w; vh[4] = b.x; vh[5] = b.y; vh[6] = b.z; vh[7] = b.w;
    }
    // (3) the diagonal block D = A(p .. p+15, p .. p+15) from both sides:
    //     y = D v, w = tau y - (tau^2 / 2)(v^T y) v, D -= v w^T + w v^T (lower triangle)
    float dv[8], y0 = 0.f, y1 = 0.f;
#pragma unroll
    for (int jj = 0; jj < 8; ++jj) {
        const int j = h8 + jj, lo = min(r, j), d = max(r, j) - lo;
        dv[jj] = band[(p + lo) * kLdb + d];
        if (jj & 1) y1 += dv[jj] * vh[jj];
        else y0 += dv[jj] * vh[jj];
    }
    float y = y0 + y1;
    y += __shfl_xor_sync(0xffffffffu, y, 16);  // every lane has read D before any writes below
    float w = tau * y, dot = w * v;
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, o);
    w -= 0.5f * tau * dot * v;
    if (lane < 16) vw[16 + r] = w;
    __syncwarp();
    {
        const float4 a = *reinterpret_cast<const float4*>(vw + 16 + h8);
        const float4 b = *reinterpret_cast<const float4*>(vw + 20 + h8);
        const float wh[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
        for (int jj = 0; jj < 8; ++jj) {
            const int j = h8 + jj;
            if (j <= r) band[(p + j) * kLdb + (r - j)] = dv[jj] - (v * wh[jj] + w * vh[jj]);
        }
    }
    if (k > 0) {
        // (2) the block on the left from the left: column j = c0 + 1 + r (r < 15), rows
        //     p + i, A(p + i, j) = band[j * kLdb + (kB - 1 - r) + i] (lane r = 15 idles)
        float* colj = band + (c0 + 1 + r) * kLdb + (kB - 1 - r) + h8;
        float a[8], w0 = 0.f, w1 = 0.f;
#pragma unroll
        for (int ii = 0; ii < 8; ++ii) {
            a[ii] = colj[ii];
            if (ii & 1) w1 += vh[ii] * a[ii];
            else w0 += vh[ii] * a[ii];
        }
        float wl = w0 + w1;
        wl = tau * (wl + __shfl_xor_sync(0xffffffffu, wl, 16));
        if (r < kB - 1)
#pragma unroll
            for (int ii = 0; ii < 8; ++ii) colj[ii] = a[ii] - vh[ii] * wl;
    }
    if (p + kB < n) {
        // (4) the block below from the right: row p + kB + r, columns p + i,
        //     A(p + kB + r, p + i) = band[(p + i) * kLdb + kB + r - i]
        float* rowr = band + (p + h8) * kLdb + kB + r - h8;  // + ii (kLdb - 1)
        float a[8], z0 = 0.f, z1 = 0.f;
#pragma unroll
        for (int ii = 0; ii < 8; ++ii) {
            a[ii] = rowr[ii * (kLdb - 1)];
            if (ii & 1) z1 += a[ii] * vh[ii];
            else z0 += a[ii] * vh[ii];
        }
        float z = z0 + z1;
        z = tau * (z + __shfl_xor_sync(0xffffffffu, z, 16));
#pragma unroll
        for (int ii = 0; ii < 8; ++ii) rowr[ii * (kLdb - 1)] = a[ii] - z * vh[ii];
    }
    __syncwarp();
}

// One CTA per chain: the band of the stage-1 matrix into shared memory, the
// wavefront of tasks (one barrier per step), then d and e. Q2: reflector
// (s, k) as kB floats (unit first element stored, zeros beyond its length) at
// q2v[(s * (ld / kB) + k) * kB], its tau at q2t[s * (ld / kB) + k].
__global__ void __launch_bounds__(kS2Warps * 32, 2)
sb2st_kernel(const ChainDesc* __restrict__ descs, const float* __restrict__ Aws, double* __restrict__ dout,
             double* __restrict__ eout, float* __restrict__ Q2, long long q2t_off) {
    extern __shared__ __align__(16) float band[];  // [n + kB][kLdb]
    __shared__ __align__(16) float vw_all[kS2Warps][32];
    const ChainDesc D = descs[blockIdx.x];
    const int n = D.n, ld = D.ld;
    const float* A = Aws + D.a_off;
    float* q2v = Q2 + D.a_off;
    float* q2t = Q2 + q2t_off + D.a_off / kB;
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int t = tid; t < (n + kB) * kLdb; t += blockDim.x) {
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

// Z <- Q2 Z for kQ2Cols columns of one chain (Z row-major, Z[i * ld + j]), two
// adjacent columns per thread, one warp per CTA. Q2 is the product of the
// sweeps' reflectors H(s, k) in sweep order; for a group of kB consecutive
// sweeps s0 .. s0+15 the reflectors of block k (rows s + 1 + kB k ..) commute
// past those of later blocks of earlier sweeps, so the group equals
// G(K) ... G(1) G(0) with G(k) = H(s0, k) H(s0+1, k) ... H(s0+15, k) acting on
// the 31 rows s0 + 1 + kB k .. s0 + 31 + kB k. Applied to a column: groups from
// the last to the first, windows k = 0, 1, .. in order, the window's rows in
// registers (a 32-row window slides down 16 rows per block: 16 loads and 16
// stores per block of 16 reflectors), the block's reflectors in shared memory
// and applied from the last sweep to the first. The next window's rows and the
// next block's reflectors are loaded while the current block is applied
// (double-buffered reflectors, one barrier per block; the rows through
// cp.async into this thread's own double-buffered slots of shared memory, which
// keeps them out of the registers). The kernel is bound by instruction issue:
// two columns per thread give 64 FMAs per five shared-memory loads of a
// reflector, and one-warp CTAs (16 per SM) fit the bench batch's 2304 warps in
// one wave.
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem, bool valid) {  // zeros when !valid
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(gmem), "r"(valid ? 8 : 0) : "memory");
}

__global__ void __launch_bounds__(kQ2Thr, 16)
q2_apply_kernel(const ChainDesc* __restrict__ descs, const float* __restrict__ Q2, long long q2t_off,
                float* __restrict__ Zws) {
    __shared__ __align__(16) float vs[2][kB][kB];  // reflector a of the block: vs[b][a][0 .. 15]
    __shared__ float ts[2][kB];
    __shared__ __align__(16) float2 zst[2][kB][kQ2Thr];  // window rows in flight: zst[b][i][thread]
    const ChainDesc D = descs[blockIdx.y];
    const int n = D.n, ld = D.ld, tid = threadIdx.x;
    if (n < 3 || (int)(blockIdx.x * kQ2Cols) >= n) return;
    const int j = blockIdx.x * kQ2Cols + 2 * tid;  // even; ld is even, so j + 1 < ld when j < n
    const bool ok0 = j < n, ok1 = j + 1 < n;       // column j + 1 >= n (padding) is computed, never stored
    const int nkm = ld / kB;
    const float* q2v = Q2 + D.a_off;
    const float* q2t = Q2 + q2t_off + D.a_off / kB;
    float* Zc = Zws + D.a_off + (ok0 ? j : 0);  // row i of these columns at Zc[i * ld]
    auto zload = [&](int i, float& a, float& b) {
        a = 0.f;
        b = 0.f;
        if (!ok0 || i >= n) return;
        const float2 x = *reinterpret_cast<const float2*>(Zc + (size_t)i * ld);
        a = x.x;
        b = x.y;
    };
    auto zfetch = [&](int i0, int buf) {  // rows i0 .. i0 + 15 into zst[buf] (zeros beyond the matrix)
#pragma unroll
        for (int i = 0; i < kB; ++i) {
            const bool ok = ok0 && i0 + i < n;
            cp_async8(&zst[buf][i][tid], Zc + (ok ? (size_t)(i0 + i) * ld : 0), ok);
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    };
    auto zstore = [&](int i, float a, float b) {
        if (!ok0 || i >= n) return;
        if (ok1) *reinterpret_cast<float2*>(Zc + (size_t)i * ld) = make_float2(a, b);
        else Zc[(size_t)i * ld] = a;
    };
    // block k of the group at s0 into vs[buf], ts[buf]: lane t copies quarter (t & 3) of reflectors
    // t / 4 and t / 4 + 8, and tau t (t < kB); zeros for reflectors that do not exist
    auto rfetch = [&](int s0, int k, int buf) {
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int a = (tid >> 2) + 8 * u, sw = s0 + a;
            const bool ok = sw <= n - 3 && sw + 1 + kB * k <= n - 2;
            const float* src = q2v + (ok ? ((size_t)sw * nkm + k) * kB + 4 * (tid & 3) : 0);
            const unsigned s = (unsigned)__cvta_generic_to_shared(&vs[buf][a][4 * (tid & 3)]);
            asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(src), "r"(ok ? 16 : 0)
                         : "memory");
        }
        if (tid < kB) {
            const int sw = s0 + tid;
            const bool ok = sw <= n - 3 && sw + 1 + kB * k <= n - 2;
            const unsigned s = (unsigned)__cvta_generic_to_shared(&ts[buf][tid]);
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(s),
                         "l"(q2t + (ok ? (size_t)sw * nkm + k : 0)), "r"(ok ? 4 : 0)
                         : "memory");
        }
    };
    const int ngroups = (n - 2 + kB - 1) / kB;  // sweeps 0 .. n-3
    for (int g = ngroups - 1; g >= 0; --g) {
        const int s0 = g * kB, base = s0 + 1;
        const int nblk = (n - 2 - base) / kB + 1;  // blocks of sweep s0 (the group's longest)
        float za[2 * kB], zb[2 * kB];
        rfetch(s0, 0, 0);
        zfetch(base + kB, 0);
#pragma unroll
        for (int i = 0; i < kB; ++i) zload(base + i, za[i], zb[i]);
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        __syncthreads();
        for (int k = 0; k < nblk; ++k) {
            const int r0 = base + kB * k, b = k & 1;  // r0: first row of the window
            const bool more = k + 1 < nblk;
#pragma unroll
            for (int i = 0; i < kB; ++i) {  // rows r0 + 16 .. r0 + 31
                const float2 x = zst[b][i][tid];
                za[kB + i] = x.x;
                zb[kB + i] = x.y;
            }
            if (more) {  // the next window's lower half and the next block's reflectors, in flight meanwhile
                rfetch(s0, k + 1, b ^ 1);
                zfetch(r0 + 2 * kB, b ^ 1);
            }
#pragma unroll
            for (int a = kB - 1; a >= 0; --a) {  // G(k) z = H(s0) (H(s0+1) (... H(s0+15) z))
                float vv[kB];
#pragma unroll
                for (int q = 0; q < kB / 4; ++q) {
                    const float4 x = *reinterpret_cast<const float4*>(&vs[b][a][4 * q]);
                    vv[4 * q] = x.x; vv[4 * q + 1] = x.y; vv[4 * q + 2] = x.z; vv[4 * q + 3] = x.w;
                }
                float d0 = 0.f, d1 = 0.f, e0 = 0.f, e1 = 0.f;
#pragma unroll
                for (int i = 0; i < kB; i += 2) {
                    d0 += vv[i] * za[a + i];
                    d1 += vv[i + 1] * za[a + i + 1];
                    e0 += vv[i] * zb[a + i];
                    e1 += vv[i + 1] * zb[a + i + 1];
                }
                const float t = ts[b][a], d = t * (d0 + d1), e = t * (e0 + e1);
#pragma unroll
                for (int i = 0; i < kB; ++i) {
                    za[a + i] -= d * vv[i];
                    zb[a + i] -= e * vv[i];
                }
            }
#pragma unroll
            for (int i = 0; i < kB; ++i) zstore(r0 + i, za[i], zb[i]);
#pragma unroll
            for (int i = 0; i < kB; ++i) {
                za[i] = za[kB + i];
                zb[i] = zb[kB + i];
            }
            asm volatile("cp.async.wait_group 0;\n" ::: "memory");  // this thread's copies of the next block
            __syncthreads();  // everyone's copies landed; buffer b is free for block k + 2
        }
#pragma unroll
        for (int i = 0; i < kB; ++i) zstore(base + kB * nblk + i, za[i], zb[i]);  // the last window's lower half
    }
}

}  // namespace

size_t sy2sb_smem_bytes(int max_ld) {
    return sizeof(float) * (s1_region_floats(max_ld) + 2 * kB * (kB + 1) + kS1Warps * (kB + 1) + 3 * kB + 2 + 2) +
           6 * 8 + 16;
}

long long sy2sb_scratch_floats(int max_ld) { return s1_scratch_floats(max_ld); }

cudaError_t launch_sy2sb(const ChainDesc* d_desc, int batch, int max_ld, const double* d_diag, float* d_A,
                         float* d_tau, const int* d_order, int* d_counter, int num_sms, int* d_status,
                         float* d_scratch, long long wait_iters, cudaStream_t st) {
    if (batch <= 0) return cudaSuccess;
    const size_t smem = sy2sb_smem_bytes(max_ld);
    cudaError_t err = cudaFuncSetAttribute(sy2sb_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    int grid = batch;
    if (d_order) {
        int per_sm = 0;
        if ((err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sy2sb_kernel, kS1Threads, smem))) return err;
        grid = max(1, min(batch, max(1, per_sm) * num_sms));
        if ((err = cudaMemsetAsync(d_counter, 0, sizeof(int), st))) return err;
    }
    sy2sb_kernel<<<grid, kS1Threads, smem, st>>>(d_desc, d_diag, d_A, d_tau, d_order, batch, d_counter, d_status,
                                                 max_ld, d_scratch, wait_iters < 0 ? kDefaultWaitIters : wait_iters);
    return cudaGetLastError();
}

cudaError_t launch_sb2st(const ChainDesc* d_desc, int batch, int max_n, const float* d_A, double* d_d, double* d_e,
                         float* d_Q2, long long q2t_off, cudaStream_t st) {
    if (batch <= 0) return cudaSuccess;
    const size_t smem = sizeof(float) * (size_t)(max_n + kB) * kLdb;
    cudaError_t err = cudaFuncSetAttribute(sb2st_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    sb2st_kernel<<<batch, kS2Warps * 32, smem, st>>>(d_desc, d_A, d_d, d_e, d_Q2, q2t_off);
    return cudaGetLastError();
}

cudaError_t launch_q2_apply(const ChainDesc* d_desc, int batch, int max_n, const float* d_Q2, long long q2t_off,
                            float* d_Z, cudaStream_t st) {
    if (batch <= 0) return cudaSuccess;
    if (batch > 65535) return cudaErrorInvalidValue;  // grid y limit
    q2_apply_kernel<<<dim3((max_n + kQ2Cols - 1) / kQ2Cols, batch), kQ2Thr, 0, st>>>(d_desc, d_Q2, q2t_off, d_Z);
    return cudaGetLastError();
}

}  // namespace fkg
