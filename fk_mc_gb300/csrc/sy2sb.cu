// sy2sb.cu — first stage of the two-stage tridiagonalisation of the mixed path
// (FP32): dense -> band (bandwidth kBand), the O(n^3) work on the tensor cores.
//
// Replaces, with the band stage of twostage.cu, the first half of
// Eigen::SelfAdjointEigenSolver at src/configuration.cpp:213; the Hamiltonian
// build (src/configuration.cpp:79-91) and the dense copy (:212) are fused into
// the matrix load.
//
// One CTA per chain (persistent over the longest-first work list when given),
// two CTAs per SM. Panel p holds columns k0 = 16 p .. k0 + 15; its QR covers
// rows r0 = k0 + 16 .. n - 1 (m rows) and its trailing matrix is
// A22 = A(r0:, r0:), stored in full (both triangles). Per panel:
//   (1) panel update: the panel's columns A(k0:, k0:k0+16) minus the previous
//       panel's V W^T + W V^T (CUDA cores, FP32, 4 x 4 tiles through shared
//       memory), the rows in registers;
//   (2) QR of rows r0.. of the panel, the rows in registers (three or four per
//       thread) rotating by one column per step (one loop body for all 16
//       columns), one barrier per column (block sums double-buffered by column
//       parity); the diagonal block and R stay in the band, reflector j (unit
//       at row r0 + j) is stored below it in column k0 + j;
//   (3) T from T^-1 = diag(1/tau) + triu(V^T V, 1); V T (FP32) into the
//       per-chunk operand slots of the chain's scratch;
//   (4) one pass over A22 in chunks of 128 rows x 32 columns that applies the
//       previous panel's update A22 -= [V W][W V]^T (tcgen05.mma kind::tf32,
//       3xTF32) and forms X = A22 (V T) from the updated chunk (FP32 FMAs);
//   (5) W = X - 1/2 V (T^T (V^T X)); [W V] (hi/lo B operand) into the slots
//       for the next pass, the rows of V | W (FP32) for the next panel update
//       and the next pass's [V W] operand.
// After the last panel its update is applied to the remaining block (fewer
// than 18 rows) by the CUDA cores. The first panel's pass forms X only.
//
// The pass (4). A22 is symmetric and stored in full, so the chunk (rows i,
// columns c) is read as the box of memory columns i, rows c: a TMA 2D load
// (cp.async.bulk.tensor, one tensor map per chain, box 32 x 128, 128-byte
// swizzle) lands it in shared memory with each of its 128 rows in one 128-byte
// line, and a TMA store puts the updated chunk back from the same buffer. A
// chunk's load and a 1D bulk copy of its operand slot ([W V] 32 x 32 hi/lo and
// V T 32 x 16) run up to four chunks ahead (four stages). Warp roles: warp 0
// issues the copies; one thread of warp 1 issues the update MMAs (M = 128,
// N = 32, K = 32 in four steps, three products each) with the A operand [V W]
// of the row block in tensor memory and the B operand from the slot, the next
// chunk's update beside the current chunk's epilogue (two accumulator sets),
// and the stores; warps 4..7 (one thread per row = tensor-memory lane) write
// the row block's [V W] (hi/lo) to tensor memory, subtract the accumulators
// from the chunk in place, meet at a named barrier of their own, and add the
// chunk's share of X in FP32 4 x 4 register tiles (rows 4 (e / 4) .., columns
// 4 (e % 4) .. for thread e). The stages and accumulators are handed on
// through mbarriers (no CTA-wide barrier inside the pass).
// Design notes from measurement on GB300: one kind::tf32 MMA with M = 128, K = 8
// costs about 47 cycles of the tensor pipe for any N <= 64 (64 at N = 128, 128
// at N = 256), so a chunk of 32 columns costs the pass the same MMA time as one
// of 16, and the N = 16 product X = A22 (V T) is no faster there than on the
// CUDA cores, where it also accumulates exactly in FP32; the occupancy API
// reports one CTA per SM for kernels that allocate tensor memory, but two such
// CTAs run side by side, so the persistent grid is sized from the kernel's own
// limits.
//
// Every mbarrier wait is bounded (wait_iters checks); a wait that gives up
// sets kStatusTimeout, the CTA stops, waits for what it has issued and frees
// its tensor memory.
#include <cuda.h>
#include <cudaTypedefs.h>

#include "fkg_common.cuh"
#include "tcgen05.cuh"

namespace fkg {
namespace {

constexpr int kB = kBand;
constexpr int kS1Threads = 256;
constexpr int kS1Warps = kS1Threads / 32;
constexpr int kMaxQR = 4;                     // panel rows per thread (kernel template QR <= kMaxQR): n <= QR * kS1Threads
constexpr int kMaxLd = kMaxQR * kS1Threads;
constexpr int kCW = 32;                       // columns of a chunk of the pass (rows of the TMA box: 128 bytes)
constexpr int kStages = 4;                    // chunks of the pass in flight
constexpr int kOldF = 128 * kCW;              // one 128 x 32 chunk of A22 (the TMA box), floats
constexpr int kSlotLo = kCW * 32;             // per chunk: [W V] kCW x 32 hi, then lo; V T kCW x 16 (FP32, rows)
constexpr int kSlotVT = 2 * kSlotLo;          // offset of V T in a slot
constexpr int kSlotF = kSlotVT + kCW * kB;
constexpr int kOffOld = 0;                    // shared memory (floats): chunks | slots
constexpr int kOffSlot = kOffOld + kStages * kOldF;
constexpr int kRegionF = kOffSlot + kStages * kSlotF;
constexpr int kSmallF = 3 * kB * (kB + 1) + 2 * kB + kB;  // Ts, G, red (two halves share 2 x 8 x 17 = 272), Pj, taus
constexpr uint32_t kTxBytes = (kOldF + kSlotF) * 4;
constexpr uint32_t kTmemCols = 256;
constexpr uint32_t kHX = 0;                   // update accumulators: two sets of [h (32 columns), x (32)]
constexpr uint32_t kVWT = 128;                // the update's A operand [V W] of the row block: hi (32), lo (32)
constexpr uint32_t kIdN = tc::idesc_tf32(kCW);
static_assert(kOldF * 4 % 1024 == 0 && kSlotF * 4 % 1024 == 0, "stage buffers on 1024-byte boundaries (128-byte swizzle)");
static_assert(kB * (kMaxLd + 1) + 32 + kS1Warps * kB * kB <= kRegionF, "the panel's V and gram16's scratch fit the pass's region");
constexpr int kVwS = 36;  // row stride of the panel update's V | W rows in shared memory (16-byte aligned)
static_assert(kB * kVwS + kMaxLd * kB <= kRegionF, "the panel update's rows fit the pass's region");
// mbarriers of the pass: chunk + slot landed (per stage), stage released (its store has read it), update
// accumulators ready / read, the chunk's epilogue done (per stage: a stage is refilled only after the
// issuing thread has waited for its epilogue, so the epilogue runs at most one phase ahead), the row
// block's [V W] written to tensor memory
constexpr int kFull = 0, kEmpty = kStages, kHxF = 2 * kStages, kHxE = kHxF + 2, kEpi = kHxE + 2, kVwr = kEpi + kStages;
constexpr int kNumBars = kVwr + 1;
constexpr int kEpiThreads = 128;  // warps 4..7
__host__ __device__ constexpr uint32_t bar_count(int b) {
    return ((b >= kHxE && b < kHxE + 2) || (b >= kEpi && b < kEpi + kStages) || b == kVwr) ? (uint32_t)kEpiThreads
                                                                                                     : 1u;
}

// per-chain scratch (floats): operand slots per chunk, rows of V | W (FP32, 32 per row), rows of X (16 per row)
__host__ __device__ inline int s1_slots(int max_ld) { return (max_ld + kCW - 1) / kCW; }
__host__ __device__ inline long long s1_scratch_floats(int max_ld) {
    return (long long)s1_slots(max_ld) * kSlotF + (long long)max_ld * 48;
}

// Sums over each warp of kB values per thread (x) and of one more (y), into
// redw[0 .. kB] (one row of shared memory per warp). The kB values by
// recursive halving (each lane keeps half of its values and adds its
// partner's copy of the same half: kB - 1 + log2(32 / kB) shuffles instead of
// 5 kB), the extra value by a butterfly.
__device__ __forceinline__ void warp_sums17(float (&x)[kB], float y, float* redw) {
    const int lane = threadIdx.x & 31;
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
    if ((lane & 1) == 0) redw[base] = t;
    if (lane == 0) redw[kB] = y;
}

// G(g, c) = sum_i a(i, g) b(i, c) over rows i < m for kB x kB results, the rows
// spread over the CTA: lane c (= lane & 15) of half h of warp w takes rows
// i = 2 w + h (mod 16) and gets a(i, g) from the lanes of its half by
// shuffles; the 16 partial results per entry are summed through `part`
// (kS1Warps * kB * kB floats of shared memory). Writes G with row stride kB + 1.
// Four rows per lane are loaded before they are used (a and b may read global
// memory: four loads in flight instead of one).
template <typename FA, typename FB>
__device__ __forceinline__ void gram16(int m, FA a, FB b, float* part, float* G) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, c = lane & 15, h = lane >> 4;
    constexpr int kStep = 2 * kS1Warps, kAhead = 4;
    float acc[kB];
#pragma unroll
    for (int g = 0; g < kB; ++g) acc[g] = 0.f;
    for (int i0 = 2 * warp; i0 < m; i0 += kAhead * kStep) {  // the trip count is the same in both halves
        float ai[kAhead], bi[kAhead];
#pragma unroll
        for (int u = 0; u < kAhead; ++u) {
            const int i = i0 + u * kStep + h;
            const bool ok = i < m;
            ai[u] = ok ? a(i, c) : 0.f;
            bi[u] = ok ? b(i, c) : 0.f;
        }
#pragma unroll
        for (int u = 0; u < kAhead; ++u)
#pragma unroll
            for (int g = 0; g < kB; ++g) acc[g] += __shfl_sync(0xffffffffu, ai[u], g + 16 * h) * bi[u];
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

// barrier of the pass's epilogue warps (4..7, named barrier 1) with the AND of their flags
__device__ __forceinline__ bool epi_barrier_and(bool v) {
    int r;
    asm volatile(
        "{\n.reg .pred p, q;\nsetp.ne.s32 p, %1, 0;\nbar.red.and.pred q, 1, 128, p;\nselp.s32 %0, 1, 0, q;\n}\n"
        : "=r"(r)
        : "r"((int)v)
        : "memory");
    return r != 0;
}

template <int kQR>
__global__ void __launch_bounds__(kS1Threads, 2)
sy2sb_kernel(const ChainDesc* __restrict__ descs, const double* __restrict__ diag, float* __restrict__ Aws,
             float* __restrict__ tauout, const int* __restrict__ order, int norder, int* __restrict__ counter,
             int* __restrict__ status, int max_ld, float* __restrict__ scratch, const CUtensorMap* __restrict__ tmaps,
             long long wait_iters) {
    extern __shared__ __align__(1024) float s1[];
    const int pst = max_ld + 1;                      // row stride of the panel's V in (2)-(3)
    float* Vs = s1;                                  // (1): the previous V | W rows 0..15; (2)-(3): V, [kB][pst]
    float* part = s1 + ((kB * pst + 31) & ~31);      // gram16 scratch
    float* Ts = s1 + kRegionF;                       // [kB][kB] (rows 16-byte aligned: vector reads)
    float* G = Ts + kB * (kB + 1);                   // [kB][kB + 1]
    float* red = G + kB * (kB + 1);                  // [2][kS1Warps][kB + 1]
    float* Pj = red + 2 * kS1Warps * (kB + 1);       // [2][kB]: the pivot row of a QR column
    float* taus = Pj + 2 * kB;                       // [kB]
    uint64_t* bars = reinterpret_cast<uint64_t*>(s1 + kRegionF + kSmallF);  // kNumBars mbarriers
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + kNumBars);
    int& s_item = *reinterpret_cast<int*>(tslot + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tc::smem_addr(s1) & 1023u) {  // the chunks' 128-byte swizzle repeats every 1024 bytes: stages start on it
        if (tid == 0 && status) atomicOr(status, kStatusBadArg);
        return;
    }

    if (tid == 0) {
        for (int b = 0; b < kNumBars; ++b) tc::mbar_init(&bars[b], bar_count(b));
        tc::mbar_fence_init();
    }
    if (warp == 0) tc::tmem_alloc(tslot, kTmemCols);
    tc::before_sync();
    __syncthreads();
    tc::after_sync();
    const uint32_t tm = *tslot;
    // the pass's epilogue (warps 4..7): this thread's chunk row = tensor-memory lane
    const int erow = (warp & 3) * 32 + lane;
    const uint32_t tlane = tm + ((uint32_t)((warp & 3) * 32) << 16);
    // chunks, update MMAs and [V W] row blocks of this CTA's passes so far (the same in every thread):
    // the mbarrier phases follow from them
    long long Q0 = 0, U0 = 0, V0 = 0;
    // the last chunk load (warp 0) and update MMA (warp 1) issued: drained on a timeout
    long long last_q = -1, last_u = -1;
    bool ok = true;

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
        const CUtensorMap* tmap = tmaps + ci;
        float* SLOTg = scratch + (size_t)ci * s1_scratch_floats(max_ld);
        float* VWP = SLOTg + (size_t)s1_slots(max_ld) * kSlotF;  // rows of V | W of the last panel
        float* XG = VWP + (size_t)max_ld * 32;                // rows of X

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
        tc::fence_async_global();  // the passes read A through the tensor map
        __syncthreads();

        int k0 = 0;
        for (; ok && k0 + kB <= n - 2; k0 += kB) {
            const int r0 = k0 + kB, m = n - r0, mp = m + kB;  // mp: panel rows k0 .. n-1
            const bool upd = k0 > 0;                          // a previous panel's update is pending
            // ---- (1) the panel's rows into registers, minus the previous panel's update ----
            float prow[kQR][kB];
            // V | W rows 0..15 of the previous panel in Vs with rows of kVwS floats (fewer bank conflicts below)
            float* Dp = s1 + kB * kVwS;  // the update of the panel's rows, [mp][kB]
            if (upd) {  // V | W rows 0..15 of the previous panel (rows k0 .. k0+15) for every thread
                for (int t = tid; t < kB * 32; t += kS1Threads) Vs[(t >> 5) * kVwS + (t & 31)] = __ldcg(VWP + t);
                __syncthreads();
                // Dp(i, l) = V(i, :) W(l, :)^T + W(i, :) V(l, :)^T for the panel rows i < mp, in 4 x 4 tiles (four
                // threads share a quad of rows, read once from shared memory per thread and tile)
                const int nt = ((mp + 3) / 4) * 4;
                for (int t = tid; t < nt; t += kS1Threads) {
                    const int i0 = 4 * (t >> 2), l0 = 4 * (t & 3);
                    float acc[4][4];
#pragma unroll
                    for (int e = 0; e < 16; ++e) acc[e >> 2][e & 3] = 0.f;
#pragma unroll
                    for (int c4 = 0; c4 < 8; ++c4) {  // four of the 32 values of row i: V (c4 < 4), then W
                        const int oc = c4 < 4 ? kB + 4 * c4 : 4 * (c4 - 4);  // its partner in row l: W, then V
                        float4 u[4], w[4];
#pragma unroll
                        for (int r = 0; r < 4; ++r)
                            u[r] = i0 + r < mp ? __ldcg(reinterpret_cast<const float4*>(VWP + (size_t)(i0 + r) * 32) + c4)
                                               : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
                        for (int k = 0; k < 4; ++k) w[k] = *reinterpret_cast<const float4*>(Vs + (l0 + k) * kVwS + oc);
#pragma unroll
                        for (int r = 0; r < 4; ++r)
#pragma unroll
                            for (int k = 0; k < 4; ++k)
                                acc[r][k] += u[r].x * w[k].x + u[r].y * w[k].y + u[r].z * w[k].z + u[r].w * w[k].w;
                    }
#pragma unroll
                    for (int r = 0; r < 4; ++r)
                        if (i0 + r < mp)
                            *reinterpret_cast<float4*>(Dp + (i0 + r) * kB + l0) =
                                make_float4(acc[r][0], acc[r][1], acc[r][2], acc[r][3]);
                }
                __syncthreads();
            }
#pragma unroll
            for (int q = 0; q < kQR; ++q) {
                const int i = tid + kS1Threads * q;
                const bool has = i < mp;
#pragma unroll
                for (int l = 0; l < kB; ++l) prow[q][l] = has ? __ldcg(A + (size_t)(k0 + l) * ld + k0 + i) : 0.f;
                if (upd && has) {
#pragma unroll
                    for (int l4 = 0; l4 < kB / 4; ++l4) {
                        const float4 d = *reinterpret_cast<const float4*>(Dp + i * kB + 4 * l4);
                        prow[q][4 * l4] -= d.x;
                        prow[q][4 * l4 + 1] -= d.y;
                        prow[q][4 * l4 + 2] -= d.z;
                        prow[q][4 * l4 + 3] -= d.w;
                    }
                }
            }
            if (tid < kB)  // the diagonal block (rows k0 .. k0+15) is final: band
#pragma unroll
                for (int l = 0; l < kB; ++l) A[(size_t)(k0 + l) * ld + k0 + tid] = prow[0][l];

            // ---- (2) QR of panel rows kB .. mp-1 (rows r0 ..): one barrier per column. The columns rotate
            //      through the registers (at step j, prow[q][l] is column j + l; zeros past the panel), so one
            //      loop body serves every column (the instruction cache holds it); column j's final values (R in
            //      the band, V below it) go to A and V to shared memory at its step ----
#pragma unroll 1
            for (int j = 0; j < kB; ++j) {
                const int buf = j & 1;
                if (tid == kB + j)  // the pivot row's owner (row kB + j < kS1Threads: q = 0)
#pragma unroll
                    for (int l = 0; l < kB; ++l) Pj[buf * kB + l] = prow[0][l];
                float pr[kB], sq = 0.f;
#pragma unroll
                for (int l = 0; l < kB; ++l) pr[l] = 0.f;
#pragma unroll
                for (int q = 0; q < kQR; ++q) {
                    const int i = tid + kS1Threads * q;
                    if (i > kB + j && i < mp) {
                        const float x = prow[q][0];
                        sq += x * x;
#pragma unroll
                        for (int l = 1; l < kB; ++l) pr[l] += x * prow[q][l];
                    }
                }
                warp_sums17(pr, sq, red + (buf * kS1Warps + warp) * (kB + 1));
                __syncthreads();
                float tot = 0.f;  // lane l <= kB: the CTA's sum l (the same order in every warp)
                if (lane <= kB)
#pragma unroll
                    for (int w = 0; w < kS1Warps; ++w) tot += red[(buf * kS1Warps + w) * (kB + 1) + lane];
                const float sigma = __shfl_sync(0xffffffffu, tot, kB), alpha = Pj[buf * kB];
                float tau = 0.f, beta = alpha, scale = 0.f;
                if (sigma != 0.f) {
                    beta = -copysignf(sqrtf(alpha * alpha + sigma), alpha);
                    tau = (beta - alpha) / beta;
                    scale = 1.f / (alpha - beta);
                }
                // w_l = tau v^T P(:, j + l) = tau (P(j, j + l) + scale d_l), v = [1; scale x], l = 1 .. 15 - j
                const float wl = (lane >= 1 && lane < kB - j) ? tau * (Pj[buf * kB + lane] + scale * tot) : 0.f;
                float wb[kB];
#pragma unroll
                for (int l = 1; l < kB; ++l) wb[l] = __shfl_sync(0xffffffffu, wl, l);
#pragma unroll
                for (int q = 0; q < kQR; ++q) {
                    const int i = tid + kS1Threads * q, ii = i - kB;
                    float out = prow[q][0];  // rows above the pivot: final since their own step
                    if (i == kB + j) {
#pragma unroll
                        for (int l = 1; l < kB; ++l) prow[q][l] -= wb[l];
                        out = beta;
                    } else if (i > kB + j && i < mp) {
                        out = prow[q][0] * scale;
#pragma unroll
                        for (int l = 1; l < kB; ++l) prow[q][l] -= out * wb[l];
                    }
                    if (ii >= 0 && ii < m) {
                        A[(size_t)(k0 + j) * ld + r0 + ii] = out;
                        Vs[j * pst + ii] = ii == j ? 1.f : (ii > j ? out : 0.f);
                    }
#pragma unroll
                    for (int l = 0; l + 1 < kB; ++l) prow[q][l] = prow[q][l + 1];
                    prow[q][kB - 1] = 0.f;
                }
                if (tid == 0) {
                    taus[j] = tau;
                    tauout[D.v_off + k0 + j] = tau;
                }
            }
            __syncthreads();

            // ---- (3) T from T^-1 = diag(1/tau) + triu(V^T V, 1); (V T)^T into the slots ----
            auto vget = [&](int i, int j) -> float { return Vs[j * pst + i]; };
            gram16(m, vget, vget, part, G);
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
                for (int r = 0; r < kB; ++r) Ts[r * kB + j] = t[r];
            }
            __syncthreads();
            const int nq = (m + kCW - 1) / kCW, nmb = (m + 127) / 128, total = nq * nmb;
            for (int ii = tid; ii < kCW * nq; ii += kS1Threads) {
                float vt[kB];
                if (ii < m) {
                    float vr[kB];
#pragma unroll
                    for (int l = 0; l < kB; ++l) vr[l] = vget(ii, l);
#pragma unroll
                    for (int c = 0; c < kB; ++c) vt[c] = 0.f;
#pragma unroll
                    for (int l = 0; l < kB; ++l) {  // T(l, c) = 0 for l > c: the sums of l <= c, in order
                        const float4* tr = reinterpret_cast<const float4*>(Ts + l * kB);
#pragma unroll
                        for (int q = 0; q < kB / 4; ++q) {
                            const float4 t4 = tr[q];
                            vt[4 * q] += vr[l] * t4.x;
                            vt[4 * q + 1] += vr[l] * t4.y;
                            vt[4 * q + 2] += vr[l] * t4.z;
                            vt[4 * q + 3] += vr[l] * t4.w;
                        }
                    }
                } else {
#pragma unroll
                    for (int c = 0; c < kB; ++c) vt[c] = 0.f;
                }
                float4* slot = reinterpret_cast<float4*>(SLOTg + (size_t)(ii / kCW) * kSlotF + kSlotVT + (ii % kCW) * kB);
#pragma unroll
                for (int c4 = 0; c4 < kB / 4; ++c4) slot[c4] = make_float4(vt[4 * c4], vt[4 * c4 + 1], vt[4 * c4 + 2], vt[4 * c4 + 3]);
            }
            tc::fence_async_global();  // the bulk copies of the pass read the slots
            tc::before_sync();
            __syncthreads();

            // ---- (4) the pass over A22: chunk q = (row block I, column chunk J), I outer. Warp 0 loads,
            //      warp 1 issues the update MMAs and the stores, warps 4..7 run the epilogue (warps 2, 3 wait) ----
            if (warp == 0 && lane == 0) {
                tc::after_sync();
                for (int q = 0; ok && q < total; ++q) {
                    const long long g = Q0 + q;
                    const int s = (int)(g % kStages), I = q / nq, J = q - I * nq;
                    if (g >= kStages)
                        ok = ok && tc::mbar_wait(&bars[kEmpty + s], (uint32_t)(((g - kStages) / kStages) & 1), wait_iters);
                    if (!ok) break;
                    tc::mbar_expect_tx(&bars[kFull + s], kTxBytes);
                    tc::tma_load_2d(s1 + kOffOld + s * kOldF, tmap, r0 + kCW * J, r0 + 128 * I, &bars[kFull + s]);
                    tc::bulk_g2s_tx(s1 + kOffSlot + s * kSlotF, SLOTg + (size_t)J * kSlotF, kSlotF * 4, &bars[kFull + s]);
                    last_q = g;
                }
            } else if (warp == 1 && lane == 0) {
                tc::after_sync();
                auto do_update = [&](int q) {  // chunk q's [V W] [W V]^T into accumulator set (U0 + q) & 1
                    const long long g = Q0 + q, u = U0 + q;
                    const int s = (int)(g % kStages), I = q / nq, J = q - I * nq;
                    if (J == 0) ok = ok && tc::mbar_wait(&bars[kVwr], (uint32_t)((V0 + I) & 1), wait_iters);
                    ok = ok && tc::mbar_wait(&bars[kFull + s], (uint32_t)((g / kStages) & 1), wait_iters);
                    if (u >= 2) ok = ok && tc::mbar_wait(&bars[kHxE + (int)(u & 1)], (uint32_t)(((u - 2) >> 1) & 1), wait_iters);
                    if (!ok) return;
                    tc::after_sync();
                    const uint32_t d = tm + kHX + 2 * kCW * (uint32_t)(u & 1), a = tm + kVWT, al = a + 32;
                    const uint64_t b = tc::sdesc(tc::smem_addr(s1 + kOffSlot + s * kSlotF)), bl = b + (kSlotLo * 4 >> 4);
#pragma unroll
                    for (int sk = 0; sk < 4; ++sk) {
                        const uint64_t o = 16 * sk;  // 256 B per K step of 8 in shared memory, 8 columns in tensor memory
                        tc::umma_ta<kIdN>(d, a + 8 * sk, b + o, sk > 0);
                        tc::umma_ta<kIdN>(d + kCW, a + 8 * sk, bl + o, sk > 0);
                        tc::umma_ta<kIdN>(d + kCW, al + 8 * sk, b + o, 1);
                    }
                    tc::umma_commit(&bars[kHxF + (int)(u & 1)]);
                    last_u = u;
                };
                if (upd && total > 0) do_update(0);
                for (int q = 0; ok && q < total; ++q) {
                    const long long g = Q0 + q;
                    const int s = (int)(g % kStages), I = q / nq, J = q - I * nq;
                    // the next chunk's update runs beside this chunk's epilogue (except across a row
                    // block: its [V W] is written by the epilogue warps after this chunk)
                    const bool next_in_block = upd && q + 1 < total && J + 1 < nq;
                    if (next_in_block) do_update(q + 1);
                    ok = ok && tc::mbar_wait(&bars[kEpi + s], (uint32_t)((g / kStages) & 1), wait_iters);
                    if (!ok) break;
                    if (upd) {  // the updated chunk back to A22
                        tc::tma_store_2d(tmap, r0 + kCW * J, r0 + 128 * I, s1 + kOffOld + s * kOldF);
                        tc::bulk_commit();
                    }
                    if (upd && q + 1 < total && !next_in_block) do_update(q + 1);
                    if (!upd) {
                        tc::mbar_arrive(&bars[kEmpty + s]);
                    } else {  // the previous chunk's store has read its stage (this chunk's may still be reading)
                        tc::bulk_wait_read<1>();
                        if (q > 0) tc::mbar_arrive(&bars[kEmpty + (int)((g - 1) % kStages)]);
                    }
                }
                if (ok && upd && total > 0) {
                    tc::bulk_wait_read<0>();
                    tc::mbar_arrive(&bars[kEmpty + (int)((Q0 + total - 1) % kStages)]);
                }
                tc::bulk_wait_all();       // the stores of A22 are complete
                tc::fence_async_global();  // ... and visible to the loads after the pass
            } else if (warp >= 4) {
                // X of the row block in 4 x 4 tiles: this thread's rows xr .. xr + 3, columns xc .. xc + 3
                float xacc[4][4];
#pragma unroll
                for (int e = 0; e < 16; ++e) xacc[e >> 2][e & 3] = 0.f;
                const int row = erow;  // the chunk's row = tensor-memory lane
                const int xr = 4 * (erow >> 2), xc = 4 * (erow & 3);
                for (int q = 0; ok && q < total; ++q) {
                    const long long g = Q0 + q, u = U0 + q;
                    const int s = (int)(g % kStages), I = q / nq, J = q - I * nq;
                    // the chunk's row in shared memory: 128 bytes, its 16-byte units permuted by the TMA's
                    // 128-byte swizzle (unit u at u ^ address bits 7..9), so that the 8 rows of a quarter warp
                    // reach 8 different bank groups
                    // (the stages start on 1024-byte boundaries: the unit permutation of row r is r & 7)
                    float* const chunk = s1 + kOffOld + s * kOldF;
                    float* old = chunk + row * kCW;
                    const int sw = row & 7;
                    if (upd && J == 0) {  // the row block's [V W] (hi, lo) into tensor memory, row = lane
                        // (the block's first update waits for it; the previous block's updates are complete:
                        // this thread waited for the last of them)
                        const int vr = kB + I * 128 + row;  // row of the previous panel's V | W
                        float v32[2 * kB];
                        if (vr < m + kB) {
                            const float4* src = reinterpret_cast<const float4*>(VWP + (size_t)vr * 32);
#pragma unroll
                            for (int u4 = 0; u4 < 8; ++u4) {
                                const float4 x = __ldcg(src + u4);
                                v32[4 * u4] = x.x; v32[4 * u4 + 1] = x.y; v32[4 * u4 + 2] = x.z; v32[4 * u4 + 3] = x.w;
                            }
                        } else {
#pragma unroll
                            for (int e = 0; e < 2 * kB; ++e) v32[e] = 0.f;
                        }
#pragma unroll
                        for (int h = 0; h < 2; ++h) {
                            float hi[16], lo[16];
#pragma unroll
                            for (int e = 0; e < 16; ++e) {
                                unsigned uh, ul;
                                split_tf32(v32[16 * h + e], uh, ul);
                                hi[e] = __uint_as_float(uh);
                                lo[e] = __uint_as_float(ul);
                            }
                            tc::tmem_st16(tlane + kVWT + 16 * h, hi);
                            tc::tmem_st16(tlane + kVWT + 32 + 16 * h, lo);
                        }
                        tc::tmem_wait_st();
                        tc::before_sync();
                        tc::mbar_arrive(&bars[kVwr]);
                    }
                    if (upd) ok = ok && tc::mbar_wait(&bars[kHxF + (int)(u & 1)], (uint32_t)((u >> 1) & 1), wait_iters);
                    ok = ok && tc::mbar_wait(&bars[kFull + s], (uint32_t)((g / kStages) & 1), wait_iters);
                    ok = __all_sync(0xffffffffu, ok);  // the tensor-memory loads below are warp-collective
                    if (ok && upd) {
                        tc::after_sync();
                        float a32[kCW];
#pragma unroll
                        for (int v4 = 0; v4 < kCW / 4; ++v4) {
                            const float4 x = *reinterpret_cast<const float4*>(old + 4 * (v4 ^ sw));
                            a32[4 * v4] = x.x; a32[4 * v4 + 1] = x.y; a32[4 * v4 + 2] = x.z; a32[4 * v4 + 3] = x.w;
                        }
                        float h[kCW];
                        const uint32_t d = tlane + kHX + 2 * kCW * (uint32_t)(u & 1);
                        tc::tmem_ld32(d + kCW, h);  // cross products first: a - (hi hi + cross)
#pragma unroll
                        for (int e = 0; e < kCW; ++e) a32[e] -= h[e];
                        tc::tmem_ld32(d, h);
                        tc::before_sync();
                        tc::mbar_arrive(&bars[kHxE + (int)(u & 1)]);  // the accumulator set is free
#pragma unroll
                        for (int e = 0; e < kCW; ++e) a32[e] -= h[e];
#pragma unroll
                        for (int v4 = 0; v4 < kCW / 4; ++v4)
                            *reinterpret_cast<float4*>(old + 4 * (v4 ^ sw)) =
                                make_float4(a32[4 * v4], a32[4 * v4 + 1], a32[4 * v4 + 2], a32[4 * v4 + 3]);
                        tc::fence_async_smem();  // the store reads the updated chunk
                    }
                    // every row of the chunk updated (X reads four rows per thread); the epilogue warps agree on ok
                    ok = epi_barrier_and(ok);
                    if (!ok) break;
                    {  // X(xr.., xc..) += A22(xr.., chunk) (V T)(chunk, xc..), FP32, one 16-byte unit of chunk columns
                       // at a time
                        const float4* vt = reinterpret_cast<const float4*>(s1 + kOffSlot + s * kSlotF + kSlotVT) + (erow & 3);
#pragma unroll
                        for (int v4 = 0; v4 < kCW / 4; ++v4) {
                            float4 a[4], w[4];
#pragma unroll
                            for (int i = 0; i < 4; ++i) {
                                const int r = xr + i;
                                a[i] = *reinterpret_cast<const float4*>(chunk + r * kCW + 4 * (v4 ^ (r & 7)));
                            }
#pragma unroll
                            for (int k = 0; k < 4; ++k) w[k] = vt[(4 * v4 + k) * (kB / 4)];
#pragma unroll
                            for (int i = 0; i < 4; ++i) {
                                const float ai[4] = {a[i].x, a[i].y, a[i].z, a[i].w};
#pragma unroll
                                for (int k = 0; k < 4; ++k) {
                                    xacc[i][0] += ai[k] * w[k].x;
                                    xacc[i][1] += ai[k] * w[k].y;
                                    xacc[i][2] += ai[k] * w[k].z;
                                    xacc[i][3] += ai[k] * w[k].w;
                                }
                            }
                        }
                    }
                    tc::mbar_arrive(&bars[kEpi + s]);  // the chunk's buffers are read (and written)
                    if (J + 1 == nq) {  // the row block's X tiles
#pragma unroll
                        for (int i = 0; i < 4; ++i) {
                            const int xrow = I * 128 + xr + i;
                            if (xrow < m)
                                *reinterpret_cast<float4*>(XG + (size_t)xrow * kB + xc) =
                                    make_float4(xacc[i][0], xacc[i][1], xacc[i][2], xacc[i][3]);
                        }
#pragma unroll
                        for (int e = 0; e < 16; ++e) xacc[e >> 2][e & 3] = 0.f;
                    }
                }
            }
            Q0 += total;
            if (upd) {
                U0 += total;
                V0 += nmb;
            }
            tc::before_sync();
            ok = __syncthreads_and(ok);
            if (!ok) break;
            tc::after_sync();

            // ---- (5) W = X - 1/2 V (T^T (V^T X)); [V W], [W V] and V | W into the scratch ----
            auto vgl = [&](int i, int j) -> float {
                return j == i ? 1.f : (i > j ? __ldcg(A + (size_t)(k0 + j) * ld + r0 + i) : 0.f);
            };
            gram16(m, vgl, [&](int i, int c) { return XG[(size_t)i * kB + c]; }, part, G);  // (V^T X)(g, c)
            float* Mt = part;  // M = T^T (V^T X), rows of kB (vector reads below); gram16's scratch is free
            {
                const int c = tid & (kB - 1), gg = tid / kB;  // M(gg, c)
                float mtc = 0.f;
                for (int l = 0; l <= gg; ++l) mtc += Ts[l * kB + gg] * G[l * (kB + 1) + c];
                Mt[gg * kB + c] = mtc;
            }
            __syncthreads();
            const int m2 = m - kB;                                      // rows of the next pass
            const int nq2 = m2 > 0 ? (m2 + kCW - 1) / kCW : 0;
            const int lim = max(m, kB + kCW * nq2);  // the last chunk's rows beyond the matrix: zeros
            for (int ii = tid; ii < lim; ii += kS1Threads) {
                float vw[2 * kB];  // V then W of row ii (zero beyond the matrix)
                if (ii < m) {
#pragma unroll
                    for (int l = 0; l < kB; ++l) vw[l] = vgl(ii, l);
                    float acc[kB];  // (V M)(ii, c), summed over l in order
#pragma unroll
                    for (int c = 0; c < kB; ++c) acc[c] = 0.f;
#pragma unroll
                    for (int l = 0; l < kB; ++l) {
                        const float4* mr = reinterpret_cast<const float4*>(Mt + l * kB);
#pragma unroll
                        for (int q = 0; q < kB / 4; ++q) {
                            const float4 mq = mr[q];
                            acc[4 * q] += vw[l] * mq.x;
                            acc[4 * q + 1] += vw[l] * mq.y;
                            acc[4 * q + 2] += vw[l] * mq.z;
                            acc[4 * q + 3] += vw[l] * mq.w;
                        }
                    }
                    const float4* xs = reinterpret_cast<const float4*>(XG + (size_t)ii * kB);
#pragma unroll
                    for (int q = 0; q < kB / 4; ++q) {
                        const float4 x = xs[q];
                        vw[kB + 4 * q] = x.x - 0.5f * acc[4 * q];
                        vw[kB + 4 * q + 1] = x.y - 0.5f * acc[4 * q + 1];
                        vw[kB + 4 * q + 2] = x.z - 0.5f * acc[4 * q + 2];
                        vw[kB + 4 * q + 3] = x.w - 0.5f * acc[4 * q + 3];
                    }
                    float4* dst = reinterpret_cast<float4*>(VWP + (size_t)ii * 32);
#pragma unroll
                    for (int u = 0; u < 8; ++u) dst[u] = make_float4(vw[4 * u], vw[4 * u + 1], vw[4 * u + 2], vw[4 * u + 3]);
                } else {
#pragma unroll
                    for (int c = 0; c < 2 * kB; ++c) vw[c] = 0.f;
                }
                if (ii >= kB && m2 > 0) {
                    const int t = ii - kB;  // row of the next pass
                    if (t < kCW * nq2) {  // B operand [W V] of the chunk's slot
                        float* sl = SLOTg + (size_t)(t / kCW) * kSlotF;
#pragma unroll
                        for (int v4 = 0; v4 < 8; ++v4) {
                            const int src = v4 < 4 ? kB + 4 * v4 : 4 * (v4 - 4);
                            const float x4[4] = {vw[src], vw[src + 1], vw[src + 2], vw[src + 3]};
                            float4 lo;
                            const float4 hi = tc::split4(x4, lo);
                            const int o = tc::kofs(t % kCW, 4 * v4);
                            *reinterpret_cast<float4*>(sl + o) = hi;
                            *reinterpret_cast<float4*>(sl + kSlotLo + o) = lo;
                        }
                    }
                }
            }
            tc::fence_async_global();  // the next pass's bulk copies read the tiles and slots
            __syncthreads();
        }
        if (!ok) break;
        if (k0 > 0) {  // the last panel's update on the remaining block A(k0:, k0:) (lower triangle)
            const int mt = n - k0;
            for (int t = tid; t < mt * mt; t += kS1Threads) {
                const int i = t % mt, c = t / mt;
                if (i < c) continue;
                const float* vi = VWP + (size_t)i * 32;
                const float* vc = VWP + (size_t)c * 32;
                float sacc = 0.f;
#pragma unroll
                for (int q = 0; q < kB; ++q) sacc += vi[q] * vc[kB + q] + vi[kB + q] * vc[q];
                float* e = A + (size_t)(k0 + c) * ld + k0 + i;
                *e = __ldcg(e) - sacc;
            }
        }
        __syncthreads();
        if (!order) break;
    }
    if (!ok) {
        if (tid == 0) atomicOr(status, kStatusTimeout);
        // the copies and MMA groups this CTA started complete before the tensor
        // memory is freed and the CTA exits: each issuing thread drains its own
        if (warp == 0 && lane == 0) {
            for (long long g = last_q - (kStages - 1); g <= last_q; ++g)
                if (g >= 0) tc::mbar_wait(&bars[kFull + (int)(g % kStages)], (uint32_t)((g / kStages) & 1), kDefaultWaitIters);
        }
        if (warp == 1 && lane == 0) {
            if (last_u >= 0) tc::mbar_wait(&bars[kHxF + (int)(last_u & 1)], (uint32_t)((last_u >> 1) & 1), kDefaultWaitIters);
            tc::bulk_wait_all();
        }
    }
    tc::before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tm, kTmemCols);
}

}  // namespace

size_t sy2sb_smem_bytes(int /*max_ld*/) { return sizeof(float) * (kRegionF + kSmallF) + kNumBars * 8 + 16; }

long long sy2sb_scratch_floats(int max_ld) { return s1_scratch_floats(max_ld); }

size_t sy2sb_tensor_map_bytes() { return sizeof(CUtensorMap); }

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library)
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

static cudaError_t encode_matrix_maps(const ChainDesc* h_desc, int batch, float* d_A, int box_rows, int box_cols,
                                      bool swizzle128, void* h_maps) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc) return cudaErrorNotSupported;
    CUtensorMap* maps = static_cast<CUtensorMap*>(h_maps);
    for (int c = 0; c < batch; ++c) {
        const ChainDesc& d = h_desc[c];
        const cuuint64_t dims[2] = {(cuuint64_t)d.ld, (cuuint64_t)d.ld};
        const cuuint64_t strides[1] = {(cuuint64_t)d.ld * sizeof(float)};
        const cuuint32_t box[2] = {(cuuint32_t)box_rows, (cuuint32_t)box_cols};
        const cuuint32_t estr[2] = {1, 1};
        const CUresult r = enc(&maps[c], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, d_A + d.a_off, dims, strides, box, estr,
                               CU_TENSOR_MAP_INTERLEAVE_NONE,
                               swizzle128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                               CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return cudaErrorInvalidValue;
    }
    return cudaSuccess;
}

// One tensor map per chain over its ld x ld FP32 matrix at d_A + a_off
// (dimension 0 the rows, contiguous; box 32 rows x 128 columns, 128-byte swizzle),
// written to h_maps (batch * sy2sb_tensor_map_bytes() bytes, 64-byte aligned).
cudaError_t sy2sb_tensor_maps(const ChainDesc* h_desc, int batch, float* d_A, void* h_maps) {
    return encode_matrix_maps(h_desc, batch, d_A, kCW, 128, true, h_maps);
}

cudaError_t launch_sy2sb(const ChainDesc* d_desc, int batch, int max_ld, const double* d_diag, float* d_A,
                         float* d_tau, const int* d_order, int* d_counter, int num_sms, int* d_status,
                         float* d_scratch, const void* d_tmaps, long long wait_iters, cudaStream_t st) {
    if (batch <= 0) return cudaSuccess;
    if (max_ld > kMaxLd || !d_tmaps) return cudaErrorInvalidValue;
    const size_t smem = sy2sb_smem_bytes(max_ld);
    // three panel rows per thread up to n = 768 (fewer registers held through the QR), four beyond
    auto kern = max_ld <= 3 * kS1Threads ? sy2sb_kernel<3> : sy2sb_kernel<4>;
    cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    // the largest shared-memory configuration: two CTAs per SM
    err = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
    if (err != cudaSuccess) return err;
    int grid = batch;
    if (d_order) {
        // CTAs per SM from the kernel's own limits: shared memory (with the per-CTA reservation),
        // registers (128 per thread) and tensor memory (512 columns per SM). The occupancy API
        // answers 1 for kernels that allocate tensor memory, but two such CTAs do run side by side.
        int dev = 0, smem_sm = 0, resv = 0, regs_sm = 0;
        if ((err = cudaGetDevice(&dev))) return err;
        if ((err = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev))) return err;
        if ((err = cudaDeviceGetAttribute(&resv, cudaDevAttrReservedSharedMemoryPerBlock, dev))) return err;
        if ((err = cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev))) return err;
        cudaFuncAttributes fa;
        if ((err = cudaFuncGetAttributes(&fa, kern))) return err;
        int per_sm = (int)(512 / kTmemCols);
        per_sm = min(per_sm, smem_sm / (int)(smem + resv));
        per_sm = min(per_sm, regs_sm / (max(fa.numRegs, 1) * kS1Threads));
        grid = max(1, min(batch, max(1, per_sm) * num_sms));
        if ((err = cudaMemsetAsync(d_counter, 0, sizeof(int), st))) return err;
    }
    kern<<<grid, kS1Threads, smem, st>>>(d_desc, d_diag, d_A, d_tau, d_order, batch, d_counter, d_status,
                                                 max_ld, d_scratch, static_cast<const CUtensorMap*>(d_tmaps),
                                                 wait_iters < 0 ? kDefaultWaitIters : wait_iters);
    return cudaGetLastError();
}

}  // namespace fkg
