// backtransform_tc5.cu — mixed path back-transformation X = Q Z on the
// fifth-generation tensor cores (tcgen05: operands in shared memory,
// accumulators in tensor memory), FP32-accurate through the 3xTF32 split.
//
// Q = H_0 H_1 ... H_{n-3} comes from the FP32 Householder reduction as panels
// of 32 reflectors, Q_p = I - V_p T_p V_p^T; larft_kernel writes V_p and
// V_p T_p split into TF32 hi/lo planes (four planes `plane` floats apart:
// (V T) hi, (V T) lo, V hi, V lo; column k0 + l, rows k0 .. ld-1). Applied
// from the last panel to the first, each panel is two GEMMs:
//   G1:  W^T = Zb^T V_p        (128 columns x 32 reflectors, K = rows)
//   G2:  Zb += (-W^T) (V_p T_p)^T   (128 columns x rows, K = 32 reflectors)
// One CTA owns 128 columns of Z (the MMAs' M = 128: tensor-memory lane c is
// column j0 + c); Z is updated in place in global memory (L2-resident for the
// CTA's 128 columns). Operand tiles are staged by the threads (Z is split into
// hi/lo on the way) into shared memory in the canonical K-major layout without
// swizzle (8-row x 16-byte core matrices; LBO = 128 B between core matrices
// along K, SBO = 1024 B between 8-row groups; a K step of 8 advances the
// descriptors by 256 B). One thread issues the tcgen05.mma instructions
// (kind::tf32, M = 128, N = 32, K = 8) and commits them to an mbarrier per
// stage buffer; stage buffers and accumulators are double-buffered: per
// 32-row step the threads stage chunk q (its global loads were issued one step
// earlier), thread 0 issues its MMAs, and the threads then read back chunk
// q - 1, whose MMAs ran during the staging.
//
// Measured on the bench workload (N = 576, 256 chains): 3.6 ms per launch
// against 3.0 ms for the mma.sync kernel of backtransform_tc.cu, which keeps
// its 32-column block of Z in shared memory: with 128 columns (M = 128) the
// block of Z does not fit on the chip (295 KB at N = 576, above both shared
// and tensor memory), so Z is re-read and re-written through L2 for every
// panel (about 11 MB per CTA) and the steps are latency bound. The autotuner
// times both per size class and picks one.
//
// Accuracy: the tensor memory accumulates with a truncating add (measured on
// GB300: about four times the error of round-to-nearest FP32 over 32 K steps,
// biased towards zero). The large products a_hi b_hi of G1 (K = all rows of
// the panel) therefore go into a fresh accumulator per 32-row chunk, which the
// threads add into FP32 registers with round-to-nearest; the cross products
// a_hi b_lo + a_lo b_hi (2^-11 smaller) accumulate in tensor memory over the
// whole panel, separately. G2 has K = 32: its a_hi b_hi products (4 steps)
// and its cross products have an accumulator each.
//
// Every mbarrier wait is bounded. A main-loop wait gives up after
// `wait_iters` checks (a kernel argument; 0 gives up without checking, which
// tests this path); the CTA then sets kStatusTimeout, stops issuing MMAs,
// waits (with the full default limit) for every MMA group it has committed,
// and frees its tensor memory.
#include <cstdint>

#include "fkg_common.cuh"
#include "tcgen05.cuh"

namespace fkg {
namespace {

constexpr int kT5C = 128;       // columns of Z per CTA (the MMAs' M)
constexpr int kT5Threads = 256;
constexpr uint32_t kT5TmemCols = 256;
// tensor-memory columns (each 32 wide: one 128 x 32 FP32 accumulator)
constexpr uint32_t kD1 = 0;     // [2] G1 chunk hi*hi
constexpr uint32_t kD1x = 64;   // G1 cross products of the panel
constexpr uint32_t kD2 = 96;    // [2] x {hi*hi, cross} of a G2 tile (64 apart)
// shared memory (bytes)
constexpr int kBig = 128 * 32 * 4;     // one 128 x 32 FP32 operand tile
constexpr int kSmall = 32 * 32 * 4;    // one 32 x 32 FP32 operand tile
constexpr int kStage = 2 * kBig + 2 * kSmall;  // G1: Zb^T hi/lo, V hi/lo; G2: (V T) hi/lo
constexpr int kA2 = 2 * kStage;        // -W^T hi/lo
constexpr int kBar = kA2 + 2 * kBig;   // two mbarriers, the tensor-memory address
constexpr int kT5Smem = kBar + 32;
// TF32 x TF32 -> FP32, both operands K-major, M = 128, N = 32
constexpr uint32_t kIdesc = tc::idesc_tf32(32);

using tc::smem_addr;
using tc::sdesc;
using tc::kofs;
using tc::umma_commit;
using tc::mbar_wait;
using tc::tmem_ld16;
using tc::fence_async_smem;
using tc::split4;
__device__ __forceinline__ void umma(uint32_t d, uint64_t a, uint64_t b, uint32_t acc) { tc::umma<kIdesc>(d, a, b, acc); }
__device__ __forceinline__ void tc_before_sync() { tc::before_sync(); }
__device__ __forceinline__ void tc_after_sync() { tc::after_sync(); }

__global__ void __launch_bounds__(kT5Threads, 2)
backtransform_tc5_kernel(const ChainDesc* __restrict__ descs, const float* __restrict__ VTs, long long plane,
                         float* __restrict__ Zws, const float* __restrict__ zscale, int* __restrict__ status,
                         long long wait_iters, int shift) {
    extern __shared__ __align__(1024) unsigned char sm5[];
    const ChainDesc D = descs[blockIdx.y];
    const int n = D.n, ld = D.ld, j0 = blockIdx.x * kT5C;
    if (j0 >= n) return;
    const float* VTh = VTs + D.a_off;
    const float* VTl = VTh + plane;
    const float* Vh = VTl + plane;
    const float* Vl = Vh + plane;
    float* Z = Zws + D.a_off;
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm5 + kBar);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm5 + kBar + 16);
    float* A2h = reinterpret_cast<float*>(sm5 + kA2);
    float* A2l = A2h + kBig / 4;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    // unit columns (the twisted factorisation's scales)
    {
        const int c = tid & (kT5C - 1), j = j0 + c;
        if (j < n) {
            const float zs = zscale[D.v_off + j];
            for (int i = tid >> 7; i < n; i += 2) Z[(size_t)i * ld + j] *= zs;
        }
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&bar[0])));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&bar[1])));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tslot)),
                     "r"(kT5TmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    const uint32_t tm = *tslot;
    const int c = (warp & 3) * 32 + lane;            // this thread's column (tensor-memory lane)
    const int half = warp >> 2;                      // this thread's 16 of an accumulator's 32 columns
    const uint32_t trow = tm + ((uint32_t)((warp & 3) * 32) << 16) + 16 * half;
    const bool colok = j0 + c < n;
    // completed waits per barrier (the same in every thread), and the MMA groups
    // thread 0 has committed to each barrier (thread 0 only)
    uint32_t uses[2] = {0u, 0u}, commits[2] = {0u, 0u};
    bool ok = true;

    // staging roles: G1's Zb^T tile (column sc, row groups 4h..4h+3), its V
    // tile and G2's (V T) tile (one float4 each of hi and lo)
    const int sc = tid & 127, sh = tid >> 7;
    const int vl = ((tid >> 6) << 3) | (tid & 7), vm = (tid >> 3) & 7;  // V tile: reflector vl, rows 4vm..
    const int ti = tid & 31, tg = tid >> 5;                             // (V T) tile: row ti, reflectors 4tg..

    const int nrefl = n - 1 - shift;  // reflector k: unit at row k + shift
    const int npanel = nrefl > 0 ? (nrefl + 31) / 32 : 0;
    for (int p = npanel - 1; p >= 0 && ok; --p) {
        const int k0 = p * 32;
        const int nq = (ld - k0) / 32;  // 32-row chunks from row k0
        // ---------------- G1: W^T = Zb^T V_p ----------------
        float wacc[16];
#pragma unroll
        for (int e = 0; e < 16; ++e) wacc[e] = 0.f;
        float pz[16];
        float4 pvh, pvl;
        auto load_g1 = [&](int q) {
            const int i0 = k0 + 32 * q;
#pragma unroll
            for (int e = 0; e < 16; ++e) {
                const int i = i0 + 4 * (4 * sh + (e >> 2)) + (e & 3);
                pz[e] = (i < n && j0 + sc < n) ? Z[(size_t)i * ld + j0 + sc] : 0.f;
            }
            const size_t g = (size_t)(k0 + vl) * ld + i0 + 4 * vm;
            pvh = *reinterpret_cast<const float4*>(Vh + g);
            pvl = *reinterpret_cast<const float4*>(Vl + g);
        };
        load_g1(0);
        for (int q = 0; q <= nq; ++q) {
            const int b = q & 1;
            unsigned char* st = sm5 + b * kStage;
            if (q < nq) {
                float* Ah = reinterpret_cast<float*>(st);
                float* Al = Ah + kBig / 4;
                float* Bh = Al + kBig / 4;
                float* Bl = Bh + kSmall / 4;
#pragma unroll
                for (int m = 0; m < 4; ++m) {
                    const float x[4] = {pz[4 * m], pz[4 * m + 1], pz[4 * m + 2], pz[4 * m + 3]};
                    float4 lo;
                    const float4 hi = split4(x, lo);
                    const int o = kofs(sc, 4 * (4 * sh + m));
                    *reinterpret_cast<float4*>(Ah + o) = hi;
                    *reinterpret_cast<float4*>(Al + o) = lo;
                }
                const int ov = kofs(vl, 4 * vm);
                *reinterpret_cast<float4*>(Bh + ov) = pvh;
                *reinterpret_cast<float4*>(Bl + ov) = pvl;
                fence_async_smem();
                if (q + 1 < nq) load_g1(q + 1);
            }
            tc_before_sync();
            ok = __syncthreads_and(ok);
            if (!ok) break;
            if (q < nq && tid == 0) {
                tc_after_sync();
                const uint64_t a = sdesc(smem_addr(st)), al = a + (kBig >> 4), bh = a + (2 * kBig >> 4),
                               bl = bh + (kSmall >> 4);
#pragma unroll
                for (int s = 0; s < 4; ++s) {
                    const uint64_t o = 16 * s;  // 256 B per K step, in descriptor units of 16 B
                    umma(tm + kD1 + 32 * b, a + o, bh + o, s > 0);
                    umma(tm + kD1x, a + o, bl + o, (q > 0 || s > 0));
                    umma(tm + kD1x, al + o, bh + o, 1);
                }
                umma_commit(&bar[b]);
                ++commits[b];
            }
            // chunk q - 1 (issued one iteration earlier): its hi*hi sums into the registers;
            // the wait also frees its stage buffer for chunk q + 1
            if (q > 0) {
                const int bp = (q - 1) & 1;
                ok = ok && mbar_wait(&bar[bp], uses[bp] & 1u, wait_iters);
                if (ok) ++uses[bp];
                tc_after_sync();
                if (ok) {
                    float v[16];
                    tmem_ld16(trow + kD1 + 32 * bp, v);
#pragma unroll
                    for (int e = 0; e < 16; ++e) wacc[e] += v[e];
                }
            }
        }
        tc_before_sync();
        ok = __syncthreads_and(ok);
        if (!ok) break;
        // W^T (columns c, reflectors 16 half ..) = registers + cross products;
        // -W^T split into A2 (all G1 products are complete)
        tc_after_sync();
        {
            float v[16];
            tmem_ld16(trow + kD1x, v);
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                const float x[4] = {-(wacc[4 * m] + v[4 * m]), -(wacc[4 * m + 1] + v[4 * m + 1]),
                                    -(wacc[4 * m + 2] + v[4 * m + 2]), -(wacc[4 * m + 3] + v[4 * m + 3])};
                float4 lo;
                const float4 hi = split4(x, lo);
                const int o = kofs(c, 16 * half + 4 * m);
                *reinterpret_cast<float4*>(A2h + o) = hi;
                *reinterpret_cast<float4*>(A2l + o) = lo;
            }
        }
        // ---------------- G2: Zb += (-W^T) (V_p T_p)^T, 32-row tiles ----------------
        float pth[4], ptl[4];
        auto load_g2 = [&](int t) {
            const int i = k0 + 32 * t + ti;
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const size_t g = (size_t)(k0 + 4 * tg + e) * ld + i;
                pth[e] = VTh[g];
                ptl[e] = VTl[g];
            }
        };
        load_g2(0);
        float zr[16];
        auto load_z = [&](int t) {  // the rows of tile t this thread updates
            const int i0 = k0 + 32 * t + 16 * half;
#pragma unroll
            for (int r = 0; r < 16; ++r) zr[r] = (colok && i0 + r < n) ? Z[(size_t)(i0 + r) * ld + j0 + c] : 0.f;
        };
        for (int t = 0; t <= nq; ++t) {
            const int b = t & 1;
            unsigned char* st = sm5 + b * kStage;
            if (t > 0) load_z(t - 1);
            if (t < nq) {
                float* Bh = reinterpret_cast<float*>(st);
                float* Bl = Bh + kSmall / 4;
                const int o = kofs(ti, 4 * tg);
                *reinterpret_cast<float4*>(Bh + o) = make_float4(pth[0], pth[1], pth[2], pth[3]);
                *reinterpret_cast<float4*>(Bl + o) = make_float4(ptl[0], ptl[1], ptl[2], ptl[3]);
                fence_async_smem();
                if (t + 1 < nq) load_g2(t + 1);
            }
            tc_before_sync();
            ok = __syncthreads_and(ok);
            if (!ok) break;
            if (t < nq && tid == 0) {
                tc_after_sync();
                const uint64_t a = sdesc(smem_addr(A2h)), al = a + (kBig >> 4), bh = sdesc(smem_addr(st)),
                               bl = bh + (kSmall >> 4);
#pragma unroll
                for (int s = 0; s < 4; ++s) {
                    const uint64_t o = 16 * s;
                    umma(tm + kD2 + 64 * b, a + o, bh + o, s > 0);
                    umma(tm + kD2 + 64 * b + 32, a + o, bl + o, s > 0);
                    umma(tm + kD2 + 64 * b + 32, al + o, bh + o, 1);
                }
                umma_commit(&bar[b]);
                ++commits[b];
            }
            if (t > 0) {  // tile t - 1 done: add its update to Z
                const int bp = (t - 1) & 1;
                ok = ok && mbar_wait(&bar[bp], uses[bp] & 1u, wait_iters);
                if (ok) ++uses[bp];
                tc_after_sync();
                if (ok) {
                    float u[16], x[16];
                    tmem_ld16(trow + kD2 + 64 * bp, u);
                    tmem_ld16(trow + kD2 + 64 * bp + 32, x);
                    const int i0 = k0 + 32 * (t - 1) + 16 * half;
                    if (colok)
#pragma unroll
                        for (int r = 0; r < 16; ++r)
                            if (i0 + r < n) Z[(size_t)(i0 + r) * ld + j0 + c] = zr[r] + (u[r] + x[r]);
                }
            }
        }
        // Z of this panel complete before the next panel reads it; ok uniform
        tc_before_sync();
        ok = __syncthreads_and(ok);
    }
    if (!ok && tid == 0) {
        atomicOr(status, kStatusTimeout);
        // every committed MMA group completes (each barrier's phases in commit
        // order) before the tensor memory is freed
        for (int b = 0; b < 2; ++b)
            while (uses[b] < commits[b] && mbar_wait(&bar[b], uses[b] & 1u, kDefaultWaitIters)) ++uses[b];
    }
    tc_before_sync();
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tm), "r"(kT5TmemCols));
}

}  // namespace

cudaError_t launch_backtransform_tc5(const ChainDesc* d_desc, int batch, int max_n, const float* d_VT, long long plane,
                                     float* d_Z, const float* d_zscale, int* d_status, long long wait_iters,
                                     int shift, cudaStream_t st) {
    if (batch <= 0) return cudaSuccess;
    if (batch > 65535) return cudaErrorInvalidValue;  // grid y limit
    cudaError_t err = cudaFuncSetAttribute(backtransform_tc5_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kT5Smem);
    if (err != cudaSuccess) return err;
    backtransform_tc5_kernel<<<dim3((max_n + kT5C - 1) / kT5C, batch), kT5Threads, kT5Smem, st>>>(
        d_desc, d_VT, plane, d_Z, d_zscale, d_status, wait_iters < 0 ? kDefaultWaitIters : wait_iters, shift);
    return cudaGetLastError();
}

}  // namespace fkg
