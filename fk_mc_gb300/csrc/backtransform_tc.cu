// backtransform_tc.cu — mixed path back-transformation X = Q Z on the tensor
// cores, FP32-accurate through the 3xTF32 split.
//
// Q = H_0 H_1 ... H_{n-3} comes from the FP32 Householder reduction as panels
// of 32 reflectors in compact-WY form, Q_p = I - V_p T_p V_p^T (V_p in the
// reduced matrix's columns; larft_kernel writes (V_p T_p) in the same layout).
// Applied from the last panel to the first, each panel is two skinny GEMMs:
//   W^T  = Zb^T V_p              (32 columns x 32 reflectors, K = rows)
//   Zb^T -= W^T (V_p T_p)^T      (32 columns x rows, K = 32 reflectors)
// One CTA owns 32 columns of Z (Zb), resident in shared memory for all
// panels (loaded with the twisted factorisation's column scales applied);
// V_p and V_p T_p stream through shared memory in 64-row chunks by
// cp.async, double-buffered. The products run as mma.sync m16n8k8 TF32 with each FP32
// operand split x = hi + lo (hi = tf32(x), lo = tf32(x - hi)) and
// a b ~ a_hi b_hi + a_hi b_lo + a_lo b_hi accumulated in FP32, which keeps
// about 22 significant bits per product (the accumulation rule is at
// mma_big). V_p and V_p T_p arrive split (larft_kernel writes hi and lo
// planes once per chain); only the Z block and W^T are split here.
//
// Shared-memory layouts ([column][row] for Zb, [reflector][row] for V) XOR the
// row index with swz(column or reflector); with that, every fragment load of
// both GEMMs and the accumulator loads/stores are free of bank conflicts, and
// groups of four rows stay contiguous for the 16-byte cp.async.
//
// The first GEMM splits its K range (rows) over the 8 warps; their partial
// W^T are summed by a fixed three-level tree, so results are bit-reproducible.
#include "fkg_common.cuh"

namespace fkg {
namespace {

constexpr int kNC = 32;        // columns of Z per CTA
constexpr int kCH = 64;        // rows of V per staged chunk
constexpr int kPanel = 32;     // reflectors per panel (the larft panel width)
constexpr int kTcThreads = 256;
constexpr int kTP = kPanel + 1;  // padded row of the 32 x 32 shared-memory matrices

__device__ __forceinline__ int swz(int r) { return ((r & 3) << 3) | (r & 4); }

// The tensor core adds the products to its accumulator input with
// truncation, so long chains of accumulation in it drift. Every product
// a_hi b_hi therefore goes into a zeroed accumulator and is added to the
// running sum with round-to-nearest FP32 adds; the two cross terms (2^-11 of
// it) may accumulate in the tensor core.
__device__ __forceinline__ void mma_big(float (&sum)[4], const unsigned (&ah)[4], const unsigned (&bh)[2]) {
    float d[4] = {0.f, 0.f, 0.f, 0.f};
    mma_tf32(d, ah, bh);
#pragma unroll
    for (int q = 0; q < 4; ++q) sum[q] += d[q];
}
__device__ __forceinline__ void mma_small(float (&cross)[4], const unsigned (&ah)[4], const unsigned (&al)[4],
                                          const unsigned (&bh)[2], const unsigned (&bl)[2]) {
    mma_tf32(cross, al, bh);
    mma_tf32(cross, ah, bl);
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Rows [i0, i0 + kCH) of the panel's columns k0 .. k0 + 31 of the split
// planes H (hi) and L (lo) of V_p, or of V_p T_p, into Vh / Vl ([column][row],
// swizzled). Columns past the last reflector (kk >= kb) and rows past ld are
// zero.
__device__ __forceinline__ void stage_chunk(const float* __restrict__ H, const float* __restrict__ L, int ld, int k0,
                                            int kb, int i0, float* __restrict__ Vh, float* __restrict__ Vl) {
#pragma unroll
    for (int u = 0; u < (kPanel * kCH / 4) / kTcThreads; ++u) {
        const int idx = threadIdx.x + kTcThreads * u;
        const int kk = idx / (kCH / 4), q = idx % (kCH / 4);
        const int o = kk * kCH + ((4 * q) ^ swz(kk));
        const int i = i0 + 4 * q;
        if (kk < kb && i < ld) {
            const size_t g = (size_t)(k0 + kk) * ld + i;
            cp_async16(Vh + o, H + g);
            cp_async16(Vl + o, L + g);
        } else {
            *reinterpret_cast<float4*>(Vh + o) = make_float4(0.f, 0.f, 0.f, 0.f);
            *reinterpret_cast<float4*>(Vl + o) = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
    cp_async_commit();
}

__global__ void __launch_bounds__(kTcThreads, 2)
backtransform_tc_kernel(const ChainDesc* __restrict__ descs, const float* __restrict__ VTs, long long plane,
                        float* __restrict__ Zws, const float* __restrict__ zscale, int shift) {
    extern __shared__ __align__(16) float smf[];
    // blockIdx.x walks the column blocks of one chain, so a chain's column
    // blocks are adjacent in launch order and run together: its V and V T
    // panels come from DRAM once and from L2 for the other column blocks
    const ChainDesc D = descs[blockIdx.y];
    const int n = D.n, ld = D.ld, j0 = blockIdx.x * kNC;
    if (j0 >= n) return;
    const float* VTh = VTs + D.a_off;      // split planes: V T hi, V T lo, V hi, V lo
    const float* VTl = VTh + plane;
    const float* Vh = VTl + plane;
    const float* Vl = Vh + plane;
    float* Z = Zws + D.a_off;
    float* Zt = smf;                       // [kNC][ld]: Zt[c * ld + (i ^ swz(c))] = Z(i, j0 + c)
    float* Vt = Zt + (size_t)kNC * ld;     // [2 buffers][hi, lo][kPanel][kCH]
    float* Wt = Vt + 4 * kPanel * kCH;     // [kNC][kTP] W^T
    float* red = Vt;                       // the partial-sum tree reuses the V buffers
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int g = lane >> 2, t = lane & 3;

    // Z block in, scaled to unit columns; zero outside the n x n matrix
    // (padding rows/columns hold no data)
    const float zs = (j0 + lane < n) ? zscale[D.v_off + j0 + lane] : 0.f;
    for (int i = warp; i < ld; i += kTcThreads / 32) {
        const float z = (i < n && j0 + lane < n) ? Z[(size_t)i * ld + j0 + lane] * zs : 0.f;
        Zt[lane * ld + (i ^ swz(lane))] = z;
    }
    const int nrefl = n - 1 - shift;  // reflector k: unit at row k + shift
    const int npanel = nrefl > 0 ? (nrefl + kPanel - 1) / kPanel : 0;
    const int mt3 = warp & 1;  // second GEMM: this warp's 16-column tile
    for (int p = npanel - 1; p >= 0; --p) {
        const int k0 = p * kPanel, kb = min(kPanel, nrefl - k0);
        __syncthreads();  // previous panel done with Vt and Zt

        // ---- W^T = Zb^T V_p: warp w takes rows i0 + 8w .. i0 + 8w + 7 of each chunk ----
        float acc[2][4][4], crs[2][4][4];
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b)
#pragma unroll
                for (int c = 0; c < 4; ++c) acc[a][b][c] = crs[a][b][c] = 0.f;
        stage_chunk(Vh, Vl, ld, k0, kb, k0, Vt, Vt + kPanel * kCH);
        int buf = 0;
        for (int i0 = k0; i0 < ld; i0 += kCH, buf ^= 1) {
            cp_async_wait_all();
            __syncthreads();
            const float* Vbh = Vt + buf * 2 * kPanel * kCH;
            const float* Vbl = Vbh + kPanel * kCH;
            if (i0 + kCH < ld) {
                float* nx = Vt + (buf ^ 1) * 2 * kPanel * kCH;
                stage_chunk(Vh, Vl, ld, k0, kb, i0 + kCH, nx, nx + kPanel * kCH);
            }
            const int r8 = i0 + 8 * warp, rr = 8 * warp;
            if (r8 < ld) {
                unsigned ah[2][4], al[2][4];
#pragma unroll
                for (int mt = 0; mt < 2; ++mt) {
                    const int c0 = mt * 16 + g, c1 = c0 + 8;
                    split_tf32(Zt[c0 * ld + ((r8 + t) ^ swz(c0))], ah[mt][0], al[mt][0]);
                    split_tf32(Zt[c1 * ld + ((r8 + t) ^ swz(c1))], ah[mt][1], al[mt][1]);
                    split_tf32(Zt[c0 * ld + ((r8 + t + 4) ^ swz(c0))], ah[mt][2], al[mt][2]);
                    split_tf32(Zt[c1 * ld + ((r8 + t + 4) ^ swz(c1))], ah[mt][3], al[mt][3]);
                }
#pragma unroll
                for (int nt = 0; nt < 4; ++nt) {
                    const int kk = nt * 8 + g;
                    const int o0 = kk * kCH + ((rr + t) ^ swz(kk)), o1 = kk * kCH + ((rr + t + 4) ^ swz(kk));
                    const unsigned bh[2] = {__float_as_uint(Vbh[o0]), __float_as_uint(Vbh[o1])};
                    const unsigned bl[2] = {__float_as_uint(Vbl[o0]), __float_as_uint(Vbl[o1])};
#pragma unroll
                    for (int mt = 0; mt < 2; ++mt) {
                        mma_small(crs[mt][nt], ah[mt], al[mt], bh, bl);
                        mma_big(acc[mt][nt], ah[mt], bh);
                    }
                }
            }
        }
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b)
#pragma unroll
                for (int c = 0; c < 4; ++c) acc[a][b][c] += crs[a][b][c];
        // ---- sum of the 8 partial W^T, fixed tree order, in fragment space ----
#pragma unroll
        for (int half = 4; half >= 1; half >>= 1) {
            __syncthreads();
            if (warp >= half && warp < 2 * half) {
                float* dst = red + (warp - half) * 1024 + lane;
#pragma unroll
                for (int a = 0; a < 2; ++a)
#pragma unroll
                    for (int b = 0; b < 4; ++b)
#pragma unroll
                        for (int c = 0; c < 4; ++c) dst[((a * 4 + b) * 4 + c) * 32] = acc[a][b][c];
            }
            __syncthreads();
            if (warp < half) {
                const float* src = red + warp * 1024 + lane;
#pragma unroll
                for (int a = 0; a < 2; ++a)
#pragma unroll
                    for (int b = 0; b < 4; ++b)
#pragma unroll
                        for (int c = 0; c < 4; ++c) acc[a][b][c] += src[((a * 4 + b) * 4 + c) * 32];
            }
        }
        if (warp == 0) {
            // accumulator (col mt*16 + g (+8), reflector nt*8 + 2t (+1))
#pragma unroll
            for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                for (int nt = 0; nt < 4; ++nt) {
                    const int c = mt * 16 + g, k = nt * 8 + 2 * t;
                    Wt[c * kTP + k] = acc[mt][nt][0];
                    Wt[c * kTP + k + 1] = acc[mt][nt][1];
                    Wt[(c + 8) * kTP + k] = acc[mt][nt][2];
                    Wt[(c + 8) * kTP + k + 1] = acc[mt][nt][3];
                }
        }
        __syncthreads();
        // ---- Zb^T -= W^T (V_p T_p)^T: warp w owns columns mt3*16.. and row tiles (w>>1), (w>>1)+4 of each chunk ----
        unsigned wh[4][4], wl[4][4];  // -W^T, split
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {
            const int c0 = mt3 * 16 + g, k1 = ks * 8 + t;
            split_tf32(-Wt[c0 * kTP + k1], wh[ks][0], wl[ks][0]);
            split_tf32(-Wt[(c0 + 8) * kTP + k1], wh[ks][1], wl[ks][1]);
            split_tf32(-Wt[c0 * kTP + k1 + 4], wh[ks][2], wl[ks][2]);
            split_tf32(-Wt[(c0 + 8) * kTP + k1 + 4], wh[ks][3], wl[ks][3]);
        }
        stage_chunk(VTh, VTl, ld, k0, kb, k0, Vt, Vt + kPanel * kCH);
        buf = 0;
        for (int i0 = k0; i0 < ld; i0 += kCH, buf ^= 1) {
            cp_async_wait_all();
            __syncthreads();
            const float* Vbh = Vt + buf * 2 * kPanel * kCH;
            const float* Vbl = Vbh + kPanel * kCH;
            if (i0 + kCH < ld) {
                float* nx = Vt + (buf ^ 1) * 2 * kPanel * kCH;
                stage_chunk(VTh, VTl, ld, k0, kb, i0 + kCH, nx, nx + kPanel * kCH);
            }
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int nt = (warp >> 1) + 4 * h;
                const int rowb = i0 + nt * 8, rr = nt * 8;
                if (rowb >= ld) continue;
                const int cA = mt3 * 16 + g, cB = cA + 8;
                float2* pA = reinterpret_cast<float2*>(Zt + cA * ld + ((rowb + 2 * t) ^ swz(cA)));
                float2* pB = reinterpret_cast<float2*>(Zt + cB * ld + ((rowb + 2 * t) ^ swz(cB)));
                // the update u = -W^T (V T)^T of this tile, summed apart from Zb
                float u[4] = {0.f, 0.f, 0.f, 0.f}, uc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
                for (int ks = 0; ks < 4; ++ks) {
                    const int k1 = ks * 8 + t, k2 = k1 + 4;
                    const int o1 = k1 * kCH + ((rr + g) ^ swz(k1)), o2 = k2 * kCH + ((rr + g) ^ swz(k2));
                    const unsigned bh[2] = {__float_as_uint(Vbh[o1]), __float_as_uint(Vbh[o2])};
                    const unsigned bl[2] = {__float_as_uint(Vbl[o1]), __float_as_uint(Vbl[o2])};
                    mma_small(uc, wh[ks], wl[ks], bh, bl);
                    mma_big(u, wh[ks], bh);
                }
                const float2 xa = *pA, xb = *pB;
                *pA = make_float2(xa.x + (u[0] + uc[0]), xa.y + (u[1] + uc[1]));
                *pB = make_float2(xb.x + (u[2] + uc[2]), xb.y + (u[3] + uc[3]));
            }
        }
    }
    __syncthreads();
    if (j0 + lane < n)
        for (int i = warp; i < n; i += kTcThreads / 32) Z[(size_t)i * ld + j0 + lane] = Zt[lane * ld + (i ^ swz(lane))];
}

}  // namespace

size_t backtransform_tc_smem_bytes(int max_ld) {
    return sizeof(float) * ((size_t)kNC * max_ld + 4 * kPanel * kCH + (size_t)kNC * kTP);
}

cudaError_t launch_backtransform_tc(const ChainDesc* d_desc, int batch, int max_n, int max_ld, const float* d_VT,
                                    long long plane, float* d_Z, const float* d_zscale, int shift, cudaStream_t st) {
    if (batch <= 0) return cudaSuccess;
    if (batch > 65535) return cudaErrorInvalidValue;  // grid y limit
    const size_t smem = backtransform_tc_smem_bytes(max_ld);
    cudaError_t err = cudaFuncSetAttribute(backtransform_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    backtransform_tc_kernel<<<dim3((max_n + kNC - 1) / kNC, batch), kTcThreads, smem, st>>>(d_desc, d_VT, plane, d_Z,
                                                                                                d_zscale, shift);
    return cudaGetLastError();
}

}  // namespace fkg
