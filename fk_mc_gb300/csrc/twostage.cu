// twostage.cu — the band stage of the two-stage tridiagonalisation of the
// mixed path (FP32): band (bandwidth kBand) -> tridiagonal, and its part of
// the back-transformation. The first stage (dense -> band) is sy2sb.cu.
//
// Replaces, with sy2sb.cu, the first half of Eigen::SelfAdjointEigenSolver at
// src/configuration.cpp:213. The one-stage reduction (sytrd_v3.cu) reads the
// whole trailing matrix for every column (a matrix-vector product per
// reflector); the two-stage reduction passes over it once per panel of kBand
// columns on the tensor cores and leaves O(b n^2) work to the band stage:
//
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

namespace fkg {
namespace {

constexpr int kB = kBand;          // bandwidth between the stages
constexpr int kLdb = 2 * kB + 2;   // band storage per column (even: conflict-free rows)
constexpr int kS2Warps = 16;      // tasks of one wavefront step run at once (about n / (3 b))
constexpr int kQ2Thr = 32;         // threads per CTA of the stage-2 back-transformation
constexpr int kQ2Cols = 2 * kQ2Thr;  // columns of Z per CTA (two per thread)

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
