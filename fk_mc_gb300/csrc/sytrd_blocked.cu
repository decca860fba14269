// sytrd_blocked.cu — blocked Householder tridiagonalisation (panel of NB
// reflectors, deferred symmetric rank-2k update), one CTA per chain.
//
// Same result as the unblocked reduction of sytrd.cu (it replaces the first
// half of Eigen::SelfAdjointEigenSolver at src/configuration.cpp:213, with the
// Hamiltonian build of :79-91 and the dense copy of :212 fused into the
// matrix load), with far less memory traffic:
//   * within a panel the trailing matrix is only READ, once per column, by
//     the symmetric matrix-vector product, and the product is corrected for
//     the panel's pending updates:  p = A v - V (W^T v) - W (V^T v);
//   * the column about to be reduced gets the pending updates applied first;
//   * after NB columns one symmetric rank-2k update A -= V W^T + W V^T
//     rewrites the trailing lower triangle.
// Per column this moves about one pass over the trailing lower triangle
// (plus 2/NB for the rank-2k update) instead of the unblocked three.
// The matrix-vector tiles issue all 32 column loads of a tile before using
// them (memory-level parallelism), and 16 warps (FP32) or 8 warps (FP64) keep
// the loads in flight. W (n x NB per chain) lives in a global scratch buffer.
#include "fkg_common.cuh"

namespace fkg {
namespace {

constexpr int kPad = kTile + 1;

template <typename T> struct BlkCfg;
template <> struct BlkCfg<float> { static constexpr int NB = 32, WARPS = 16; };
template <> struct BlkCfg<double> { static constexpr int NB = 16, WARPS = 8; };

template <typename T>
__device__ __forceinline__ T vget(const T* __restrict__ A, int ld, int n, int k, int i) {
    if (i == k + 1) return T(1);
    if (i > k + 1 && i < n) return A[(size_t)k * ld + i];
    return T(0);
}

template <typename T>
__global__ void __launch_bounds__(BlkCfg<T>::WARPS * 32, 1)
sytrd_blk_kernel(const ChainDesc* __restrict__ descs, const double* __restrict__ diag, T* __restrict__ Aws,
                 T* __restrict__ Wws, double* __restrict__ dout, double* __restrict__ eout, T* __restrict__ tauout) {
    constexpr int NB = BlkCfg<T>::NB, WARPS = BlkCfg<T>::WARPS, NT = WARPS * 32;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sm = reinterpret_cast<T*>(smem_raw);
    const ChainDesc D = descs[blockIdx.x];
    const int n = D.n, ld = D.ld;
    T* __restrict__ A = Aws + D.a_off;
    T* __restrict__ W = Wws + D.v_off * NB;  // W_l(i) at W[l*ld + i]
    T* v = sm;                                // [ld]
    T* p = v + ld;                            // [ld]
    T* pw = p + ld;                           // [WARPS][ld]
    T* stage = pw + (size_t)WARPS * ld;       // [WARPS][2][32][kPad]
    T* c1 = stage + (size_t)WARPS * 2 * kTile * kPad;  // [NB]  W^T v
    T* c2 = c1 + NB;                                   // [NB]  V^T v
    T* vk = c2 + NB;                                   // [NB]
    T* wk = vk + NB;                                   // [NB]
    T* red = wk + NB;                                  // [WARPS]
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    T* mytile = stage + (size_t)warp * 2 * kTile * kPad;
    T* mypw = pw + (size_t)warp * ld;

    // ---- build the lower triangle of H = hopping + diag(-mu_c + U f) ----
    for (long long t = tid; t < (long long)n * ld; t += NT) {
        const int i = (int)(t % ld), j = (int)(t / ld);
        if (i >= j && i < n) A[(size_t)j * ld + i] = T(0);
    }
    __syncthreads();
    for (int i = tid; i < n; i += NT) {
        for (int q = D.rowptr[i]; q < D.rowptr[i + 1]; ++q) {
            const int j = D.col[q];
            if (j <= i) A[(size_t)j * ld + i] += T(D.val[q]);
        }
        A[(size_t)i * ld + i] += T(diag[D.v_off + i]);
    }
    for (int i = tid; i < ld; i += NT) { v[i] = T(0); p[i] = T(0); }
    __syncthreads();

    const int nt = (n + kTile - 1) / kTile;
    for (int k0 = 0; k0 < n - 2; k0 += NB) {
        const int nbk = min(NB, n - 2 - k0);
        for (int j = 0; j < nbk; ++j) {
            const int k = k0 + j, s = k + 1;
            T* colk = A + (size_t)k * ld;
            // ---- (1) pending updates of this panel on column k (rows k..n-1) ----
            if (tid < j) { vk[tid] = vget(A, ld, n, k0 + tid, k); wk[tid] = W[(size_t)tid * ld + k]; }
            __syncthreads();
            if (j > 0)
                for (int i = k + tid; i < n; i += NT) {
                    T a = colk[i];
                    for (int l = 0; l < j; ++l)
                        a -= vget(A, ld, n, k0 + l, i) * wk[l] + W[(size_t)l * ld + i] * vk[l];
                    colk[i] = a;
                }
            __syncthreads();
            // ---- (2) reflector from A(s:, k) ----
            T part = T(0);
            for (int i = s + 1 + tid; i < n; i += NT) { const T x = colk[i]; part += x * x; }
            const T sigma = block_sum(part, red);
            const T alpha = colk[s];
            T tau = T(0), beta = alpha, scale = T(0);
            if (sigma != T(0)) {
                const T xnorm = sqrt(alpha * alpha + sigma);
                beta = alpha >= T(0) ? -xnorm : xnorm;
                tau = (beta - alpha) / beta;
                scale = T(1) / (alpha - beta);
            }
            if (tid == 0) {
                eout[D.v_off + k] = (double)beta;
                dout[D.v_off + k] = (double)colk[k];
                tauout[D.v_off + k] = tau;
            }
            for (int i = tid; i < n; i += NT) {
                T vi = T(0);
                if (i == s) vi = T(1);
                else if (i > s) { vi = colk[i] * scale; colk[i] = vi; }
                v[i] = vi;
            }
            for (int t = tid; t < WARPS * ld; t += NT) pw[t] = T(0);
            __syncthreads();
            if (tau == T(0)) {
                for (int i = tid; i < ld; i += NT) W[(size_t)j * ld + i] = T(0);
                __syncthreads();
                continue;
            }
            // ---- (3a) p = A22 v with the stale trailing matrix (lower tiles) ----
            const int I0 = s / kTile;
            int cnt = 0;
            for (int I = I0; I < nt; ++I) {
                for (int J = I0; J <= I; ++J, ++cnt) {
                    if ((cnt % WARPS) != warp) continue;
                    const int i = I * kTile + lane;
                    const bool dg = (I == J);
                    const bool row_ok = (i < n) && (i >= s);
                    T a[kTile];
#pragma unroll
                    for (int c = 0; c < kTile; ++c) {
                        const int jj = J * kTile + c;
                        a[c] = (row_ok && jj < n && jj >= s && (!dg || i >= jj)) ? A[(size_t)jj * ld + i] : T(0);
                    }
                    T rs0 = T(0), rs1 = T(0), rs2 = T(0), rs3 = T(0);  // independent chains
#pragma unroll
                    for (int c = 0; c < kTile; c += 4) {
                        rs0 += a[c] * v[J * kTile + c];
                        rs1 += a[c + 1] * v[J * kTile + c + 1];
                        rs2 += a[c + 2] * v[J * kTile + c + 2];
                        rs3 += a[c + 3] * v[J * kTile + c + 3];
                    }
#pragma unroll
                    for (int c = 0; c < kTile; ++c) mytile[c * kPad + lane] = (dg && c == lane) ? T(0) : a[c];
                    const T rs = (rs0 + rs1) + (rs2 + rs3);
                    __syncwarp();
                    T cs0 = T(0), cs1 = T(0), cs2 = T(0), cs3 = T(0);
#pragma unroll
                    for (int r = 0; r < kTile; r += 4) {
                        cs0 += mytile[lane * kPad + r] * v[I * kTile + r];
                        cs1 += mytile[lane * kPad + r + 1] * v[I * kTile + r + 1];
                        cs2 += mytile[lane * kPad + r + 2] * v[I * kTile + r + 2];
                        cs3 += mytile[lane * kPad + r + 3] * v[I * kTile + r + 3];
                    }
                    const T cs = (cs0 + cs1) + (cs2 + cs3);
                    mypw[i] += rs;
                    mypw[J * kTile + lane] += cs;
                    __syncwarp();
                }
            }
            // ---- (3b) c1 = W^T v, c2 = V^T v over the panel's previous reflectors ----
            for (int l = warp; l < j; l += WARPS) {
                T s1 = T(0), s2 = T(0);
                for (int i = s + lane; i < n; i += 32) {
                    s1 += W[(size_t)l * ld + i] * v[i];
                    s2 += vget(A, ld, n, k0 + l, i) * v[i];
                }
                s1 = warp_sum(s1);
                s2 = warp_sum(s2);
                if (lane == 0) { c1[l] = s1; c2[l] = s2; }
            }
            __syncthreads();
            // ---- (3c)+(4) w = tau p - (tau/2)(tau p.v) v, p corrected for the pending updates ----
            part = T(0);
            for (int i = s + tid; i < n; i += NT) {
                T q = T(0);
#pragma unroll
                for (int w8 = 0; w8 < WARPS; ++w8) q += pw[(size_t)w8 * ld + i];
                for (int l = 0; l < j; ++l) q -= vget(A, ld, n, k0 + l, i) * c1[l] + W[(size_t)l * ld + i] * c2[l];
                q *= tau;
                p[i] = q;
                part += q * v[i];
            }
            const T pv = block_sum(part, red);
            const T K = T(0.5) * tau * pv;
            for (int i = tid; i < ld; i += NT) W[(size_t)j * ld + i] = (i >= s && i < n) ? p[i] - K * v[i] : T(0);
            __syncthreads();
        }
        // ---- (5) A(tb:, tb:) -= V W^T + W V^T on the lower tiles, tb = k0 + nbk ----
        const int tb = k0 + nbk;
        const int I0 = tb / kTile;
        T* VJs = mytile;                 // [32][kPad]: VJs[c][l] = V_l(32J + c)
        T* WJs = mytile + kTile * kPad;  // [32][kPad]
        int cnt = 0;
        for (int I = I0; I < nt; ++I) {
            for (int J = I0; J <= I; ++J, ++cnt) {
                if ((cnt % WARPS) != warp) continue;
                const int i = I * kTile + lane;
                const bool dg = (I == J);
                // stage V_l, W_l at the tile's columns (lane = column)
                const int jc = J * kTile + lane;
                for (int l = 0; l < NB; ++l) {
                    VJs[lane * kPad + l] = l < nbk ? vget(A, ld, n, k0 + l, jc) : T(0);
                    WJs[lane * kPad + l] = (l < nbk && jc < n) ? W[(size_t)l * ld + jc] : T(0);
                }
                T VI[NB], WI[NB];
#pragma unroll
                for (int l = 0; l < NB; ++l) {
                    VI[l] = l < nbk ? vget(A, ld, n, k0 + l, i) : T(0);
                    WI[l] = (l < nbk && i < n) ? W[(size_t)l * ld + i] : T(0);
                }
                __syncwarp();
                if (i < n && i >= tb) {
                    // four columns at a time: independent accumulation chains
                    for (int c = 0; c < kTile; c += 4) {
                        T acc[4];
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            const int jj = J * kTile + c + q;
                            acc[q] = (jj < n && jj >= tb && !(dg && i < jj)) ? A[(size_t)jj * ld + i] : T(0);
                        }
#pragma unroll
                        for (int l = 0; l < NB; ++l) {
#pragma unroll
                            for (int q = 0; q < 4; ++q)
                                acc[q] -= VI[l] * WJs[(c + q) * kPad + l] + WI[l] * VJs[(c + q) * kPad + l];
                        }
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            const int jj = J * kTile + c + q;
                            if (jj < n && jj >= tb && !(dg && i < jj)) A[(size_t)jj * ld + i] = acc[q];
                        }
                    }
                }
                __syncwarp();
            }
        }
        __syncthreads();
    }
    // ---- the trailing 2 x 2 block ----
    if (tid == 0 && n >= 2) {
        dout[D.v_off + n - 2] = (double)A[(size_t)(n - 2) * ld + n - 2];
        eout[D.v_off + n - 2] = (double)A[(size_t)(n - 2) * ld + n - 1];
        tauout[D.v_off + n - 2] = T(0);
    }
    if (tid == 0) dout[D.v_off + n - 1] = (double)A[(size_t)(n - 1) * ld + n - 1];
}

template <typename T>
size_t blk_smem(int max_ld) {
    constexpr int NB = BlkCfg<T>::NB, WARPS = BlkCfg<T>::WARPS;
    return sizeof(T) * ((size_t)(2 + WARPS) * max_ld + (size_t)WARPS * 2 * kTile * kPad + 4 * NB + WARPS);
}

template <typename T>
cudaError_t launch_blk(const ChainDesc* d_desc, int batch, int max_ld, const double* d_diag, T* d_A, T* d_W,
                       double* d_d, double* d_e, T* d_tau, cudaStream_t st) {
    if (batch <= 0) return cudaSuccess;
    const size_t smem = blk_smem<T>(max_ld);
    cudaError_t err = cudaFuncSetAttribute(sytrd_blk_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    sytrd_blk_kernel<T><<<batch, BlkCfg<T>::WARPS * 32, smem, st>>>(d_desc, d_diag, d_A, d_W, d_d, d_e, d_tau);
    return cudaGetLastError();
}

}  // namespace

size_t sytrd_blk_scratch_elems(int v_total, bool fp32) {
    return (size_t)v_total * (fp32 ? BlkCfg<float>::NB : BlkCfg<double>::NB);
}

cudaError_t launch_sytrd_blk_f64(const ChainDesc* d_desc, int batch, int max_ld, const double* d_diag, double* d_A,
                                 double* d_W, double* d_d, double* d_e, double* d_tau, cudaStream_t st) {
    return launch_blk<double>(d_desc, batch, max_ld, d_diag, d_A, d_W, d_d, d_e, d_tau, st);
}

cudaError_t launch_sytrd_blk_f32(const ChainDesc* d_desc, int batch, int max_ld, const double* d_diag, float* d_A,
                                 float* d_W, double* d_d, double* d_e, float* d_tau, cudaStream_t st) {
    return launch_blk<float>(d_desc, batch, max_ld, d_diag, d_A, d_W, d_d, d_e, d_tau, st);
}

}  // namespace fkg
