// sytrd.cu — Householder tridiagonalisation, one CTA per chain, in FP64 (the
// plain path) or FP32 (the mixed path).
//
// Replaces the first half of Eigen::SelfAdjointEigenSolver at
// src/configuration.cpp:213 (with the sparse->dense copy of :212 and the
// Hamiltonian build of :79-91 fused into the matrix load).
//
// Outputs: the diagonal d and off-diagonal e of T (always stored as FP64, the
// tridiagonal eigen-solve runs in FP64), tau_k, and the Householder vectors
// v_k in A(k+2:, k) (v_k(k+1) = 1 implicit) for the back-transformation.
//
// Roofline (FP64 variant): on GB300 the FP64 pipe (about 1.2 TFLOP/s for the whole GPU, two
// DFMA per clock per SM) is far below what HBM can feed, so this kernel is
// FP64-compute bound. The algorithm does the minimum FP64 work of an
// unblocked symmetric reduction, 4/3 n^3 flops: per reflector one symmetric
// matrix-vector product on the lower triangle (2 DFMA per stored element) and
// one symmetric rank-2 update of the lower triangle (2 DFMA per element).
//
// Work split: the trailing matrix is cut on a fixed grid of 32 x 32 tiles;
// the lower tiles are dealt to the 8 warps round robin. In the matrix-vector
// pass a warp loads its tile with coalesced column reads (lane = row), forms
// the row sums in registers and the column sums from a padded shared-memory
// copy of the tile (lane = column), and adds both into a private per-warp
// partial vector; the partial vectors are summed after the pass, so no
// atomics are needed and the result is deterministic.
#include "fkg_common.cuh"

namespace fkg {
namespace {

constexpr int kWarps = 8;
constexpr int kThreads = kWarps * 32;
constexpr int kPad = kTile + 1;

__device__ __forceinline__ size_t aidx(int i, int j, int ld) { return (size_t)j * ld + i; }

template <typename T>
__global__ void __launch_bounds__(kThreads, 1)
sytrd_kernel(const ChainDesc* __restrict__ descs, const double* __restrict__ diag, T* __restrict__ Aws,
             double* __restrict__ dout, double* __restrict__ eout, T* __restrict__ tauout) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* smem = reinterpret_cast<T*>(smem_raw);
    const ChainDesc D = descs[blockIdx.x];
    const int n = D.n, ld = D.ld;
    T* __restrict__ A = Aws + D.a_off;
    T* v = smem;                    // [ld]  Householder vector (0 outside [s, n))
    T* w = v + ld;                  // [ld]  w = p - K v
    T* pw = w + ld;                 // [kWarps][ld] per-warp partial products
    T* tile = pw + kWarps * ld;     // [kWarps][32*33]
    T* red = tile + kWarps * kTile * kPad;  // [kWarps]
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    T* mytile = tile + warp * kTile * kPad;
    T* mypw = pw + warp * ld;

    // ---- build the lower triangle of H = hopping + diag(-mu_c + U f) ----
    for (long long t = tid; t < (long long)n * ld; t += kThreads) {
        int i = (int)(t % ld), j = (int)(t / ld);
        if (i >= j && i < n) A[aidx(i, j, ld)] = T(0);
    }
    __syncthreads();
    for (int i = tid; i < n; i += kThreads) {
        for (int p = D.rowptr[i]; p < D.rowptr[i + 1]; ++p) {
            int j = D.col[p];
            if (j <= i) A[aidx(i, j, ld)] += T(D.val[p]);
        }
        A[aidx(i, i, ld)] += T(diag[D.v_off + i]);
    }
    for (int i = tid; i < ld; i += kThreads) { v[i] = T(0); w[i] = T(0); }
    __syncthreads();

    const int nt = (n + kTile - 1) / kTile;
    for (int k = 0; k + 2 < n; ++k) {
        const int s = k + 1;
        T* colk = A + (size_t)k * ld;
        // ---- reflector H_k = I - tau v v^T annihilating A(s+1:, k) ----
        T part = T(0);
        for (int i = s + 1 + tid; i < n; i += kThreads) { T x = colk[i]; part += x * x; }
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
            tauout[D.v_off + k] = tau;
        }
        if (tau == T(0)) {
            __syncthreads();
            continue;
        }
        for (int i = tid; i < n; i += kThreads) {
            T vi = T(0);
            if (i == s) vi = T(1);
            else if (i > s) { vi = colk[i] * scale; colk[i] = vi; }  // keep v for the back-transform
            v[i] = vi;
        }
        for (int t = tid; t < kWarps * ld; t += kThreads) pw[t] = T(0);
        __syncthreads();

        // ---- p = A22 v over the lower tiles of A(s:n, s:n) ----
        const int I0 = s / kTile;
        int cnt = 0;
        for (int I = I0; I < nt; ++I) {
            for (int J = I0; J <= I; ++J, ++cnt) {
                if ((cnt % kWarps) != warp) continue;
                const int i = I * kTile + lane;
                const bool diag_tile = (I == J);
                const bool row_ok = (i < n) && (i >= s);
                T rs = T(0);
#pragma unroll 8
                for (int c = 0; c < kTile; ++c) {
                    const int j = J * kTile + c;
                    T a = T(0);
                    if (row_ok && j < n && j >= s && (!diag_tile || i >= j)) a = A[aidx(i, j, ld)];
                    rs = fma(a, v[j], rs);
                    mytile[c * kPad + lane] = (diag_tile && i == j) ? T(0) : a;
                }
                __syncwarp();
                T cs = T(0);
#pragma unroll 8
                for (int r = 0; r < kTile; ++r) {
                    const int ii = I * kTile + r;
                    cs = fma(mytile[lane * kPad + r], v[ii], cs);
                }
                mypw[i] += rs;  // i, j < nt*32 <= ld
                mypw[J * kTile + lane] += cs;
                __syncwarp();
            }
        }
        __syncthreads();

        // ---- w = tau p - (tau/2)(tau p . v) v ----
        part = T(0);
        for (int i = s + tid; i < n; i += kThreads) {
            T p = T(0);
#pragma unroll
            for (int q = 0; q < kWarps; ++q) p += pw[q * ld + i];
            p *= tau;
            w[i] = p;
            part += p * v[i];
        }
        const T pv = block_sum(part, red);
        const T K = T(0.5) * tau * pv;
        for (int i = s + tid; i < n; i += kThreads) w[i] -= K * v[i];
        __syncthreads();

        // ---- A22 -= v w^T + w v^T on the lower tiles ----
        cnt = 0;
        for (int I = I0; I < nt; ++I) {
            for (int J = I0; J <= I; ++J, ++cnt) {
                if ((cnt % kWarps) != warp) continue;
                const int i = I * kTile + lane;
                if (i >= n || i < s) continue;
                const T vi = v[i], wi = w[i];
                const bool diag_tile = (I == J);
#pragma unroll 8
                for (int c = 0; c < kTile; ++c) {
                    const int j = J * kTile + c;
                    if (j < n && j >= s && (!diag_tile || i >= j)) {
                        T a = A[aidx(i, j, ld)];
                        a = fma(-vi, w[j], a);
                        a = fma(-wi, v[j], a);
                        A[aidx(i, j, ld)] = a;
                    }
                }
            }
        }
        __syncthreads();
    }
    // ---- diagonal and last off-diagonal ----
    for (int i = tid; i < n; i += kThreads) dout[D.v_off + i] = (double)A[aidx(i, i, ld)];
    if (tid == 0 && n >= 2) {
        eout[D.v_off + n - 2] = (double)A[aidx(n - 1, n - 2, ld)];
        tauout[D.v_off + n - 2] = T(0);
    }
}

template <typename T>
cudaError_t launch_sytrd_t(const ChainDesc* d_desc, int batch, int max_ld, const double* d_diag, T* d_A,
                           double* d_d, double* d_e, T* d_tau, cudaStream_t st) {
    if (batch <= 0) return cudaSuccess;
    const size_t smem = sizeof(T) * ((size_t)(2 + kWarps) * max_ld + kWarps * kTile * kPad + kWarps);
    cudaError_t err = cudaFuncSetAttribute(sytrd_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    sytrd_kernel<T><<<batch, kThreads, smem, st>>>(d_desc, d_diag, d_A, d_d, d_e, d_tau);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_sytrd_f64(const ChainDesc* d_desc, int batch, int max_ld, const double* d_diag, double* d_A,
                             double* d_d, double* d_e, double* d_tau, cudaStream_t st) {
    return launch_sytrd_t<double>(d_desc, batch, max_ld, d_diag, d_A, d_d, d_e, d_tau, st);
}

cudaError_t launch_sytrd_f32(const ChainDesc* d_desc, int batch, int max_ld, const double* d_diag, float* d_A,
                             double* d_d, double* d_e, float* d_tau, cudaStream_t st) {
    return launch_sytrd_t<float>(d_desc, batch, max_ld, d_diag, d_A, d_d, d_e, d_tau, st);
}

}  // namespace fkg
