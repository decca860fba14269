// grad.cu — derivatives of the free energy F = -logZ / beta of one
// configuration (the quantity calc_ed caches as logZ, src/configuration.cpp:244)
// with respect to H and to the model parameters.
//
// dF/dH = rho = V diag(f) V^T, f_k = 1 / (1 + exp(beta eps_k)) (the Fermi
// factors, ed_cache::cached_fermi). With H = hopping(t) + diag(U n_f - mu_c)
// and the hopping linear in t:
//   dF/dU    = sum_i n_f(i) rho_ii
//   dF/dmu   = -sum_i rho_ii = -sum_k f_k
//   dF/dt    = tr(rho hopping) / t = (E_c - U dF/dU - mu dF/dmu) / t,  E_c = sum_k f_k eps_k
//   dF/dbeta = (E_c - F) / beta      (at fixed H)
// so only the diagonal of rho needs the eigenvectors; the full rho
// (optional) is the weighted Gram matrix X diag(f) X^T.
#include "fkg_common.cuh"

namespace fkg {
namespace {

constexpr int kThreads = 256;

// One CTA per chain. X row-major (X[i*ld + k] = component i of eigenvector k),
// eps[k] the eigenvalue paired with column k.
template <typename T>
__global__ void __launch_bounds__(kThreads)
grad_kernel(const ChainDesc* __restrict__ descs, const T* __restrict__ Xws, const double* __restrict__ eps,
            const int32_t* __restrict__ f, const double* __restrict__ U, const double* __restrict__ mu,
            const double* __restrict__ t, const double* __restrict__ beta, double* __restrict__ out /*[batch][5]*/,
            double* __restrict__ fermi_ws) {
    const ChainDesc D = descs[blockIdx.x];
    const int n = D.n, ld = D.ld, c = blockIdx.x;
    const T* X = Xws + D.a_off;
    const double b = beta[c];
    double* fk = fermi_ws + D.v_off;
    __shared__ double red[6][kThreads / 32];
    // Fermi factors, E_c, sum f, logZ (Neumaier-compensated)
    double ec = 0.0, sf = 0.0, lz = 0.0, lzc = 0.0;
    for (int k = threadIdx.x; k < n; k += kThreads) {
        const double e = eps[D.v_off + k];
        const double fe = 1.0 / (1.0 + exp(b * e));
        fk[k] = fe;
        ec += fe * e;
        sf += fe;
        const double x = -b * e, term = fmax(x, 0.0) + log1p(exp(-fabs(x)));
        const double tt = lz + term;
        lzc += fabs(lz) >= fabs(term) ? (lz - tt) + term : (term - tt) + lz;
        lz = tt;
    }
    __syncthreads();
    // dF/dU = sum_i n_f(i) rho_ii, one warp per row i (coalesced row of X)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double du = 0.0;
    for (int i = warp; i < n; i += kThreads / 32) {
        if (!f[D.v_off + i]) continue;
        double r = 0.0;
        for (int k = lane; k < n; k += 32) {
            const double x = (double)X[(size_t)i * ld + k];
            r += fk[k] * x * x;
        }
        du += warp_sum(r);
    }
    ec = warp_sum(ec); sf = warp_sum(sf); lz = warp_sum(lz); lzc = warp_sum(lzc);
    if (lane == 0) {
        red[0][warp] = ec; red[1][warp] = sf; red[2][warp] = lz; red[3][warp] = lzc; red[4][warp] = du;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double E = 0, S = 0, Z = 0, Zc = 0, DU = 0;
        for (int q = 0; q < kThreads / 32; ++q) { E += red[0][q]; S += red[1][q]; Z += red[2][q]; Zc += red[3][q]; DU += red[4][q]; }
        const double logz = Z + Zc, F = -logz / b;
        const double dmu = -S;
        double* o = out + 5 * (size_t)c;
        o[0] = F;
        o[1] = DU;
        o[2] = (E - U[c] * DU - mu[c] * dmu) / t[c];
        o[3] = dmu;
        o[4] = (E - F) / b;
    }
}

// rho = X diag(f) X^T (full density matrix), 32 x 32 output tiles per CTA.
template <typename T>
__global__ void __launch_bounds__(256)
rho_kernel(const ChainDesc* __restrict__ descs, const T* __restrict__ Xws, const double* __restrict__ fermi_ws,
           double* __restrict__ rho_ws) {
    const ChainDesc D = descs[blockIdx.x];
    const int n = D.n, ld = D.ld;
    const int ti = blockIdx.y / ((n + 31) / 32), tj = blockIdx.y % ((n + 31) / 32);
    if (ti * 32 >= n) return;
    const T* X = Xws + D.a_off;
    const double* fk = fermi_ws + D.v_off;
    __shared__ double Xi[32][33], Xj[32][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 8 rows of 4 outputs each
    double acc[4] = {0, 0, 0, 0};
    for (int k0 = 0; k0 < n; k0 += 32) {
        for (int q = ty; q < 32; q += 8) {
            const int ri = ti * 32 + q, rj = tj * 32 + q, k = k0 + tx;
            Xi[q][tx] = (ri < n && k < n) ? (double)X[(size_t)ri * ld + k] * fk[k] : 0.0;
            Xj[q][tx] = (rj < n && k < n) ? (double)X[(size_t)rj * ld + k] : 0.0;
        }
        __syncthreads();
        for (int k = 0; k < 32; ++k)
#pragma unroll
            for (int u = 0; u < 4; ++u) acc[u] = fma(Xi[ty + 8 * u][k], Xj[tx][k], acc[u]);
        __syncthreads();
    }
    double* R = rho_ws + D.a_off;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int i = ti * 32 + ty + 8 * u, j = tj * 32 + tx;
        if (i < n && j < n) R[(size_t)j * ld + i] = acc[u];  // column-major
    }
}

}  // namespace

cudaError_t launch_grad(const ChainDesc* d_desc, int batch, bool fp32, const void* d_X, const double* d_eps,
                        const int32_t* d_f, const double* d_U, const double* d_mu, const double* d_t,
                        const double* d_beta, double* d_out, double* d_fermi, cudaStream_t st) {
    if (batch <= 0) return cudaSuccess;
    if (fp32)
        grad_kernel<float><<<batch, kThreads, 0, st>>>(d_desc, (const float*)d_X, d_eps, d_f, d_U, d_mu, d_t, d_beta,
                                                       d_out, d_fermi);
    else
        grad_kernel<double><<<batch, kThreads, 0, st>>>(d_desc, (const double*)d_X, d_eps, d_f, d_U, d_mu, d_t,
                                                        d_beta, d_out, d_fermi);
    return cudaGetLastError();
}

cudaError_t launch_rho(const ChainDesc* d_desc, int batch, int max_n, bool fp32, const void* d_X,
                       const double* d_fermi, double* d_rho, cudaStream_t st) {
    if (batch <= 0) return cudaSuccess;
    const int nt = (max_n + 31) / 32;
    dim3 grid(batch, nt * nt);
    if (fp32) rho_kernel<float><<<grid, 256, 0, st>>>(d_desc, (const float*)d_X, d_fermi, d_rho);
    else rho_kernel<double><<<grid, 256, 0, st>>>(d_desc, (const double*)d_X, d_fermi, d_rho);
    return cudaGetLastError();
}

}  // namespace fkg
