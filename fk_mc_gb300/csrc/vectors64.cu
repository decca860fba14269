// vectors64.cu — FP64 eigenvectors of the tridiagonal T for the plain path's
// calc_ed(true) (src/configuration.cpp:216-219: cached_evecs, used by
// measure_ipr, measure_stiffness and measure_eigenfunctions) and for the
// FP64 free-energy gradient.
//
// Inverse iteration: for eigenvalue lambda_j, Gaussian elimination with row
// interchanges factors T - lambda_j I = P L U (U has three diagonals), and
// three solves U^{-1} L^{-1} P^T x from a fixed start vector converge to the
// eigenvector. Eigenvalues closer than 1e-5 ||T|| form a cluster: one thread
// computes the cluster's vectors in order and orthogonalises each iterate
// against the cluster's earlier vectors (modified Gram-Schmidt), so exactly
// degenerate eigenvalues (the U = 0 lattices) still get an orthonormal basis.
// Vectors outside a cluster are orthogonal to about eps ||T|| / gap < 1e-11.
// Output row-major Z[i*ld + j] = component i of eigenvector j.
#include <cfloat>

#include "fkg_common.cuh"

namespace fkg {
namespace {

constexpr int kThreads = 128;

struct LU {
    double* r0;   // reciprocals of the diagonal of U
    double* u1;   // first superdiagonal of U
    double* u2;   // second superdiagonal of U (fill-in from interchanges)
    double* m;    // multipliers of L
    int* piv;     // 1 where rows i and i+1 were interchanged
};

// The pivots are kept as reciprocals: one FP64 division per elimination step
// serves the multiplier and the three back substitutions, which then only
// multiply (a division is a long dependent sequence on the FP64 pipe; the
// solves are chains of n dependent steps). A pivot below pivmin is replaced by
// +-pivmin before its reciprocal is taken.
__device__ void factor(const double* d, const double* e, int n, double lam, double pivmin, LU f) {
    auto guard = [&](double x) { return fabs(x) < pivmin ? (x < 0.0 ? -pivmin : pivmin) : x; };
    double cd = d[0] - lam, cs = n > 1 ? e[0] : 0.0;  // active row: diagonal and superdiagonal
    for (int i = 0; i + 1 < n; ++i) {
        const double sub = e[i], an = d[i + 1] - lam, en = i + 2 < n ? e[i + 1] : 0.0;
        if (fabs(cd) >= fabs(sub)) {
            const double r = 1.0 / guard(cd), mu = sub * r;
            f.r0[i] = r; f.u1[i] = cs; f.u2[i] = 0.0; f.m[i] = mu; f.piv[i] = 0;
            cd = an - mu * cs;
            cs = en;
        } else {
            const double r = 1.0 / guard(sub), mu = cd * r;
            f.r0[i] = r; f.u1[i] = an; f.u2[i] = en; f.m[i] = mu; f.piv[i] = 1;
            cd = cs - mu * an;
            cs = -mu * en;
        }
    }
    f.r0[n - 1] = 1.0 / guard(cd);
}

// x <- (P L U)^{-1} x, in place
__device__ void solve(LU f, int n, double* x) {
    for (int i = 0; i + 1 < n; ++i) {
        if (f.piv[i]) { const double t = x[i]; x[i] = x[i + 1]; x[i + 1] = t; }
        x[i + 1] -= f.m[i] * x[i];
    }
    x[n - 1] *= f.r0[n - 1];
    if (n >= 2) x[n - 2] = (x[n - 2] - f.u1[n - 2] * x[n - 1]) * f.r0[n - 2];
    for (int i = n - 3; i >= 0; --i) x[i] = (x[i] - f.u1[i] * x[i + 1] - f.u2[i] * x[i + 2]) * f.r0[i];
}

__global__ void __launch_bounds__(kThreads)
stein_kernel(const ChainDesc* __restrict__ descs, const double* __restrict__ dd, const double* __restrict__ ee,
             const double* __restrict__ ww, double* __restrict__ Zws, double* __restrict__ scratch) {
    extern __shared__ double sme[];
    const ChainDesc D = descs[blockIdx.x];
    const int n = D.n, ld = D.ld;
    if ((int)(blockIdx.y * blockDim.x) >= n) return;
    double* d = sme;
    double* e = sme + ld;
    __shared__ double red[2][kThreads / 32];
    double gl = DBL_MAX, gu = -DBL_MAX;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        d[i] = dd[D.v_off + i];
        e[i] = i + 1 < n ? ee[D.v_off + i] : 0.0;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double r = (i > 0 ? fabs(e[i - 1]) : 0.0) + (i + 1 < n ? fabs(e[i]) : 0.0);
        gl = fmin(gl, d[i] - r);
        gu = fmax(gu, d[i] + r);
    }
    gl = warp_min(gl);
    gu = warp_max(gu);
    if ((threadIdx.x & 31) == 0) { red[0][threadIdx.x >> 5] = gl; red[1][threadIdx.x >> 5] = gu; }
    __syncthreads();
    for (int q = 0; q < kThreads / 32; ++q) { gl = fmin(gl, red[0][q]); gu = fmax(gu, red[1][q]); }
    const double tnorm = fmax(fabs(gl), fabs(gu));
    const double ortol = 1e-5 * tnorm, pivmin = DBL_EPSILON * tnorm + DBL_MIN;
    const int j = blockIdx.y * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const double* w = ww + D.v_off;
    if (j > 0 && w[j] - w[j - 1] <= ortol) return;  // not a cluster leader
    double* Z = Zws + D.a_off;
    // per-thread scratch: 5 ld doubles (r0, u1, u2, m, piv) + the work vector;
    // chain c owns [6 a_off_c, 6 a_off_c + 6 ld_c^2)
    double* base = scratch + 6 * (size_t)D.a_off + (size_t)j * 6 * ld;
    LU f{base, base + ld, base + 2 * ld, base + 3 * ld, reinterpret_cast<int*>(base + 4 * ld)};
    double* x = base + 5 * ld;
    for (int jj = j; jj < n && (jj == j || w[jj] - w[jj - 1] <= ortol); ++jj) {
        // a perturbation of 2 eps ||T|| keeps identical eigenvalues of a cluster apart
        const double lam = w[jj] + (jj - j) * 2.0 * DBL_EPSILON * tnorm;
        factor(d, e, n, lam, pivmin, f);
        for (int i = 0; i < n; ++i) x[i] = 1.0 + 0.25 * sin(0.7 * i + 1.3 * jj);  // fixed start vector
        for (int it = 0; it < 3; ++it) {
            solve(f, n, x);
            for (int q = j; q < jj; ++q) {  // orthogonalise against the cluster's earlier vectors
                double dot = 0.0;
                for (int i = 0; i < n; ++i) dot += Z[(size_t)i * ld + q] * x[i];
                for (int i = 0; i < n; ++i) x[i] -= dot * Z[(size_t)i * ld + q];
            }
            double nrm = 0.0;
            for (int i = 0; i < n; ++i) nrm += x[i] * x[i];
            const double sc = 1.0 / sqrt(nrm);
            for (int i = 0; i < n; ++i) x[i] *= sc;
        }
        // sign: largest component positive (deterministic output)
        int imax = 0;
        for (int i = 1; i < n; ++i)
            if (fabs(x[i]) > fabs(x[imax])) imax = i;
        const double sg = x[imax] < 0.0 ? -1.0 : 1.0;
        for (int i = 0; i < n; ++i) Z[(size_t)i * ld + jj] = sg * x[i];
    }
}

// Mixed path: the twisted-factorisation vectors are accurate for isolated
// eigenvalues but may coincide inside clusters of (nearly) equal eigenvalues
// (gaps <= 1e-5 ||T||; the twisted factorisation skips those members, and
// this kernel runs beside it on a second stream). One CTA per chain computes
// the clusters' vectors by FP64 inverse iteration, the members of several
// clusters at once: thread g
// owns member g (its LU factors and iterate in the chain's scratch, 6 ld
// doubles), and after each of the three solves one warp per cluster
// orthonormalises the cluster's iterates in order (modified Gram-Schmidt,
// lanes over the rows). A wave holds at most min(256, ld / 6) members; a
// longer cluster is done in chunks, each chunk's iterates first made
// orthogonal to the cluster's vectors finished in earlier waves. Chains
// without a cluster leave after the scan.
constexpr int kCfThreads = 256;

__global__ void __launch_bounds__(kCfThreads)
cluster_fix_kernel(const ChainDesc* __restrict__ descs, const double* __restrict__ dd, const double* __restrict__ ee,
                   const double* __restrict__ ww, const double* __restrict__ ctol, float* __restrict__ Zws,
                   float* __restrict__ zscale, double* __restrict__ scratch) {
    extern __shared__ double smc[];
    const ChainDesc D = descs[blockIdx.x];
    const int n = D.n, ld = D.ld;
    double* d = smc;
    double* e = d + ld;
    double* w = e + ld;
    __shared__ int sj[kCfThreads], sr[kCfThreads], cls[kCfThreads + 1], cfin[kCfThreads];
    __shared__ int s_nslots, s_ncl, s_pos, s_cstart, s_cend;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int i = tid; i < n; i += blockDim.x) {
        d[i] = dd[D.v_off + i];
        e[i] = i + 1 < n ? ee[D.v_off + i] : 0.0;
        w[i] = ww[D.v_off + i];
    }
    __syncthreads();
    // the tolerance the shift kernel recorded (the twisted factorisation skips
    // exactly these members)
    const double ortol = ctol[blockIdx.x], tnorm = ortol / kClusterTol;
    const double pivmin = DBL_EPSILON * tnorm + DBL_MIN;
    int any = 0;
    for (int i = tid + 1; i < n; i += blockDim.x) any |= (w[i] - w[i - 1] <= ortol);
    if (!__syncthreads_or(any)) return;
    float* Z = Zws + D.a_off;
    double* base0 = scratch + D.a_off;  // ld * ld doubles of this chain
    const int cap = min(kCfThreads, ld / 6);
    if (tid == 0) { s_pos = 0; s_cstart = 0; s_cend = 0; }
    __syncthreads();
    for (;;) {
        // ---- the next wave (thread 0 walks the spectrum): whole clusters, or
        //      a chunk of one that does not fit; cfin[c] = the cluster's first
        //      member, members cfin[c] .. sj[cls[c]] - 1 are finished ----
        if (tid == 0) {
            int pos = s_pos, cstart = s_cstart, cend = s_cend, g = 0, c = 0;
            while (pos < n && g < cap) {
                if (pos >= cend) {  // at a cluster boundary: find the next cluster
                    int end = pos + 1;
                    while (end < n && w[end] - w[end - 1] <= ortol) ++end;
                    if (end - pos < 2) { pos = end; continue; }
                    cstart = pos;
                    cend = end;
                }
                const int take = min(cend - pos, cap - g);
                cls[c] = g;
                cfin[c] = cstart;
                ++c;
                for (int q = 0; q < take; ++q) { sj[g + q] = pos + q; sr[g + q] = pos + q - cstart; }
                g += take;
                pos += take;
            }
            cls[c] = g;
            s_nslots = g;
            s_ncl = c;
            s_pos = pos;
            s_cstart = cstart;
            s_cend = cend;
        }
        __syncthreads();
        const int nslots = s_nslots, ncl = s_ncl;
        if (nslots == 0) break;
        double* base = base0 + (size_t)min(tid, cap - 1) * 6 * ld;
        LU f{base, base + ld, base + 2 * ld, base + 3 * ld, reinterpret_cast<int*>(base + 4 * ld)};
        double* x = base + 5 * ld;
        if (tid < nslots) {
            const int jj = sj[tid];
            // a perturbation of 2 eps ||T|| per rank keeps identical eigenvalues apart
            const double lam = w[jj] + sr[tid] * 2.0 * DBL_EPSILON * tnorm;
            factor(d, e, n, lam, pivmin, f);
            for (int i = 0; i < n; ++i) x[i] = 1.0 + 0.25 * sin(0.7 * i + 1.3 * jj);  // fixed start vector
        }
        for (int it = 0; it < 3; ++it) {
            if (tid < nslots) solve(f, n, x);
            __syncthreads();
            for (int c = warp; c < ncl; c += kCfThreads / 32) {
                const int g0 = cls[c], k = cls[c + 1] - g0;
                for (int f = cfin[c]; f < sj[g0]; ++f) {  // the cluster's vectors from earlier waves
                    for (int m = 0; m < k; ++m) {
                        double* xm = base0 + (size_t)(g0 + m) * 6 * ld + 5 * ld;
                        double dp = 0.0;
                        for (int i = lane; i < n; i += 32) dp += (double)Z[(size_t)i * ld + f] * xm[i];
                        const double dot = warp_sum(dp);
                        for (int i = lane; i < n; i += 32) xm[i] -= dot * (double)Z[(size_t)i * ld + f];
                        __syncwarp();
                    }
                }
                for (int q = 0; q < k; ++q) {
                    double* xq = base0 + (size_t)(g0 + q) * 6 * ld + 5 * ld;
                    double part = 0.0;
                    for (int i = lane; i < n; i += 32) part += xq[i] * xq[i];
                    const double sc = 1.0 / sqrt(warp_sum(part));
                    for (int i = lane; i < n; i += 32) xq[i] *= sc;
                    __syncwarp();
                    for (int m = q + 1; m < k; ++m) {
                        double* xm = base0 + (size_t)(g0 + m) * 6 * ld + 5 * ld;
                        double dp = 0.0;
                        for (int i = lane; i < n; i += 32) dp += xq[i] * xm[i];
                        const double dot = warp_sum(dp);
                        for (int i = lane; i < n; i += 32) xm[i] -= dot * xq[i];
                        __syncwarp();
                    }
                }
            }
            __syncthreads();
        }
        for (int g = warp; g < nslots; g += kCfThreads / 32) {
            const double* xg = base0 + (size_t)g * 6 * ld + 5 * ld;
            const int jj = sj[g];
            for (int i = lane; i < n; i += 32) Z[(size_t)i * ld + jj] = (float)xg[i];
            if (lane == 0) zscale[D.v_off + jj] = 1.f;  // written normalised
        }
        __syncthreads();
    }
}

}  // namespace

cudaError_t launch_cluster_fix_f32(const ChainDesc* d_desc, int batch, int max_ld, const double* d_d,
                                   const double* d_e, const double* d_w, const double* d_ctol, float* d_Z,
                                   float* d_zscale, double* d_scratch, cudaStream_t st) {
    if (batch <= 0) return cudaSuccess;
    const size_t smem = sizeof(double) * 3 * (size_t)max_ld;
    cudaError_t err = cudaFuncSetAttribute(cluster_fix_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    cluster_fix_kernel<<<batch, kCfThreads, smem, st>>>(d_desc, d_d, d_e, d_w, d_ctol, d_Z, d_zscale,
                                                         d_scratch);
    return cudaGetLastError();
}

size_t stein_scratch_elems(long long a_total) { return (size_t)6 * a_total; }

cudaError_t launch_stein_f64(const ChainDesc* d_desc, int batch, int max_n, int max_ld, const double* d_d,
                             const double* d_e, const double* d_w, double* d_Z, double* d_scratch, cudaStream_t st) {
    if (batch <= 0) return cudaSuccess;
    const size_t smem = sizeof(double) * 2 * max_ld;
    cudaError_t err = cudaFuncSetAttribute(stein_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    stein_kernel<<<dim3(batch, (max_n + kThreads - 1) / kThreads), kThreads, smem, st>>>(d_desc, d_d, d_e, d_w, d_Z,
                                                                                          d_scratch);
    return cudaGetLastError();
}

}  // namespace fkg
