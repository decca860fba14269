// measures.cu — the eigenvector-consuming measures of fk_mc on the GPU, from
// calc_ed(true) of a batch (eigenvectors X, their eigenvalues, Fermi factors):
//   * measure_ipr (include/fk_mc/measures/ipr.hpp:39-56):
//       ipr_k = ||x_k||_4 / ||x_k||_2^2 for every eigenvector;
//   * the Drude stiffness of measure_stiffness
//     (include/fk_mc/measures/stiffness.hpp:129-187), with the kinetic and
//     current operators Tm, Jm of the lattice's first axis:
//       T = -pi sum_k fermi_k x_k^T Tm x_k,
//       V = sum over pairs i > j with |e_i - e_j| > 1e-12 and |sigma| > 1e-13 of
//           2 sigma / (e_i - e_j),  sigma = pi (f_j - f_i) mJ(j,i) mJ(i,j),
//       mJ = X^T Jm X, stiffness = (V + T) / n,
//     and, on a frequency grid w with width eta, the conductivity history:
//       cond(w) = sum over the same pairs of
//                 sigma (L(w + e_j - e_i) - L(w + e_i - e_j)),  L(x) = eta / pi / (x^2 + eta^2)
//     (the resonant terms of stiffness.hpp:160-185).
// Jm is antisymmetric (-1 to the left neighbour, +1 to the right), so
// mJ(j,i) mJ(i,j) = -mJ(j,i)^2, and every term is symmetric in (i, j): the
// pairs are summed over the columns of X in storage order (the mixed path
// keeps its columns unsorted) with each column's own eigenvalue.
//
// Layout: X row-major per chain (X[i * ld + k] = component i of vector k, FP64
// on the plain path, FP32 on the mixed path); JX = Jm X in the same layout.
// mJ is never stored: one CTA per 32 x 32 tile of X^T JX (upper tiles only)
// forms the tile and sums its pairs' terms; per-tile partial sums are added
// in a fixed order, so the result is reproducible.
#include <cfloat>

#include "fkg_common.cuh"

namespace fkg {
namespace {

constexpr int kMt = 32;  // tile of mJ

// ipr of the k-th eigenvector in ascending eigenvalue order (perm: storage
// column of the k-th, or null when the columns are already sorted)
template <typename TX>
__global__ void __launch_bounds__(128)
ipr_kernel(const ChainDesc* __restrict__ descs, const TX* __restrict__ Xws, const int* __restrict__ perm,
           double* __restrict__ out) {
    const ChainDesc D = descs[blockIdx.x];
    const int n = D.n, ld = D.ld;
    const int k = blockIdx.y * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int col = perm ? perm[D.v_off + k] : k;
    const TX* X = Xws + D.a_off;
    double s2 = 0.0, s4 = 0.0;
    for (int i = 0; i < n; ++i) {
        const double x = (double)X[(size_t)i * ld + col];
        const double x2 = x * x;
        s2 += x2;
        s4 = fma(x2, x2, s4);
    }
    out[D.v_off + k] = sqrt(sqrt(s4)) / s2;
}

// Per storage column b: eigenvalue and Fermi factor, the kinetic expectation
// t_b = x_b^T Tm x_b, and the column b of JX = Jm X. Per CTA: sum_b f_b t_b.
template <typename TX>
__global__ void __launch_bounds__(128)
stiff_columns_kernel(const ChainDesc* __restrict__ descs, const StiffOps* __restrict__ ops,
                     const TX* __restrict__ Xws, const double* __restrict__ eps, const double* __restrict__ beta,
                     TX* __restrict__ JXws, double2* __restrict__ ef, double* __restrict__ tpart) {
    __shared__ double red[4];
    const ChainDesc D = descs[blockIdx.x];
    const int* __restrict__ srow = ops[blockIdx.x].rowptr;
    const int* __restrict__ scol = ops[blockIdx.x].col;
    const double* __restrict__ tval = ops[blockIdx.x].tval;
    const double* __restrict__ jval = ops[blockIdx.x].jval;
    const int n = D.n, ld = D.ld;
    const int b = blockIdx.y * blockDim.x + threadIdx.x;
    double ft = 0.0;
    if (b < n) {
        const TX* X = Xws + D.a_off;
        TX* JX = JXws + D.a_off;
        double tb = 0.0;
        for (int i = 0; i < n; ++i) {
            double tx = 0.0, jx = 0.0;
            for (int p = srow[i]; p < srow[i + 1]; ++p) {
                const double xc = (double)X[(size_t)scol[p] * ld + b];
                tx = fma(tval[p], xc, tx);
                jx = fma(jval[p], xc, jx);
            }
            tb = fma((double)X[(size_t)i * ld + b], tx, tb);
            JX[(size_t)i * ld + b] = (TX)jx;
        }
        const double e = eps[D.v_off + b];
        const double f = 1.0 / (1.0 + exp(beta[blockIdx.x] * e));
        ef[D.v_off + b] = make_double2(e, f);
        ft = f * tb;
    }
    ft = warp_sum(ft);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = ft;
    __syncthreads();
    if (threadIdx.x == 0) tpart[(size_t)blockIdx.x * gridDim.y + blockIdx.y] = (red[0] + red[1]) + (red[2] + red[3]);
}

// One 32 x 32 tile (ja <= ib) of S = X^T JX, S(a, b) = x_a . (Jm x_b), and its
// pairs a < b: V += 2 pi (f_a - f_b) (-S(a,b)^2) / (e_b - e_a) where the
// reference's conditions hold. 256 threads, 4 outputs each. With a frequency
// grid the tile's terms (energy difference, sigma) are gathered in shared
// memory and summed per frequency in a fixed order (FP32 terms on the mixed
// path, FP64 on the plain path).
template <typename TX>
__global__ void __launch_bounds__(256)
stiff_pairs_kernel(const ChainDesc* __restrict__ descs, const TX* __restrict__ Xws, const TX* __restrict__ JXws,
                   const double2* __restrict__ ef, int ntile, double* __restrict__ vpart, int nw,
                   const double* __restrict__ wgrid, double eta, double* __restrict__ cpart) {
    __shared__ TX Xa[kMt][kMt + 1];
    __shared__ TX Jb[kMt][kMt + 1];
    __shared__ double red[8];
    __shared__ double2 terms[kMt * kMt];  // (e_i - e_j, sigma) of the tile's pairs, e_i > e_j
    __shared__ double cbuf[256];          // per-slice conductivity sums (S * nw <= 256)
    __shared__ float2 termf[sizeof(TX) == 4 ? kMt * kMt : 1];  // the terms in FP32 (mixed path)
    __shared__ int wcnt[8];
    __shared__ int nterm;
    // blockIdx.x = tile, blockIdx.y = chain: one chain's tiles are adjacent in
    // launch order, so its X and JX columns are served from L2 after the
    // first reads
    const ChainDesc D = descs[blockIdx.y];
    const int n = D.n, ld = D.ld;
    // tile index -> (ja, ib), ja <= ib, row-major over ib
    int ib = 0, q = blockIdx.x;
    while (q > ib) { q -= ib + 1; ++ib; }
    const int ja = q;
    double* out = vpart + (size_t)blockIdx.y * ntile + blockIdx.x;
    double* cout = cpart ? cpart + ((size_t)blockIdx.y * ntile + blockIdx.x) * nw : nullptr;
    if (ib * kMt >= n) {
        if (threadIdx.x == 0) *out = 0.0;
        if (cout)
            for (int q = threadIdx.x; q < nw; q += blockDim.x) cout[q] = 0.0;
        return;
    }
    if (threadIdx.x == 0) nterm = 0;
    const TX* X = Xws + D.a_off;
    const TX* JX = JXws + D.a_off;
    const int t = threadIdx.x, tc = t & 31, tr = t >> 5;  // this thread: column b = ib*32 + tc, rows a = ja*32 + tr + 8u
    TX acc[4] = {TX(0), TX(0), TX(0), TX(0)};
    for (int r0 = 0; r0 < n; r0 += kMt) {
        for (int u = tr; u < kMt; u += 8) {
            const int r = r0 + u;
            Xa[u][tc] = (r < n && ja * kMt + tc < n) ? X[(size_t)r * ld + ja * kMt + tc] : TX(0);
            Jb[u][tc] = (r < n && ib * kMt + tc < n) ? JX[(size_t)r * ld + ib * kMt + tc] : TX(0);
        }
        __syncthreads();
#pragma unroll 8
        for (int u = 0; u < kMt; ++u) {
            const TX jb = Jb[u][tc];
#pragma unroll
            for (int v = 0; v < 4; ++v) acc[v] = fma(Xa[u][tr + 8 * v], jb, acc[v]);
        }
        __syncthreads();
    }
    double vsum = 0.0;
    const int bcol = ib * kMt + tc;
    if (cout && bcol >= n)
#pragma unroll
        for (int v = 0; v < 4; ++v) terms[(tr + 8 * v) * kMt + tc] = make_double2(0.0, 0.0);
    if (bcol < n) {
        const double2 efb = ef[D.v_off + bcol];
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int a = ja * kMt + tr + 8 * v;
            if (cout) terms[(tr + 8 * v) * kMt + tc] = make_double2(0.0, 0.0);
            if (a >= n || (ja == ib && a >= bcol)) continue;
            const double2 efa = ef[D.v_off + a];
            if (!(fabs(efb.x - efa.x) > 1e-12)) continue;
            const double s = (double)acc[v];
            const double sigma = M_PI * (efa.y - efb.y) * (-s * s);
            if (fabs(sigma) > 1e-13) {
                vsum += 2.0 * sigma / (efb.x - efa.x);
                // the reference's sigma_ij takes i as the higher eigenvalue
                if (cout)
                    terms[(tr + 8 * v) * kMt + tc] = make_double2(fabs(efb.x - efa.x), efb.x > efa.x ? sigma : -sigma);
            }
        }
    }
    vsum = warp_sum(vsum);
    if ((t & 31) == 0) red[t >> 5] = vsum;
    if (cout) {
        // compact the tile's terms in a fixed (row-major) order; entries that
        // are no pair of the tile were zeroed above
        __syncthreads();
        if constexpr (sizeof(TX) == 4) {
            // FP32 copies, in parallel: thread t takes entries 4t .. 4t+3, its
            // output offset is the block's exclusive prefix sum of the counts
            int cnt = 0;
#pragma unroll
            for (int u = 0; u < 4; ++u) cnt += terms[4 * t + u].y != 0.0;
            int incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, incl, o);
                if ((t & 31) >= o) incl += y;
            }
            if ((t & 31) == 31) wcnt[t >> 5] = incl;
            __syncthreads();
            int off = incl - cnt;
            for (int w = 0; w < (t >> 5); ++w) off += wcnt[w];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const double2 x = terms[4 * t + u];
                if (x.y != 0.0) termf[off++] = make_float2((float)x.x, (float)x.y);
            }
            if (t == blockDim.x - 1) nterm = off;
        } else if (t == 0) {
            int m = 0;
            for (int e = 0; e < kMt * kMt; ++e) {
                const double2 x = terms[e];
                if (x.y != 0.0) terms[m++] = x;
            }
            nterm = m;
        }
    }
    __syncthreads();
    if (t == 0) {
        double s = 0.0;
        for (int w = 0; w < 8; ++w) s += red[w];
        *out = s;
    }
    if (cout) {
        // L(w - d) - L(w + d) = (eta / pi) 4 w d / (((w - d)^2 + eta^2) ((w + d)^2 + eta^2)):
        // one quotient per term and frequency, free of the cancellation of
        // the two Lorentzians. With nw < 256 the terms are split into S
        // slices (k = s, s + S, ...) so that every thread works; the slices
        // are added in order.
        const int m = nterm;
        const int S = nw * 2 <= (int)blockDim.x ? (int)blockDim.x / nw : 1;
        const double scale = 4.0 * eta / M_PI, eta2 = eta * eta;
        for (int q0 = 0; q0 < nw; q0 += (S > 1 ? nw : (int)blockDim.x)) {
            const int q = q0 + (S > 1 ? t % nw : t), s = S > 1 ? t / nw : 0;
            double c = 0.0;
            if (q < nw && s < S) {
                if constexpr (sizeof(TX) == 4) {
                    // the mixed path: terms in FP32 (its eigenvectors are FP32-accurate),
                    // blocks of 16 terms summed in FP32, the blocks in FP64
                    const float w = (float)wgrid[q], e2 = (float)eta2;
                    int k = s;
                    while (k < m) {
                        float cb = 0.f;
                        for (int u = 0; u < 16 && k < m; ++u, k += S) {
                            const float de = termf[k].x, sg = termf[k].y;
                            const float a = w - de, b = w + de;
                            const float p = fmaf(a, a, e2) * fmaf(b, b, e2);
                            cb += __fdividef(sg * (w * de), p);
                        }
                        c += (double)cb;
                    }
                } else {
                    const double w = wgrid[q];
                    for (int k = s; k < m; k += S) {
                        const double de = terms[k].x;  // e_i - e_j > 0
                        const double a = w - de, b = w + de;
                        c += terms[k].y * (w * de) / (fma(a, a, eta2) * fma(b, b, eta2));
                    }
                }
            }
            if (S > 1) {
                __syncthreads();  // cbuf free (previous round read)
                if (s < S && q < nw) cbuf[s * nw + (q - q0)] = c;
                __syncthreads();
                if (t < nw && q0 + t < nw) {
                    double tot = 0.0;
                    for (int u = 0; u < S; ++u) tot += cbuf[u * nw + t];
                    cout[q0 + t] = tot * scale;
                }
            } else if (q < nw) {
                cout[q] = c * scale;
            }
        }
    }
}

// stiffness = (V + T) / n, partial sums added in a fixed order
__global__ void stiff_final_kernel(const ChainDesc* __restrict__ descs, int batch, const double* __restrict__ tpart,
                                   int ntb, const double* __restrict__ vpart, int ntile, double* __restrict__ out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= batch) return;
    double t = 0.0, v = 0.0;
    for (int q = 0; q < ntb; ++q) t += tpart[(size_t)c * ntb + q];
    for (int q = 0; q < ntile; ++q) v += vpart[(size_t)c * ntile + q];
    out[c] = (v - M_PI * t) / descs[c].n;
}

// cond[c][w] = sum over tiles, fixed order
__global__ void cond_final_kernel(int batch, int ntile, int nw, const double* __restrict__ cpart,
                                  double* __restrict__ cond) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= batch * nw) return;
    const int c = idx / nw, w = idx % nw;
    double s = 0.0;
    for (int q = 0; q < ntile; ++q) s += cpart[((size_t)c * ntile + q) * nw + w];
    cond[idx] = s;
}

}  // namespace

cudaError_t launch_ipr(const ChainDesc* d_desc, int batch, int max_n, bool f32, const void* d_X, const int* d_perm,
                       double* d_out, cudaStream_t st) {
    if (batch <= 0) return cudaSuccess;
    dim3 grid(batch, (max_n + 127) / 128);
    if (f32) ipr_kernel<float><<<grid, 128, 0, st>>>(d_desc, (const float*)d_X, d_perm, d_out);
    else ipr_kernel<double><<<grid, 128, 0, st>>>(d_desc, (const double*)d_X, nullptr, d_out);
    return cudaGetLastError();
}

size_t stiffness_scratch_bytes(int batch, int max_n, int nw) {
    const int ntb = (max_n + 127) / 128, nb = (max_n + kMt - 1) / kMt, ntile = nb * (nb + 1) / 2;
    return sizeof(double) * (size_t)batch * (ntb + (size_t)ntile * (1 + nw));
}

cudaError_t launch_stiffness(const ChainDesc* d_desc, const StiffOps* d_ops, int batch, int max_n, bool f32,
                             const void* d_X, const double* d_eps, const double* d_beta, void* d_JX, double2* d_ef,
                             double* d_scratch, double* d_out, int nw, const double* d_wgrid, double eta,
                             double* d_cond, cudaStream_t st) {
    if (batch <= 0) return cudaSuccess;
    if (batch > 65535) return cudaErrorInvalidValue;  // grid y limit of the pair kernel
    const int ntb = (max_n + 127) / 128, nb = (max_n + kMt - 1) / kMt, ntile = nb * (nb + 1) / 2;
    double* tpart = d_scratch;
    double* vpart = d_scratch + (size_t)batch * ntb;
    double* cpart = nw > 0 ? vpart + (size_t)batch * ntile : nullptr;
    if (f32) {
        stiff_columns_kernel<float><<<dim3(batch, ntb), 128, 0, st>>>(d_desc, d_ops, (const float*)d_X, d_eps, d_beta,
                                                                      (float*)d_JX, d_ef, tpart);
        stiff_pairs_kernel<float><<<dim3(ntile, batch), 256, 0, st>>>(d_desc, (const float*)d_X, (const float*)d_JX,
                                                                      d_ef, ntile, vpart, nw, d_wgrid, eta, cpart);
    } else {
        stiff_columns_kernel<double><<<dim3(batch, ntb), 128, 0, st>>>(d_desc, d_ops, (const double*)d_X, d_eps,
                                                                       d_beta, (double*)d_JX, d_ef, tpart);
        stiff_pairs_kernel<double><<<dim3(ntile, batch), 256, 0, st>>>(d_desc, (const double*)d_X,
                                                                       (const double*)d_JX, d_ef, ntile, vpart, nw,
                                                                       d_wgrid, eta, cpart);
    }
    stiff_final_kernel<<<(batch + 127) / 128, 128, 0, st>>>(d_desc, batch, tpart, ntb, vpart, ntile, d_out);
    if (nw > 0) cond_final_kernel<<<(batch * nw + 127) / 128, 128, 0, st>>>(batch, ntile, nw, cpart, d_cond);
    return cudaGetLastError();
}

}  // namespace fkg
