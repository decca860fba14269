// fkg_common.cuh — shared device-side definitions of the fk_mc GB300 solver.
//
// Data layout in HBM (one context, many chains):
//   * per-chain dense workspace A_c: ld_c x ld_c doubles (or floats for the
//     mixed path), column-major, ld_c = n_c rounded up to a multiple of 32;
//     only the lower triangle is kept up to date by the reductions;
//   * per-chain vectors of length ld_c (diagonal of H, tridiagonal d/e/tau,
//     eigenvalues, f-occupations) packed back to back at offset v_off_c;
//   * per-lattice sparse hopping (CSR) shared by every chain on that lattice.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace fkg {

constexpr int kTile = 32;  // tile edge of the tiled symmetric kernels
constexpr int kBand = 16;  // band width between the two stages of the two-stage reduction (twostage.cu)

// One entry per chain (or per proposal) of a batched launch.
struct ChainDesc {
    int n;             // matrix order (number of lattice sites)
    int ld;            // leading dimension of A_c (multiple of 32)
    int lattice;       // lattice id
    int pad;
    long long a_off;   // element offset of A_c inside the dense workspace
    long long v_off;   // element offset of this chain's vectors (spacing ld)
    const int* rowptr; // CSR hopping of the lattice (device)
    const int* col;
    const double* val;
    const float2* valf; // the same values as FP32 pairs hi + lo (mixed-path refinement)
};

// Eigenvalues of the tridiagonal closer than this times ||T|| form a cluster
// whose eigenvectors the mixed path recomputes in FP64 (cluster fix-up).
constexpr double kClusterTol = 1e-5;

// Kinetic (tval) and current (jval) operators of measure_stiffness along the
// lattice's first axis, CSR with one pattern, per chain (device pointers).
struct StiffOps {
    const int* rowptr;
    const int* col;
    const double* tval;
    const double* jval;
};

// One chain of a Chebyshev-expansion logZ (chebyshev.cu): its lattice's CSR
// hopping, the hopping's diagonal, and the balls of radius R around every
// site: ball j holds the sites within R hops of j in hop order (bsite[bptr[j]
// ..bptr[j+1]), local row 0 = j), bcnt[j*(R+1) + d] of them within d hops, and
// the ball's own CSR of the off-diagonal hopping (local row g = bptr[j] + r:
// entries blrp[g]..blrp[g+1] with local columns blcol and values blval).
struct KpmDesc {
    int n, ld, R, bmax;     // order, vector spacing, ball radius, largest ball
    long long v_off;        // offset of this chain's vectors (spacing ld)
    const int* rowptr;      // CSR hopping of the lattice
    const int* col;
    const double* val;
    const double* hdiag;    // diagonal of the hopping matrix
    const int* bptr;
    const int* bsite;
    const int* bcnt;
    const int* blrp;
    const int* blcol;
    const double* blval;
    const float2* blv2;     // blval as FP32 pairs hi + lo
    const float2* valf;     // val as FP32 pairs hi + lo
};

// Spectral bounds of one chain's Chebyshev expansion: x = (H - b)/a.
struct KpmAB {
    double e_min, e_max, a, b;
};

// Status word bits written by kernels (host reads them after the launch).
enum : int {
    kStatusNaN = 1,          // a NaN/Inf appeared in an eigenvalue or logZ
    kStatusNoConverge = 2,   // an iterative step ran into its iteration cap
    kStatusBadArg = 4,       // a descriptor was out of range
    kStatusTimeout = 8,      // a bounded device wait (mbarrier) ran out
};

// Default iteration limit of the bounded mbarrier waits of the tensor-core
// kernels' main loops (fkg_set_wait_limit changes it per context).
constexpr long long kDefaultWaitIters = 1ll << 24;

__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}
__device__ __forceinline__ float warp_sum(float x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}
__device__ __forceinline__ double warp_min(double x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x = fmin(x, __shfl_xor_sync(0xffffffffu, x, o));
    return x;
}
__device__ __forceinline__ double warp_max(double x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x = fmax(x, __shfl_xor_sync(0xffffffffu, x, o));
    return x;
}

// Block-wide min/max; every thread gets the result. `red` needs blockDim/32 slots.
__device__ __forceinline__ double block_min(double x, double* red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    x = warp_min(x);
    __syncthreads();
    if (lane == 0) red[wid] = x;
    __syncthreads();
    double s = red[0];
    for (int i = 1; i < nw; ++i) s = fmin(s, red[i]);
    return s;
}
__device__ __forceinline__ double block_max(double x, double* red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    x = warp_max(x);
    __syncthreads();
    if (lane == 0) red[wid] = x;
    __syncthreads();
    double s = red[0];
    for (int i = 1; i < nw; ++i) s = fmax(s, red[i]);
    return s;
}

// Block-wide sum; every thread gets the result. `red` needs blockDim/32 slots.
template <typename T>
__device__ __forceinline__ T block_sum(T x, T* red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    x = warp_sum(x);
    __syncthreads();
    if (lane == 0) red[wid] = x;
    __syncthreads();
    T s = 0;
    for (int i = 0; i < nw; ++i) s += red[i];
    return s;
}

// TF32 tensor-core helpers (mma.sync m16n8k8, the 3xTF32 split): x = hi + lo
// with hi = tf32(x) and lo = tf32(x - hi); a b ~ a_hi b_hi + a_hi b_lo + a_lo b_hi.
__device__ __forceinline__ void split_tf32(float x, unsigned& hi, unsigned& lo) {
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(hi) : "f"(x));
    const float r = x - __uint_as_float(hi);
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(lo) : "f"(r));
}
__device__ __forceinline__ void mma_tf32(float (&d)[4], const unsigned (&a)[4], const unsigned (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Double-float arithmetic (an unevaluated sum hi + lo of two FP32 numbers,
// about 48 significant bits; Dekker 1971, Knuth's TwoSum), for FP64-grade
// sums on the FP32 pipe, which is about sixty times wider than GB300's FP64
// pipe (rank-one roots, Chebyshev moments).
struct dfl {
    float hi, lo;
};
__device__ __forceinline__ dfl df_of(double x) {
    const float h = (float)x;
    return {h, (float)(x - (double)h)};
}
__device__ __forceinline__ dfl df_add(dfl a, dfl b) {
    const float s = a.hi + b.hi, bb = s - a.hi;
    float e = (a.hi - (s - bb)) + (b.hi - bb);
    e += a.lo + b.lo;
    const float h = s + e;
    return {h, e - (h - s)};
}
__device__ __forceinline__ dfl df_mul(dfl a, dfl b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    const float h = p + e;
    return {h, e - (h - p)};
}
// 1/a: the FP32 reciprocal of a.hi corrected by one Newton step carried in
// double-float (r = q + q (1 - a q), the residual formed exactly by fma)
__device__ __forceinline__ dfl df_rcp(dfl a) {
    const float q = 1.0f / a.hi;
    const float p = a.hi * q, pe = fmaf(a.hi, q, -p);
    const float e = ((1.0f - p) - pe) - a.lo * q;
    const float rl = q * e, h = q + rl;
    return {h, rl - (h - q)};
}
__device__ __forceinline__ double df_val(dfl a) { return (double)a.hi + (double)a.lo; }

// butterfly sum over the warp (lane 0's value is the one to use)
__device__ __forceinline__ dfl warp_sum_df(dfl x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        x = df_add(x, {__shfl_xor_sync(0xffffffffu, x.hi, o), __shfl_xor_sync(0xffffffffu, x.lo, o)});
    return x;
}

// Error-free sum of two doubles (Knuth's TwoSum).
__device__ __forceinline__ void two_sum(double a, double b, double& s, double& err) {
    s = a + b;
    double bb = s - a;
    err = (a - (s - bb)) + (b - bb);
}

}  // namespace fkg

// Host-side launch wrappers implemented in the .cu files.
namespace fkg {
// Chebyshev-expansion logZ (chebyshev.cu): bounds by Lanczos (at most kmax
// steps; d_steps, may be null: the steps each chain took), moments of M (even)
// Chebyshev polynomials on balls of radius R = M/2 (d_part: 3R doubles per
// site), coefficients on a G-point Lobatto grid. d_ab: the bounds
// per chain; d_mu (may be null): M moments per chain.
cudaError_t launch_kpm(const KpmDesc* d_kdesc, int batch, int max_n, int max_ld, int max_bmax, int R, int M, int G,
                       int kmax, const double* d_diag, const double* d_beta, KpmAB* d_ab, int* d_steps,
                       double* d_part, double* d_mu, double* d_logz, int* d_status, cudaStream_t st);
int kpm_warps_per_cta(int bmax);
// variant: index into kSytrdF64Nb / kSytrdF32Nb (panel width); d_order (may be
// null): chain indices longest first for the persistent schedule; d_status
// (may be null): kStatusBadArg when a CSR column lies outside [0, n)
extern const int kSytrdF32Nb[3];
extern const int kSytrdF64Nb[2];
cudaError_t launch_sytrd_v3_f64(const ChainDesc* d_desc, int batch, int max_ld, const double* d_diag, double* d_A,
                                double* d_d, double* d_e, double* d_tau, cudaStream_t st, int variant = 1,
                                const int* d_order = nullptr, int* d_counter = nullptr, int num_sms = 0,
                                int* d_status = nullptr);
cudaError_t launch_sytrd_v3_f32(const ChainDesc* d_desc, int batch, int max_ld, const double* d_diag, float* d_A,
                                double* d_d, double* d_e, float* d_tau, cudaStream_t st, int variant = 1,
                                const int* d_order = nullptr, int* d_counter = nullptr, int num_sms = 0,
                                int* d_status = nullptr);
// shift: reflector k has its unit at row k + shift (1: one-stage reduction,
// kBand: the two-stage reduction's first stage)
cudaError_t launch_larft_vt(const ChainDesc* d_desc, int batch, int max_n, const float* d_A32, const float* d_tau32,
                            float* d_Tf, float* d_VT, long long plane, int shift, cudaStream_t st);
// two-stage reduction: dense -> band kBand (sy2sb.cu; A32 in place, the
// reflectors below the band, their tau in d_tau; n <= 1024), band ->
// tridiagonal (twostage.cu; d, e; the band stage's reflectors in d_Q2: [ld][ld]
// vectors per chain, then their tau from q2t_off on, ld / kBand per sweep), and
// Z <- Q2 Z. The first stage reads and writes A32 through one TMA tensor map
// per chain (sy2sb_tensor_maps, host side, sy2sb_tensor_map_bytes() each).
size_t sy2sb_smem_bytes(int max_ld);
long long sy2sb_scratch_floats(int max_ld);  // per chain: operand tiles and rows of the tensor-core pass
size_t sy2sb_tensor_map_bytes();
cudaError_t sy2sb_tensor_maps(const ChainDesc* h_desc, int batch, float* d_A, void* h_maps);
cudaError_t launch_sy2sb(const ChainDesc* d_desc, int batch, int max_ld, const double* d_diag, float* d_A,
                         float* d_tau, const int* d_order, int* d_counter, int num_sms, int* d_status,
                         float* d_scratch, const void* d_tmaps, long long wait_iters, cudaStream_t st);
cudaError_t launch_sb2st(const ChainDesc* d_desc, int batch, int max_n, const float* d_A, double* d_d, double* d_e,
                         float* d_Q2, long long q2t_off, cudaStream_t st);
cudaError_t launch_q2_apply(const ChainDesc* d_desc, int batch, int max_n, const float* d_Q2, long long q2t_off,
                            float* d_Z, cudaStream_t st);
cudaError_t launch_mixed_refine(const ChainDesc* d_desc, int batch, int max_n, int max_ld, const double* d_diag,
                                const float* d_A32, const float* d_VT, long long vt_plane, const double* d_d,
                                const double* d_e,
                                double* d_w, const double* d_ctol, float* d_Z, float* d_zscale, double* d_theta,
                                int* d_perm, double* d_scratch, int* d_status, cudaStream_t st, cudaStream_t aux,
                                cudaEvent_t ev_fork, cudaEvent_t ev_join, cudaEvent_t ev_larft, int bt_variant,
                                long long wait_iters, int shift, const float* d_Q2, long long q2t_off,
                                void (*stage)(void*, int, int), void* sctx);
cudaError_t launch_backtransform_f64(const ChainDesc* d_desc, int batch, int max_n, int max_ld, const double* d_A,
                                     const double* d_tau, double* d_Tf, double* d_Z, cudaStream_t st);
size_t stein_scratch_elems(long long a_total);
cudaError_t launch_cluster_fix_f32(const ChainDesc* d_desc, int batch, int max_ld, const double* d_d,
                                   const double* d_e, const double* d_w, const double* d_ctol, float* d_Z,
                                   float* d_zscale, double* d_scratch, cudaStream_t st);
cudaError_t launch_stein_f64(const ChainDesc* d_desc, int batch, int max_n, int max_ld, const double* d_d,
                             const double* d_e, const double* d_w, double* d_Z, double* d_scratch, cudaStream_t st);
cudaError_t launch_grad(const ChainDesc* d_desc, int batch, bool fp32, const void* d_X, const double* d_eps,
                        const int32_t* d_f, const double* d_U, const double* d_mu, const double* d_t,
                        const double* d_beta, double* d_out, double* d_fermi, cudaStream_t st);
cudaError_t launch_rho(const ChainDesc* d_desc, int batch, int max_n, bool fp32, const void* d_X,
                       const double* d_fermi, double* d_rho, cudaStream_t st);
cudaError_t launch_trieig_values(const ChainDesc* d_desc, int batch, int max_n, int max_ld, const double* d_d,
                                 const double* d_e, double* d_w, int* d_status, cudaStream_t st);
// mixed path: eigenvalues of T as shifts for the twisted factorisation (FP32
// bracket, double-float Newton; FP64 only where a bracket is not confirmed)
cudaError_t launch_trieig_shifts(const ChainDesc* d_desc, int batch, int max_n, int max_ld, const double* d_d,
                                 const double* d_e, double* d_w, double* d_ctol, int* d_status, cudaStream_t st);
// mixed path X = Q Z, 3xTF32 tensor-core GEMMs (backtransform_tc.cu)
// d_VT: the four split planes larft_kernel writes (`plane` floats apart)
cudaError_t launch_backtransform_tc(const ChainDesc* d_desc, int batch, int max_n, int max_ld, const float* d_VT,
                                    long long plane, float* d_Z, const float* d_zscale, int shift, cudaStream_t st);
// the same on the tcgen05 tensor cores (backtransform_tc5.cu); sets
// kStatusTimeout in d_status if one of its main-loop mbarrier waits gives up
// after wait_iters checks (0: without checking, a test setting)
cudaError_t launch_backtransform_tc5(const ChainDesc* d_desc, int batch, int max_n, const float* d_VT, long long plane,
                                     float* d_Z, const float* d_zscale, int* d_status, long long wait_iters,
                                     int shift, cudaStream_t st);
// measures.cu: ipr per eigenvector (ascending order); Drude stiffness per chain
cudaError_t launch_ipr(const ChainDesc* d_desc, int batch, int max_n, bool f32, const void* d_X, const int* d_perm,
                       double* d_out, cudaStream_t st);
size_t stiffness_scratch_bytes(int batch, int max_n, int nw);
cudaError_t launch_stiffness(const ChainDesc* d_desc, const StiffOps* d_ops, int batch, int max_n, bool f32,
                             const void* d_X, const double* d_eps, const double* d_beta, void* d_JX, double2* d_ef,
                             double* d_scratch, double* d_out, int nw, const double* d_wgrid, double eta,
                             double* d_cond, cudaStream_t st);
cudaError_t launch_logz(const ChainDesc* d_desc, int batch, int max_n, const double* d_w, const double* d_beta,
                        double* d_logz, double* d_exp, double* d_fermi, int* d_status, cudaStream_t st);
// logZ of each chain and, in the same launch, its Metropolis decision and
// state update (the eigen-solve path's proposal step; equal to launch_logz
// followed by launch_accept)
cudaError_t launch_logz_accept(const ChainDesc* d_desc, int batch, const double* d_w, const double* d_beta,
                               double* d_logz, const int32_t* d_site, const double* d_u, const double* d_ebmf,
                               int32_t* d_f, double* d_logz_cur, double* d_w_cur, int32_t* d_accepted,
                               double* d_dlogz, int* d_status, cudaStream_t st, const int* d_step);
cudaError_t launch_proposal_diag(const ChainDesc* d_desc, int batch, int max_n, const int32_t* d_f,
                                 const int32_t* d_site, const double* d_U, const double* d_mu_c, double* d_diag,
                                 int* d_status, cudaStream_t st, const int* d_step = nullptr);
cudaError_t launch_accept(const ChainDesc* d_desc, int batch, int max_n, const int32_t* d_site, const double* d_u,
                          const double* d_logz_new, const double* d_w_new, const double* d_ebmf, int32_t* d_f,
                          double* d_logz_cur, double* d_w_cur, int32_t* d_accepted, double* d_dlogz,
                          int* d_status, cudaStream_t st, const int* d_step = nullptr);
cudaError_t launch_step_inc(int* d_step, cudaStream_t st);
}  // namespace fkg
