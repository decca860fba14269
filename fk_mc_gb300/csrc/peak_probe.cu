// peak_probe.cu — throughput probes of the FP64 and FP32 FMA pipes and of the
// TF32 mma.sync path.
//
// The measured peaks (HBM copy, bf16 GEMM) do not cover the FP64 pipe
// (the plain path), the FP32 pipe or the TF32 mma.sync rate (the mixed
// path's back-transformation); bench.py measures them with these kernels on
// the same GPU and uses them as roofline denominators. FMA: eight independent
// chains per thread, 8 CTAs of 256 threads per SM. TF32: four independent
// m16n8k8 accumulators per warp, same grid.
#include "fkg_common.cuh"

namespace fkg {
namespace {
template <typename T>
__global__ void fma_probe_kernel(T* out, int iters, T a, T b) {
    T x0 = (T)threadIdx.x * (T)1e-9, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
      x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
__global__ void mma_tf32_probe_kernel(float* out, int iters) {
    unsigned a[4], b[2];
    const float av[4] = {threadIdx.x * 1e-3f, 1.f, 2.f, 3.f}, bv[2] = {0.5f, 0.25f};
#pragma unroll
    for (int q = 0; q < 4; ++q) asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(a[q]) : "f"(av[q]));
#pragma unroll
    for (int q = 0; q < 2; ++q) asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(b[q]) : "f"(bv[q]));
    float d[4][4] = {};
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < 4; ++c)
            asm volatile(
                "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                "{%0,%1,%2,%3};\n"
                : "+f"(d[c][0]), "+f"(d[c][1]), "+f"(d[c][2]), "+f"(d[c][3])
                : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = d[0][0] + d[1][1] + d[2][2] + d[3][3];
}
}  // namespace

// Returns FLOP/s (2 per FMA) of the FP64 (which = 0) or FP32 (which = 1) pipe,
// or of TF32 mma.sync m16n8k8 (which = 2, 2 x 16 x 8 x 8 per instruction).
cudaError_t run_fma_probe(int which, int num_sms, double* flops, cudaStream_t st) {
    const int nb = num_sms * 8, nt = 256;
    void* buf = nullptr;
    cudaError_t e = cudaMallocAsync(&buf, sizeof(double) * nb * nt, st);
    if (e != cudaSuccess) return e;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int iters = which == 0 ? 4096 : which == 1 ? 65536 : 8192;
    float ms = 0.f;
    for (int rep = 0; rep < 2; ++rep) {  // first launch warms up
        cudaEventRecord(e0, st);
        if (which == 0) fma_probe_kernel<double><<<nb, nt, 0, st>>>((double*)buf, iters, 0.999, 1e-3);
        else if (which == 1) fma_probe_kernel<float><<<nb, nt, 0, st>>>((float*)buf, iters, 0.999f, 1e-3f);
        else mma_tf32_probe_kernel<<<nb, nt, 0, st>>>((float*)buf, iters);
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
    }
    if (which == 2) *flops = 2.0 * 16 * 8 * 8 * 4.0 * (double)iters * nb * (nt / 32) / (ms * 1e-3);
    else *flops = 2.0 * 8 * (double)iters * nb * nt / (ms * 1e-3);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFreeAsync(buf, st);
    e = cudaStreamSynchronize(st);
    return e != cudaSuccess ? e : cudaGetLastError();
}
}  // namespace fkg
