// peak_probe.cu — FMA throughput probe of the FP64 and FP32 pipes.
//
// The FP64 path is bound by the FP64 pipe, whose rate the driver-measured
// peaks (HBM copy, bf16 GEMM) do not cover; bench.py measures it with this
// kernel on the same GPU and uses it as the roofline denominator.
// Eight independent FMA chains per thread, 8 CTAs of 256 threads per SM.
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
}  // namespace

// Returns FLOP/s (2 per FMA) of the FP64 (which = 0) or FP32 (which = 1) pipe.
cudaError_t run_fma_probe(int which, int num_sms, double* flops, cudaStream_t st) {
    const int nb = num_sms * 8, nt = 256;
    void* buf = nullptr;
    cudaError_t e = cudaMallocAsync(&buf, sizeof(double) * nb * nt, st);
    if (e != cudaSuccess) return e;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int iters = which == 0 ? 4096 : 65536;
    float ms = 0.f;
    for (int rep = 0; rep < 2; ++rep) {  // first launch warms up
        cudaEventRecord(e0, st);
        if (which == 0) fma_probe_kernel<double><<<nb, nt, 0, st>>>((double*)buf, iters, 0.999, 1e-3);
        else fma_probe_kernel<float><<<nb, nt, 0, st>>>((float*)buf, iters, 0.999f, 1e-3f);
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
    }
    *flops = 2.0 * 8 * (double)iters * nb * nt / (ms * 1e-3);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFreeAsync(buf, st);
    e = cudaStreamSynchronize(st);
    return e != cudaSuccess ? e : cudaGetLastError();
}
}  // namespace fkg
