// noalloc.cu — fkg_eigh_logz_noalloc: the FP64 batched eigen-solve + logZ for
// callers that cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: a Monte Carlo rank that
// runs inside a host application whose pool allocator has already reserved
// the whole device, or a latency-critical step in which a device allocation
// (which synchronises the device) is not allowed. This entry point takes the
// caller's device buffers for its inputs and outputs and keeps all of its
// scratch (the dense matrices, the tridiagonal, the batch descriptors and the
// status word) in one file-scope
// device array of fixed size, so it never allocates.
//
// Every call shares that array, which keeps the previous call's contents:
// the status word is cleared at the start of each call, and every other
// scratch region is fully rewritten before it is read. Calls that overlap on
// the GPU (issued concurrently on different streams, or from several host
// threads) race on the array: serialise them.
#include <cstring>
#include <mutex>

#include "../../include/fkg.h"
#include "fkg_common.cuh"

namespace fkg {
namespace {

constexpr int kMaxN = FKG_NOALLOC_MAX_N;
constexpr int kMaxBatch = FKG_NOALLOC_MAX_BATCH;
constexpr int kLd = (kMaxN + kTile - 1) / kTile * kTile;
constexpr size_t kAlign = 256;
constexpr size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

// byte offsets of the regions inside the scratch array
constexpr size_t kOffDesc = 0;
constexpr size_t kOffStatus = align_up(kOffDesc + sizeof(ChainDesc) * kMaxBatch);
constexpr size_t kOffA = align_up(kOffStatus + sizeof(int));
constexpr size_t kOffVec = align_up(kOffA + sizeof(double) * (size_t)kMaxBatch * kLd * kLd);
constexpr size_t kVecBytes = sizeof(double) * (size_t)kMaxBatch * kLd;
constexpr size_t kScratchBytes = align_up(kOffVec + 5 * kVecBytes);  // diag, d, e, tau, w

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch_addr[kMaxDevices] = {nullptr};

int fail(char* errbuf, int errlen, int code, const char* msg) {
    if (errbuf && errlen > 0) {
        std::strncpy(errbuf, msg, (size_t)errlen - 1);
        errbuf[errlen - 1] = '\0';
    }
    return code;
}

}  // namespace
}  // namespace fkg

using namespace fkg;

extern "C" int fkg_eigh_logz_noalloc(int batch, int n, const int32_t* d_rowptr, const int32_t* d_col,
                                     const double* d_val, const double* d_diag, const double* d_beta,
                                     double* d_evals, double* d_logz, void* stream, char* errbuf, int errlen) {
    if (batch < 1 || batch > kMaxBatch)
        return fail(errbuf, errlen, FKG_ERR_ARG, "batch must be in [1, FKG_NOALLOC_MAX_BATCH]");
    if (n < 1 || n > kMaxN) return fail(errbuf, errlen, FKG_ERR_ARG, "n must be in [1, FKG_NOALLOC_MAX_N]");
    if (!d_rowptr || !d_col || !d_val || !d_diag || !d_beta || !d_evals || !d_logz)
        return fail(errbuf, errlen, FKG_ERR_ARG, "null device pointer");
    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return fail(errbuf, errlen, FKG_ERR_CUDA, "cudaGetDevice failed");
    }
    // once per device, with that device current: the device address of the
    // scratch array (the host-side symbol is only a stand-in for it)
    unsigned char* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (!g_scratch_addr[dev]) {
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) {
                cudaGetLastError();
                return fail(errbuf, errlen, FKG_ERR_CUDA, "cudaGetSymbolAddress of the scratch array failed");
            }
            g_scratch_addr[dev] = p;
        }
        base = (unsigned char*)g_scratch_addr[dev];
    }
    ChainDesc* d_desc = (ChainDesc*)(base + kOffDesc);
    int* d_status = (int*)(base + kOffStatus);
    double* A = (double*)(base + kOffA);
    double* vdiag = (double*)(base + kOffVec);
    double* vd = vdiag + (size_t)kMaxBatch * kLd;
    double* ve = vd + (size_t)kMaxBatch * kLd;
    double* vtau = ve + (size_t)kMaxBatch * kLd;
    double* vw = vtau + (size_t)kMaxBatch * kLd;
    const int ld = (n + kTile - 1) / kTile * kTile;
    ChainDesc h[kMaxBatch];
    for (int c = 0; c < batch; ++c) {
        h[c].n = n;
        h[c].ld = ld;
        h[c].lattice = 0;
        h[c].pad = 0;
        h[c].a_off = (long long)c * ld * ld;
        h[c].v_off = (long long)c * ld;
        h[c].rowptr = d_rowptr;
        h[c].col = d_col;
        h[c].val = d_val;
        h[c].valf = nullptr;  // the FP64 path never reads the pairs
    }
#define NA_CUDA(call)                                                                   \
    do {                                                                                \
        cudaError_t _e = (call);                                                        \
        if (_e != cudaSuccess) return fail(errbuf, errlen, FKG_ERR_CUDA, cudaGetErrorString(_e)); \
    } while (0)
    NA_CUDA(cudaMemsetAsync(d_status, 0, sizeof(int), st));
    NA_CUDA(cudaMemcpyAsync(d_desc, h, sizeof(ChainDesc) * batch, cudaMemcpyHostToDevice, st));
    // packed (spacing n) diagonal -> scratch with spacing ld
    NA_CUDA(cudaMemcpy2DAsync(vdiag, sizeof(double) * ld, d_diag, sizeof(double) * n, sizeof(double) * n, batch,
                              cudaMemcpyDeviceToDevice, st));
    NA_CUDA(launch_sytrd_v3_f64(d_desc, batch, ld, vdiag, A, vd, ve, vtau, st, 1, nullptr, nullptr, 0, d_status));
    NA_CUDA(launch_trieig_values(d_desc, batch, n, ld, vd, ve, vw, d_status, st));
    NA_CUDA(launch_logz(d_desc, batch, n, vw, d_beta, d_logz, nullptr, nullptr, d_status, st));
    NA_CUDA(cudaMemcpy2DAsync(d_evals, sizeof(double) * n, vw, sizeof(double) * ld, sizeof(double) * n, batch,
                              cudaMemcpyDeviceToDevice, st));
    int hstatus = 0;
    NA_CUDA(cudaMemcpyAsync(&hstatus, d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
    NA_CUDA(cudaStreamSynchronize(st));
#undef NA_CUDA
    if (hstatus & kStatusNaN) return fail(errbuf, errlen, FKG_ERR_NUMERIC, "NaN or Inf in eigenvalues or logZ");
    if (hstatus & kStatusNoConverge) return fail(errbuf, errlen, FKG_ERR_NUMERIC, "eigenvalue iteration did not converge");
    if (hstatus & kStatusBadArg)
        return fail(errbuf, errlen, FKG_ERR_ARG, "a CSR column index lies outside [0, n)");
    if (hstatus) return fail(errbuf, errlen, FKG_ERR_NUMERIC, "device-side check failed");
    return fail(errbuf, errlen, FKG_OK, "");
}
