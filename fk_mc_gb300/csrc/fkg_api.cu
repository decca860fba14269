// fkg_api.cu — the C ABI of include/fkg.h: context, device buffers, batch
// layout and the launch sequence of each entry point.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/fkg.h"
#include "fkg_common.cuh"
#include "fkg_internal.h"

using namespace fkg;

namespace {

int set_err(fkg_ctx* ctx, int code, const std::string& msg) {
    if (ctx) ctx->err = msg;
    return code;
}

#define FKG_CUDA(ctx, call)                                                                      \
    do {                                                                                         \
        cudaError_t _e = (call);                                                                 \
        if (_e != cudaSuccess)                                                                   \
            return set_err(ctx, FKG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
    } while (0)

int round_ld(int n) { return (n + kTile - 1) / kTile * kTile; }

}  // namespace

namespace fkg {

int ensure_dev(fkg_ctx* ctx, DevBuf& b, size_t bytes) {
    if (bytes <= b.bytes && b.p) return FKG_OK;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
    size_t want = bytes < 256 ? 256 : bytes;
    cudaError_t e = cudaMalloc(&b.p, want);
    if (e != cudaSuccess) {
        b.p = nullptr;
        cudaGetLastError();
        return set_err(ctx, FKG_ERR_ALLOC, std::string("cudaMalloc(") + std::to_string(want) + "): " + cudaGetErrorString(e));
    }
    b.bytes = want;
    return FKG_OK;
}

int ensure_pinned(fkg_ctx* ctx, size_t bytes) {
    if (bytes <= ctx->pin_bytes && ctx->pin) return FKG_OK;
    if (ctx->pin) cudaFreeHost(ctx->pin);
    ctx->pin = nullptr;
    ctx->pin_bytes = 0;
    cudaError_t e = cudaMallocHost(&ctx->pin, bytes);
    if (e != cudaSuccess) {
        ctx->pin = nullptr;
        cudaGetLastError();
        return set_err(ctx, FKG_ERR_ALLOC, std::string("cudaMallocHost: ") + cudaGetErrorString(e));
    }
    ctx->pin_bytes = bytes;
    return FKG_OK;
}

// Lay out a batch: per-chain descriptor with vector offsets (spacing ld) and
// dense-workspace offsets (ld*ld each).
int make_layout(fkg_ctx* ctx, int batch, const int32_t* lattice_id, Layout& L) {
    if (batch <= 0) return set_err(ctx, FKG_ERR_ARG, "batch must be positive");
    if (!lattice_id) return set_err(ctx, FKG_ERR_ARG, "lattice_id is NULL");
    L.batch = batch;
    L.desc.resize(batch);
    L.n_total = 0;
    L.v_total = 0;
    L.a_total = 0;
    L.max_n = 0;
    L.max_ld = 0;
    L.min_n = 1 << 30;
    for (int c = 0; c < batch; ++c) {
        int id = lattice_id[c];
        if (id < 0 || id >= kMaxLattices || ctx->lat[id].n <= 0)
            return set_err(ctx, FKG_ERR_ARG, "lattice id " + std::to_string(id) + " is not registered");
        const LatticeDev& lt = ctx->lat[id];
        ChainDesc& d = L.desc[c];
        d.n = lt.n;
        d.ld = round_ld(lt.n);
        d.lattice = id;
        d.pad = 0;
        d.a_off = L.a_total;
        d.v_off = L.v_total;
        d.rowptr = lt.rowptr;
        d.col = lt.col;
        d.val = lt.val;
        d.valf = lt.valf;
        L.a_total += (long long)d.ld * d.ld;
        L.v_total += d.ld;
        L.n_total += d.n;
        if (d.n > L.max_n) L.max_n = d.n;
        if (d.n < L.min_n) L.min_n = d.n;
        if (d.ld > L.max_ld) L.max_ld = d.ld;
    }
    L.order.resize(batch);
    for (int c = 0; c < batch; ++c) L.order[c] = c;
    std::stable_sort(L.order.begin(), L.order.end(), [&](int x, int y) { return L.desc[x].n > L.desc[y].n; });
    return FKG_OK;
}

// Descriptors and the work list of a layout to the device (async on ctx->st).
int upload_layout(fkg_ctx* ctx, Workspace& ws, const Layout& L) {
    FKG_CUDA(ctx, cudaMemcpyAsync(ws.desc.p, L.desc.data(), sizeof(ChainDesc) * L.batch, cudaMemcpyHostToDevice, ctx->st));
    FKG_CUDA(ctx, cudaMemcpyAsync(ws.order.p, L.order.data(), sizeof(int) * L.batch, cudaMemcpyHostToDevice, ctx->st));
    return FKG_OK;
}

// Variant of the reduction: the tuning entry of the size bucket that carries
// most of the batch's n^3 work (defaults: NB = 8 FP32, 4 FP64). The two-stage
// reduction runs for a whole batch, so it is taken only where every chain's
// bucket selects it: a batch that also holds smaller chains keeps the
// one-stage kernel, whose persistent longest-first schedule balances them
// (measured on the uneven batch of n = 144 .. 1024: 14.7k against 12.7k
// proposals/s).
static int pick_variant(const fkg_ctx* ctx, const Layout& L, bool f32) {
    double work[17] = {0};
    for (const ChainDesc& d : L.desc) work[std::min(16, (d.n + 63) / 64)] += (double)d.n * d.n * d.n;
    int best = 0;
    for (int b = 1; b < 17; ++b)
        if (work[b] > work[best]) best = b;
    const int v = f32 ? ctx->tune_f32[best] : ctx->tune_f64[best];
    if (f32 && v == kTwoStageVariant)
        for (const ChainDesc& d : L.desc)
            if (ctx->tune_f32[std::min(16, (d.n + 63) / 64)] != kTwoStageVariant) return 1;
    return v >= 0 ? v : 1;
}

// Back-transformation kernel of the mixed path (0: mma.sync, backtransform_tc.cu;
// 1: tcgen05, backtransform_tc5.cu) for the size bucket with most of the work.
static int pick_bt(const fkg_ctx* ctx, const Layout& L) {
    double work[17] = {0};
    for (const ChainDesc& d : L.desc) work[std::min(16, (d.n + 63) / 64)] += (double)d.n * d.n * d.n;
    int best = 0;
    for (int b = 1; b < 17; ++b)
        if (work[b] > work[best]) best = b;
    return ctx->tune_bt[best] >= 0 ? ctx->tune_bt[best] : 0;
}

// Device buffers for one batched solve on `ws`.
int ensure_solve_ws(fkg_ctx* ctx, Workspace& ws, const Layout& L, bool need_vecs) {
    int rc;
    const size_t V = (size_t)L.v_total;
    if ((rc = ensure_dev(ctx, ws.desc, sizeof(ChainDesc) * L.batch))) return rc;
    if ((rc = ensure_dev(ctx, ws.order, sizeof(int) * L.batch))) return rc;
    if ((rc = ensure_dev(ctx, ws.counter, sizeof(int)))) return rc;
    if ((rc = ensure_dev(ctx, ws.A, sizeof(double) * (size_t)L.a_total))) return rc;
    if ((rc = ensure_dev(ctx, ws.diag, sizeof(double) * V))) return rc;
    if ((rc = ensure_dev(ctx, ws.d, sizeof(double) * V))) return rc;
    if ((rc = ensure_dev(ctx, ws.e, sizeof(double) * V))) return rc;
    if ((rc = ensure_dev(ctx, ws.tau, sizeof(double) * V))) return rc;
    if ((rc = ensure_dev(ctx, ws.w, sizeof(double) * V))) return rc;
    if ((rc = ensure_dev(ctx, ws.beta, sizeof(double) * L.batch))) return rc;
    if ((rc = ensure_dev(ctx, ws.logz, sizeof(double) * L.batch))) return rc;
    if (need_vecs) {
        if ((rc = ensure_dev(ctx, ws.exp_e, sizeof(double) * V))) return rc;
        if ((rc = ensure_dev(ctx, ws.fermi, sizeof(double) * V))) return rc;
    }
    if (ctx->precision == FKG_PREC_MIXED) {
        if ((rc = ensure_dev(ctx, ws.A32, sizeof(float) * (size_t)L.a_total))) return rc;
        if ((rc = ensure_dev(ctx, ws.Z, sizeof(float) * (size_t)L.a_total))) return rc;
        if ((rc = ensure_dev(ctx, ws.aux32, sizeof(float) * V))) return rc;
        if ((rc = ensure_dev(ctx, ws.Tf, sizeof(float) * 32 * V))) return rc;
        if ((rc = ensure_dev(ctx, ws.aux64, sizeof(double) * V))) return rc;
        if ((rc = ensure_dev(ctx, ws.perm, sizeof(int) * V))) return rc;
        if ((rc = ensure_dev(ctx, ws.VT, sizeof(float) * 4 * (size_t)L.a_total))) return rc;  // split V T and V
        if ((rc = ensure_dev(ctx, ws.zsc, sizeof(float) * V))) return rc;
        if ((rc = ensure_dev(ctx, ws.ctol, sizeof(double) * L.batch))) return rc;
        // two-stage reduction: the band stage's reflectors ([ld][ld] per chain) and their tau
        if ((rc = ensure_dev(ctx, ws.Q2, sizeof(float) * (size_t)(L.a_total + L.a_total / kBand)))) return rc;
        if ((rc = ensure_dev(ctx, ws.S1, sizeof(float) * (size_t)sy2sb_scratch_floats(L.max_ld) * L.batch))) return rc;
        if ((rc = ensure_dev(ctx, ws.TM, sy2sb_tensor_map_bytes() * L.batch))) return rc;
    }
    return FKG_OK;
}

// The first stage's tensor maps (one per chain over its A32 matrix) into ws.TM,
// encoded on the host when the A32 buffer or the layout changed since the last
// upload (a graph captured afterwards replays the upload from ws.tm_host).
static int upload_tensor_maps(fkg_ctx* ctx, Workspace& ws, const Layout& L) {
    std::vector<long long> key;
    key.reserve(1 + 2 * (size_t)L.batch);
    key.push_back((long long)(uintptr_t)ws.A32.p);
    for (const ChainDesc& d : L.desc) {
        key.push_back(d.a_off);
        key.push_back(d.ld);
    }
    if (key == ws.tm_key) return FKG_OK;
    const size_t mb = sy2sb_tensor_map_bytes();
    ws.tm_host.assign(mb * L.batch + 64, 0);
    unsigned char* h = ws.tm_host.data();
    h += (64 - (uintptr_t)h % 64) % 64;  // the encoder writes 64-byte aligned maps
    const cudaError_t e = sy2sb_tensor_maps(L.desc.data(), L.batch, (float*)ws.A32.p, h);
    if (e != cudaSuccess) {
        ws.tm_key.clear();
        return set_err(ctx, FKG_ERR_CUDA, std::string("tensor maps of the two-stage reduction: ") + cudaGetErrorString(e));
    }
    FKG_CUDA(ctx, cudaMemcpyAsync(ws.TM.p, h, mb * L.batch, cudaMemcpyHostToDevice, ctx->st));
    ws.tm_key = std::move(key);
    return FKG_OK;
}

static void stage_cb(void* c, int stage, int end) {
    if (end) stage_end((fkg_ctx*)c, stage);
    else stage_begin((fkg_ctx*)c, stage);
}

// Enqueue one batched eigenvalue solve + logZ on ctx->st. Inputs already on the
// device in ws.desc / ws.diag / ws.beta.
int enqueue_solve(fkg_ctx* ctx, Workspace& ws, const Layout& L, bool want_exp, const StepIO* io) {
    const ChainDesc* dd = (const ChainDesc*)ws.desc.p;
    double* A = (double*)ws.A.p;
    bool two_stage = false;
    if (ctx->precision == FKG_PREC_F64) {
        stage_begin(ctx, FKG_STAGE_REDUCE);
        FKG_CUDA(ctx, launch_sytrd_v3_f64(dd, L.batch, L.max_ld, (const double*)ws.diag.p, A, (double*)ws.d.p,
                                          (double*)ws.e.p, (double*)ws.tau.p, ctx->st, pick_variant(ctx, L, false),
                                          (const int*)ws.order.p, (int*)ws.counter.p, ctx->num_sms,
                                          (int*)ctx->status.p));
        stage_end(ctx, FKG_STAGE_REDUCE);
        ctx->launches++;
    } else {
        if (!ws.A32.p || !ws.Z.p || !ws.Tf.p || !ws.VT.p || !ws.zsc.p || !ws.Q2.p || !ws.S1.p)
            return set_err(ctx, FKG_ERR_STATE, "mixed workspace not allocated");
        two_stage = pick_variant(ctx, L, true) == kTwoStageVariant;
        if (two_stage) {
            const int rc = upload_tensor_maps(ctx, ws, L);
            if (rc) return rc;
        }
        stage_begin(ctx, FKG_STAGE_REDUCE);
        if (two_stage) {  // dense -> band -> tridiagonal
            FKG_CUDA(ctx, launch_sy2sb(dd, L.batch, L.max_ld, (const double*)ws.diag.p, (float*)ws.A32.p,
                                       (float*)ws.aux32.p, (const int*)ws.order.p, (int*)ws.counter.p, ctx->num_sms,
                                       (int*)ctx->status.p, (float*)ws.S1.p, ws.TM.p, ctx->wait_iters, ctx->st));
            FKG_CUDA(ctx, launch_sb2st(dd, L.batch, L.max_n, (const float*)ws.A32.p, (double*)ws.d.p,
                                       (double*)ws.e.p, (float*)ws.Q2.p, L.a_total, ctx->st));
            ctx->launches += 2;
        } else {
            FKG_CUDA(ctx, launch_sytrd_v3_f32(dd, L.batch, L.max_ld, (const double*)ws.diag.p, (float*)ws.A32.p,
                                              (double*)ws.d.p, (double*)ws.e.p, (float*)ws.aux32.p, ctx->st,
                                              pick_variant(ctx, L, true), (const int*)ws.order.p, (int*)ws.counter.p,
                                              ctx->num_sms, (int*)ctx->status.p));
            ctx->launches++;
        }
        stage_end(ctx, FKG_STAGE_REDUCE);
        // larft + V T on the second stream, joined before the back-transformation
        FKG_CUDA(ctx, cudaEventRecord(ctx->ev_red, ctx->st));
        FKG_CUDA(ctx, cudaStreamWaitEvent(ctx->aux_st, ctx->ev_red, 0));
        FKG_CUDA(ctx, launch_larft_vt(dd, L.batch, L.max_n, (const float*)ws.A32.p, (const float*)ws.aux32.p,
                                      (float*)ws.Tf.p, (float*)ws.VT.p, L.a_total, two_stage ? kBand : 1,
                                      ctx->aux_st));
        FKG_CUDA(ctx, cudaEventRecord(ctx->ev_larft, ctx->aux_st));
        ctx->launches++;
    }
    stage_begin(ctx, FKG_STAGE_TRIEIG);
    if (ctx->precision == FKG_PREC_F64) {
        FKG_CUDA(ctx, launch_trieig_values(dd, L.batch, L.max_n, L.max_ld, (const double*)ws.d.p,
                                           (const double*)ws.e.p, (double*)ws.w.p, (int*)ctx->status.p, ctx->st));
        ctx->launches++;
    } else {
        FKG_CUDA(ctx, launch_trieig_shifts(dd, L.batch, L.max_n, L.max_ld, (const double*)ws.d.p,
                                           (const double*)ws.e.p, (double*)ws.w.p, (double*)ws.ctol.p,
                                           (int*)ctx->status.p, ctx->st));
        ctx->launches++;
    }
    stage_end(ctx, FKG_STAGE_TRIEIG);
    if (ctx->precision == FKG_PREC_MIXED) {
        FKG_CUDA(ctx, launch_mixed_refine(dd, L.batch, L.max_n, L.max_ld, (const double*)ws.diag.p,
                                          (const float*)ws.A32.p, (const float*)ws.VT.p, L.a_total, (const double*)ws.d.p,
                                          (const double*)ws.e.p, (double*)ws.w.p, (const double*)ws.ctol.p,
                                          (float*)ws.Z.p, (float*)ws.zsc.p, (double*)ws.aux64.p, (int*)ws.perm.p,
                                          A /* the FP64 matrix workspace is idle on this path: cluster scratch */,
                                          (int*)ctx->status.p, ctx->st, ctx->aux2_st, ctx->ev_fork, ctx->ev_join,
                                          ctx->ev_larft, pick_bt(ctx, L), ctx->wait_iters, two_stage ? kBand : 1,
                                          two_stage ? (const float*)ws.Q2.p : nullptr, L.a_total, stage_cb, ctx));
        ctx->launches += two_stage ? 6 : 5;  // cluster fix-up, twisted, (band stage,) back-transformation, refine, sort
    }
    stage_begin(ctx, FKG_STAGE_LOGZ);
    if (io)  // the proposal step: logZ, decision and state update in one launch
        FKG_CUDA(ctx, launch_logz_accept(dd, L.batch, (const double*)ws.w.p, (const double*)ws.beta.p,
                                         (double*)ws.logz.p, io->site, io->u, (const double*)ctx->ch_ebmf.p,
                                         (int32_t*)ctx->ch_f.p, (double*)ctx->ch_logz_cur.p,
                                         (double*)ctx->ch_w_cur.p, io->acc, io->dl, (int*)ctx->status.p, ctx->st,
                                         io->step));
    else
        FKG_CUDA(ctx, launch_logz(dd, L.batch, L.max_n, (const double*)ws.w.p, (const double*)ws.beta.p,
                                  (double*)ws.logz.p, want_exp ? (double*)ws.exp_e.p : nullptr,
                                  want_exp ? (double*)ws.fermi.p : nullptr, (int*)ctx->status.p, ctx->st));
    stage_end(ctx, FKG_STAGE_LOGZ);
    ctx->launches++;
    return FKG_OK;
}

void stage_begin(fkg_ctx* ctx, int stage) {
    if (!ctx->profiling) return;
    StageTimer& t = ctx->timers[stage];
    while (t.ev.size() < t.used + 2) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) { cudaGetLastError(); return; }
        t.ev.push_back(e);
    }
    cudaEventRecord(t.ev[t.used], ctx->st);
}

void stage_end(fkg_ctx* ctx, int stage) {
    if (!ctx->profiling) return;
    StageTimer& t = ctx->timers[stage];
    if (t.ev.size() < t.used + 2) return;
    cudaEventRecord(t.ev[t.used + 1], ctx->st);
    t.used += 2;
    t.launches++;
}

int check_status(fkg_ctx* ctx) {
    int h = 0;
    FKG_CUDA(ctx, cudaMemcpyAsync(&h, ctx->status.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
    FKG_CUDA(ctx, cudaStreamSynchronize(ctx->st));
    if (h & kStatusNaN) return set_err(ctx, FKG_ERR_NUMERIC, "NaN or Inf in eigenvalues or logZ");
    if (h & kStatusNoConverge) return set_err(ctx, FKG_ERR_NUMERIC, "an eigenvalue iteration did not converge");
    if (h & kStatusTimeout) return set_err(ctx, FKG_ERR_TIMEOUT, "a bounded device wait ran out");
    if (h & kStatusBadArg) return set_err(ctx, FKG_ERR_ARG, "a device-side argument check failed");
    return FKG_OK;
}

}  // namespace fkg

extern "C" {

fkg_ctx* fkg_create(int max_n, int max_batch, unsigned flags) {
    if (max_n < 0 || max_batch < 0) return nullptr;
    fkg_ctx* ctx = new (std::nothrow) fkg_ctx();
    if (!ctx) return nullptr;
    ctx->max_n = max_n;
    ctx->max_batch = max_batch;
    ctx->flags = flags;
    // Stream priorities: the step's own stream and the cluster fix-up's (both on
    // the path to the back-transformation) high; larft's lowest, so that its
    // CTAs fill the SMs the shifts and the twisted factorisation leave free
    // (it only has to finish before the back-transformation)
    int prio_low = 0, prio_high = 0;
    if (cudaGetDevice(&ctx->device) != cudaSuccess ||
        cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, ctx->device) != cudaSuccess ||
        cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high) != cudaSuccess ||
        cudaStreamCreateWithPriority(&ctx->own_st, cudaStreamNonBlocking, prio_high) != cudaSuccess) {
        cudaGetLastError();
        delete ctx;
        return nullptr;
    }
    ctx->st = ctx->own_st;
    if (cudaStreamCreateWithPriority(&ctx->aux_st, cudaStreamNonBlocking, prio_low) != cudaSuccess ||
        cudaStreamCreateWithPriority(&ctx->aux2_st, cudaStreamNonBlocking, prio_high) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_red, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_larft, cudaEventDisableTiming) != cudaSuccess ||
        ensure_dev(ctx, ctx->status, sizeof(int)) != FKG_OK) {
        cudaGetLastError();
        for (cudaEvent_t ev : {ctx->ev_fork, ctx->ev_join, ctx->ev_red, ctx->ev_larft})
            if (ev) cudaEventDestroy(ev);
        if (ctx->aux_st) cudaStreamDestroy(ctx->aux_st);
        if (ctx->aux2_st) cudaStreamDestroy(ctx->aux2_st);
        cudaStreamDestroy(ctx->own_st);
        delete ctx;
        return nullptr;
    }
    return ctx;
}

void fkg_destroy(fkg_ctx* ctx) {
    if (!ctx) return;
    cudaStreamSynchronize(ctx->st);
    for (auto& l : ctx->lat) l.free_all();
    for (DevBuf* b : ctx->all_buffers()) if (b->p) cudaFree(b->p);
    if (ctx->pin) cudaFreeHost(ctx->pin);
    for (auto& t : ctx->timers)
        for (cudaEvent_t e : t.ev) cudaEventDestroy(e);
    ctx->drop_graph();
    cudaStreamSynchronize(ctx->own_st);
    cudaStreamSynchronize(ctx->aux_st);
    cudaStreamSynchronize(ctx->aux2_st);
    for (cudaEvent_t ev : {ctx->ev_fork, ctx->ev_join, ctx->ev_red, ctx->ev_larft}) cudaEventDestroy(ev);
    cudaStreamDestroy(ctx->aux_st);
    cudaStreamDestroy(ctx->aux2_st);
    cudaStreamDestroy(ctx->own_st);
    delete ctx;
}

int fkg_set_tuning(fkg_ctx* ctx, int precision, int n_max, int variant) {
    if (!ctx) return FKG_ERR_ARG;
    if (precision != FKG_PREC_F64 && precision != FKG_PREC_MIXED) return set_err(ctx, FKG_ERR_ARG, "unknown precision");
    if (n_max < 1 || n_max > kMaxN) return set_err(ctx, FKG_ERR_ARG, "n_max out of range");
    // mixed: 0..2 the one-stage panel widths, 3 the two-stage reduction (band kBand)
    const int nvar = precision == FKG_PREC_MIXED ? kMixedVariants : 2;
    if (variant < -1 || variant >= nvar) return set_err(ctx, FKG_ERR_ARG, "variant out of range");
    (precision == FKG_PREC_MIXED ? ctx->tune_f32 : ctx->tune_f64)[std::min(16, (n_max + 63) / 64)] = variant;
    ctx->drop_graph();
    return FKG_OK;
}

int fkg_set_tuning_back(fkg_ctx* ctx, int n_max, int variant) {
    if (!ctx) return FKG_ERR_ARG;
    if (n_max < 1 || n_max > kMaxN) return set_err(ctx, FKG_ERR_ARG, "n_max out of range");
    if (variant < -1 || variant > 1) return set_err(ctx, FKG_ERR_ARG, "variant out of range");
    ctx->tune_bt[std::min(16, (n_max + 63) / 64)] = variant;
    ctx->drop_graph();
    return FKG_OK;
}

int fkg_set_wait_limit(fkg_ctx* ctx, long long iters) {
    if (!ctx) return FKG_ERR_ARG;
    ctx->wait_iters = iters < 0 ? kDefaultWaitIters : iters;
    ctx->drop_graph();  // the limit is a kernel argument of the captured step
    return FKG_OK;
}

int fkg_set_graphs(fkg_ctx* ctx, int enable) {
    if (!ctx) return FKG_ERR_ARG;
    FKG_CUDA(ctx, cudaStreamSynchronize(ctx->st));
    ctx->use_graphs = enable != 0;
    ctx->drop_graph();
    return FKG_OK;
}

int fkg_set_stream(fkg_ctx* ctx, void* cuda_stream) {
    if (!ctx) return FKG_ERR_ARG;
    FKG_CUDA(ctx, cudaStreamSynchronize(ctx->st));
    ctx->st = cuda_stream ? (cudaStream_t)cuda_stream : ctx->own_st;
    return FKG_OK;
}

int fkg_profile(fkg_ctx* ctx, int enable) {
    if (!ctx) return FKG_ERR_ARG;
    FKG_CUDA(ctx, cudaStreamSynchronize(ctx->st));
    for (auto& t : ctx->timers) {
        t.used = 0;
        t.acc_ms = 0.0;
        t.launches = 0;
    }
    ctx->profiling = enable != 0;
    return FKG_OK;
}

int fkg_stage_time(fkg_ctx* ctx, int stage, double* total_ms, long long* launches) {
    if (!ctx) return FKG_ERR_ARG;
    if (stage < 0 || stage >= FKG_NUM_STAGES) return set_err(ctx, FKG_ERR_ARG, "unknown stage");
    StageTimer& t = ctx->timers[stage];
    for (size_t i = 0; i + 1 < t.used; i += 2) {
        FKG_CUDA(ctx, cudaEventSynchronize(t.ev[i + 1]));
        float ms = 0.f;
        FKG_CUDA(ctx, cudaEventElapsedTime(&ms, t.ev[i], t.ev[i + 1]));
        t.acc_ms += ms;
    }
    t.used = 0;
    if (total_ms) *total_ms = t.acc_ms;
    if (launches) *launches = t.launches;
    return FKG_OK;
}

const char* fkg_last_error(const fkg_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

long long fkg_launch_count(const fkg_ctx* ctx) { return ctx ? ctx->launches : 0; }

int fkg_set_precision(fkg_ctx* ctx, int precision) {
    if (!ctx) return FKG_ERR_ARG;
    if (precision != FKG_PREC_F64 && precision != FKG_PREC_MIXED) return set_err(ctx, FKG_ERR_ARG, "unknown precision");
    if (ctx->precision != precision) ctx->drop_graph();
    ctx->precision = precision;
    return FKG_OK;
}

int fkg_set_hopping(fkg_ctx* ctx, int lattice_id, int n, const int32_t* rowptr, const int32_t* col,
                    const double* val) {
    if (!ctx) return FKG_ERR_ARG;
    if (lattice_id < 0 || lattice_id >= kMaxLattices) return set_err(ctx, FKG_ERR_ARG, "lattice_id out of range");
    if (n <= 0 || n > kMaxN) return set_err(ctx, FKG_ERR_ARG, "n out of range (1.." + std::to_string(kMaxN) + ")");
    if (!rowptr || (!col && rowptr[n] > 0) || (!val && rowptr[n] > 0)) return set_err(ctx, FKG_ERR_ARG, "null CSR array");
    const int nnz = rowptr[n];
    if (rowptr[0] != 0 || nnz < 0) return set_err(ctx, FKG_ERR_ARG, "bad rowptr");
    for (int i = 0; i < n; ++i)
        if (rowptr[i + 1] < rowptr[i]) return set_err(ctx, FKG_ERR_ARG, "rowptr not monotone");
    for (int p = 0; p < nnz; ++p) {
        if (col[p] < 0 || col[p] >= n) return set_err(ctx, FKG_ERR_ARG, "column index out of range");
        if (!(val[p] == val[p]) || val[p] - val[p] != 0.0) return set_err(ctx, FKG_ERR_NUMERIC, "NaN/Inf in hopping");
    }
    LatticeDev& l = ctx->lat[lattice_id];
    l.free_all();
    l = LatticeDev();
    l.h_rowptr.assign(rowptr, rowptr + n + 1);
    l.h_col.assign(col, col + nnz);
    l.h_val.assign(val, val + nnz);
    FKG_CUDA(ctx, cudaMalloc(&l.rowptr, sizeof(int32_t) * (n + 1)));
    FKG_CUDA(ctx, cudaMalloc(&l.col, sizeof(int32_t) * (nnz > 0 ? nnz : 1)));
    FKG_CUDA(ctx, cudaMalloc(&l.val, sizeof(double) * (nnz > 0 ? nnz : 1)));
    FKG_CUDA(ctx, cudaMalloc(&l.valf, sizeof(float2) * (nnz > 0 ? nnz : 1)));
    FKG_CUDA(ctx, cudaMemcpy(l.rowptr, rowptr, sizeof(int32_t) * (n + 1), cudaMemcpyHostToDevice));
    if (nnz > 0) {
        std::vector<float2> vf(nnz);
        for (int p = 0; p < nnz; ++p) {
            const float hi = (float)val[p];
            vf[p] = make_float2(hi, (float)(val[p] - (double)hi));
        }
        FKG_CUDA(ctx, cudaMemcpy(l.col, col, sizeof(int32_t) * nnz, cudaMemcpyHostToDevice));
        FKG_CUDA(ctx, cudaMemcpy(l.val, val, sizeof(double) * nnz, cudaMemcpyHostToDevice));
        FKG_CUDA(ctx, cudaMemcpy(l.valf, vf.data(), sizeof(float2) * nnz, cudaMemcpyHostToDevice));
    }
    l.n = n;
    l.nnz = nnz;
    ctx->chains_ready = false;  // descriptors of existing chains point at the old arrays
    return FKG_OK;
}

int fkg_eigh_logz(fkg_ctx* ctx, int batch, const int32_t* lattice_id, const double* diag, const double* beta,
                  double* evals, double* exp_e, double* fermi, double* evecs, double* logz) {
    if (!ctx) return FKG_ERR_ARG;
    if (!diag || !beta) return set_err(ctx, FKG_ERR_ARG, "diag/beta is NULL");
    if (evecs) return eigh_vectors(ctx, batch, lattice_id, diag, beta, evals, exp_e, fermi, evecs, logz);
    Layout& L = ctx->solve_layout;
    int rc;
    if ((rc = make_layout(ctx, batch, lattice_id, L))) return rc;
    const bool want_exp = exp_e || fermi;
    if ((rc = ensure_solve_ws(ctx, ctx->solve, L, want_exp))) return rc;
    const size_t V = (size_t)L.v_total;
    // pinned staging: diag (V) + beta (batch) in; evals, exp, fermi (3V) + logz (batch) out
    if ((rc = ensure_pinned(ctx, sizeof(double) * (4 * V + 2 * batch)))) return rc;
    double* hin = (double*)ctx->pin;
    double* hb = hin + V;
    double* hout = hb + batch;
    long long src = 0;
    for (int c = 0; c < batch; ++c) {
        const ChainDesc& d = L.desc[c];
        for (int i = 0; i < d.ld; ++i) hin[d.v_off + i] = i < d.n ? diag[src + i] : 0.0;
        if (!(beta[c] > 0.0) || beta[c] - beta[c] != 0.0) return set_err(ctx, FKG_ERR_ARG, "beta must be finite and > 0");
        hb[c] = beta[c];
        src += d.n;
    }
    FKG_CUDA(ctx, cudaMemsetAsync(ctx->status.p, 0, sizeof(int), ctx->st));
    if ((rc = upload_layout(ctx, ctx->solve, L))) return rc;
    FKG_CUDA(ctx, cudaMemcpyAsync(ctx->solve.diag.p, hin, sizeof(double) * V, cudaMemcpyHostToDevice, ctx->st));
    FKG_CUDA(ctx, cudaMemcpyAsync(ctx->solve.beta.p, hb, sizeof(double) * batch, cudaMemcpyHostToDevice, ctx->st));
    if ((rc = enqueue_solve(ctx, ctx->solve, L, want_exp))) return rc;
    double* ow = hout;
    double* oe = ow + V;
    double* of = oe + V;
    double* oz = of + V;
    if (evals) FKG_CUDA(ctx, cudaMemcpyAsync(ow, ctx->solve.w.p, sizeof(double) * V, cudaMemcpyDeviceToHost, ctx->st));
    if (exp_e) FKG_CUDA(ctx, cudaMemcpyAsync(oe, ctx->solve.exp_e.p, sizeof(double) * V, cudaMemcpyDeviceToHost, ctx->st));
    if (fermi) FKG_CUDA(ctx, cudaMemcpyAsync(of, ctx->solve.fermi.p, sizeof(double) * V, cudaMemcpyDeviceToHost, ctx->st));
    FKG_CUDA(ctx, cudaMemcpyAsync(oz, ctx->solve.logz.p, sizeof(double) * batch, cudaMemcpyDeviceToHost, ctx->st));
    if ((rc = check_status(ctx))) return rc;
    long long dst = 0;
    for (int c = 0; c < batch; ++c) {
        const ChainDesc& d = L.desc[c];
        if (evals) std::memcpy(evals + dst, ow + d.v_off, sizeof(double) * d.n);
        if (exp_e) std::memcpy(exp_e + dst, oe + d.v_off, sizeof(double) * d.n);
        if (fermi) std::memcpy(fermi + dst, of + d.v_off, sizeof(double) * d.n);
        if (logz) logz[c] = oz[c];
        dst += d.n;
    }
    return FKG_OK;
}

int fkg_chains_init(fkg_ctx* ctx, int batch, const int32_t* lattice_id, const int32_t* f, const double* U,
                    const double* mu_c, const double* mu_f, const double* beta) {
    if (!ctx) return FKG_ERR_ARG;
    if (!f || !U || !mu_c || !mu_f || !beta) return set_err(ctx, FKG_ERR_ARG, "null chain parameter array");
    ctx->chains_ready = false;
    ctx->drop_graph();
    Layout& L = ctx->chain_layout;
    int rc;
    if ((rc = make_layout(ctx, batch, lattice_id, L))) return rc;
    Workspace& ws = ctx->chain;
    if ((rc = ensure_solve_ws(ctx, ws, L, false))) return rc;
    const size_t V = (size_t)L.v_total;
    if ((rc = ensure_dev(ctx, ctx->ch_f, sizeof(int32_t) * V))) return rc;
    if ((rc = ensure_dev(ctx, ctx->ch_U, sizeof(double) * batch))) return rc;
    if ((rc = ensure_dev(ctx, ctx->ch_mu_c, sizeof(double) * batch))) return rc;
    if ((rc = ensure_dev(ctx, ctx->ch_ebmf, sizeof(double) * batch))) return rc;
    if ((rc = ensure_dev(ctx, ctx->ch_logz_cur, sizeof(double) * batch))) return rc;
    if ((rc = ensure_dev(ctx, ctx->ch_w_cur, sizeof(double) * V))) return rc;
    if ((rc = ensure_pinned(ctx, sizeof(double) * (4 * (size_t)batch) + sizeof(int32_t) * V))) return rc;
    double* hU = (double*)ctx->pin;
    double* hmu = hU + batch;
    double* heb = hmu + batch;
    double* hbeta = heb + batch;
    int32_t* hf = (int32_t*)(hbeta + batch);
    long long src = 0;
    for (int c = 0; c < batch; ++c) {
        const ChainDesc& d = L.desc[c];
        for (int i = 0; i < d.ld; ++i) {
            int fi = i < d.n ? f[src + i] : 0;
            if (fi != 0 && fi != 1) return set_err(ctx, FKG_ERR_ARG, "f occupations must be 0 or 1");
            hf[d.v_off + i] = fi;
        }
        src += d.n;
        if (!(beta[c] > 0.0) || beta[c] - beta[c] != 0.0) return set_err(ctx, FKG_ERR_ARG, "beta must be finite and > 0");
        hU[c] = U[c];
        hmu[c] = mu_c[c];
        heb[c] = std::exp(beta[c] * mu_f[c]);  // move_addremove::exp_beta_mu_f (include/fk_mc/moves.hpp:44)
        hbeta[c] = beta[c];
    }
    cudaStream_t st = ctx->st;
    FKG_CUDA(ctx, cudaMemsetAsync(ctx->status.p, 0, sizeof(int), st));
    if ((rc = upload_layout(ctx, ws, L))) return rc;
    FKG_CUDA(ctx, cudaMemcpyAsync(ctx->ch_f.p, hf, sizeof(int32_t) * V, cudaMemcpyHostToDevice, st));
    FKG_CUDA(ctx, cudaMemcpyAsync(ctx->ch_U.p, hU, sizeof(double) * batch, cudaMemcpyHostToDevice, st));
    FKG_CUDA(ctx, cudaMemcpyAsync(ctx->ch_mu_c.p, hmu, sizeof(double) * batch, cudaMemcpyHostToDevice, st));
    FKG_CUDA(ctx, cudaMemcpyAsync(ctx->ch_ebmf.p, heb, sizeof(double) * batch, cudaMemcpyHostToDevice, st));
    FKG_CUDA(ctx, cudaMemcpyAsync(ws.beta.p, hbeta, sizeof(double) * batch, cudaMemcpyHostToDevice, st));
    // current configuration: diag, solve, keep logZ and spectrum
    FKG_CUDA(ctx, launch_proposal_diag((const ChainDesc*)ws.desc.p, batch, L.max_n, (const int32_t*)ctx->ch_f.p,
                                       nullptr, (const double*)ctx->ch_U.p, (const double*)ctx->ch_mu_c.p,
                                       (double*)ws.diag.p, (int*)ctx->status.p, st));
    ctx->launches++;
    if (ctx->method == FKG_METHOD_CHEBYSHEV) {
        if ((rc = prepare_kpm(ctx, ws, L))) return rc;
        if ((rc = enqueue_kpm(ctx, ws, L, nullptr))) return rc;
        FKG_CUDA(ctx, cudaMemsetAsync(ctx->ch_w_cur.p, 0, sizeof(double) * V, st));  // no spectrum kept
    } else {
        if ((rc = enqueue_solve(ctx, ws, L, false))) return rc;
        FKG_CUDA(ctx, cudaMemcpyAsync(ctx->ch_w_cur.p, ws.w.p, sizeof(double) * V, cudaMemcpyDeviceToDevice, st));
    }
    FKG_CUDA(ctx, cudaMemcpyAsync(ctx->ch_logz_cur.p, ws.logz.p, sizeof(double) * batch, cudaMemcpyDeviceToDevice, st));
    if ((rc = check_status(ctx))) return rc;
    ctx->chains_ready = true;
    return FKG_OK;
}

int fkg_propose_accept_device(fkg_ctx* ctx, int nsteps, const int32_t* d_site, const double* d_u,
                              int32_t* d_accepted, double* d_dlogz) {
    if (!ctx) return FKG_ERR_ARG;
    if (!ctx->chains_ready) return set_err(ctx, FKG_ERR_STATE, "fkg_chains_init has not been called");
    if (nsteps < 0 || !d_site || !d_u || !d_accepted || !d_dlogz) return set_err(ctx, FKG_ERR_ARG, "bad step arguments");
    int rc = enqueue_steps(ctx, nsteps, d_site, d_u, d_accepted, d_dlogz);
    if (rc) return rc;
    return check_status(ctx);
}

int fkg_propose_accept(fkg_ctx* ctx, int nsteps, const int32_t* site, const double* u, int32_t* accepted,
                       double* dlogz) {
    if (!ctx) return FKG_ERR_ARG;
    if (!ctx->chains_ready) return set_err(ctx, FKG_ERR_STATE, "fkg_chains_init has not been called");
    if (nsteps < 0 || !site || !u) return set_err(ctx, FKG_ERR_ARG, "bad step arguments");
    const Layout& L = ctx->chain_layout;
    const int B = L.batch;
    const size_t tot = (size_t)nsteps * B;
    for (size_t k = 0; k < tot; ++k) {
        const int c = (int)(k % B);
        if (site[k] < 0 || site[k] >= L.desc[c].n) return set_err(ctx, FKG_ERR_ARG, "site index out of range");
    }
    int rc;
    // a captured step graph holds the addresses of these buffers: drop it if one moves
    const void* old[4] = {ctx->st_site.p, ctx->st_u.p, ctx->st_acc.p, ctx->st_dlogz.p};
    if ((rc = ensure_dev(ctx, ctx->st_site, sizeof(int32_t) * tot))) return rc;
    if ((rc = ensure_dev(ctx, ctx->st_u, sizeof(double) * tot))) return rc;
    if ((rc = ensure_dev(ctx, ctx->st_acc, sizeof(int32_t) * tot))) return rc;
    if ((rc = ensure_dev(ctx, ctx->st_dlogz, sizeof(double) * tot))) return rc;
    if (old[0] != ctx->st_site.p || old[1] != ctx->st_u.p || old[2] != ctx->st_acc.p || old[3] != ctx->st_dlogz.p)
        ctx->drop_graph();
    if ((rc = ensure_pinned(ctx, (sizeof(double) + sizeof(int32_t)) * 2 * tot + 64))) return rc;
    double* hu = (double*)ctx->pin;
    double* hd = hu + tot;
    int32_t* hs = (int32_t*)(hd + tot);
    int32_t* ha = hs + tot;
    std::memcpy(hs, site, sizeof(int32_t) * tot);
    std::memcpy(hu, u, sizeof(double) * tot);
    cudaStream_t st = ctx->st;
    FKG_CUDA(ctx, cudaMemcpyAsync(ctx->st_site.p, hs, sizeof(int32_t) * tot, cudaMemcpyHostToDevice, st));
    FKG_CUDA(ctx, cudaMemcpyAsync(ctx->st_u.p, hu, sizeof(double) * tot, cudaMemcpyHostToDevice, st));
    if ((rc = enqueue_steps(ctx, nsteps, (const int32_t*)ctx->st_site.p, (const double*)ctx->st_u.p,
                            (int32_t*)ctx->st_acc.p, (double*)ctx->st_dlogz.p)))
        return rc;
    FKG_CUDA(ctx, cudaMemcpyAsync(ha, ctx->st_acc.p, sizeof(int32_t) * tot, cudaMemcpyDeviceToHost, st));
    FKG_CUDA(ctx, cudaMemcpyAsync(hd, ctx->st_dlogz.p, sizeof(double) * tot, cudaMemcpyDeviceToHost, st));
    if ((rc = check_status(ctx))) return rc;
    if (accepted) std::memcpy(accepted, ha, sizeof(int32_t) * tot);
    if (dlogz) std::memcpy(dlogz, hd, sizeof(double) * tot);
    return FKG_OK;
}

int fkg_free_energy_grad(fkg_ctx* ctx, int batch, const int32_t* lattice_id, const int32_t* f, const double* U,
                         const double* mu_c, const double* t, const double* beta, double* F, double* dF_dU,
                         double* dF_dt, double* dF_dmu, double* dF_dbeta, double* rho) {
    if (!ctx) return FKG_ERR_ARG;
    if (!f || !U || !mu_c || !t || !beta) return set_err(ctx, FKG_ERR_ARG, "null parameter array");
    Layout& L = ctx->solve_layout;
    int rc;
    if ((rc = make_layout(ctx, batch, lattice_id, L))) return rc;
    Workspace& ws = ctx->solve;
    if ((rc = ensure_solve_ws(ctx, ws, L, false))) return rc;
    const size_t V = (size_t)L.v_total;
    if ((rc = ensure_dev(ctx, ws.fint, sizeof(int32_t) * V))) return rc;
    if ((rc = ensure_dev(ctx, ws.gout, sizeof(double) * 5 * batch))) return rc;
    if ((rc = ensure_dev(ctx, ws.fermiw, sizeof(double) * V))) return rc;
    if ((rc = ensure_dev(ctx, ws.Ulist, sizeof(double) * 3 * batch))) return rc;
    if (rho && (rc = ensure_dev(ctx, ws.rho, sizeof(double) * (size_t)L.a_total))) return rc;
    if ((rc = ensure_pinned(ctx, sizeof(double) * (V + 4 * (size_t)batch + 5 * (size_t)batch) + sizeof(int32_t) * V)))
        return rc;
    double* hdiag = (double*)ctx->pin;
    double* hb = hdiag + V;
    double* hprm = hb + batch;        // U, mu, t
    double* hout = hprm + 3 * batch;  // [batch][5]
    int32_t* hf = (int32_t*)(hout + 5 * batch);
    long long src = 0;
    for (int c = 0; c < batch; ++c) {
        const ChainDesc& d = L.desc[c];
        if (!(beta[c] > 0.0) || beta[c] - beta[c] != 0.0) return set_err(ctx, FKG_ERR_ARG, "beta must be finite and > 0");
        if (t[c] == 0.0) return set_err(ctx, FKG_ERR_ARG, "t must be nonzero (dF/dt divides by t)");
        for (int i = 0; i < d.ld; ++i) {
            const int fi = i < d.n ? f[src + i] : 0;
            if (fi != 0 && fi != 1) return set_err(ctx, FKG_ERR_ARG, "f occupations must be 0 or 1");
            hf[d.v_off + i] = fi;
            hdiag[d.v_off + i] = i < d.n ? -mu_c[c] + U[c] * fi : 0.0;
        }
        src += d.n;
        hb[c] = beta[c];
        hprm[c] = U[c];
        hprm[batch + c] = mu_c[c];
        hprm[2 * batch + c] = t[c];
    }
    cudaStream_t st = ctx->st;
    FKG_CUDA(ctx, cudaMemsetAsync(ctx->status.p, 0, sizeof(int), st));
    if ((rc = upload_layout(ctx, ws, L))) return rc;
    FKG_CUDA(ctx, cudaMemcpyAsync(ws.diag.p, hdiag, sizeof(double) * V, cudaMemcpyHostToDevice, st));
    FKG_CUDA(ctx, cudaMemcpyAsync(ws.beta.p, hb, sizeof(double) * batch, cudaMemcpyHostToDevice, st));
    FKG_CUDA(ctx, cudaMemcpyAsync(ws.Ulist.p, hprm, sizeof(double) * 3 * batch, cudaMemcpyHostToDevice, st));
    FKG_CUDA(ctx, cudaMemcpyAsync(ws.fint.p, hf, sizeof(int32_t) * V, cudaMemcpyHostToDevice, st));
    if ((rc = enqueue_solve(ctx, ws, L, false))) return rc;
    const bool f32 = ctx->precision == FKG_PREC_MIXED;
    if (!f32 && (rc = enqueue_vectors(ctx, ws, L))) return rc;
    const void* X = f32 ? ws.Z.p : ws.Z64.p;
    const double* eps = f32 ? (const double*)ws.aux64.p : (const double*)ws.w.p;  // paired with X's columns
    const double* dU = (const double*)ws.Ulist.p;
    FKG_CUDA(ctx, launch_grad((const ChainDesc*)ws.desc.p, batch, f32, X, eps, (const int32_t*)ws.fint.p, dU,
                              dU + batch, dU + 2 * batch, (const double*)ws.beta.p, (double*)ws.gout.p,
                              (double*)ws.fermiw.p, st));
    ctx->launches++;
    if (rho) {
        FKG_CUDA(ctx, launch_rho((const ChainDesc*)ws.desc.p, batch, L.max_n, f32, X, (const double*)ws.fermiw.p,
                                 (double*)ws.rho.p, st));
        ctx->launches++;
    }
    FKG_CUDA(ctx, cudaMemcpyAsync(hout, ws.gout.p, sizeof(double) * 5 * batch, cudaMemcpyDeviceToHost, st));
    if ((rc = check_status(ctx))) return rc;
    for (int c = 0; c < batch; ++c) {
        if (F) F[c] = hout[5 * c];
        if (dF_dU) dF_dU[c] = hout[5 * c + 1];
        if (dF_dt) dF_dt[c] = hout[5 * c + 2];
        if (dF_dmu) dF_dmu[c] = hout[5 * c + 3];
        if (dF_dbeta) dF_dbeta[c] = hout[5 * c + 4];
    }
    if (rho) {
        if ((rc = ensure_pinned(ctx, sizeof(double) * (size_t)L.a_total))) return rc;
        double* hr = (double*)ctx->pin;
        FKG_CUDA(ctx, cudaMemcpyAsync(hr, ws.rho.p, sizeof(double) * (size_t)L.a_total, cudaMemcpyDeviceToHost, st));
        FKG_CUDA(ctx, cudaStreamSynchronize(st));
        size_t dst = 0;
        for (int c = 0; c < batch; ++c) {
            const ChainDesc& d = L.desc[c];
            for (int j = 0; j < d.n; ++j)
                for (int i = 0; i < d.n; ++i) rho[dst + (size_t)j * d.n + i] = hr[d.a_off + (size_t)j * d.ld + i];
            dst += (size_t)d.n * d.n;
        }
    }
    return FKG_OK;
}

int fkg_set_stiffness_ops(fkg_ctx* ctx, int lattice_id, int n, const int32_t* rowptr, const int32_t* col,
                          const double* tval, const double* jval) {
    if (!ctx) return FKG_ERR_ARG;
    if (lattice_id < 0 || lattice_id >= kMaxLattices) return set_err(ctx, FKG_ERR_ARG, "lattice_id out of range");
    LatticeDev& l = ctx->lat[lattice_id];
    if (l.n <= 0 || n != l.n) return set_err(ctx, FKG_ERR_ARG, "register the lattice's hopping first, with the same n");
    if (!rowptr || !col || !tval || !jval) return set_err(ctx, FKG_ERR_ARG, "null CSR array");
    const int nnz = rowptr[n];
    if (rowptr[0] != 0 || nnz < 0) return set_err(ctx, FKG_ERR_ARG, "bad rowptr");
    for (int i = 0; i < n; ++i)
        if (rowptr[i + 1] < rowptr[i]) return set_err(ctx, FKG_ERR_ARG, "rowptr not monotone");
    for (int p = 0; p < nnz; ++p) {
        if (col[p] < 0 || col[p] >= n) return set_err(ctx, FKG_ERR_ARG, "column index out of range");
        if (tval[p] - tval[p] != 0.0 || jval[p] - jval[p] != 0.0) return set_err(ctx, FKG_ERR_NUMERIC, "NaN/Inf in operator");
    }
    for (void* q : {(void*)l.srow, (void*)l.scol, (void*)l.stval, (void*)l.sjval})
        if (q) cudaFree(q);
    l.srow = nullptr; l.scol = nullptr; l.stval = nullptr; l.sjval = nullptr; l.snnz = -1;
    const size_t m = nnz > 0 ? nnz : 1;
    FKG_CUDA(ctx, cudaMalloc(&l.srow, sizeof(int32_t) * (n + 1)));
    FKG_CUDA(ctx, cudaMalloc(&l.scol, sizeof(int32_t) * m));
    FKG_CUDA(ctx, cudaMalloc(&l.stval, sizeof(double) * m));
    FKG_CUDA(ctx, cudaMalloc(&l.sjval, sizeof(double) * m));
    FKG_CUDA(ctx, cudaMemcpy(l.srow, rowptr, sizeof(int32_t) * (n + 1), cudaMemcpyHostToDevice));
    if (nnz > 0) {
        FKG_CUDA(ctx, cudaMemcpy(l.scol, col, sizeof(int32_t) * nnz, cudaMemcpyHostToDevice));
        FKG_CUDA(ctx, cudaMemcpy(l.stval, tval, sizeof(double) * nnz, cudaMemcpyHostToDevice));
        FKG_CUDA(ctx, cudaMemcpy(l.sjval, jval, sizeof(double) * nnz, cudaMemcpyHostToDevice));
    }
    l.snnz = nnz;
    return FKG_OK;
}

// calc_ed(true) of a batch, eigenvectors left in the solve workspace (X,
// each column's eigenvalue, the column order); used by the measures.
static int solve_with_vectors(fkg_ctx* ctx, int batch, const int32_t* lattice_id, const double* diag,
                              const double* beta, const void** X, const double** eps, const int** perm) {
    int rc = fkg_eigh_logz(ctx, batch, lattice_id, diag, beta, nullptr, nullptr, nullptr, nullptr, nullptr);
    if (rc) return rc;
    Workspace& ws = ctx->solve;
    const bool f32 = ctx->precision == FKG_PREC_MIXED;
    if (!f32 && (rc = enqueue_vectors(ctx, ws, ctx->solve_layout))) return rc;
    *X = f32 ? ws.Z.p : ws.Z64.p;
    *eps = f32 ? (const double*)ws.aux64.p : (const double*)ws.w.p;  // paired with X's columns
    *perm = f32 ? (const int*)ws.perm.p : nullptr;
    return FKG_OK;
}

int fkg_measure_ipr(fkg_ctx* ctx, int batch, const int32_t* lattice_id, const double* diag, const double* beta,
                    double* ipr) {
    if (!ctx) return FKG_ERR_ARG;
    if (!ipr) return set_err(ctx, FKG_ERR_ARG, "ipr is NULL");
    const void* X;
    const double* eps;
    const int* perm;
    int rc = solve_with_vectors(ctx, batch, lattice_id, diag, beta, &X, &eps, &perm);
    if (rc) return rc;
    Layout& L = ctx->solve_layout;
    Workspace& ws = ctx->solve;
    const size_t V = (size_t)L.v_total;
    if ((rc = ensure_dev(ctx, ws.mout, sizeof(double) * V))) return rc;
    FKG_CUDA(ctx, launch_ipr((const ChainDesc*)ws.desc.p, batch, L.max_n, ctx->precision == FKG_PREC_MIXED, X, perm,
                             (double*)ws.mout.p, ctx->st));
    ctx->launches++;
    if ((rc = ensure_pinned(ctx, sizeof(double) * V))) return rc;
    double* h = (double*)ctx->pin;
    FKG_CUDA(ctx, cudaMemcpyAsync(h, ws.mout.p, sizeof(double) * V, cudaMemcpyDeviceToHost, ctx->st));
    if ((rc = check_status(ctx))) return rc;
    size_t dst = 0;
    for (int c = 0; c < batch; ++c) {
        std::memcpy(ipr + dst, h + L.desc[c].v_off, sizeof(double) * L.desc[c].n);
        dst += L.desc[c].n;
    }
    return FKG_OK;
}

int fkg_measure_stiffness(fkg_ctx* ctx, int batch, const int32_t* lattice_id, const double* diag,
                          const double* beta, double* stiffness, int nw, const double* wgrid, double eta,
                          double* cond) {
    if (!ctx) return FKG_ERR_ARG;
    if (!stiffness || !lattice_id) return set_err(ctx, FKG_ERR_ARG, "null argument");
    if (nw < 0 || (nw > 0 && (!wgrid || !cond))) return set_err(ctx, FKG_ERR_ARG, "frequency grid or cond missing");
    if (nw > 0 && !(eta > 0.0)) return set_err(ctx, FKG_ERR_ARG, "eta must be > 0");
    for (int c = 0; c < batch; ++c) {
        const int id = lattice_id[c];
        if (id < 0 || id >= kMaxLattices || ctx->lat[id].snnz < 0)
            return set_err(ctx, FKG_ERR_STATE, "stiffness operators not set for lattice " + std::to_string(id));
    }
    const void* X;
    const double* eps;
    const int* perm;
    int rc = solve_with_vectors(ctx, batch, lattice_id, diag, beta, &X, &eps, &perm);
    if (rc) return rc;
    Layout& L = ctx->solve_layout;
    Workspace& ws = ctx->solve;
    const size_t V = (size_t)L.v_total;
    if ((rc = ensure_dev(ctx, ws.mout, sizeof(double) * (V > (size_t)batch ? V : batch)))) return rc;
    if ((rc = ensure_dev(ctx, ws.ef, sizeof(double2) * V))) return rc;
    if ((rc = ensure_dev(ctx, ws.mscr, stiffness_scratch_bytes(batch, L.max_n, nw)))) return rc;
    if ((rc = ensure_dev(ctx, ws.sops, sizeof(StiffOps) * batch))) return rc;
    // frequency grid in, conductivity out: after the operators in the same buffer
    if ((rc = ensure_dev(ctx, ws.mcond, sizeof(double) * ((size_t)nw + (size_t)batch * nw)))) return rc;
    std::vector<StiffOps> ops(batch);
    for (int c = 0; c < batch; ++c) {
        const LatticeDev& l = ctx->lat[lattice_id[c]];
        ops[c] = StiffOps{l.srow, l.scol, l.stval, l.sjval};
    }
    const size_t ncond = (size_t)batch * nw;
    if ((rc = ensure_pinned(ctx, sizeof(double) * (batch + nw + ncond) + sizeof(StiffOps) * batch))) return rc;
    StiffOps* hops = (StiffOps*)ctx->pin;
    double* h = (double*)(hops + batch);  // [batch] stiffness, [nw] grid, [batch * nw] cond
    std::memcpy(hops, ops.data(), sizeof(StiffOps) * batch);
    FKG_CUDA(ctx, cudaMemcpyAsync(ws.sops.p, hops, sizeof(StiffOps) * batch, cudaMemcpyHostToDevice, ctx->st));
    double* d_w = (double*)ws.mcond.p;
    double* d_cond = d_w + nw;
    if (nw > 0) {
        std::memcpy(h + batch, wgrid, sizeof(double) * nw);
        FKG_CUDA(ctx, cudaMemcpyAsync(d_w, h + batch, sizeof(double) * nw, cudaMemcpyHostToDevice, ctx->st));
    }
    // J X goes to the FP64 matrix workspace, whose reduced matrix the vectors no longer need
    FKG_CUDA(ctx, launch_stiffness((const ChainDesc*)ws.desc.p, (const StiffOps*)ws.sops.p, batch, L.max_n,
                                   ctx->precision == FKG_PREC_MIXED, X, eps, (const double*)ws.beta.p, ws.A.p,
                                   (double2*)ws.ef.p, (double*)ws.mscr.p, (double*)ws.mout.p, nw, d_w, eta, d_cond,
                                   ctx->st));
    ctx->launches += nw > 0 ? 4 : 3;
    FKG_CUDA(ctx, cudaMemcpyAsync(h, ws.mout.p, sizeof(double) * batch, cudaMemcpyDeviceToHost, ctx->st));
    if (nw > 0)
        FKG_CUDA(ctx, cudaMemcpyAsync(h + batch + nw, d_cond, sizeof(double) * ncond, cudaMemcpyDeviceToHost, ctx->st));
    if ((rc = check_status(ctx))) return rc;
    std::memcpy(stiffness, h, sizeof(double) * batch);
    if (nw > 0) std::memcpy(cond, h + batch + nw, sizeof(double) * ncond);
    return FKG_OK;
}

int fkg_chains_get(fkg_ctx* ctx, int32_t* f, double* logz, double* evals) {
    if (!ctx) return FKG_ERR_ARG;
    if (!ctx->chains_ready) return set_err(ctx, FKG_ERR_STATE, "fkg_chains_init has not been called");
    const Layout& L = ctx->chain_layout;
    const size_t V = (size_t)L.v_total;
    int rc;
    if ((rc = ensure_pinned(ctx, (sizeof(double) + sizeof(int32_t)) * V + sizeof(double) * L.batch))) return rc;
    double* hw = (double*)ctx->pin;
    double* hz = hw + V;
    int32_t* hf = (int32_t*)(hz + L.batch);
    cudaStream_t st = ctx->st;
    FKG_CUDA(ctx, cudaMemcpyAsync(hw, ctx->ch_w_cur.p, sizeof(double) * V, cudaMemcpyDeviceToHost, st));
    FKG_CUDA(ctx, cudaMemcpyAsync(hz, ctx->ch_logz_cur.p, sizeof(double) * L.batch, cudaMemcpyDeviceToHost, st));
    FKG_CUDA(ctx, cudaMemcpyAsync(hf, ctx->ch_f.p, sizeof(int32_t) * V, cudaMemcpyDeviceToHost, st));
    FKG_CUDA(ctx, cudaStreamSynchronize(st));
    long long dst = 0;
    for (int c = 0; c < L.batch; ++c) {
        const ChainDesc& d = L.desc[c];
        if (f) std::memcpy(f + dst, hf + d.v_off, sizeof(int32_t) * d.n);
        if (evals) std::memcpy(evals + dst, hw + d.v_off, sizeof(double) * d.n);
        if (logz) logz[c] = hz[c];
        dst += d.n;
    }
    return FKG_OK;
}

}  // extern "C"

namespace fkg {

// The per-step launch sequence of fkg_propose_accept: proposed diagonal,
// eigen-solve + logZ, Metropolis decision. Device pointers; no sync.
// One proposal step for all chains: proposed diagonal, eigen-solve + logZ,
// Metropolis decision. step (may be null): device step index that offsets the
// per-step inputs and outputs (graph replay).
static int enqueue_one_step(fkg_ctx* ctx, const int32_t* site, const double* u, int32_t* acc, double* dl,
                            const int* step) {
    const Layout& L = ctx->chain_layout;
    Workspace& ws = ctx->chain;
    const int B = L.batch;
    cudaStream_t st = ctx->st;
    const ChainDesc* dd = (const ChainDesc*)ws.desc.p;
    stage_begin(ctx, FKG_STAGE_LOGZ);
    FKG_CUDA(ctx, launch_proposal_diag(dd, B, L.max_n, (const int32_t*)ctx->ch_f.p, site, (const double*)ctx->ch_U.p,
                                       (const double*)ctx->ch_mu_c.p, (double*)ws.diag.p, (int*)ctx->status.p, st, step));
    stage_end(ctx, FKG_STAGE_LOGZ);
    ctx->launches++;
    const bool cheb = ctx->method == FKG_METHOD_CHEBYSHEV;
    if (!cheb) {  // eigen-solve; its logZ kernel takes the decisions
        const StepIO io{site, u, acc, dl, step};
        return enqueue_solve(ctx, ws, L, false, &io);
    }
    int rc = enqueue_kpm(ctx, ws, L, nullptr);
    if (rc) return rc;
    stage_begin(ctx, FKG_STAGE_LOGZ);
    FKG_CUDA(ctx, launch_accept(dd, B, L.max_n, site, u, (const double*)ws.logz.p, cheb ? nullptr : (const double*)ws.w.p,
                                (const double*)ctx->ch_ebmf.p, (int32_t*)ctx->ch_f.p, (double*)ctx->ch_logz_cur.p,
                                cheb ? nullptr : (double*)ctx->ch_w_cur.p, acc, dl, (int*)ctx->status.p, st, step));
    stage_end(ctx, FKG_STAGE_LOGZ);
    ctx->launches++;
    return FKG_OK;
}

// The per-step launch sequence of fkg_propose_accept. Without profiling, one
// step is captured once into a CUDA graph whose kernels read the step index
// from device memory, and the graph is replayed nsteps times; the inputs and
// outputs then live in the context's step buffers (copied from/to the
// caller's pointers when they differ). Device pointers; no sync.
int enqueue_steps(fkg_ctx* ctx, int nsteps, const int32_t* d_site, const double* d_u, int32_t* d_acc,
                  double* d_dlogz) {
    const Layout& L = ctx->chain_layout;
    const int B = L.batch;
    cudaStream_t st = ctx->st;
    FKG_CUDA(ctx, cudaMemsetAsync(ctx->status.p, 0, sizeof(int), st));
    if (!ctx->use_graphs || ctx->profiling) {
        for (int s = 0; s < nsteps; ++s) {
            const size_t off = (size_t)s * B;
            int rc = enqueue_one_step(ctx, d_site + off, d_u + off, d_acc + off, d_dlogz + off, nullptr);
            if (rc) return rc;
        }
        return FKG_OK;
    }
    int rc;
    const size_t tot = (size_t)nsteps * B;
    const void* old[4] = {ctx->st_site.p, ctx->st_u.p, ctx->st_acc.p, ctx->st_dlogz.p};
    if ((rc = ensure_dev(ctx, ctx->st_site, sizeof(int32_t) * tot))) return rc;
    if ((rc = ensure_dev(ctx, ctx->st_u, sizeof(double) * tot))) return rc;
    if ((rc = ensure_dev(ctx, ctx->st_acc, sizeof(int32_t) * tot))) return rc;
    if ((rc = ensure_dev(ctx, ctx->st_dlogz, sizeof(double) * tot))) return rc;
    if ((rc = ensure_dev(ctx, ctx->d_step, sizeof(int)))) return rc;
    if (old[0] != ctx->st_site.p || old[1] != ctx->st_u.p || old[2] != ctx->st_acc.p || old[3] != ctx->st_dlogz.p)
        ctx->drop_graph();
    int32_t* site = (int32_t*)ctx->st_site.p;
    double* u = (double*)ctx->st_u.p;
    int32_t* acc = (int32_t*)ctx->st_acc.p;
    double* dl = (double*)ctx->st_dlogz.p;
    if (d_site != site) FKG_CUDA(ctx, cudaMemcpyAsync(site, d_site, sizeof(int32_t) * tot, cudaMemcpyDeviceToDevice, st));
    if (d_u != u) FKG_CUDA(ctx, cudaMemcpyAsync(u, d_u, sizeof(double) * tot, cudaMemcpyDeviceToDevice, st));
    FKG_CUDA(ctx, cudaMemsetAsync(ctx->d_step.p, 0, sizeof(int), st));
    if (!ctx->graph_exec) {
        const long long before = ctx->launches;
        FKG_CUDA(ctx, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        rc = enqueue_one_step(ctx, site, u, acc, dl, (const int*)ctx->d_step.p);
        ctx->graph_kernels = (int)(ctx->launches - before) + 1;  // + the step-index increment
        ctx->launches = before;  // captured, not launched
        if (rc == FKG_OK && launch_step_inc((int*)ctx->d_step.p, st) != cudaSuccess) rc = FKG_ERR_CUDA;
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(st, &g);
        if (rc) { if (g) cudaGraphDestroy(g); return rc; }
        if (e != cudaSuccess) return set_err(ctx, FKG_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
        ctx->graph = g;
        e = cudaGraphInstantiate(&ctx->graph_exec, g, 0);
        if (e != cudaSuccess) { ctx->drop_graph(); return set_err(ctx, FKG_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e)); }
    }
    for (int s = 0; s < nsteps; ++s) {
        FKG_CUDA(ctx, cudaGraphLaunch(ctx->graph_exec, st));
        ctx->launches += ctx->graph_kernels;
    }
    if (d_acc != acc) FKG_CUDA(ctx, cudaMemcpyAsync(d_acc, acc, sizeof(int32_t) * tot, cudaMemcpyDeviceToDevice, st));
    if (d_dlogz != dl) FKG_CUDA(ctx, cudaMemcpyAsync(d_dlogz, dl, sizeof(double) * tot, cudaMemcpyDeviceToDevice, st));
    return FKG_OK;
}

// FP64 eigenvectors after an FP64 enqueue_solve: inverse iteration on T, then
// X = Q Z; the result (row-major, column j <-> eigenvalue j) is left in ws.Z64.
int enqueue_vectors(fkg_ctx* ctx, Workspace& ws, const Layout& L) {
    int rc;
    const size_t V = (size_t)L.v_total;
    if ((rc = ensure_dev(ctx, ws.Z64, sizeof(double) * (size_t)L.a_total))) return rc;
    if ((rc = ensure_dev(ctx, ws.stein, sizeof(double) * stein_scratch_elems(L.a_total)))) return rc;
    if ((rc = ensure_dev(ctx, ws.Tf64, sizeof(double) * 32 * V))) return rc;
    const ChainDesc* dd = (const ChainDesc*)ws.desc.p;
    stage_begin(ctx, FKG_STAGE_TRIEIG);
    FKG_CUDA(ctx, launch_stein_f64(dd, L.batch, L.max_n, L.max_ld, (const double*)ws.d.p, (const double*)ws.e.p,
                                   (const double*)ws.w.p, (double*)ws.Z64.p, (double*)ws.stein.p, ctx->st));
    stage_end(ctx, FKG_STAGE_TRIEIG);
    stage_begin(ctx, FKG_STAGE_BACK);
    FKG_CUDA(ctx, launch_backtransform_f64(dd, L.batch, L.max_n, L.max_ld, (const double*)ws.A.p,
                                           (const double*)ws.tau.p, (double*)ws.Tf64.p, (double*)ws.Z64.p, ctx->st));
    stage_end(ctx, FKG_STAGE_BACK);
    ctx->launches += 3;
    return FKG_OK;
}

// Copies the eigenvectors of the last solve on `ws` to host, column-major
// n x n per chain, in ascending eigenvalue order.
static int fetch_vectors(fkg_ctx* ctx, Workspace& ws, const Layout& L, double* evecs) {
    int rc;
    const bool f32 = ctx->precision == FKG_PREC_MIXED;
    const size_t A = (size_t)L.a_total, V = (size_t)L.v_total;
    if ((rc = ensure_pinned(ctx, (f32 ? sizeof(float) : sizeof(double)) * A + sizeof(int) * V))) return rc;
    int* hp = (int*)ctx->pin;
    void* hx = (void*)(hp + V + (V & 1));
    if (f32) {
        FKG_CUDA(ctx, cudaMemcpyAsync(hp, ws.perm.p, sizeof(int) * V, cudaMemcpyDeviceToHost, ctx->st));
        FKG_CUDA(ctx, cudaMemcpyAsync(hx, ws.Z.p, sizeof(float) * A, cudaMemcpyDeviceToHost, ctx->st));
    } else {
        FKG_CUDA(ctx, cudaMemcpyAsync(hx, ws.Z64.p, sizeof(double) * A, cudaMemcpyDeviceToHost, ctx->st));
    }
    if ((rc = check_status(ctx))) return rc;
    size_t dst = 0;
    for (int c = 0; c < L.batch; ++c) {
        const ChainDesc& d = L.desc[c];
        for (int k = 0; k < d.n; ++k) {
            const int col = f32 ? hp[d.v_off + k] : k;
            for (int i = 0; i < d.n; ++i) {
                const size_t src = (size_t)d.a_off + (size_t)i * d.ld + col;
                evecs[dst + (size_t)k * d.n + i] = f32 ? (double)((const float*)hx)[src] : ((const double*)hx)[src];
            }
        }
        dst += (size_t)d.n * d.n;
    }
    return FKG_OK;
}

int eigh_vectors(fkg_ctx* ctx, int batch, const int32_t* lattice_id, const double* diag, const double* beta,
                 double* evals, double* exp_e, double* fermi, double* evecs, double* logz) {
    // values, exp, fermi, logZ as fkg_eigh_logz without vectors, then the vectors
    int rc = fkg_eigh_logz(ctx, batch, lattice_id, diag, beta, evals, exp_e, fermi, nullptr, logz);
    if (rc) return rc;
    Layout& L = ctx->solve_layout;
    if (ctx->precision == FKG_PREC_F64 && (rc = enqueue_vectors(ctx, ctx->solve, L))) return rc;
    return fetch_vectors(ctx, ctx->solve, L, evecs);
}

}  // namespace fkg
