// kpm_api.cu — host side of the Chebyshev-expansion logZ (chebyshev.cu):
// the balls around every site of a lattice, the per-chain descriptors and
// the entry points fkg_set_chebyshev, fkg_chebyshev_logz and fkg_set_method.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "fkg_internal.h"

#define FKG_CUDA(ctx, call)                                                                   \
    do {                                                                                      \
        cudaError_t _e = (call);                                                              \
        if (_e != cudaSuccess) {                                                              \
            cudaGetLastError();                                                               \
            return kpm_err(ctx, FKG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
        }                                                                                     \
    } while (0)

namespace fkg {
namespace {

int kpm_err(fkg_ctx* ctx, int code, const std::string& msg) {
    ctx->err = msg;
    return code;
}

template <typename T>
int upload(fkg_ctx* ctx, T*& dst, const std::vector<T>& src) {
    FKG_CUDA(ctx, cudaMalloc(&dst, sizeof(T) * std::max<size_t>(src.size(), 1)));
    if (!src.empty()) FKG_CUDA(ctx, cudaMemcpy(dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice));
    return FKG_OK;
}

// Ball of radius R around every site: breadth-first search over the
// off-diagonal hopping, sites in hop order, and the ball's own CSR (only
// entries between two ball sites; a column of T_m(x), m <= R, never needs
// another). Also the hopping's diagonal.
int build_balls(fkg_ctx* ctx, LatticeDev& l, int R) {
    const int n = l.n;
    const std::vector<int32_t>& rp = l.h_rowptr;
    const std::vector<int32_t>& cl = l.h_col;
    const std::vector<double>& vl = l.h_val;
    std::vector<double> hdiag(n, 0.0);
    for (int i = 0; i < n; ++i)
        for (int p = rp[i]; p < rp[i + 1]; ++p)
            if (cl[p] == i) hdiag[i] += vl[p];
    std::vector<int32_t> bptr(n + 1, 0), bsite, bcnt((size_t)n * (R + 1)), blrp(1, 0), blcol;
    std::vector<double> blval;
    std::vector<int> loc(n, -1);
    int bmax = 0;
    for (int j = 0; j < n; ++j) {
        const size_t start = bsite.size();
        bsite.push_back(j);
        loc[j] = 0;
        size_t front_begin = start, front_end = bsite.size();
        bcnt[(size_t)j * (R + 1)] = 1;
        for (int d = 1; d <= R; ++d) {
            for (size_t q = front_begin; q < front_end; ++q) {
                const int s = bsite[q];
                for (int p = rp[s]; p < rp[s + 1]; ++p) {
                    const int t = cl[p];
                    if (t != s && loc[t] < 0) {
                        loc[t] = (int)(bsite.size() - start);
                        bsite.push_back(t);
                    }
                }
            }
            front_begin = front_end;
            front_end = bsite.size();
            bcnt[(size_t)j * (R + 1) + d] = (int32_t)(front_end - start);
        }
        const int size = (int)(bsite.size() - start);
        bmax = std::max(bmax, size);
        for (int r = 0; r < size; ++r) {
            const int s = bsite[start + r];
            for (int p = rp[s]; p < rp[s + 1]; ++p) {
                const int t = cl[p];
                if (t != s && loc[t] >= 0) {
                    blcol.push_back(loc[t]);
                    blval.push_back(vl[p]);
                }
            }
            blrp.push_back((int32_t)blcol.size());
        }
        for (size_t q = start; q < bsite.size(); ++q) loc[bsite[q]] = -1;
        bptr[j + 1] = (int32_t)bsite.size();
        if (bsite.size() > (size_t)0x7fffffff || blcol.size() > (size_t)0x7fffffff)
            return kpm_err(ctx, FKG_ERR_ALLOC, "Chebyshev balls too large (reduce cheb_size)");
    }
    std::vector<float2> blv2(blval.size());
    for (size_t p = 0; p < blval.size(); ++p) {
        const float h = (float)blval[p];
        blv2[p] = make_float2(h, (float)(blval[p] - (double)h));
    }
    l.free_kpm();
    int rc;
    if ((rc = upload(ctx, l.kpm_bptr, bptr)) || (rc = upload(ctx, l.kpm_bsite, bsite)) ||
        (rc = upload(ctx, l.kpm_bcnt, bcnt)) || (rc = upload(ctx, l.kpm_blrp, blrp)) ||
        (rc = upload(ctx, l.kpm_blcol, blcol)) || (rc = upload(ctx, l.kpm_blval, blval)) ||
        (rc = upload(ctx, l.kpm_blv2, blv2)) || (rc = upload(ctx, l.kpm_hdiag, hdiag))) {
        l.free_kpm();
        return rc;
    }
    l.kpm_R = R;
    l.kpm_bmax = bmax;
    return FKG_OK;
}

int kpm_kmax(int max_n) { return std::min(2 * max_n + 64, 2048); }

}  // namespace

int prepare_kpm(fkg_ctx* ctx, Workspace& ws, const Layout& L) {
    if (ctx->kpm_M < 2) return kpm_err(ctx, FKG_ERR_STATE, "fkg_set_chebyshev has not been called");
    const int R = ctx->kpm_M / 2;
    std::vector<KpmDesc> kd(L.batch);
    for (int c = 0; c < L.batch; ++c) {
        LatticeDev& l = ctx->lat[L.desc[c].lattice];
        if (l.kpm_R != R) {
            int rc = build_balls(ctx, l, R);
            if (rc) return rc;
        }
        const ChainDesc& d = L.desc[c];
        kd[c] = KpmDesc{d.n, d.ld, R, l.kpm_bmax, d.v_off, l.rowptr, l.col, l.val, l.kpm_hdiag,
                        l.kpm_bptr, l.kpm_bsite, l.kpm_bcnt, l.kpm_blrp, l.kpm_blcol, l.kpm_blval, l.kpm_blv2,
                        l.valf};
    }
    const size_t V = (size_t)L.v_total;
    int rc;
    if ((rc = ensure_dev(ctx, ws.kdesc, sizeof(KpmDesc) * L.batch))) return rc;
    if ((rc = ensure_dev(ctx, ws.ksteps, sizeof(int) * L.batch))) return rc;
    if ((rc = ensure_dev(ctx, ws.kab, sizeof(KpmAB) * L.batch))) return rc;
    if ((rc = ensure_dev(ctx, ws.kpart, sizeof(double) * 3 * (size_t)R * V))) return rc;
    if ((rc = ensure_dev(ctx, ws.kmu, sizeof(double) * (size_t)ctx->kpm_M * L.batch))) return rc;
    FKG_CUDA(ctx, cudaMemcpyAsync(ws.kdesc.p, kd.data(), sizeof(KpmDesc) * L.batch, cudaMemcpyHostToDevice, ctx->st));
    FKG_CUDA(ctx, cudaStreamSynchronize(ctx->st));  // kd is a local array
    ws.kpm_batch = L.batch;
    return FKG_OK;
}

int enqueue_kpm(fkg_ctx* ctx, Workspace& ws, const Layout& L, double* d_mu) {
    if (ws.kpm_batch != L.batch) return kpm_err(ctx, FKG_ERR_STATE, "Chebyshev descriptors are not set up");
    int bmax = 1;
    for (int c = 0; c < L.batch; ++c) bmax = std::max(bmax, ctx->lat[L.desc[c].lattice].kpm_bmax);
    stage_begin(ctx, FKG_STAGE_LOGZ);
    FKG_CUDA(ctx, launch_kpm((const KpmDesc*)ws.kdesc.p, L.batch, L.max_n, L.max_ld, bmax, ctx->kpm_M / 2,
                             ctx->kpm_M, ctx->kpm_G, kpm_kmax(L.max_n), (const double*)ws.diag.p,
                             (const double*)ws.beta.p, (KpmAB*)ws.kab.p, (int*)ws.ksteps.p, (double*)ws.kpart.p,
                             d_mu, (double*)ws.logz.p, (int*)ctx->status.p, ctx->st));
    stage_end(ctx, FKG_STAGE_LOGZ);
    ctx->launches += 3;
    return FKG_OK;
}

}  // namespace fkg

using namespace fkg;

extern "C" {

int fkg_set_chebyshev(fkg_ctx* ctx, int cheb_size, int grid_size) {
    if (!ctx) return FKG_ERR_ARG;
    if (cheb_size < 2 || cheb_size > 1024) return kpm_err(ctx, FKG_ERR_ARG, "cheb_size must be in [2, 1024]");
    if (grid_size < 2 || grid_size > 4096) return kpm_err(ctx, FKG_ERR_ARG, "grid_size must be in [2, 4096]");
    ctx->kpm_M = cheb_size + cheb_size % 2;  // chebyshev_eval rounds the moment count up to even
    ctx->kpm_G = grid_size;
    ctx->solve.kpm_batch = 0;
    if (ctx->method == FKG_METHOD_CHEBYSHEV) ctx->chains_ready = false;
    ctx->drop_graph();
    return FKG_OK;
}

int fkg_set_method(fkg_ctx* ctx, int method) {
    if (!ctx) return FKG_ERR_ARG;
    if (method != FKG_METHOD_ED && method != FKG_METHOD_CHEBYSHEV) return kpm_err(ctx, FKG_ERR_ARG, "unknown method");
    if (method != ctx->method) {
        ctx->method = method;
        ctx->chains_ready = false;
        ctx->drop_graph();
    }
    return FKG_OK;
}

int fkg_chebyshev_logz(fkg_ctx* ctx, int batch, const int32_t* lattice_id, const double* diag, const double* beta,
                       double* logz, double* e_min, double* e_max, double* moments, int32_t* lanczos_steps) {
    if (!ctx) return FKG_ERR_ARG;
    if (!diag || !beta || !logz) return kpm_err(ctx, FKG_ERR_ARG, "diag/beta/logz is NULL");
    Layout& L = ctx->solve_layout;
    int rc;
    if ((rc = make_layout(ctx, batch, lattice_id, L))) return rc;
    Workspace& ws = ctx->solve;
    const size_t V = (size_t)L.v_total;
    if ((rc = ensure_dev(ctx, ws.desc, sizeof(ChainDesc) * L.batch))) return rc;
    if ((rc = ensure_dev(ctx, ws.order, sizeof(int) * L.batch))) return rc;
    if ((rc = ensure_dev(ctx, ws.counter, sizeof(int)))) return rc;
    if ((rc = ensure_dev(ctx, ws.diag, sizeof(double) * V))) return rc;
    if ((rc = ensure_dev(ctx, ws.beta, sizeof(double) * L.batch))) return rc;
    if ((rc = ensure_dev(ctx, ws.logz, sizeof(double) * L.batch))) return rc;
    if ((rc = prepare_kpm(ctx, ws, L))) return rc;
    const int M = ctx->kpm_M;
    if ((rc = ensure_pinned(ctx, sizeof(double) * (V + 4 * (size_t)batch + (size_t)M * batch)))) return rc;
    double* hin = (double*)ctx->pin;
    double* hb = hin + V;
    long long src = 0;
    for (int c = 0; c < batch; ++c) {
        const ChainDesc& d = L.desc[c];
        for (int i = 0; i < d.ld; ++i) hin[d.v_off + i] = i < d.n ? diag[src + i] : 0.0;
        if (!(beta[c] > 0.0) || beta[c] - beta[c] != 0.0) return kpm_err(ctx, FKG_ERR_ARG, "beta must be finite and > 0");
        hb[c] = beta[c];
        src += d.n;
    }
    cudaStream_t st = ctx->st;
    FKG_CUDA(ctx, cudaMemsetAsync(ctx->status.p, 0, sizeof(int), st));
    if ((rc = upload_layout(ctx, ws, L))) return rc;
    FKG_CUDA(ctx, cudaMemcpyAsync(ws.diag.p, hin, sizeof(double) * V, cudaMemcpyHostToDevice, st));
    FKG_CUDA(ctx, cudaMemcpyAsync(ws.beta.p, hb, sizeof(double) * batch, cudaMemcpyHostToDevice, st));
    if ((rc = enqueue_kpm(ctx, ws, L, moments ? (double*)ws.kmu.p : nullptr))) return rc;
    double* oz = hb + batch;
    std::vector<KpmAB> ab(batch);
    FKG_CUDA(ctx, cudaMemcpyAsync(oz, ws.logz.p, sizeof(double) * batch, cudaMemcpyDeviceToHost, st));
    if (moments) FKG_CUDA(ctx, cudaMemcpyAsync(moments, ws.kmu.p, sizeof(double) * M * batch, cudaMemcpyDeviceToHost, st));
    FKG_CUDA(ctx, cudaMemcpyAsync(ab.data(), ws.kab.p, sizeof(KpmAB) * batch, cudaMemcpyDeviceToHost, st));
    if (lanczos_steps)
        FKG_CUDA(ctx, cudaMemcpyAsync(lanczos_steps, ws.ksteps.p, sizeof(int32_t) * batch, cudaMemcpyDeviceToHost, st));
    if ((rc = check_status(ctx))) return rc;
    for (int c = 0; c < batch; ++c) {
        logz[c] = oz[c];
        if (e_min) e_min[c] = ab[c].e_min;
        if (e_max) e_max[c] = ab[c].e_max;
    }
    return FKG_OK;
}

}  // extern "C"
