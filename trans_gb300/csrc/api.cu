// api.cu -- the C ABI of include/trans_gpu.h over the engine (engine.h).
//
// The single-case entry points (trans_create ...) drive a context holding one case; the batch
// entry points (trans_batch_*, batch.cu) add and remove cases of a context while it runs, each
// case with its own parameters, iteration counter and norms, all advanced by the same launches.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "engine.h"

using namespace tg;
using namespace tg::eng;

namespace {

Ctx* as_ctx(void* p) { return static_cast<Ctx*>(p); }

CaseRec* first_case(Ctx* c) { return (c && !c->cases.empty()) ? c->cases[0] : nullptr; }

void set_ki(Ctx* c, int ki) {
    for (CaseRec* cs : c->cases) cs->KI = ki;
}

}  // namespace

extern "C" {

int trans_create(const trans_params* p, int nblocks, const trans_block* blocks, void** out) {
    if (!out) return TRANS_E_ARG;
    *out = nullptr;
    if (validate_case(p, nblocks, blocks) != TRANS_OK) return TRANS_E_ARG;   // before any device work
    Ctx* c = new Ctx();
    int rc = ctx_init(c, p->precision, 0);
    if (!rc) rc = case_add(c, p, nblocks, blocks, nullptr);
    if (!rc) rc = rebuild(c);
    if (rc) { ctx_free(c); delete c; return rc; }
    *out = c;
    return TRANS_OK;
}

int trans_destroy(void* ctx) {
    Ctx* c = as_ctx(ctx);
    if (!c) return TRANS_OK;
    ctx_free(c);
    delete c;
    return TRANS_OK;
}

int trans_set_field(void* ctx, int ib, int f, const double* a) {
    Ctx* c = as_ctx(ctx);
    return c ? field_io(c, first_case(c), ib, f, const_cast<double*>(a), true) : TRANS_E_ARG;
}

int trans_get_field(void* ctx, int ib, int f, double* a) {
    Ctx* c = as_ctx(ctx);
    return c ? field_io(c, first_case(c), ib, f, a, false) : TRANS_E_ARG;
}

int trans_set_fields(void* ctx, int n, const int* ib, const int* field, const double* const* arrays) {
    Ctx* c = as_ctx(ctx);
    return c ? fields_io(c, first_case(c), n, ib, field, const_cast<double* const*>(arrays), true) : TRANS_E_ARG;
}

int trans_get_fields(void* ctx, int n, const int* ib, const int* field, double* const* arrays) {
    Ctx* c = as_ctx(ctx);
    return c ? fields_io(c, first_case(c), n, ib, field, arrays, false) : TRANS_E_ARG;
}

int trans_run_stage(void* ctx, int stage, int ki, int itr_chld) {
    Ctx* c = as_ctx(ctx);
    if (!c) return TRANS_E_ARG;
    set_ki(c, ki);
    return run_stage(c, stage, itr_chld);
}

int trans_iterate(void* ctx, int ki, trans_norms* norms) {
    Ctx* c = as_ctx(ctx);
    if (!c || c->cases.empty()) return TRANS_E_ARG;
    set_ki(c, ki);
    int rc = run_iterations(c, 1);          // replayed as a one-iteration graph once tuned
    if (rc) return rc;
    if (norms) std::copy(c->cases[0]->norms.begin(), c->cases[0]->norms.end(), norms);
    return TRANS_OK;
}

int trans_stage_times(void* ctx, int ki, double* ms) {
    Ctx* c = as_ctx(ctx);
    if (!c || !ms || c->cases.empty()) return TRANS_E_ARG;
    set_ki(c, ki);
    cudaEvent_t ev[TRANS_NSTAGES + 1];
    for (int q = 0; q <= TRANS_NSTAGES; ++q) CK(cudaEventCreate(&ev[q]));
    for (int q = 0; q < TRANS_NSTAGES; ++q) ms[q] = 0.0;
    const CaseRec* c0 = c->cases[0];
    int nsub = sub_iterations(c0->p);
    int rc = TRANS_OK;
    for (int it = 1; it <= nsub && rc == TRANS_OK; ++it)
        for (int st = TRANS_STAGE_SPECRAD; st <= TRANS_STAGE_UPDATE_U && rc == TRANS_OK; ++st) {
            if (st == TRANS_STAGE_UPDATE_U && it != nsub) continue;
            CK(cudaEventRecord(ev[st], c->stream));
            rc = run_stage(c, st, it);
            CK(cudaEventRecord(ev[st + 1], c->stream));
            CK(cudaEventSynchronize(ev[st + 1]));
            float t = 0;
            CK(cudaEventElapsedTime(&t, ev[st], ev[st + 1]));
            ms[st] += t;
        }
    for (int q = 0; q <= TRANS_NSTAGES; ++q) cudaEventDestroy(ev[q]);
    return rc;
}

double trans_probe_fma_gflops(int fp64) { return probe_fma_gflops(fp64); }

double trans_probe_chain_us(int chained, int grid) { return probe_chain_us(chained, grid); }

int trans_time_iterations(void* ctx, int ki_first, int n, double* ms, trans_norms* norms) {
    Ctx* c = as_ctx(ctx);
    if (!c || !ms || n < 0 || c->cases.empty()) return TRANS_E_ARG;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaEventRecord(e0, c->stream));
    set_ki(c, ki_first);
    int rc = run_iterations(c, n);
    CK(cudaEventRecord(e1, c->stream));
    CK(cudaEventSynchronize(e1));
    float t = 0;
    CK(cudaEventElapsedTime(&t, e0, e1));
    *ms = t;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (norms) std::copy(c->cases[0]->norms.begin(), c->cases[0]->norms.end(), norms);
    return rc;
}

int trans_prepare(void* ctx, int ki) {
    Ctx* c = as_ctx(ctx);
    if (!c || c->cases.empty()) return TRANS_E_ARG;
    if (ki >= 0) set_ki(c, ki);
    else
        for (CaseRec* cs : c->cases) cs->KI = cs->p.KI_ini + cs->iters + 1;
    return prepare(c);
}

int trans_get_norms(void* ctx, trans_norms* norms) {
    Ctx* c = as_ctx(ctx);
    if (!c || !norms || c->cases.empty()) return TRANS_E_ARG;
    std::copy(c->cases[0]->norms.begin(), c->cases[0]->norms.end(), norms);
    return TRANS_OK;
}

int trans_get_integrals(void* ctx, trans_integrals* out) {
    Ctx* c = as_ctx(ctx);
    return c ? integrals(c, first_case(c), out) : TRANS_E_ARG;
}

int trans_get_wall_cp(void* ctx, int ib, int iconn, double* cp) {
    Ctx* c = as_ctx(ctx);
    return c ? wall_cp(c, first_case(c), ib, iconn, cp) : TRANS_E_ARG;
}

int trans_get_wall_forces(void* ctx, int ib, int iconn, double* forces) {
    Ctx* c = as_ctx(ctx);
    return c ? wall_cp(c, first_case(c), ib, iconn, forces, true) : TRANS_E_ARG;
}

int trans_halo_pack(void* ctx, int sweep, int ib, int iconn, double* buf) {
    Ctx* c = as_ctx(ctx);
    return c ? halo_io(c, first_case(c), sweep, ib, iconn, nullptr, buf, true) : TRANS_E_ARG;
}

int trans_halo_unpack(void* ctx, int sweep, int ib, int iconn, const trans_conn* partner, const double* buf) {
    Ctx* c = as_ctx(ctx);
    return c ? halo_io(c, first_case(c), sweep, ib, iconn, partner, const_cast<double*>(buf), false) : TRANS_E_ARG;
}

int trans_sync(void* ctx) {
    Ctx* c = as_ctx(ctx);
    if (!c) return TRANS_E_ARG;
    CK(cudaStreamSynchronize(c->stream));
    return TRANS_OK;
}

long long trans_device_bytes(void* ctx) {
    Ctx* c = as_ctx(ctx);
    if (!c) return 0;
    long long b = 0;
    for (const CaseRec* cs : c->cases)
        b += (long long)(cs->arena_doubles * (sizeof(double) + (cs->farena ? sizeof(float) : 0)));
    const long long dq_arrays = c->fl->sweep_pair ? 2 : 1;      // the mixed path's two-plane schedule keeps a second one
    b += (c->sv.n + 31) / 32 * 32 * ((long long)(c->fl->rec_width + dq_arrays * DQ_STRIDE) * (long long)c->fl->elem + 8LL * (long long)sizeof(int));
    return b;
}

long long trans_kernel_launches(void* ctx) {
    Ctx* c = as_ctx(ctx);
    return c ? c->launches : 0;
}

int trans_kernel_times(void* ctx, int ki, double* ms, int* launches, int n) {
    Ctx* c = as_ctx(ctx);
    if (!c || !ms || !launches || n < NKCLASS || c->cases.empty()) return TRANS_E_ARG;
    for (int k = 0; k < n; ++k) { ms[k] = 0.0; launches[k] = 0; }
    if (c->sweep_mode < 0) {                   // tune outside the timed iteration
        int rc = trans_iterate(ctx, ki, nullptr);
        if (rc) return rc;
        ++ki;
    }
    set_ki(c, ki);
    return kernel_times(c, ms, launches);
}

int trans_check_conversions(long long n, unsigned long long seed, long long* mismatches) {
    if (n < 1 || n > (1LL << 32) || !mismatches) {
        g_stateless_err = "trans_check_conversions: n must be 1..2^32 and mismatches non-NULL";
        return TRANS_E_ARG;
    }
    const cudaError_t e = check_conversions(n, seed, mismatches);
    if (e != cudaSuccess) {
        g_stateless_err = std::string("trans_check_conversions: ") + cudaGetErrorString(e);
        return TRANS_E_CUDA;
    }
    return TRANS_OK;
}

const char* trans_kernel_class(int k) { return (k >= 0 && k < NKCLASS) ? kclass_name[k] : ""; }

const char* trans_tuning(void* ctx) {
    Ctx* c = as_ctx(ctx);
    if (!c) return "no context";
    static thread_local std::string out;
    const std::string tiles = c->sweep_mode == 3 ? std::to_string(c->tile_shape[0]) + "x" + std::to_string(c->tile_shape[1]) + "x"
                                                       + std::to_string(c->tile_shape[2]) + "/" : std::string();
    const std::string chain = c->pdl ? (c->pdl == 2 ? "-early" : "-chained") : "";
    out = "sweep=" + std::string(c->sweep_mode == 5 ? "pairs" + chain
                                 : c->sweep_mode >= 1 ? std::string(c->sweep_mode == 1 ? "coop " : c->sweep_mode == 2 ? "flow " : c->sweep_mode == 4 ? "clusters " : "tiles ")
                                                      + tiles + std::to_string(c->sweep_grid) + "x" + std::to_string(c->sweep_block)
                                 : c->sweep_mode == 0 ? (c->pdl ? (c->pdl == 2 ? "planes-early" : "planes-chained") : "planes") : "untuned")
          + (c->sweep_wpc ? "/wpc" : "")
          + (c->sweep_pf && (c->sweep_mode == 0 || c->sweep_mode == 4 || c->sweep_mode == 5) ? "/pf" + std::to_string(c->sweep_pf) : "")
          + (c->sweep_cta && (c->sweep_mode == 0 || c->sweep_mode == 5) ? "/cta" + std::to_string(c->sweep_cta) : "")
          + "; measured: " + c->sweep_tuning
          + (c->mixed ? std::string("; residual=") + (c->resid_tma == 1 ? "tma" : c->resid_tma == 0 ? "gather" : "untuned")
                            + (c->resid_tuning.empty() ? std::string() : " (" + c->resid_tuning + ")")
                      : std::string());
    return out.c_str();
}

const char* trans_last_error(void* ctx) {
    Ctx* c = as_ctx(ctx);
    return c ? c->err.c_str() : stateless_error();
}

}  // extern "C"
