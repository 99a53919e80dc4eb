// batch.cu -- the batch entry points of include/trans_gpu.h: a context whose cases are added
// and removed while it runs (continuous batching), within a device-memory budget.
#include <algorithm>

#include "engine.h"

using namespace tg;
using namespace tg::eng;

extern "C" {

int trans_batch_create(int precision, long long device_budget_bytes, void** out) {
    if (!out || (precision != TRANS_FP64 && precision != TRANS_MIXED) || device_budget_bytes < 0) return TRANS_E_ARG;
    *out = nullptr;
    Ctx* c = new Ctx();
    int rc = ctx_init(c, precision, device_budget_bytes);
    if (rc) { ctx_free(c); delete c; return rc; }
    *out = c;
    return TRANS_OK;
}

long long trans_batch_case_bytes(const trans_params* p, int nblocks, const trans_block* blocks) {
    if (validate_case(p, nblocks, blocks) != TRANS_OK) return -1;
    return case_bytes(p, nblocks, blocks);
}

int trans_batch_add(void* ctx, const trans_params* p, int nblocks, const trans_block* blocks, int* case_id) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !case_id) return TRANS_E_ARG;
    if (validate_case(p, nblocks, blocks) != TRANS_OK) return fail(c, TRANS_E_ARG, "case outside the supported configurations");
    CaseRec* cs = nullptr;
    int rc = case_add(c, p, nblocks, blocks, &cs);
    if (rc) return rc;
    *case_id = cs->id;
    return TRANS_OK;
}

int trans_batch_remove(void* ctx, int case_id) {
    Ctx* c = static_cast<Ctx*>(ctx);
    return c ? case_remove(c, case_id) : TRANS_E_ARG;
}

int trans_batch_set_field(void* ctx, int case_id, int ib, int field, const double* a) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return TRANS_E_ARG;
    CaseRec* cs = case_find(c, case_id);
    if (!cs) return fail(c, TRANS_E_ARG, "no such case");
    return field_io(c, cs, ib, field, const_cast<double*>(a), true);
}

int trans_batch_get_field(void* ctx, int case_id, int ib, int field, double* a) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return TRANS_E_ARG;
    CaseRec* cs = case_find(c, case_id);
    if (!cs) return fail(c, TRANS_E_ARG, "no such case");
    return field_io(c, cs, ib, field, a, false);
}

int trans_batch_set_fields(void* ctx, int case_id, int n, const int* ib, const int* field, const double* const* arrays) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return TRANS_E_ARG;
    CaseRec* cs = case_find(c, case_id);
    if (!cs) return fail(c, TRANS_E_ARG, "no such case");
    return fields_io(c, cs, n, ib, field, const_cast<double* const*>(arrays), true);
}

int trans_batch_get_fields(void* ctx, int case_id, int n, const int* ib, const int* field, double* const* arrays) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return TRANS_E_ARG;
    CaseRec* cs = case_find(c, case_id);
    if (!cs) return fail(c, TRANS_E_ARG, "no such case");
    return fields_io(c, cs, n, ib, field, arrays, false);
}

int trans_batch_iterate(void* ctx, int n) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || n < 0) return TRANS_E_ARG;
    if (c->cases.empty() || n == 0) return TRANS_OK;
    for (CaseRec* cs : c->cases) cs->KI = cs->p.KI_ini + cs->iters + 1;
    return run_iterations(c, n);         // TRANS_E_NAN: norms are final; the caller retires the case(s)
}

int trans_batch_time_iterations(void* ctx, int n, double* ms) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || n < 0 || !ms) return TRANS_E_ARG;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaEventRecord(e0, c->stream));
    int rc = trans_batch_iterate(ctx, n);
    CK(cudaEventRecord(e1, c->stream));
    CK(cudaEventSynchronize(e1));
    float t = 0;
    CK(cudaEventElapsedTime(&t, e0, e1));
    *ms = t;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

int trans_batch_case_norms(void* ctx, int case_id, int* iterations, trans_norms* first, trans_norms* last) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return TRANS_E_ARG;
    CaseRec* cs = case_find(c, case_id);
    if (!cs) return fail(c, TRANS_E_ARG, "no such case");
    if (iterations) *iterations = cs->iters;
    if (first) std::copy(cs->first_norms.begin(), cs->first_norms.end(), first);
    if (last) std::copy(cs->norms.begin(), cs->norms.end(), last);
    return TRANS_OK;
}

long long trans_batch_bytes_in_use(void* ctx) {
    Ctx* c = static_cast<Ctx*>(ctx);
    return c ? c->in_use : 0;
}

int trans_batch_get_integrals(void* ctx, int case_id, trans_integrals* out) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return TRANS_E_ARG;
    CaseRec* cs = case_find(c, case_id);
    if (!cs) return fail(c, TRANS_E_ARG, "no such case");
    return integrals(c, cs, out);
}

int trans_batch_integrals(void* ctx, int* ids, trans_integrals* out, int n) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || n < 0 || (n > 0 && (!ids || !out))) return TRANS_E_ARG;
    if (c->cases.empty() || n == 0) return 0;
    std::vector<trans_integrals> all;
    int rc = all_integrals(c, all);
    if (rc) return rc;
    int m = std::min(n, (int)all.size());
    for (int q = 0; q < m; ++q) { ids[q] = c->cases[q]->id; out[q] = all[q]; }
    return m;
}

int trans_batch_get_wall_cp(void* ctx, int case_id, int ib, int iconn, double* cp) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return TRANS_E_ARG;
    CaseRec* cs = case_find(c, case_id);
    if (!cs) return fail(c, TRANS_E_ARG, "no such case");
    return wall_cp(c, cs, ib, iconn, cp);
}

int trans_batch_cases(void* ctx, int* ids, int max) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return TRANS_E_ARG;
    int n = (int)c->cases.size();
    for (int q = 0; q < n && q < max && ids; ++q) ids[q] = c->cases[q]->id;
    return n;
}

}  // extern "C"
