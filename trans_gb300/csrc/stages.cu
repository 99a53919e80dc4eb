// stages.cu -- one outer iteration of every case of a context, stage by stage in the order of
// main.F90:54-197, with the LU-SGS sweep schedules, the residual norms and field transfer.
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <initializer_list>
#include <utility>

#include "engine.h"

namespace tg {
namespace eng {

namespace {

struct FieldMap { int slot; int ncomp; int lb; };
FieldMap field_map(int f) {
    switch (f) {
        case TRANS_V: return {S_V, 7, -2};
        case TRANS_PP: return {S_PP, 1, -2};
        case TRANS_T: return {S_T, 1, -2};
        case TRANS_RMIU: return {S_RMIU, 1, -2};
        case TRANS_WT0: return {S_WT0, 7, 1};
        case TRANS_WT1: return {S_WT1, 7, 1};
        case TRANS_SD: return {S_SD, 9, -2};
        case TRANS_GRAD: return {S_GRAD, 3, -2};
        case TRANS_VOL: return {S_VOL, 1, -2};
        case TRANS_ALAGM: return {S_ALAGM, 3, -2};
        case TRANS_DST: return {S_DST, 1, -2};
        case TRANS_ALENG: return {S_ALENG, 1, -2};
        case TRANS_ASENG: return {S_ASENG, 1, 1};
        case TRANS_XC: return {S_XC, 1, 0};
        case TRANS_YC: return {S_YC, 1, 0};
        case TRANS_ZC: return {S_ZC, 1, 0};
        case TRANS_RAD: return {S_RAD, 1, -2};
        case TRANS_THTC: return {S_THTC, 1, -2};
        case TRANS_D: return {S_D, 7, 0};
        case TRANS_RDS: return {S_RDS, 3, 0};
        case TRANS_DTM: return {S_DTM, 1, 1};
        case TRANS_DQDXYZ: return {S_DQ, 18, -1};
        case TRANS_SHOCK: return {S_SHOCK, 1, -2};
        case TRANS_WT2: return {S_WT2, 7, 1};
        default: return {-1, 0, 0};
    }
}

bool is_geometry(int f) { return f >= TRANS_SD && f <= TRANS_THTC; }

// FP32 copies of slot ranges {first, count} of every block (mixed path); to_fp64 copies back
void mirror(Ctx* c, std::initializer_list<std::pair<int, int>> ranges, int to_fp64 = 0) {
    MirrorList ml;
    std::memset(&ml, 0, sizeof(ml));
    ml.to_fp64 = to_fp64;
    for (auto& r : ranges) { ml.first[ml.n] = r.first; ml.count[ml.n] = r.second; ml.n++; }
    launch_mirror(c->stream, c->d_blk, (int)c->blk.size(), c->total_cells, c->d_off, ml);
    c->launches++;
}

}  // namespace

int finalize_geometry(Ctx* c) {
    bool dirty = false;
    for (CaseRec* cs : c->cases) dirty |= cs->geom_dirty;
    if (!dirty) return TRANS_OK;
    launch_geom_static(c->stream, c->d_blk, (int)c->blk.size(), c->total_cells, c->d_off);
    c->launches++;
    if (c->mixed) mirror(c, {{S_SD, S_WALL + 3 - S_SD}});
    CK(cudaGetLastError());
    for (CaseRec* cs : c->cases) cs->geom_dirty = false;
    return TRANS_OK;
}

namespace {

// switches of one case for its current KI (Time/SpectralRadius.F90:159-160, main.F90:60-64)
CaseDev case_dev(const CaseRec* cs) {
    const trans_params& p = cs->p;
    CaseDev d;
    std::memset(&d, 0, sizeof(d));
    d.p = cs->dp;
    d.pf = params_as<float>(cs->dp);
    double CFL_sub = p.CFL_Sub_start + (p.CFL_Sub_end - p.CFL_Sub_start) * (double)(cs->KI - p.KI_ini) / (double)p.CFL_Sub_step;
    d.CFL_sub = std::min(CFL_sub, p.CFL_Sub_end);
    d.turb = (p.IF_Euler == 0 && p.IF_Turb_org == 1 && (cs->KI >= p.KItm || p.Kind_Hybrid > 0)) ? 1 : 0;
    d.turb_upd = (p.IF_Euler == 0 && d.turb == 1 && cs->KI >= p.KItm) ? 1 : 0;
    return d;
}

}  // namespace

int upload_cdev(Ctx* c) {
    const size_t n = c->cases.size();
    std::vector<CaseDev> now(n);
    for (size_t k = 0; k < n; ++k) now[k] = case_dev(c->cases[k]);
    if (c->cdev_last.size() == n && std::memcmp(now.data(), c->cdev_last.data(), n * sizeof(CaseDev)) == 0) return TRANS_OK;
    CK(cudaStreamSynchronize(c->stream));          // the pinned copy may still be in flight
    std::memcpy(c->h_cdev, now.data(), n * sizeof(CaseDev));
    CK(cudaMemcpyAsync(c->d_cdev, c->h_cdev, n * sizeof(CaseDev), cudaMemcpyHostToDevice, c->stream));
    c->cdev_last = now;
    return TRANS_OK;
}

namespace {

bool any_case(const Ctx* c, bool (*pred)(const CaseRec*)) {
    for (const CaseRec* cs : c->cases)
        if (pred(cs)) return true;
    return false;
}

}  // namespace

// Per-block norms from the per-tile partials in c->h_parts, summed in tile order
// (deterministic), then handed to the blocks' cases.
int reduce_norms(Ctx* c) {
    int nan = 0;
    for (size_t b = 0; b < c->blk.size(); ++b) {
        trans_norms& N = c->norms[b];
        double sa = 0, sk = 0, so = 0, ma = -1, mk = 0, mo = 0;
        long long ia = 0;
        int bnan = 0;
        for (size_t t = 0; t < c->cell_tiles.size(); ++t) {
            if (c->cell_tile_blk[t] != (int)b) continue;
            const NormPart& P = c->h_parts[t];
            sa += P.sa; sk += P.sk; so += P.so;
            if (P.ma > ma || (P.ma == ma && P.ia > ia)) { ma = P.ma; ia = P.ia; }
            mk = std::max(mk, P.mk); mo = std::max(mo, P.mo);
            bnan |= P.nan;
        }
        const DevBlock& B = c->blk[b];
        N.DRSa = std::sqrt(sa / B.NI1 / B.NJ1 / B.NK1);
        N.DRSk = std::sqrt(sk / B.NI1 / B.NJ1 / B.NK1);
        N.DRSo = std::sqrt(so / B.NI1 / B.NJ1 / B.NK1);
        N.DUa = ma; N.DUk = mk; N.DUo = mo;
        N.Ima = (int)(ia % B.NI1) + 1; N.Jma = (int)((ia / B.NI1) % B.NJ1) + 1; N.Kma = (int)(ia / ((long long)B.NI1 * B.NJ1)) + 1;
        N.nan_flag = bnan;
        nan |= bnan;
    }
    for (CaseRec* cs : c->cases)
        std::copy(c->norms.begin() + cs->blk0, c->norms.begin() + cs->blk0 + cs->blk.size(), cs->norms.begin());
    if (nan) return fail(c, TRANS_E_NAN, "NaN in the density increment");
    return TRANS_OK;
}

// Norms of every block (from k_block_norms, BlockNorms = trans_norms layout) into the context
// and its cases.
static_assert(sizeof(BlockNorms) == sizeof(trans_norms), "BlockNorms mirrors trans_norms");
int collect_norms(Ctx* c, const BlockNorms* hn) {
    std::memcpy(c->norms.data(), hn, sizeof(trans_norms) * c->norms.size());
    int nan = 0;
    for (const trans_norms& N : c->norms) nan |= N.nan_flag;
    for (CaseRec* cs : c->cases)
        std::copy(c->norms.begin() + cs->blk0, c->norms.begin() + cs->blk0 + cs->blk.size(), cs->norms.begin());
    if (nan) return fail(c, TRANS_E_NAN, "NaN in the density increment");
    return TRANS_OK;
}

namespace {

// The device address of a page-locked host array of `bytes` bytes registered with this
// device (cudaHostAlloc, cudaHostRegister), or null: the transpose kernel then reads or writes
// the caller's array in place over the host link, with no staging copy.  Both ends of the
// array must be page-locked host memory at a linear device mapping.
double* mapped_host(const double* host, size_t bytes) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return nullptr; }
    cudaPointerAttributes a0{}, a1{};
    const char* last = (const char*)host + bytes - 1;
    if (cudaPointerGetAttributes(&a0, host) != cudaSuccess || cudaPointerGetAttributes(&a1, last) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a0.type != cudaMemoryTypeHost || a1.type != cudaMemoryTypeHost || !a0.devicePointer || !a1.devicePointer)
        return nullptr;
    if (a0.device != dev || a1.device != dev) return nullptr;
    if ((const char*)a1.devicePointer - (const char*)a0.devicePointer != (std::ptrdiff_t)(bytes - 1)) return nullptr;
    return (double*)a0.devicePointer;
}

}  // namespace

int field_io(Ctx* c, CaseRec* cs, int ib, int f, double* host, bool upload, bool sync) {
    if (!c || !cs || ib < 0 || ib >= (int)cs->blk.size() || !host) return TRANS_E_ARG;
    FieldMap fm = field_map(f);
    if (fm.slot < 0) return fail(c, TRANS_E_ARG, "bad field id");
    if (f == TRANS_WT2 && cs->p.IF_RK != 1) return fail(c, TRANS_E_ARG, "Wt2 exists in Runge-Kutta cases only");
    // the FP32 copies of D, DQdxyz and shock go through the work lists; every other field only
    // needs the case's own block (so adding a case and filling it does not rebuild the lists)
    const bool mirrored = c->mixed && (f == TRANS_D || f == TRANS_DQDXYZ || f == TRANS_SHOCK);
    if (mirrored && !c->built) {
        int rc = rebuild(c);
        if (rc) return rc;
    }
    const DevBlock& b = cs->blk[ib];
    size_t ncells = (size_t)(b.NI + 3 - fm.lb) * (b.NJ + 3 - fm.lb) * (b.NK + 3 - fm.lb);
    size_t bytes = ncells * fm.ncomp * sizeof(double);
    cudaStream_t s = c->stream;
    int is_sd = f == TRANS_SD ? 1 : 0;
    double* mapped = f == TRANS_THTC || !c->xfer_mapped ? nullptr : mapped_host(host, bytes);
    if (mapped) {       // page-locked caller array: transpose in place over the host link
        if (!upload) {
            if (c->mixed && f == TRANS_D) mirror(c, {{S_D, 7}}, 1);
            if (c->mixed && f == TRANS_DQDXYZ) mirror(c, {{S_DQ, 18}}, 1);
            if (c->mixed && f == TRANS_SHOCK) mirror(c, {{S_SHOCK, 1}}, 1);
        }
        launch_field_xfer(s, b, fm.slot, fm.ncomp, fm.lb, is_sd, mapped, upload ? 1 : 0);
        c->launches++;
        if (upload) {
            if (is_geometry(f)) cs->geom_dirty = true;
            if (c->mixed && f == TRANS_D) mirror(c, {{S_D, 7}});
            if (c->mixed && f == TRANS_DQDXYZ) mirror(c, {{S_DQ, 18}});
            if (c->mixed && f == TRANS_SHOCK) mirror(c, {{S_SHOCK, 1}});
        }
        CK(cudaGetLastError());
        if (sync) CK(cudaStreamSynchronize(s));
        return TRANS_OK;
    }
    if (!c->d_stage || c->stage_doubles < ncells * fm.ncomp) {          // staging for the largest field so far
        CK(cudaStreamSynchronize(s));
        if (c->d_stage) cudaFree(c->d_stage);
        c->d_stage = nullptr;
        c->stage_doubles = 0;
        size_t mx = (size_t)(b.NI + 4) * (b.NJ + 4) * (b.NK + 4) * 18;  // DQdxyz of this block
        mx = std::max(mx, ncells * fm.ncomp);
        CK(cudaMalloc(&c->d_stage, mx * sizeof(double)));
        c->stage_doubles = mx;
    }
    if (upload) {
        CK(cudaMemcpyAsync(c->d_stage, host, bytes, cudaMemcpyHostToDevice, s));
        if (!c->copy_done) CK(cudaEventCreateWithFlags(&c->copy_done, cudaEventDisableTiming));
        CK(cudaEventRecord(c->copy_done, s));
        launch_field_xfer(s, b, fm.slot, fm.ncomp, fm.lb, is_sd, c->d_stage, 1);
        c->launches++;
        if (f == TRANS_THTC) {      // sin/cos of the outlet recurrence, evaluated once on the host
            std::vector<double> sn(ncells), co(ncells);
            for (size_t q = 0; q < ncells; ++q) { sn[q] = std::sin(host[q]); co[q] = std::cos(host[q]); }
            CK(cudaMemcpyAsync(c->d_stage, sn.data(), ncells * sizeof(double), cudaMemcpyHostToDevice, s));
            launch_field_xfer(s, b, S_SINT, 1, fm.lb, 0, c->d_stage, 1);
            CK(cudaMemcpyAsync(c->d_stage, co.data(), ncells * sizeof(double), cudaMemcpyHostToDevice, s));
            launch_field_xfer(s, b, S_COST, 1, fm.lb, 0, c->d_stage, 1);
            CK(cudaStreamSynchronize(s));
        }
        if (is_geometry(f)) cs->geom_dirty = true;
        if (c->mixed && f == TRANS_D) mirror(c, {{S_D, 7}});
        if (c->mixed && f == TRANS_DQDXYZ) mirror(c, {{S_DQ, 18}});
        if (c->mixed && f == TRANS_SHOCK) mirror(c, {{S_SHOCK, 1}});
        // the caller's buffer is free once the copy is done; the transpose into the slots runs
        // on in stream order (later copies into the staging buffer queue behind it)
        CK(cudaGetLastError());
        if (sync) CK(cudaEventSynchronize(c->copy_done));
        return TRANS_OK;
    } else {
        // the mixed path keeps DeltaQ, the gradients and the shock sensor in FP32
        if (c->mixed && f == TRANS_D) mirror(c, {{S_D, 7}}, 1);
        if (c->mixed && f == TRANS_DQDXYZ) mirror(c, {{S_DQ, 18}}, 1);
        if (c->mixed && f == TRANS_SHOCK) mirror(c, {{S_SHOCK, 1}}, 1);
        launch_field_xfer(s, b, fm.slot, fm.ncomp, fm.lb, is_sd, c->d_stage, 0);
        c->launches++;
        CK(cudaMemcpyAsync(host, c->d_stage, bytes, cudaMemcpyDeviceToHost, s));
    }
    CK(cudaGetLastError());
    if (sync) CK(cudaStreamSynchronize(s));
    return TRANS_OK;
}

// ---------------------------------------------------------------------------------------
// LU-SGS sweep schedules (all compute every DeltaQ with the same operations)
// ---------------------------------------------------------------------------------------
namespace {

int sweep_once(Ctx* c, int mode, int grid, int block, bool capture = false) {
    const int lanes = c->sweep_lanes | c->sweep_wpc;
    if ((mode == 0 || mode == 5) && c->sweep_exec &&
        (c->sweep_exec_mode != mode || c->sweep_exec_pdl != c->pdl || c->sweep_exec_wpc != c->sweep_wpc || c->sweep_exec_pf != c->sweep_pf ||
         c->sweep_exec_cta != c->sweep_cta)) {   // changed
        cudaGraphExecDestroy(c->sweep_exec);
        c->sweep_exec = nullptr;
    }
    cudaStream_t s = c->stream;
    const int nh = (int)c->plane_off.size() - 1;
    if (mode == 3) {
        if (!c->d_tiles) {
            if (capture) return fail(c, TRANS_E_CUDA, "tiled sweep captured before its tiles were built");
            int rc = build_tiles(c, c->tile_default[0], c->tile_default[1], c->tile_default[2]);
            if (rc) return rc;
        }
        const int nt = c->tv.ntiles;
        CK(cudaMemsetAsync(c->d_tflags, 0, sizeof(int) * ((size_t)2 * nt + 1), s));
        CK(cudaMemsetAsync(c->d_sync, 0, sizeof(SweepSync), s));
        CK(c->fl->sweep_tiles(s, c->sv, c->tv, lanes, c->d_tflags, c->d_tflags + 2 * nt, c->d_sync, grid, block,
                                   c->spin_limit));
        CK(cudaMemcpyAsync(c->h_sync, c->d_sync, sizeof(SweepSync), cudaMemcpyDeviceToHost, s));
        c->launches++;
        return TRANS_OK;
    }
    if (mode == 4) {
        CK(launch_sweep_cluster(s, c->sv, c->d_pb_off, nh, (int)c->blk.size(), c->sweep_lanes, grid, block, c->sweep_pf));
        c->launches++;
        return TRANS_OK;
    }
    if (mode == 2) {
        const size_t np = (size_t)((c->sv.n + 31) / 32 * 32);
        CK(cudaMemsetAsync(c->d_flags, 0, 2 * np * sizeof(int), s));
        CK(cudaMemsetAsync(c->d_sync, 0, sizeof(SweepSync), s));
        CK(c->fl->sweep_flow(s, c->sv, c->d_flags, c->d_flags + np, c->sweep_lanes, c->d_sync, grid, block, c->spin_limit));
        CK(cudaMemcpyAsync(c->h_sync, c->d_sync, sizeof(SweepSync), cudaMemcpyDeviceToHost, s));
        c->launches++;
        return TRANS_OK;
    }
    if (mode == 1) {
        CK(cudaMemsetAsync(c->d_sync, 0, sizeof(SweepSync), s));
        CK(c->fl->sweep_all(s, c->sv, c->d_plane_off, nh, lanes, c->d_sync, grid, block, c->spin_limit));
        CK(cudaMemcpyAsync(c->h_sync, c->d_sync, sizeof(SweepSync), cudaMemcpyDeviceToHost, s));
        c->launches++;
        return TRANS_OK;
    }
    // one launch per hyperplane (mode 0) or per two (mode 5), L ascending then U descending,
    // replayed as one graph (or captured directly into the caller's graph)
    // hyperplane h of the L sweep prefetches hyperplane h + sweep_pf into L2, the U sweep h - sweep_pf
    // (mode 5: the planes of the pair sweep_pf launches ahead)
    if (mode == 5 && !c->fl->sweep_pair) return fail(c, TRANS_E_ARG, "two-plane sweeps are a mixed-path schedule");
    auto pairs = [&]() {
        const int d = c->sweep_pf;
        const int np = (int)c->pair_lo.size();
        auto pf_range = [&](const std::vector<Ctx::SweepPair>& v, int k, int& first, int& count) {
            first = 0; count = 0;
            if (!d || k + d >= (int)v.size()) return;
            const Ctx::SweepPair& a = v[k + d];
            if (a.p_count) { first = a.p_first; count = a.p_count; }
        };
        for (int k = 0; k < np; ++k) {
            const Ctx::SweepPair& a = c->pair_lo[k];
            int pf0, pfn;
            pf_range(c->pair_lo, k, pf0, pfn);
            c->fl->sweep_pair(s, c->sv, c->d_dq2, true, a.p_first, a.p_count, c->d_orph + a.o_off, a.o_count, lanes,
                              c->pdl, pf0, pfn, c->sweep_cta);
        }
        for (int k = 0; k < (int)c->pair_up.size(); ++k) {
            const Ctx::SweepPair& a = c->pair_up[k];
            int pf0, pfn;
            pf_range(c->pair_up, k, pf0, pfn);
            c->fl->sweep_pair(s, c->sv, c->d_dq2, false, a.p_first, a.p_count, c->d_orph + a.o_off, a.o_count, lanes,
                              c->pdl, pf0, pfn, c->sweep_cta);
        }
    };
    auto planes = [&]() {
        if (mode == 5) { pairs(); return; }
        const int d = c->sweep_pf;
        auto cnt = [&](int h) { return (h >= 0 && h < nh) ? c->plane_off[h + 1] - c->plane_off[h] : 0; };
        for (int h = 0; h < nh; ++h)
            if (cnt(h))
                c->fl->sweep_lower(s, c->sv, c->plane_off[h], cnt(h), lanes, c->pdl, d && h + d < nh ? c->plane_off[h + d] : 0,
                                   d ? cnt(h + d) : 0, c->sweep_cta);
        for (int h = nh - 1; h >= 0; --h)
            if (cnt(h))
                c->fl->sweep_upper(s, c->sv, c->plane_off[h], cnt(h), lanes, c->pdl, d && h - d >= 0 ? c->plane_off[h - d] : 0,
                                   d ? cnt(h - d) : 0, c->sweep_cta);
    };
    auto count_planes = [&]() {
        if (mode == 5) {
            for (const auto* v : {&c->pair_lo, &c->pair_up})
                for (const Ctx::SweepPair& a : *v) c->launches += (a.p_count + a.o_count > 0) ? 1 : 0;
            return;
        }
        for (int h = 0; h < nh; ++h) c->launches += (c->plane_off[h + 1] > c->plane_off[h]) ? 2 : 0;
    };
    if (capture) {              // captured into the caller's graph: every hyperplane launch counts per replay
        planes();
        count_planes();
        return TRANS_OK;
    }
    if (!c->sweep_exec) {
        cudaGraph_t g = nullptr;
        CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        planes();
        cudaError_t e = cudaStreamEndCapture(s, &g);
        if (e != cudaSuccess) return fail(c, TRANS_E_CUDA, std::string("sweep graph capture: ") + cudaGetErrorString(e));
        e = cudaGraphInstantiate(&c->sweep_exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return fail(c, TRANS_E_CUDA, std::string("sweep graph instantiate: ") + cudaGetErrorString(e));
        c->sweep_exec_mode = mode;
        c->sweep_exec_pdl = c->pdl;
        c->sweep_exec_wpc = c->sweep_wpc;
        c->sweep_exec_pf = c->sweep_pf;
        c->sweep_exec_cta = c->sweep_cta;
    }
    CK(cudaGraphLaunch(c->sweep_exec, s));
    count_planes();
    return TRANS_OK;
}

// keep a copy of the sweep-order DeltaQ (restore = copy it back)
int save_dq(Ctx* c, bool restore) {
    size_t bytes = (size_t)DQ_STRIDE * (size_t)((c->sv.n + 31) / 32 * 32) * c->fl->elem;
    if (!c->d_dq_save) CK(cudaMalloc(&c->d_dq_save, bytes));
    CK(cudaMemcpyAsync(restore ? c->sv.dq : c->d_dq_save, restore ? c->d_dq_save : c->sv.dq, bytes, cudaMemcpyDeviceToDevice,
                       c->stream));
    return TRANS_OK;
}

// Schedule tuner: time every candidate schedule on the live right-hand side (DeltaQ saved and
// restored around each trial), keep the fastest.
int tune_sweeps(Ctx* c) {
    int dev = 0, nsm = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    struct Cand { int mode, grid, block, pdl, ti, tj, tk, wpc, pf, cta = 0; };
    std::vector<Cand> cands;
    const bool fp32 = c->fl->elem == 4;
    if (fp32) {
        // mixed path: one thread per position; plain launches, or chained with the next
        // hyperplane released after the wait (1) or at entry (2); prefetch distance; CTA size
        for (int pdl : {0, 1, 2})
            for (int pf : {0, 2})
                for (int cta : {32, 64, 128}) cands.push_back({0, 0, 0, pdl, 0, 0, 0, 0, pf, cta});
        // two hyperplanes per launch, chained
        for (int pdl : {1, 2})
            for (int pf : {0, 1})
                for (int cta : {32, 64, 128}) cands.push_back({5, 0, 0, pdl, 0, 0, 0, 0, pf, cta});
        const int occ = c->fl->sweep_all_occupancy(256);
        if (occ >= 1) cands.push_back({1, nsm, 256, 0, 0, 0, 0, 0, 0});
        const int tocc = c->fl->sweep_tiles_occupancy(256);
        if (tocc >= 1) cands.push_back({3, tocc * nsm, 256, 0, 16, 4, 4, 0, 0});
        // one cluster per block: CTAs per cluster x CTA size, records prefetched 0 or 2 ahead
        for (int cs : {8, 16})
            for (int bs : {256, 512})
                if (sweep_cluster_fits(cs, bs) >= 1)
                    for (int pf : {0, 2}) cands.push_back({4, cs, bs, 0, 0, 0, 0, 0, pf});
    }
    for (int wpc : {0, SWEEP_WPC}) {
        if (fp32) break;
        for (int pf : {0, 1, 2, 4}) {             // prefetch distance (hyperplanes) of the plane launches
            cands.push_back({0, 0, 0, 1, 0, 0, 0, wpc, pf});
            cands.push_back({0, 0, 0, 0, 0, 0, 0, wpc, pf});
            cands.push_back({0, 0, 0, 2, 0, 0, 0, wpc, pf});     // next launch released at entry
        }
        for (int block : {128, 256, 512}) {
            int occ = c->fl->sweep_all_occupancy(block);
            for (int per : {1, 2, 4})
                if (per <= occ) cands.push_back({1, per * nsm, block, 0, 0, 0, 0, wpc, 0});
        }
        // tiled wavefront: tile shapes x CTA sizes, one resident wave of CTAs
        const int shapes[][3] = {{16, 4, 4}, {8, 4, 4}, {4, 4, 4}};
        for (const auto& sh : shapes)
            for (int block : {256, 512}) {
                const int occ = c->fl->sweep_tiles_occupancy(block);
                if (occ >= 1) cands.push_back({3, occ * nsm, block, 0, sh[0], sh[1], sh[2], wpc, 0});
            }
    }
    if (!fp32 && c->fl->sweep_flow_occupancy(256) >= 4) cands.push_back({2, 4 * nsm, 256, 0, 0, 0, 0, 0, 0});
    const int pdl0 = c->pdl_allowed;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    float best = 1e30f;
    Cand pick = cands[0];
    c->sweep_tuning.clear();
    int rc = save_dq(c, false);
    for (const Cand& k : cands) {
        if (k.mode == 0 || k.mode == 5) c->pdl = pdl0 ? k.pdl : 0;
        c->sweep_wpc = k.wpc;
        c->sweep_pf = k.pf;
        c->sweep_cta = k.cta;
        if (k.mode == 3 && (rc = build_tiles(c, k.ti, k.tj, k.tk))) break;
        for (int rep = 0; rep < 2 && rc == TRANS_OK; ++rep) {      // first run warms up (graph build)
            if ((rc = save_dq(c, true))) break;
            CK(cudaEventRecord(e0, c->stream));
            if ((rc = sweep_once(c, k.mode, k.grid, k.block))) break;
            CK(cudaEventRecord(e1, c->stream));
            CK(cudaEventSynchronize(e1));
            if (k.mode >= 1 && k.mode <= 3 && c->h_sync->err) { rc = -100; break; }   // the cooperative schedules report there
            float ms = 0;
            CK(cudaEventElapsedTime(&ms, e0, e1));
            if (rep == 1) {
                const std::string chain = c->pdl ? (c->pdl == 2 ? "-early" : "-chained") : "";
                c->sweep_tuning += (k.mode == 5 ? "pairs" + chain
                                    : k.mode ? std::string(k.mode == 1 ? "coop " : k.mode == 2 ? "flow " : k.mode == 4 ? "clusters " : "tiles ")
                                                 + (k.mode == 3 ? std::to_string(k.ti) + "x" + std::to_string(k.tj) + "x"
                                                                      + std::to_string(k.tk) + "/" : std::string())
                                                 + std::to_string(k.grid) + "x" + std::to_string(k.block)
                                           : std::string(c->pdl ? (c->pdl == 2 ? "planes-early" : "planes-chained") : "planes"))
                                   + (k.wpc ? "/wpc" : "") + (k.pf ? "/pf" + std::to_string(k.pf) : "")
                                   + (k.cta ? "/cta" + std::to_string(k.cta) : "")
                                   + ":" + std::to_string(ms) + "ms ";
                if (ms < best) { best = ms; pick = k; }
            }
        }
        if (rc == -100) rc = TRANS_OK;         // a schedule that timed out is just not picked
        if (rc) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    if ((rc = save_dq(c, true))) return rc;
    if (pick.mode == 3) {
        if ((rc = build_tiles(c, pick.ti, pick.tj, pick.tk))) return rc;
        c->tile_default[0] = pick.ti; c->tile_default[1] = pick.tj; c->tile_default[2] = pick.tk;   // kept over rebuilds
    }
    c->tuned_positions = c->sv.n;
    c->sweep_mode = pick.mode; c->sweep_grid = pick.grid; c->sweep_block = pick.block;
    c->sweep_wpc = pick.wpc;
    c->sweep_pf = pick.pf;
    c->sweep_cta = pick.cta;
    c->pdl = (pick.mode == 0 || pick.mode == 5) ? (pdl0 ? pick.pdl : 0) : 0;
    return TRANS_OK;
}

// The mixed path's two residual implementations (TMA-staged tiles, or k_face_flux + k_gather)
// compute the same FP32 face fluxes: time both on the live state (the residual stage only
// writes D and the FX slots), keep the faster.
int tune_resid(Ctx* c) {
    cudaStream_t s = c->stream;
    const int nct = (int)c->cell_tiles.size();
    auto run = [&](int tma) {
        if (tma) {
            for (int d = 0; d < 3; ++d)
                launch_resid_tma(d + 1, s, c->d_blk, c->d_rtiles[d], c->n_rtiles[d], c->d_cdev, c->d_rmaps, c->d_kerr,
                                 c->resid_spin);
        } else {
            for (int d = 0; d < 3; ++d) c->fl->face_flux[d](s, c->d_blk, c->d_face[d], (int)c->face_tiles[d].size(), c->d_cdev);
            c->fl->gather(s, c->d_blk, c->d_cell, nct, c->d_cdev);
        }
    };
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    float ms[2] = {0.f, 0.f};
    for (int v = 0; v < 2; ++v) {
        run(v);                                  // warm-up
        CK(cudaEventRecord(e0, s));
        for (int rep = 0; rep < 3; ++rep) run(v);
        CK(cudaEventRecord(e1, s));
        CK(cudaEventSynchronize(e1));
        CK(cudaEventElapsedTime(&ms[v], e0, e1));
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    CK(cudaGetLastError());
    c->resid_tma = ms[1] < ms[0] ? 1 : 0;
    c->resid_tuning = "tma:" + std::to_string(ms[1] / 3) + "ms gather:" + std::to_string(ms[0] / 3) + "ms";
    return TRANS_OK;
}

int run_sweeps(Ctx* c) {
    if (c->sweep_mode < 0) {
        int rc = tune_sweeps(c);
        if (rc) return rc;
    }
    return sweep_once(c, c->sweep_mode, c->sweep_grid, c->sweep_block);
}

bool wants_des(const CaseRec* cs) { return cs->p.Kind_Hybrid == 3; }
bool wants_dual(const CaseRec* cs) { return cs->p.Kind_Dual != 0; }

}  // namespace

// ---------------------------------------------------------------------------------------
// One hot-path subroutine over every block of every case (trans_run_stage)
// ---------------------------------------------------------------------------------------
namespace {

// One stage.  capture: inside a CUDA-graph capture (no host synchronisation, no parameter
// upload, the norms go to history slot `slot`).
int stage_exec(Ctx* c, int stage, int itr, bool capture, int slot) {
    if (c->cases.empty()) return fail(c, TRANS_E_ARG, "no case");
    int rc;
    if (!capture) {
        if (!c->built && (rc = rebuild(c))) return rc;
        if ((rc = finalize_geometry(c))) return rc;
    }
    cudaStream_t s = c->stream;
    const int nct = (int)c->cell_tiles.size();
    switch (stage) {
        case TRANS_STAGE_SPECRAD: {
            if (!capture && (rc = upload_cdev(c))) return rc;
            KScope t(c, K_SPECRAD);
            if (c->mixed) launch_specrad_mixed(s, c->d_blk, c->d_cell, nct, c->d_cdev);
            else launch_specrad(s, c->d_blk, c->d_cell, nct, c->d_cdev);
            c->launches++;
            break;
        }
        case TRANS_STAGE_BC_STATE:
            if (!capture && (rc = upload_cdev(c))) return rc;
            { KScope t(c, K_BC_STATE); launch_bc_state(s, c->d_blk, c->d_bc, (int)c->bc.size(), c->d_cdev); }
            {
                KScope t(c, K_BC_OUTLET);
                if (c->mixed) launch_bc_outlet_mixed(s, c->d_blk, c->d_outlet, c->d_lines, (int)c->lines.size(), c->d_cdev);
                else launch_bc_outlet(s, c->d_blk, c->d_outlet, c->d_lines, (int)c->lines.size(), c->d_cdev);
            }
            c->launches += 1 + (c->lines.empty() ? 0 : 1);
            break;
        case TRANS_STAGE_GRADIENT:
            if (!capture && (rc = upload_cdev(c))) return rc;
            if (c->mixed) {
                // the FP32 kernels read FP32 copies of this sub-iteration's state, primitives and radii
                KScope t(c, K_PRIMS);
                launch_prims_mixed(s, c->d_blk, (int)c->blk.size(), c->total_cells, c->d_off);
            } else {
                KScope t(c, K_PRIMS);
                launch_prims(s, c->d_blk, (int)c->blk.size(), c->total_cells, c->d_off);
            }
            { KScope t(c, K_GRADIENT); c->fl->gradient(s, c->d_blk, c->d_cell, nct, c->d_cdev); }
            { KScope t(c, K_SHOCK_GHOST); c->fl->shock_ghost(s, c->d_blk, c->d_ghost, (int)c->ghost_tiles.size()); }
            c->launches += 3;
            break;
        case TRANS_STAGE_BC_GRAD:
            { KScope t(c, K_BC_GRAD); c->fl->bc_grad(s, c->d_blk, c->d_bc, (int)c->bc.size()); }
            c->launches++;
            break;
        case TRANS_STAGE_RESIDUAL:
            if (!capture && (rc = upload_cdev(c))) return rc;
            if (c->mixed && c->resid_tma < 0 && !capture && (rc = tune_resid(c))) return rc;
            if (c->mixed && c->resid_tma == 1) {
                // FP32: fluxes from TMA-staged tiles, summed into D per direction
                for (int d = 0; d < 3; ++d) {
                    KScope t(c, K_RESID_TMA);
                    launch_resid_tma(d + 1, s, c->d_blk, c->d_rtiles[d], c->n_rtiles[d], c->d_cdev, c->d_rmaps, c->d_kerr,
                                     c->resid_spin);
                }
                c->launches += 3;
                break;
            }
            for (int d = 0; d < 3; ++d) {
                // the viscous and the convective fluxes of a direction are two launches
                KScope t(c, K_FACE, 2);
                c->fl->face_flux[d](s, c->d_blk, c->d_face[d], (int)c->face_tiles[d].size(), c->d_cdev);
            }
            { KScope t(c, K_GATHER); c->fl->gather(s, c->d_blk, c->d_cell, nct, c->d_cdev); }
            c->launches += 7;
            break;
        case TRANS_STAGE_LUSGS: {
            if (!capture && (rc = upload_cdev(c))) return rc;
            if (c->sweep_lanes == 2) {
                // Runge-Kutta: TIME_RK_Save + TIME_RK on the mean flow, then the k-omega LU-SGS
                // of TURBTWO_TIME_LUSGS_SST on the new state (main.F90:152-158)
                KScope t(c, K_UPDATE);
                launch_rk_update(s, c->d_blk, c->d_cell, nct, c->d_parts, c->mixed ? 1 : 0, itr);
                c->launches++;
            }
            if (any_case(c, wants_des)) {
                KScope t(c, K_SST_FC1);
                c->fl->sst_fc1(s, c->d_blk, c->d_cell, nct, c->d_cdev);
                c->launches++;
            }
            {
                KScope t(c, K_PREP);
                c->fl->prep(s, c->d_blk, c->d_cell, nct, c->d_qpos, c->sv, c->d_cdev);
                c->fl->jac(s, c->d_blk, c->sv, c->d_cdev);
            }
            c->launches += 2;
            {
                int nh = (int)c->plane_off.size() - 1, nl = 0;
                if (c->sweep_mode == 5) {
                    for (const auto* v : {&c->pair_lo, &c->pair_up})
                        for (const Ctx::SweepPair& a : *v) nl += (a.p_count + a.o_count > 0) ? 1 : 0;
                } else {
                    for (int h = 0; h < nh; ++h) nl += (c->plane_off[h + 1] > c->plane_off[h]) ? 2 : 0;
                }
                KScope t(c, K_SWEEP, (c->sweep_mode >= 1 && c->sweep_mode != 5) ? 1 : nl);
                if (capture) rc = sweep_once(c, c->sweep_mode, c->sweep_grid, c->sweep_block, true);
                else rc = run_sweeps(c);
                if (rc) return rc;
            }
            { KScope t(c, K_SCATTER); c->fl->scatter(s, c->d_blk, c->d_cell, nct, c->d_qpos, c->sv, c->sweep_lanes == 2 ? 5 : 0); }
            c->launches++;
            break;
        }
        case TRANS_STAGE_UPDATE: {
            if (!capture && (rc = upload_cdev(c))) return rc;
            const int nblk = (int)c->blk.size();
            {
                KScope t(c, K_UPDATE);
                if (c->sweep_lanes == 2) launch_rk_vupdate(s, c->d_blk, c->d_cell, nct, c->d_cdev, c->d_parts, c->mixed ? 1 : 0);
                else if (c->mixed) launch_update_mixed(s, c->d_blk, c->d_cell, nct, c->d_cdev, c->d_parts);
                else launch_update(s, c->d_blk, c->d_cell, nct, c->d_cdev, c->d_parts, 0);
                launch_block_norms(s, c->d_blk, nblk, c->d_parts, c->d_tile_first, c->d_norms + (size_t)slot * nblk);
            }
            c->launches += 2;
            if (capture) break;
            CK(cudaMemcpyAsync(c->h_norms, c->d_norms, sizeof(BlockNorms) * nblk, cudaMemcpyDeviceToHost, s));
            CK(cudaMemcpyAsync(c->h_kerr, c->d_kerr, sizeof(int), cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            if (c->sweep_mode >= 1 && c->sweep_mode <= 3 && c->h_sync->err) return fail(c, TRANS_E_TIMEOUT, "LU-SGS sweep wait timed out");
            if (*c->h_kerr) return fail(c, TRANS_E_TIMEOUT, "residual tile staging wait timed out");
            if ((rc = collect_norms(c, c->h_norms))) return rc;
            break;
        }
        case TRANS_STAGE_UPDATE_U:
            if (!capture && (rc = upload_cdev(c))) return rc;
            if (any_case(c, wants_dual)) {
                KScope t(c, K_UPDATE_U);
                launch_update_u(s, c->d_blk, c->d_cell, nct, c->d_cdev);
                c->launches++;
            }
            break;
        default:
            return fail(c, TRANS_E_ARG, "bad stage");
    }
    if (!capture) CK(cudaGetLastError());
    return TRANS_OK;
}

}  // namespace

int run_stage(Ctx* c, int stage, int itr) { return stage_exec(c, stage, itr, false, 0); }

// One outer iteration (main.F90:54-171 + :192-197) of every case at its current KI.
int run_iteration(Ctx* c) {
    if (c->cases.empty()) return fail(c, TRANS_E_ARG, "no case");
    const CaseRec* c0 = c->cases[0];
    const int nsub = sub_iterations(c0->p);
    int rc = TRANS_OK;
    for (int it = 1; it <= nsub && rc == TRANS_OK; ++it)
        for (int st = TRANS_STAGE_SPECRAD; st <= TRANS_STAGE_UPDATE && rc == TRANS_OK; ++st)
            rc = run_stage(c, st, it);
    if (rc == TRANS_OK) rc = run_stage(c, TRANS_STAGE_UPDATE_U, nsub);
    if (rc != TRANS_OK && rc != TRANS_E_NAN) return rc;
    for (CaseRec* cs : c->cases) {               // a NaN iteration still has its norms
        if (cs->iters == 0) cs->first_norms = cs->norms;
        cs->iters++;
    }
    return rc;
}

namespace {

// the cases' switches are the same for their next n KI values (graphs replay fixed parameters)
bool switches_fixed(Ctx* c, int n) {
    for (CaseRec* cs : c->cases) {
        const int ki = cs->KI;
        const CaseDev a = case_dev(cs);
        cs->KI = ki + n - 1;
        const CaseDev b = case_dev(cs);
        cs->KI = ki;
        if (a.CFL_sub != b.CFL_sub || a.turb != b.turb || a.turb_upd != b.turb_upd) return false;
        if (cs->p.CFL_Sub_end != cs->p.CFL_Sub_start && ki - cs->p.KI_ini < cs->p.CFL_Sub_step) return false;
    }
    return true;
}

// capture n iterations into c->iter_exec (n = GRAPH_ITERS) or c->iter1_exec (n = 1)
int capture_iterations(Ctx* c, int n) {
    cudaGraphExec_t& exec = n == 1 ? c->iter1_exec : c->iter_exec;
    if (exec) { cudaGraphExecDestroy(exec); exec = nullptr; }
    if (n != 1) c->iter_n = 0;
    if (c->sweep_mode == 3 && !c->d_tiles) {          // allocations cannot happen inside the capture
        int rc = build_tiles(c, c->tile_default[0], c->tile_default[1], c->tile_default[2]);
        if (rc) return rc;
    }
    const CaseRec* c0 = c->cases[0];
    const int nsub = sub_iterations(c0->p);
    const int nblk = (int)c->blk.size();
    cudaStream_t s = c->stream;
    cudaGraph_t g = nullptr;
    const long long launches0 = c->launches;
    CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    int rc = TRANS_OK;
    for (int q = 0; q < n && rc == TRANS_OK; ++q) {
        for (int it = 1; it <= nsub && rc == TRANS_OK; ++it)
            for (int st = TRANS_STAGE_SPECRAD; st <= TRANS_STAGE_UPDATE && rc == TRANS_OK; ++st)
                rc = stage_exec(c, st, it, true, q);
        if (rc == TRANS_OK) rc = stage_exec(c, TRANS_STAGE_UPDATE_U, nsub, true, q);
    }
    if (rc == TRANS_OK) {
        cudaMemcpyAsync(c->h_norms, c->d_norms, sizeof(BlockNorms) * (size_t)nblk * n, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(c->h_sync, c->d_sync, sizeof(SweepSync), cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(c->h_kerr, c->d_kerr, sizeof(int), cudaMemcpyDeviceToHost, s);
    }
    cudaError_t e = cudaStreamEndCapture(s, &g);
    if (rc) { if (g) cudaGraphDestroy(g); return rc; }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(c, TRANS_E_CUDA, std::string("iteration graph capture: ") + cudaGetErrorString(e));
    }
    e = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(c, TRANS_E_CUDA, std::string("iteration graph instantiate: ") + cudaGetErrorString(e));
    }
    if (n == 1) {
        c->iter1_launches = c->launches - launches0;
    } else {
        c->iter_n = n;
        c->iter_launches = c->launches - launches0;       // kernels per replay
    }
    c->launches = launches0;
    return TRANS_OK;
}

}  // namespace

int run_iterations(Ctx* c, int n) {
    if (c->cases.empty()) return fail(c, TRANS_E_ARG, "no case");
    int rc, done = 0;
    bool first = true;
    auto advance = [&]() {
        for (CaseRec* cs : c->cases) cs->KI++;
    };
    while (done < n) {
        if (!first) advance();                  // KI of this iteration
        first = false;
        // an ordinary iteration builds the work lists and the geometry terms and tunes the
        // sweeps; graphs replay iterations whose switches (CFL ramp, turbulence) are fixed
        // (a single iteration replays a one-iteration graph: its switches are uploaded with it)
        const bool tuned = c->graphs && c->built && c->sweep_mode >= 0 && !(c->mixed && c->resid_tma < 0);
        const bool graph = tuned && n - done >= GRAPH_ITERS && switches_fixed(c, GRAPH_ITERS);
        const bool graph1 = tuned && !graph && n - done < GRAPH_ITERS;
        if (!graph && !graph1) {
            if ((rc = run_iteration(c))) return rc;
            ++done;
            continue;
        }
        const int m = graph ? GRAPH_ITERS : 1;
        if ((rc = finalize_geometry(c)) || (rc = upload_cdev(c))) return rc;
        const bool have = graph ? (c->iter_exec && c->iter_n == m) : c->iter1_exec != nullptr;
        if (!have && capture_iterations(c, m) != TRANS_OK) {
            c->graphs = false;                  // not capturable here: launch directly from now on
            if ((rc = run_iteration(c))) return rc;
            ++done;
            continue;
        }
        CK(cudaGraphLaunch(graph ? c->iter_exec : c->iter1_exec, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        c->launches += graph ? c->iter_launches : c->iter1_launches;
        const int nblk = (int)c->blk.size();
        int nan = 0;
        for (int q = 0; q < m; ++q) {
            nan |= collect_norms(c, c->h_norms + (size_t)q * nblk) == TRANS_E_NAN;
            for (CaseRec* cs : c->cases) {
                if (cs->iters == 0) cs->first_norms = cs->norms;
                cs->iters++;
            }
        }
        for (int q = 1; q < m; ++q) advance();  // KI of the last replayed iteration
        done += m;
        if (c->sweep_mode >= 1 && c->sweep_mode <= 3 && c->h_sync->err) return fail(c, TRANS_E_TIMEOUT, "LU-SGS sweep wait timed out");
        if (*c->h_kerr) return fail(c, TRANS_E_TIMEOUT, "residual tile staging wait timed out");
        if (nan) return fail(c, TRANS_E_NAN, "NaN in the density increment");
    }
    return TRANS_OK;
}

int prepare(Ctx* c) {
    if (c->cases.empty()) return fail(c, TRANS_E_ARG, "no case");
    int rc;
    for (int st = TRANS_STAGE_SPECRAD; st <= TRANS_STAGE_LUSGS; ++st)
        if ((rc = run_stage(c, st, 1))) return rc;
    CK(cudaStreamSynchronize(c->stream));
    if (c->graphs && switches_fixed(c, GRAPH_ITERS) && (!c->iter_exec || c->iter_n != GRAPH_ITERS)) {
        if ((rc = upload_cdev(c))) return rc;
        if (capture_iterations(c, GRAPH_ITERS) != TRANS_OK) c->graphs = false;
    }
    return TRANS_OK;
}

int kernel_times(Ctx* c, double* ms, int* launches) {
    for (int k = 0; k < NKCLASS; ++k) { ms[k] = 0.0; launches[k] = 0; }
    c->ktime_on = true;
    c->kev.clear();
    int rc = run_iteration(c);
    c->ktime_on = false;
    cudaStreamSynchronize(c->stream);
    for (auto& e : c->kev) {
        float t = 0;
        if (cudaEventElapsedTime(&t, e.a, e.b) == cudaSuccess) { ms[e.k] += t; launches[e.k] += e.n; }
        cudaEventDestroy(e.a);
        cudaEventDestroy(e.b);
    }
    c->kev.clear();
    return rc;
}


// ---- integrated quantities (trans_get_integrals, trans_get_wall_cp) ----
int all_integrals(Ctx* c, std::vector<trans_integrals>& out) {
    if (c->cases.empty()) return fail(c, TRANS_E_ARG, "no case");
    int rc;
    if (!c->built && (rc = rebuild(c))) return rc;
    if ((rc = upload_cdev(c))) return rc;
    const int nc = (int)c->cases.size();
    launch_integrals(c->stream, c->d_blk, c->d_bc, c->d_bc_first, nc, c->d_cdev, c->d_intg);
    c->launches++;
    CK(cudaGetLastError());
    std::vector<double> h((size_t)NINTG * nc);
    CK(cudaMemcpyAsync(h.data(), c->d_intg, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    out.assign(nc, trans_integrals{});
    for (int k = 0; k < nc; ++k) {
        const double* q = &h[(size_t)NINTG * k];
        trans_integrals& r = out[k];
        r.mass_in = q[0];
        r.p0_in = q[0] != 0.0 ? q[1] / q[0] : 0.0;
        r.p_in = q[0] != 0.0 ? q[2] / q[0] : 0.0;
        r.mass_out = q[3];
        r.p0_out = q[3] != 0.0 ? q[4] / q[3] : 0.0;
        r.p_out = q[3] != 0.0 ? q[5] / q[3] : 0.0;
        r.loss = r.p0_in != r.p_in ? (r.p0_in - r.p0_out) / (r.p0_in - r.p_in) : 0.0;
        for (int d = 0; d < 3; ++d) { r.force_p[d] = q[6 + d]; r.force_v[d] = q[9 + d]; }
    }
    return TRANS_OK;
}

int integrals(Ctx* c, CaseRec* cs, trans_integrals* out) {
    if (!c || !cs || !out) return TRANS_E_ARG;
    std::vector<trans_integrals> all;
    int rc = all_integrals(c, all);
    if (rc) return rc;
    for (size_t k = 0; k < c->cases.size(); ++k)
        if (c->cases[k] == cs) { *out = all[k]; return TRANS_OK; }
    return fail(c, TRANS_E_ARG, "case not in the context");
}

int wall_cp(Ctx* c, CaseRec* cs, int ib, int iconn, double* cp, bool forces) {
    if (!c || !cs || !cp) return TRANS_E_ARG;
    if (ib < 0 || ib >= (int)cs->hb.size()) return fail(c, TRANS_E_ARG, "bad block index");
    const HostBlock& h = cs->hb[ib];
    if (iconn < 1 || iconn > (int)h.conn.size()) return fail(c, TRANS_E_ARG, "bad connection index");
    if (h.conn[iconn - 1].BCType != 1) return fail(c, TRANS_E_ARG, "connection is not a wall (kind 1)");
    int rc;
    if (!c->built && (rc = rebuild(c))) return rc;
    if ((rc = upload_cdev(c))) return rc;
    // entries of the segment in the context's table: cases, blocks and connections in order
    size_t k = 0;
    while (k < c->cases.size() && c->cases[k] != cs) ++k;
    if (k == c->cases.size()) return fail(c, TRANS_E_ARG, "case not in the context");
    long long e0 = c->bc_first[k], n = 0;
    for (int nb = 0; nb <= ib; ++nb)
        for (int ic = 0; ic < (int)cs->hb[nb].conn.size(); ++ic) {
            const trans_conn& a = cs->hb[nb].conn[ic];
            if (a.BCType == 9 && block_index(cs, a.TargetBlock) < 0) continue;     // cross-rank: not in the table
            long long cnt = 1;
            for (int q = 0; q < 3; ++q) cnt *= (long long)(a.pointEnd[q] - a.pointStart[q] + 1);
            if (nb == ib && ic == iconn - 1) { n = cnt; break; }
            e0 += cnt;
        }
    if (e0 + n > c->bc_first[k + 1]) return fail(c, TRANS_E_ARG, "wall segment outside the boundary table");
    const size_t words = (size_t)n * (forces ? 6 : 1);
    if (!c->d_stage || c->stage_doubles < words) {      // the staging buffer holds the segment's values
        CK(cudaStreamSynchronize(c->stream));
        if (c->d_stage) cudaFree(c->d_stage);
        c->d_stage = nullptr;
        c->stage_doubles = 0;
        CK(cudaMalloc(&c->d_stage, words * sizeof(double)));
        c->stage_doubles = words;
    }
    if (forces) launch_wall_forces(c->stream, c->d_blk, c->d_bc, (int)e0, (int)n, c->d_cdev, c->d_stage);
    else launch_wall_cp(c->stream, c->d_blk, c->d_bc, (int)e0, (int)n, c->d_cdev, c->d_stage);
    c->launches++;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(cp, c->d_stage, sizeof(double) * words, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return TRANS_OK;
}

// Cross-rank 1-to-1 interfaces (BC/PARALLEL_BC_P2P.F90:1-257, Common/PARALLEL_Funcs.F90:57-87):
// the caller exchanges the words of a segment whose target block is in another context after
// BC_STATE (sweep -1) and BC_GRAD (sweep 0).  Pack: this segment's interior layers, face cells in
// the segment's K, J, I order.  Unpack: this segment's ghost layers from the partner segment's
// words, through the same index transform and rotation as the same-rank copy.  The buffers are
// host memory; the tables and words go through a device staging area of the context.
int halo_io(Ctx* c, CaseRec* cs, int sweep, int ib, int iconn, const trans_conn* partner, double* buf, bool pack) {
    if (!c || !cs || !buf || (sweep != -1 && sweep != 0) || (!pack && !partner)) return TRANS_E_ARG;
    if (ib < 0 || ib >= (int)cs->hb.size()) return fail(c, TRANS_E_ARG, "bad block index");
    const HostBlock& h = cs->hb[ib];
    if (iconn < 1 || iconn > (int)h.conn.size() || h.conn[iconn - 1].BCType != 9)
        return fail(c, TRANS_E_ARG, "connection is not a 1-to-1 interface (kind 9)");
    int rc;
    if (!c->built && (rc = rebuild(c))) return rc;
    const trans_conn& a = h.conn[iconn - 1];
    const DevBlock& b = cs->blk[ib];
    const int W = sweep == -1 ? 36 : 18;
    std::vector<int> tab;
    int n = 0;
    const int* S3[3] = {a.CIJKAdd, a.CIJKAdd1, a.CIJKAdd2};
    const int* E3[3] = {a.CEIJKAdd, a.CEIJKAdd1, a.CEIJKAdd2};
    long long nwords = 0;
    if (pack) {
        for (int K = a.pointStart[2]; K <= a.pointEnd[2]; ++K)
            for (int J = a.pointStart[1]; J <= a.pointEnd[1]; ++J)
                for (int I = a.pointStart[0]; I <= a.pointEnd[0]; ++I, ++n)
                    for (int L = 0; L < 3; ++L) tab.push_back(cidx(b, I + S3[L][0], J + S3[L][1], K + S3[L][2]));
        nwords = (long long)n * W;
    } else {
        const trans_conn& t = *partner;
        const int ti = t.pointEnd[0] - t.pointStart[0] + 1, tj = t.pointEnd[1] - t.pointStart[1] + 1;
        const int tk = t.pointEnd[2] - t.pointStart[2] + 1;
        if (ti < 1 || tj < 1 || tk < 1) return fail(c, TRANS_E_ARG, "bad partner segment");
        const int IIadd = a.pointEnd[0] - a.pointStart[0] + 2, JJadd = a.pointEnd[1] - a.pointStart[1] + 2;
        const int KKadd = a.pointEnd[2] - a.pointStart[2] + 2;
        for (int K = a.pointStart[2]; K <= a.pointEnd[2]; ++K)
            for (int J = a.pointStart[1]; J <= a.pointEnd[1]; ++J)
                for (int I = a.pointStart[0]; I <= a.pointEnd[0]; ++I, ++n) {
                    int iL = I - a.pointStart[0] + 1, jL = J - a.pointStart[1] + 1, kL = K - a.pointStart[2] + 1;
                    iL = a.revMatrix[0] * IIadd + (1 - 2 * a.revMatrix[0]) * iL;
                    jL = a.revMatrix[1] * JJadd + (1 - 2 * a.revMatrix[1]) * jL;
                    kL = a.revMatrix[2] * KKadd + (1 - 2 * a.revMatrix[2]) * kL;
                    int pb, pj, pk;
                    ijk_start_end(iL, jL, kL, pb, pj, pk, a.Transform, a.TransformT, a.lcross);
                    pb -= 1; pj -= 1; pk -= 1;
                    if (pb < 0 || pb >= ti || pj < 0 || pj >= tj || pk < 0 || pk >= tk)
                        return fail(c, TRANS_E_ARG, "partner face cell outside the partner segment");
                    tab.push_back(pb + ti * (pj + tj * pk));
                    for (int L = 0; L < 3; ++L) tab.push_back(cidx(b, I + E3[L][0], J + E3[L][1], K + E3[L][2]));
                }
        nwords = (long long)ti * tj * tk * W;
    }
    // device staging: the table, then the words (16-byte aligned)
    const size_t tbytes = (tab.size() * sizeof(int) + 15) / 16 * 16;
    const size_t need = tbytes + (size_t)nwords * sizeof(double);
    if (c->halo_bytes < need) {
        CK(cudaStreamSynchronize(c->stream));
        if (c->d_halo) cudaFree(c->d_halo);
        c->d_halo = nullptr;
        c->halo_bytes = 0;
        CK(cudaMalloc(&c->d_halo, need));
        c->halo_bytes = need;
    }
    int* d_tab = (int*)c->d_halo;
    double* d_words = (double*)((char*)c->d_halo + tbytes);
    cudaStream_t s = c->stream;
    CK(cudaMemcpyAsync(d_tab, tab.data(), tab.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    if (pack) {
        launch_halo_pack(s, b, d_tab, n, sweep, c->mixed ? 1 : 0, d_words);
        CK(cudaMemcpyAsync(buf, d_words, (size_t)nwords * sizeof(double), cudaMemcpyDeviceToHost, s));
    } else {
        CK(cudaMemcpyAsync(d_words, buf, (size_t)nwords * sizeof(double), cudaMemcpyHostToDevice, s));
        // the state in FP64 (the FP64 unit's contraction, as k_bc_state); the gradients in the
        // context's precision (as k_bc_grad of that precision)
        const FluxLaunchers& fl = sweep == -1 ? flux_launchers_f64() : *c->fl;
        fl.halo_unpack(s, b, d_tab, n, sweep, std::cos(a.rotateAngle), std::sin(a.rotateAngle), d_words);
    }
    c->launches++;
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s));
    return TRANS_OK;
}

int fields_io(Ctx* c, CaseRec* cs, int n, const int* ib, const int* f, double* const* host, bool upload) {
    if (!c || !cs || n < 0 || (n > 0 && (!ib || !f || !host))) return TRANS_E_ARG;
    // page-locked arrays of plain fields go in batches, one launch each over the host link; the
    // rest (pageable arrays, fields with FP32 copies or derived slots) one by one, in the
    // caller's order (a batch is launched before the next array that is not in it, or that
    // names a block and field the batch already holds)
    XferBatch x;
    std::memset(&x, 0, sizeof(x));
    long long total = 0;
    const int ch = upload ? XFER_CHUNK : 1;      // elements per thread
    std::vector<std::pair<int, int>> held;
    auto flush = [&]() {
        if (x.n == 0) return;
        launch_fields_xfer(c->stream, x, total, upload ? 1 : 0, ch);
        c->launches++;
        std::memset(&x, 0, sizeof(x));
        total = 0;
        held.clear();
    };
    for (int q = 0; q < n; ++q) {
        const int fq = f[q];
        const FieldMap fm = field_map(fq);
        double* mapped = nullptr;
        long long cnt = 0;
        if (c->xfer_batch && ib[q] >= 0 && ib[q] < (int)cs->blk.size() && host[q] && fm.slot >= 0 && fq != TRANS_THTC &&
            fq != TRANS_D && fq != TRANS_DQDXYZ && fq != TRANS_SHOCK && !(fq == TRANS_WT2 && cs->p.IF_RK != 1)) {
            const DevBlock& bq = cs->blk[ib[q]];
            cnt = (long long)(bq.NI + 3 - fm.lb) * (bq.NJ + 3 - fm.lb) * (bq.NK + 3 - fm.lb) * fm.ncomp;
            mapped = c->xfer_mapped ? mapped_host(host[q], (size_t)cnt * sizeof(double)) : nullptr;
        }
        if (!mapped) {
            flush();
            int rc = field_io(c, cs, ib[q], fq, host[q], upload, false);
            if (rc) {
                cudaStreamSynchronize(c->stream);    // the arrays already queued are settled either way
                return rc;
            }
            continue;
        }
        if ((uintptr_t)mapped & 15) {          // 16-byte host accesses need an aligned array
            flush();
            int rc = field_io(c, cs, ib[q], fq, host[q], upload, false);
            if (rc) {
                cudaStreamSynchronize(c->stream);
                return rc;
            }
            continue;
        }
        if (x.n == XFER_MAX || std::find(held.begin(), held.end(), std::make_pair(ib[q], fq)) != held.end()) flush();
        const DevBlock& b = cs->blk[ib[q]];
        XferEntry& E = x.e[x.n++];
        E.base = b.base; E.host = mapped; E.off = total; E.count = cnt;
        E.ncell = b.ncell; E.PI = b.PI; E.PJ = b.PJ; E.ei = b.NI + 3 - fm.lb; E.ej = b.NJ + 3 - fm.lb;
        E.slot0 = fm.slot; E.ncomp = fm.ncomp; E.lb = fm.lb; E.is_sd = fq == TRANS_SD ? 1 : 0;
        total += (cnt + ch - 1) / ch;      // chunks
        held.emplace_back(ib[q], fq);
        if (upload && is_geometry(fq)) cs->geom_dirty = true;
    }
    flush();
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->stream));
    return TRANS_OK;
}

}  // namespace eng
}  // namespace tg
