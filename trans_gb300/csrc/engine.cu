// engine.cu -- contexts and cases: validation, device arenas, the work lists that cover every
// case of a context, and the boundary gather tables (from the reference's ConnectivityStruct).
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>

#include "engine.h"

namespace tg {
namespace eng {

const char* const kclass_name[NKCLASS] = {"k_specrad", "k_bc_state", "k_bc_outlet", "k_prims", "k_mirror", "k_gradient",
    "k_shock_ghost", "k_bc_grad", "k_face_flux", "k_gather", "k_sst_fc1", "k_lusgs_prep", "k_sweep", "k_sweep_scatter",
    "k_update", "k_update_u", "k_resid_tma"};

int fail(Ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}

KScope::KScope(Ctx* c_, int k_, int n_) : c(c_), k(k_), n(n_) {
    if (c->ktime_on && cudaEventCreate(&a) == cudaSuccess && cudaEventCreate(&b) == cudaSuccess) cudaEventRecord(a, c->stream);
}
KScope::~KScope() {
    if (c->ktime_on && a && b) { cudaEventRecord(b, c->stream); c->kev.push_back({k, n, a, b}); }
}

namespace {

template <typename T> void dfree(T*& p) { if (p) cudaFree((void*)p); p = nullptr; }

// module globals of one case as the kernels read them (trans_params + derived)
Params make_params(const trans_params& p) {
    Params d;
    std::memset(&d, 0, sizeof(d));
    d.XM = p.XM; d.RXM2 = p.RXM2; d.PPF = p.PPF; d.Csthlnd = p.Csthlnd; d.Csth1 = p.Csth1; d.Ref = p.Ref;
    d.Tiny = p.Tiny; d.VxF = p.VxF; d.VyF = p.VyF; d.VzF = p.VzF; d.omega0 = p.omega[0];
    d.P0in = p.P0in; d.T0in = p.T0in; d.Pouthub = p.Pouthub; d.VisRatio = p.VisRatio; d.FSTI = p.FSTI;
    d.A1 = p.A1; d.Beta_star = p.Beta_star; d.Sigk1 = p.Sigk1; d.Sigo1 = p.Sigo1; d.Beta1 = p.Beta1;
    d.Gama1 = p.Gama1; d.Sigk2 = p.Sigk2; d.Sigo2 = p.Sigo2; d.Beta2 = p.Beta2; d.Gama2 = p.Gama2;
    d.Prod_Lmt = p.Prod_Lmt; d.gama_max = p.gama_max; d.gama_min = p.gama_min; d.F_limiter1 = p.F_limiter1; d.F_limiter2 = p.F_limiter2; d.Alscale = p.Alscale;
    d.DT_LUSGS_Main = p.DT_LUSGS_Main; d.DT_LUSGS_Sub = p.DT_LUSGS_Sub; d.CFL_Main = p.CFL_Main;
    d.Trans_location = p.Trans_location;
    d.Kind_Spatial = p.Kind_Spatial; d.Kind_Roe = p.Kind_Roe; d.Kind_Hybrid = p.Kind_Hybrid;
    d.Kind_SubHY = p.Kind_SubHY; d.Kind_Dual = p.Kind_Dual; d.IF_Local_Main = p.IF_Local_Main;
    d.IF_Local_Sub = p.IF_Local_Sub; d.IF_Comppress = p.IF_Comppress; d.If_fix_Transition = p.If_fix_Transition;
    d.Kind_Model = p.Kind_Model; d.IF_Precondition = p.IF_Precondition; d.Kind_RotMod = p.Kind_RotMod;
    return d;
}

}  // namespace

// options outside the configurations of this hot path are rejected, never approximated
bool params_supported(const trans_params* p) {
    // RC correction (Kind_RotMod 1; 2 computes a factor nothing reads)
    if ((p->IF_Precondition != 0 && p->IF_Precondition != 1) || p->Kind_RotMod < 0 || p->Kind_RotMod > 2 ||
        (p->Kind_Model != 1 && p->Kind_Model != 2) || p->IF_Euler != 0)
        return false;
    // low-Mach preconditioning: LU-SGS marching, FP64 path
    if (p->IF_Precondition == 1 && (p->IF_RK != 0 || p->precision != TRANS_FP64)) return false;
    if (p->IF_RK != 0 && p->IF_RK != 1) return false;
    if (p->Kind_Spatial < 1 || p->Kind_Spatial > 4 || p->Kind_Roe < 1 || p->Kind_Roe > 3) return false;
    if (p->Kind_Hybrid != 0 && p->Kind_Hybrid != 3) return false;
    // DES (0), the DDES shielding functions (1-3) and IDDES (5); FSST is undefined for 4
    if (p->Kind_Hybrid == 3 && (p->Kind_SubHY < 0 || p->Kind_SubHY > 5 || p->Kind_SubHY == 4)) return false;
    // a frame rotating about the x axis at omega(1); omega(2) and omega(3) are read by no
    // routine of the path
    if (!std::isfinite(p->omega[0])) return false;
    if (p->precision != TRANS_FP64 && p->precision != TRANS_MIXED) return false;
    // the rotated Roe scheme splits its dissipation along the direction of the velocity jump,
    // which FP32 rounding turns into noise where the two states nearly agree: FP64 path only
    if (p->precision == TRANS_MIXED && p->Kind_Roe == 2) return false;
    if (p->Kind_Dual != 0 && p->Kchld < 1) return false;
    return true;
}

bool block_ok(const trans_block& tb) {
    if (tb.ni < 4 || tb.nj < 4 || tb.nk < 4 || tb.nconn < 0 || (tb.nconn > 0 && !tb.conn)) return false;
    return (long long)padded_pi(tb.ni) * (tb.nj + 5) * (tb.nk + 5) <= (1LL << 30);
}

int validate_case(const trans_params* p, int nblocks, const trans_block* blocks) {
    if (!p || !blocks || nblocks <= 0 || !params_supported(p)) return TRANS_E_ARG;
    for (int n = 0; n < nblocks; ++n)
        if (!block_ok(blocks[n])) return TRANS_E_ARG;
    return TRANS_OK;
}

namespace {

// wall marks on faces (Input/Read_BlockDimensions.F90:240-283) into the S_WALL slots
int upload_walls(Ctx* c, const HostBlock& h, const DevBlock& b) {
    for (int d = 0; d < 3; ++d) {
        std::vector<double> w(b.ncell, 0.0);
        bool any = false;
        for (int side = 0; side < 2; ++side) {
            const std::vector<int>& m = h.mw[2 * d + side];
            if (m.empty()) continue;
            int na = d == 0 ? b.NJ1 : b.NI1, nb2 = d == 2 ? b.NJ1 : b.NK1;
            for (int q = 0; q < nb2; ++q)
                for (int a = 0; a < na; ++a) {
                    if (m[(size_t)a + (size_t)na * q] != 1) continue;
                    int fi, fj, fk;
                    int face = side ? (d == 0 ? b.NI : d == 1 ? b.NJ : b.NK) : 1;
                    if (d == 0) { fi = face; fj = a + 1; fk = q + 1; }
                    else if (d == 1) { fi = a + 1; fj = face; fk = q + 1; }
                    else { fi = a + 1; fj = q + 1; fk = face; }
                    w[cidx(b, fi, fj, fk)] = 1.0;
                    any = true;
                }
        }
        if (any) CK(cudaMemcpy(b.base + (size_t)(S_WALL + d) * b.ncell, w.data(), sizeof(double) * b.ncell, cudaMemcpyHostToDevice));
    }
    return TRANS_OK;
}

}  // namespace

// Device bytes one case takes: its slot arena (+ FP32 copies in the mixed path) and its share
// of the sweep-order arrays and work lists.
long long case_bytes(const trans_params* p, int nblocks, const trans_block* blocks) {
    const int precision = p->precision;
    long long padded = 0, interior = 0;
    for (int n = 0; n < nblocks; ++n) {
        padded += (long long)padded_pi(blocks[n].ni) * (blocks[n].nj + 5) * (blocks[n].nk + 5);
        interior += (long long)(blocks[n].ni - 1) * (blocks[n].nj - 1) * (blocks[n].nk - 1);
    }
    const long long elem = precision == TRANS_MIXED ? 4 : 8;
    long long b = padded * case_slots(*p) * (8 + (precision == TRANS_MIXED ? 4 : 0));
    const long long rec = precision == TRANS_MIXED ? NCREC : NREC;      // sweep record entries per position
    // DeltaQ arrays: the sweep's, the tuner's copy, and in the mixed path the two-plane schedule's second one
    const long long ndq = precision == TRANS_MIXED ? 3 : 2;
    b += interior * ((rec + ndq * DQ_STRIDE) * elem + 8LL * 4 + (long long)sizeof(SweepCell));
    if (p->IF_Precondition == 1) b += interior * 6LL * NPC * 8;          // the neighbours' PrecondDW coefficients
    b += interior / 16 + 4096;           // tiles, norm partials, boundary tables (rounded up)
    return b;
}

int ctx_init(Ctx* c, int precision, long long budget) {
    c->precision = precision;
    c->mixed = precision == TRANS_MIXED;
    c->fl = c->mixed ? &flux_launchers_f32() : &flux_launchers_f64();
    c->budget = budget;
    CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    CK(cudaMalloc(&c->d_sync, sizeof(SweepSync)));
    CK(cudaMallocHost(&c->h_sync, sizeof(SweepSync)));
    std::memset(c->h_sync, 0, sizeof(SweepSync));
    CK(cudaMalloc(&c->d_kerr, sizeof(int)));
    CK(cudaMemset(c->d_kerr, 0, sizeof(int)));
    CK(cudaMallocHost(&c->h_kerr, sizeof(int)));
    *c->h_kerr = 0;
    // TRANS_RESID_TMA=0 | 1 | auto: the mixed path's residual from k_face_flux + k_gather (the
    // default), from the TMA-staged tiles, or the faster of the two on the context's first
    // residual
    const char* rt = std::getenv("TRANS_RESID_TMA");
    if (rt && std::string(rt) == "0") c->resid_tma = 0;
    if (rt && std::string(rt) == "1") c->resid_tma = 1;
    if (rt && std::string(rt) == "auto") c->resid_tma = -1;
    // TRANS_XFER_BATCH=0: trans_set/get_fields transfer the arrays one launch each (for comparisons)
    const char* xb = std::getenv("TRANS_XFER_BATCH");
    if (xb && std::string(xb) == "0") c->xfer_batch = false;
    // TRANS_XFER_DMA=1: page-locked arrays too go through the staging buffer by DMA copies
    const char* xd = std::getenv("TRANS_XFER_DMA");
    if (xd && std::string(xd) == "1") c->xfer_mapped = false;
    // TRANS_RESID_SPIN=n: polls of the tile staging wait before it gives up (for tests)
    const char* rsp = std::getenv("TRANS_RESID_SPIN");
    if (rsp) c->resid_spin = (unsigned)std::max(0L, std::atol(rsp));
    // TRANS_GRAPHS=0 turns the whole-iteration graphs off (every iteration launched directly)
    const char* gr = std::getenv("TRANS_GRAPHS");
    if (gr && std::string(gr) == "0") c->graphs = false;
    // TRANS_PDL=0 launches the hyperplanes without programmatic dependent launch; TRANS_PDL=2
    // releases the next hyperplane's launch at entry (mixed path)
    const char* pd = std::getenv("TRANS_PDL");
    if (pd && std::string(pd) == "0") c->pdl = c->pdl_allowed = 0;
    if (pd && std::string(pd) == "2") c->pdl = 2;
    // TRANS_SWEEP_CTA=n: CTA size of the mixed path's hyperplane launches (for tests and captures)
    const char* sc = std::getenv("TRANS_SWEEP_CTA");
    if (sc) c->sweep_cta = std::max(0, std::atoi(sc));
    // TRANS_SWEEP_MAP=wpc forces the warp-per-component thread mapping of the sweeps (for tests)
    const char* wm = std::getenv("TRANS_SWEEP_MAP");
    if (wm && std::string(wm) == "wpc") c->sweep_wpc = SWEEP_WPC;
    // TRANS_SWEEP_PF=n forces an L2 prefetch distance of n hyperplanes (for tests)
    const char* pf = std::getenv("TRANS_SWEEP_PF");
    if (pf) c->sweep_pf = std::max(0, std::atoi(pf));
    // TRANS_SWEEP_SPIN=n bounds every device-side wait of the cooperative sweep schedules at n
    // polls (for tests of the timeout path: a small n makes the waits run out)
    const char* sp = std::getenv("TRANS_SWEEP_SPIN");
    if (sp) c->spin_limit = (unsigned)std::max(0L, std::strtol(sp, nullptr, 10));
    // sweep schedule: TRANS_SWEEP=planes | coop | flow | tiles | clusters | pairs forces one (for tests);
    // default: tuned
    const char* m = std::getenv("TRANS_SWEEP");
    std::string ms = m ? m : "";
    // clusters: the mixed path's cluster-barrier schedule (the FP64 path takes planes)
    if (ms == "clusters") ms = c->mixed ? "clusters" : "planes";
    if (ms == "clusters") {
        c->sweep_forced = true;
        c->sweep_mode = 4; c->sweep_grid = 8; c->sweep_block = 256;
        const char* pfs = std::getenv("TRANS_SWEEP_PF");
        c->sweep_pf = pfs ? std::max(0, std::atoi(pfs)) : 0;
    }
    // pairs: two hyperplanes per launch (mixed path; the FP64 path takes planes)
    if (ms == "pairs" && !c->mixed) ms = "planes";
    if (ms == "pairs") {
        c->sweep_forced = true;
        c->sweep_mode = 5;
    }
    if (ms == "planes" || ms == "coop" || ms == "flow" || ms == "tiles") {
        int dev = 0, nsm = 0;
        CK(cudaGetDevice(&dev));
        CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
        c->sweep_forced = true;
        if (ms == "planes") c->sweep_mode = 0;
        if (ms == "coop") { c->sweep_mode = 1; c->sweep_block = 256; c->sweep_grid = nsm * std::max(1, std::min(2, c->fl->sweep_all_occupancy(256))); }
        if (ms == "flow") { c->sweep_mode = 2; c->sweep_block = 256; c->sweep_grid = nsm * std::max(1, std::min(4, c->fl->sweep_flow_occupancy(256))); }
        if (ms == "tiles") {
            c->sweep_mode = 3; c->sweep_block = 256; c->sweep_grid = nsm * std::max(1, c->fl->sweep_tiles_occupancy(256));
            const char* ts = std::getenv("TRANS_TILE");
            int a = 0, b = 0, d = 0;
            if (ts && std::sscanf(ts, "%dx%dx%d", &a, &b, &d) == 3 && a > 0 && b > 0 && d > 0) {
                c->tile_default[0] = a; c->tile_default[1] = b; c->tile_default[2] = d;
            }
        }
    }
    return TRANS_OK;
}

void free_worklists(Ctx* c) {
    dfree(c->d_blk); dfree(c->d_off); dfree(c->d_cell); dfree(c->d_ghost);
    for (int d = 0; d < 3; ++d) { dfree(c->d_face[d]); dfree(c->d_rtiles[d]); c->n_rtiles[d] = 0; }
    dfree(c->d_rmaps);
    dfree(c->d_bc); dfree(c->d_outlet); dfree(c->d_lines); dfree(c->d_sweep); dfree(c->d_plane_off); dfree(c->d_pb_off);
    dfree(c->d_nbp); dfree(c->d_flags); dfree(c->d_rec); dfree(c->d_dqs); dfree(c->d_dq2); dfree(c->d_orph); dfree(c->d_dq_save);
    c->pair_lo.clear(); c->pair_up.clear(); dfree(c->d_parts); dfree(c->d_pc);
    dfree(c->d_cdev); dfree(c->d_stage); dfree(c->d_tile_first); dfree(c->d_norms);
    dfree(c->d_tiles); dfree(c->d_tflags); dfree(c->d_qpos); dfree(c->d_bc_first); dfree(c->d_intg);
    c->tv = TileView{};
    c->tile_shape[0] = c->tile_shape[1] = c->tile_shape[2] = 0;
    if (c->h_norms) { cudaFreeHost(c->h_norms); c->h_norms = nullptr; }
    if (c->iter_exec) { cudaGraphExecDestroy(c->iter_exec); c->iter_exec = nullptr; }
    if (c->iter1_exec) { cudaGraphExecDestroy(c->iter1_exec); c->iter1_exec = nullptr; }
    c->iter_n = 0;
    if (c->h_cdev) { cudaFreeHost(c->h_cdev); c->h_cdev = nullptr; }
    if (c->sweep_exec) { cudaGraphExecDestroy(c->sweep_exec); c->sweep_exec = nullptr; }
    c->built = false;
}

void ctx_free(Ctx* c) {
    if (c->stream) cudaStreamSynchronize(c->stream);
    free_worklists(c);
    for (CaseRec* cs : c->cases) {
        cudaFree(cs->arena);
        if (cs->farena) cudaFree(cs->farena);
        delete cs;
    }
    c->cases.clear();
    dfree(c->d_sync);
    if (c->h_sync) { cudaFreeHost(c->h_sync); c->h_sync = nullptr; }
    dfree(c->d_kerr);
    dfree(c->d_halo);
    c->halo_bytes = 0;
    if (c->h_kerr) { cudaFreeHost(c->h_kerr); c->h_kerr = nullptr; }
    if (c->copy_done) { cudaEventDestroy(c->copy_done); c->copy_done = nullptr; }
    if (c->stream) { cudaStreamDestroy(c->stream); c->stream = nullptr; }
}

CaseRec* case_find(Ctx* c, int id) {
    for (CaseRec* cs : c->cases)
        if (cs->id == id) return cs;
    return nullptr;
}

int case_add(Ctx* c, const trans_params* p, int nblocks, const trans_block* blocks, CaseRec** out) {
    if (!p || !blocks || nblocks <= 0) return fail(c, TRANS_E_ARG, "null case");
    if (!params_supported(p)) return fail(c, TRANS_E_ARG, "option outside the supported configurations");
    if (p->precision != c->precision) return fail(c, TRANS_E_ARG, "a context holds cases of one precision mode");
    for (CaseRec* o : c->cases) {
        if (o->p.IF_RK != p->IF_RK) return fail(c, TRANS_E_ARG, "cases of one context share the time integrator");
        if (o->p.IF_Precondition != p->IF_Precondition)
            return fail(c, TRANS_E_ARG, "cases of one context share the preconditioning switch");
        if (sub_iterations(o->p) != sub_iterations(*p) || (o->p.Kind_Dual != 0) != (p->Kind_Dual != 0))
            return fail(c, TRANS_E_ARG, "cases of one context share the sub-iteration count");
    }
    for (int n = 0; n < nblocks; ++n)
        if (!block_ok(blocks[n])) return fail(c, TRANS_E_ARG, "bad block dimensions or connectivity");
    const long long need = case_bytes(p, nblocks, blocks);
    const int nslot = case_slots(*p);
    if (c->budget > 0 && c->in_use + need > c->budget) return fail(c, TRANS_E_MEMORY, "case does not fit the device budget");
    CaseRec* cs = new CaseRec();
    cs->p = *p;
    cs->dp = make_params(*p);
    cs->KI = p->KI_ini;
    cs->hb.resize(nblocks);
    cs->blk.resize(nblocks);
    size_t total = 0;
    for (int n = 0; n < nblocks; ++n) {
        const trans_block& tb = blocks[n];
        HostBlock& h = cs->hb[n];
        h.NI = tb.ni; h.NJ = tb.nj; h.NK = tb.nk; h.id = tb.id;
        h.conn.assign(tb.conn, tb.conn + tb.nconn);
        int n1[6] = {tb.nj - 1, tb.nj - 1, tb.ni - 1, tb.ni - 1, tb.ni - 1, tb.ni - 1};
        int n2[6] = {tb.nk - 1, tb.nk - 1, tb.nk - 1, tb.nk - 1, tb.nj - 1, tb.nj - 1};
        for (int f = 0; f < 6; ++f)
            if (tb.markwall[f]) h.mw[f].assign(tb.markwall[f], tb.markwall[f] + (size_t)n1[f] * n2[f]);
        DevBlock& b = cs->blk[n];
        std::memset(&b, 0, sizeof(b));
        b.NI = tb.ni; b.NJ = tb.nj; b.NK = tb.nk;
        b.NI1 = b.NI - 1; b.NJ1 = b.NJ - 1; b.NK1 = b.NK - 1;
        b.PI = padded_pi(b.NI); b.PJ = b.NJ + 5; b.PK = b.NK + 5;
        b.ncell = b.PI * b.PJ * b.PK;
        b.nint = b.NI1 * b.NJ1 * b.NK1;
        total += (size_t)nslot * (size_t)b.ncell;
    }
    cs->arena_doubles = total;
    auto bail = [&](int code, const char* what) {
        if (cs->arena) cudaFree(cs->arena);
        if (cs->farena) cudaFree(cs->farena);
        delete cs;
        return fail(c, code, what);
    };
    if (cudaMalloc(&cs->arena, total * sizeof(double)) != cudaSuccess) return bail(TRANS_E_MEMORY, "device arena");
    if (cudaMemset(cs->arena, 0, total * sizeof(double)) != cudaSuccess) return bail(TRANS_E_CUDA, "arena clear");
    if (c->mixed) {
        if (cudaMalloc(&cs->farena, total * sizeof(float)) != cudaSuccess) return bail(TRANS_E_MEMORY, "FP32 arena");
        if (cudaMemset(cs->farena, 0, total * sizeof(float)) != cudaSuccess) return bail(TRANS_E_CUDA, "FP32 arena clear");
    }
    size_t pos = 0;
    for (int n = 0; n < nblocks; ++n) {
        cs->blk[n].base = cs->arena + pos;
        cs->blk[n].fbase = cs->farena ? cs->farena + pos : nullptr;
        pos += (size_t)nslot * (size_t)cs->blk[n].ncell;
        if (upload_walls(c, cs->hb[n], cs->blk[n])) return bail(TRANS_E_CUDA, "wall flags");
    }
    cs->norms.assign(nblocks, trans_norms{});
    cs->first_norms.assign(nblocks, trans_norms{});
    cs->id = c->next_id++;
    cs->bytes = need;
    c->in_use += need;
    c->cases.push_back(cs);
    c->built = false;
    if (out) *out = cs;
    return TRANS_OK;
}

int case_remove(Ctx* c, int id) {
    for (size_t q = 0; q < c->cases.size(); ++q) {
        CaseRec* cs = c->cases[q];
        if (cs->id != id) continue;
        CK(cudaStreamSynchronize(c->stream));
        cudaFree(cs->arena);
        if (cs->farena) cudaFree(cs->farena);
        c->in_use -= cs->bytes;
        delete cs;
        c->cases.erase(c->cases.begin() + q);
        c->built = false;
        return TRANS_OK;
    }
    return fail(c, TRANS_E_ARG, "no such case");
}

}  // namespace eng
}  // namespace tg
