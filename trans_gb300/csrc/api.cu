// api.cu -- the C ABI of include/trans_gpu.h over the CUDA kernels.
//
// Host responsibilities: validate the options, lay the blocks out in one device arena, turn the
// reference's connectivity (ConnectivityStruct) into gather tables for the boundary kernels,
// order the interior cells of every block on i+j+k hyperplanes for the LU-SGS sweeps, move
// Fortran-layout arrays in and out, and sequence the kernels as main.F90:54-197 does.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>
#include <initializer_list>
#include <mutex>
#include <utility>

#include "../../include/trans_gpu.h"
#include "types.cuh"
#include "launch.h"

using namespace tg;

namespace {

struct HostBlock {
    int NI, NJ, NK, id;
    std::vector<trans_conn> conn;
    std::vector<int> mw[6];
};

struct Ctx {
    trans_params p;
    Params dp;
    std::vector<HostBlock> hb;
    std::vector<DevBlock> blk;
    DevBlock* d_blk = nullptr;
    double* arena = nullptr;
    size_t arena_doubles = 0;
    float* farena = nullptr;             // FP32 copies of the slots (mixed path only)
    bool mixed = false;
    long long* d_off = nullptr;          // padded-cell offsets of the blocks (for flat kernels)
    long long total_cells = 0;
    std::vector<Tile> cell_tiles, face_tiles[3], ghost_tiles;
    Tile *d_cell = nullptr, *d_face[3] = {nullptr, nullptr, nullptr}, *d_ghost = nullptr;
    std::vector<int> cell_tile_blk;      // block of each cell tile (norm reduction)
    std::vector<BCEntry> bc, outlet;
    std::vector<OutletLine> lines;
    BCEntry *d_bc = nullptr, *d_outlet = nullptr;
    OutletLine* d_lines = nullptr;
    std::vector<SweepCell> sweep;
    std::vector<int> plane_off;          // sweep cells of hyperplane h: [plane_off[h], plane_off[h+1])
    SweepCell* d_sweep = nullptr;
    NormPart* d_parts = nullptr;
    std::vector<NormPart> h_parts;
    std::vector<trans_norms> norms;
    cudaStream_t stream = nullptr;
    bool geom_dirty = true;
    long long launches = 0;
    int KI = 1;
    std::string err;
    const FluxLaunchers* fl = nullptr;
    double* d_stage = nullptr;           // Fortran-layout staging buffer of trans_set/get_field
    cudaGraphExec_t sweep_exec[2] = {nullptr, nullptr};   // both sweeps as one CUDA graph (per turb flag)
    // sweep schedule: 0 = one launch per hyperplane (graph), 1 = one cooperative launch with
    // grid barriers; -1 = pick the faster on first use (both give bit-identical DeltaQ)
    int sweep_mode = -1, sweep_grid = 0, sweep_block = 0;
    int* d_plane_off = nullptr;
    SweepView sv{};                      // sweep-order arrays (cells, neighbour positions, records, DeltaQ)
    int* d_nbp = nullptr;
    void* d_rec = nullptr;
    void* d_dqs = nullptr;
    void* d_dq_save = nullptr;           // DeltaQ backup while the schedule tuner runs trials
    SweepSync* d_sync = nullptr;
    SweepSync* h_sync = nullptr;         // pinned
    std::string sweep_tuning;            // what the schedule tuner measured
    // per-kernel timing (trans_kernel_times): events around each launch while enabled
    bool ktime_on = false;
    struct KEv { int k, n; cudaEvent_t a, b; };
    std::vector<KEv> kev;
    size_t stage_doubles = 0;
};

// kernel classes of trans_kernel_times
enum KClass { K_SPECRAD, K_BC_STATE, K_BC_OUTLET, K_PRIMS, K_MIRROR, K_GRADIENT, K_SHOCK_GHOST, K_BC_GRAD,
              K_FACE, K_GATHER, K_SST_FC1, K_PREP, K_SWEEP, K_SCATTER, K_UPDATE, K_UPDATE_U, NKCLASS };
const char* const kclass_name[NKCLASS] = {"k_specrad", "k_bc_state", "k_bc_outlet", "k_prims", "k_mirror", "k_gradient",
    "k_shock_ghost", "k_bc_grad", "k_face_flux", "k_gather", "k_sst_fc1", "k_lusgs_prep", "k_sweep", "k_sweep_scatter",
    "k_update", "k_update_u"};

// times the launches issued in its lifetime as kernel class k (n launches) when enabled
struct KScope {
    Ctx* c; int k, n; cudaEvent_t a = nullptr, b = nullptr;
    KScope(Ctx* c_, int k_, int n_ = 1) : c(c_), k(k_), n(n_) {
        if (c->ktime_on && cudaEventCreate(&a) == cudaSuccess && cudaEventCreate(&b) == cudaSuccess) cudaEventRecord(a, c->stream);
    }
    ~KScope() {
        if (c->ktime_on && a && b) { cudaEventRecord(b, c->stream); c->kev.push_back({k, n, a, b}); }
    }
};

int fail(Ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}

#define CK(call)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) return fail(c, TRANS_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// Geom/startup.F90:1-25
void ijk_start_end(int I, int J, int K, int& Is, int& Js, int& Ks, const int* TL, const int* TT, int lcross) {
    int l1 = 1 - lcross;
    int t1 = TL[0] * I + TL[1] * J + TL[2] * K;
    int t2 = TL[0] * (J * l1 + K * lcross) + TL[1] * (I * l1 + K * lcross) + TL[2] * (I * l1 + J * lcross);
    int t3 = TL[0] * (J * lcross + K * l1) + TL[1] * (I * lcross + K * l1) + TL[2] * (I * lcross + J * l1);
    Is = TT[0] * t1 + (TT[1] + TT[2]) * t2;
    Js = TT[1] * t1 + TT[0] * t2 + TT[2] * t3;
    Ks = TT[2] * t1 + (TT[0] + TT[1]) * t3;
}

int block_index(Ctx* c, int id) {
    for (size_t n = 0; n < c->hb.size(); ++n)
        if (c->hb[n].id == id) return (int)n;
    return -1;
}

// Gather tables of BC_Boundarys (BC/Boundary.F90:22-47): one entry per boundary face cell,
// in block / connection / (k,j,i) order; outlets in a separate table ordered line by line.
int build_bc(Ctx* c) {
    for (size_t nb = 0; nb < c->hb.size(); ++nb) {
        const HostBlock& h = c->hb[nb];
        const DevBlock& b = c->blk[nb];
        for (size_t ic = 0; ic < h.conn.size(); ++ic) {
            const trans_conn& a = h.conn[ic];
            int kind = a.BCType;
            if (kind != 1 && kind != 2 && kind != 3 && kind != 5 && kind != 7 && kind != 9)
                return fail(c, TRANS_E_ARG, "unsupported BC kind " + std::to_string(kind));
            int tb = -1;
            const trans_conn* ta = nullptr;
            if (kind == 9) {
                tb = block_index(c, a.TargetBlock);
                if (tb < 0 || a.TargetConn < 1 || a.TargetConn > (int)c->hb[tb].conn.size())
                    return fail(c, TRANS_E_ARG, "bad 1-to-1 target");
                ta = &c->hb[tb].conn[a.TargetConn - 1];
            }
            {   // the face cells must lie on one face of the block, tangential indices interior
                const int n3[3] = {b.NI, b.NJ, b.NK};
                int d = a.IJKDirect - 1;
                if (d < 0 || d > 2) return fail(c, TRANS_E_ARG, "bad IJKDirect");
                for (int q = 0; q < 3; ++q) {
                    int lo = a.pointStart[q], hi = a.pointEnd[q];
                    bool ok = (q == d) ? (lo == hi && (lo == 1 || lo == n3[q])) : (lo >= 1 && hi <= n3[q] - 1 && lo <= hi);
                    if (!ok) return fail(c, TRANS_E_ARG, "connection range outside the block");
                }
                if (b.NI1 < 3 || b.NJ1 < 3 || b.NK1 < 3) return fail(c, TRANS_E_ARG, "blocks need 3 interior cells per direction");
            }
            std::vector<BCEntry> seg;
            for (int K = a.pointStart[2]; K <= a.pointEnd[2]; ++K)
            for (int J = a.pointStart[1]; J <= a.pointEnd[1]; ++J)
            for (int I = a.pointStart[0]; I <= a.pointEnd[0]; ++I) {
                BCEntry E;
                std::memset(&E, 0, sizeof(E));
                E.kind = kind; E.blk = (int)nb; E.conn = (int)ic; E.i = I; E.j = J; E.k = K;
                E.dir = a.IJKDirect; E.lor = a.LeftOrRight;
                E.sub = (J == a.pointStart[1]) ? 1 : 0;
                const int* E3[3] = {a.CEIJKAdd, a.CEIJKAdd1, a.CEIJKAdd2};
                for (int L = 0; L < 3; ++L) E.l[L] = cidx(b, I + E3[L][0], J + E3[L][1], K + E3[L][2]);
                E.face = cidx(b, I + a.IJKAdd[0], J + a.IJKAdd[1], K + a.IJKAdd[2]);
                if (kind == 9) {
                    int IIadd = a.pointEnd[0] - a.pointStart[0] + 2, JJadd = a.pointEnd[1] - a.pointStart[1] + 2;
                    int KKadd = a.pointEnd[2] - a.pointStart[2] + 2;
                    int iL = I - a.pointStart[0] + 1, jL = J - a.pointStart[1] + 1, kL = K - a.pointStart[2] + 1;
                    iL = a.revMatrix[0] * IIadd + (1 - 2 * a.revMatrix[0]) * iL;
                    jL = a.revMatrix[1] * JJadd + (1 - 2 * a.revMatrix[1]) * jL;
                    kL = a.revMatrix[2] * KKadd + (1 - 2 * a.revMatrix[2]) * kL;
                    int ib, jb, kb;
                    ijk_start_end(iL, jL, kL, ib, jb, kb, a.Transform, a.TransformT, a.lcross);
                    ib += ta->pointStart[0] - 1; jb += ta->pointStart[1] - 1; kb += ta->pointStart[2] - 1;
                    const int* S3[3] = {ta->CIJKAdd, ta->CIJKAdd1, ta->CIJKAdd2};
                    const DevBlock& r = c->blk[tb];
                    for (int L = 0; L < 3; ++L) {
                        int ii = ib + S3[L][0], jj = jb + S3[L][1], kk = kb + S3[L][2];
                        if (ii < 1 || ii > r.NI1 || jj < 1 || jj > r.NJ1 || kk < 1 || kk > r.NK1)
                            return fail(c, TRANS_E_ARG, "1-to-1 source cell outside the target block");
                        E.s[L] = cidx(r, ii, jj, kk);
                    }
                    E.src_blk = tb;
                    E.cost = std::cos(a.rotateAngle);
                    E.sint = std::sin(a.rotateAngle);
                } else {
                    const int* S3[3] = {a.CIJKAdd, a.CIJKAdd1, a.CIJKAdd2};
                    for (int L = 0; L < 3; ++L) E.s[L] = cidx(b, I + S3[L][0], J + S3[L][1], K + S3[L][2]);
                    E.src_blk = (int)nb;
                    E.cost = 1.0; E.sint = 0.0;
                }
                seg.push_back(E);
            }
            c->bc.insert(c->bc.end(), seg.begin(), seg.end());
            if (kind == 7) {
                // lines along j: key = (k for i-faces, i for k-faces, cell for j-faces)
                std::stable_sort(seg.begin(), seg.end(), [&](const BCEntry& x, const BCEntry& y) {
                    int kx = a.IJKDirect == 1 ? x.k : (a.IJKDirect == 3 ? x.i : x.i + 100000 * x.k);
                    int ky = a.IJKDirect == 1 ? y.k : (a.IJKDirect == 3 ? y.i : y.i + 100000 * y.k);
                    if (kx != ky) return kx < ky;
                    return x.j < y.j;
                });
                size_t q = 0;
                while (q < seg.size()) {
                    size_t r = q + 1;
                    if (a.IJKDirect != 2)
                        while (r < seg.size() && ((a.IJKDirect == 1 && seg[r].k == seg[q].k) || (a.IJKDirect == 3 && seg[r].i == seg[q].i))) ++r;
                    OutletLine L;
                    L.blk = (int)nb; L.first = (int)(c->outlet.size() + q); L.n = (int)(r - q); L.pad_ = 0;
                    c->lines.push_back(L);
                    q = r;
                }
                c->outlet.insert(c->outlet.end(), seg.begin(), seg.end());
            }
        }
    }
    return TRANS_OK;
}

int upload_vec(Ctx* c, const void* h, size_t bytes, void** d) {
    if (bytes == 0) { *d = nullptr; return TRANS_OK; }
    CK(cudaMalloc(d, bytes));
    CK(cudaMemcpy(*d, h, bytes, cudaMemcpyHostToDevice));
    return TRANS_OK;
}

void make_tiles(int nblk, const std::vector<long long>& counts, int tile, std::vector<Tile>& out, std::vector<int>* owner) {
    for (int b = 0; b < nblk; ++b)
        for (long long s = 0; s < counts[b]; s += tile) {
            Tile t;
            t.blk = b; t.start = (int)s; t.count = (int)std::min<long long>(tile, counts[b] - s); t.pad_ = 0;
            out.push_back(t);
            if (owner) owner->push_back(b);
        }
}

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
        default: return {-1, 0, 0};
    }
}

bool is_geometry(int f) { return f >= TRANS_SD && f <= TRANS_THTC; }

// SD(dir,comp,...) arrives with dir fastest; slot S_SD + 3*(dir-1) + (comp-1)
inline int comp_slot(int f, int m) {
    if (f == TRANS_SD) { int dir = m % 3, comp = m / 3; return 3 * dir + comp; }
    return m;
}

void fill_params(Ctx* c) {
    const trans_params& p = c->p;
    Params& d = c->dp;
    std::memset(&d, 0, sizeof(d));
    d.XM = p.XM; d.RXM2 = p.RXM2; d.PPF = p.PPF; d.Csthlnd = p.Csthlnd; d.Csth1 = p.Csth1; d.Ref = p.Ref;
    d.Tiny = p.Tiny; d.VxF = p.VxF; d.VyF = p.VyF; d.VzF = p.VzF; d.omega0 = p.omega[0];
    d.P0in = p.P0in; d.T0in = p.T0in; d.Pouthub = p.Pouthub; d.VisRatio = p.VisRatio; d.FSTI = p.FSTI;
    d.A1 = p.A1; d.Beta_star = p.Beta_star; d.Sigk1 = p.Sigk1; d.Sigo1 = p.Sigo1; d.Beta1 = p.Beta1;
    d.Gama1 = p.Gama1; d.Sigk2 = p.Sigk2; d.Sigo2 = p.Sigo2; d.Beta2 = p.Beta2; d.Gama2 = p.Gama2;
    d.Prod_Lmt = p.Prod_Lmt; d.gama_max = p.gama_max; d.gama_min = p.gama_min;
    d.DT_LUSGS_Main = p.DT_LUSGS_Main; d.DT_LUSGS_Sub = p.DT_LUSGS_Sub; d.CFL_Main = p.CFL_Main;
    d.Trans_location = p.Trans_location;
    d.Kind_Spatial = p.Kind_Spatial; d.Kind_Roe = p.Kind_Roe; d.Kind_Hybrid = p.Kind_Hybrid;
    d.Kind_SubHY = p.Kind_SubHY; d.Kind_Dual = p.Kind_Dual; d.IF_Local_Main = p.IF_Local_Main;
    d.IF_Local_Sub = p.IF_Local_Sub; d.IF_Comppress = p.IF_Comppress; d.If_fix_Transition = p.If_fix_Transition;
}

int turb_on(const Ctx* c) {
    const trans_params& p = c->p;
    return (p.IF_Euler == 0 && p.IF_Turb_org == 1 && (c->KI >= p.KItm || p.Kind_Hybrid > 0)) ? 1 : 0;
}

// FP32 copies of slot ranges {first, count} (mixed path); to_fp64 copies back
void mirror(Ctx* c, std::initializer_list<std::pair<int, int>> ranges, int to_fp64 = 0) {
    MirrorList ml;
    std::memset(&ml, 0, sizeof(ml));
    ml.to_fp64 = to_fp64;
    for (auto& r : ranges) { ml.first[ml.n] = r.first; ml.count[ml.n] = r.second; ml.n++; }
    launch_mirror(c->stream, c->d_blk, (int)c->blk.size(), c->total_cells, c->d_off, ml);
    c->launches++;
}

int finalize_geometry(Ctx* c) {
    if (!c->geom_dirty) return TRANS_OK;
    launch_geom_static(c->stream, c->d_blk, (int)c->blk.size(), c->total_cells, c->d_off);
    c->launches++;
    if (c->mixed) mirror(c, {{S_SD, S_WALL + 3 - S_SD}});
    CK(cudaGetLastError());
    c->geom_dirty = false;
    return TRANS_OK;
}

// Per-block norms from the per-tile partials in c->h_parts, summed in tile order (deterministic).
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
    if (nan) return fail(c, TRANS_E_NAN, "NaN in the density increment");
    return TRANS_OK;
}

// both LU-SGS sweeps with the schedule `mode` (grid/block for the cooperative one)
int sweep_once(Ctx* c, int turb, int mode, int grid, int block) {
    cudaStream_t s = c->stream;
    int nh = (int)c->plane_off.size() - 1;
    if (mode == 1) {
        CK(cudaMemsetAsync(c->d_sync, 0, sizeof(SweepSync), s));
        CK(c->fl->sweep_all(s, c->sv, c->d_plane_off, nh, turb, c->d_sync, grid, block));
        CK(cudaMemcpyAsync(c->h_sync, c->d_sync, sizeof(SweepSync), cudaMemcpyDeviceToHost, s));
        c->launches++;
        return TRANS_OK;
    }
    // one launch per hyperplane, L ascending then U descending, replayed as one graph
    if (!c->sweep_exec[turb]) {
        cudaGraph_t g = nullptr;
        CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        for (int h = 0; h < nh; ++h) {
            int cnt = c->plane_off[h + 1] - c->plane_off[h];
            if (cnt) c->fl->sweep_lower(s, c->sv, c->plane_off[h], cnt, turb);
        }
        for (int h = nh - 1; h >= 0; --h) {
            int cnt = c->plane_off[h + 1] - c->plane_off[h];
            if (cnt) c->fl->sweep_upper(s, c->sv, c->plane_off[h], cnt, turb);
        }
        cudaError_t e = cudaStreamEndCapture(s, &g);
        if (e != cudaSuccess) return fail(c, TRANS_E_CUDA, std::string("sweep graph capture: ") + cudaGetErrorString(e));
        e = cudaGraphInstantiate(&c->sweep_exec[turb], g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return fail(c, TRANS_E_CUDA, std::string("sweep graph instantiate: ") + cudaGetErrorString(e));
    }
    CK(cudaGraphLaunch(c->sweep_exec[turb], s));
    for (int h = 0; h < nh; ++h) c->launches += (c->plane_off[h + 1] > c->plane_off[h]) ? 2 : 0;
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
int tune_sweeps(Ctx* c, int turb) {
    int dev = 0, nsm = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    struct Cand { int mode, grid, block; };
    std::vector<Cand> cands = {{0, 0, 0}};
    for (int block : {128, 256, 512}) {
        int occ = c->fl->sweep_all_occupancy(block);
        for (int per : {1, 2, 4})
            if (per <= occ) cands.push_back({1, per * nsm, block});
    }
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    float best = 1e30f;
    Cand pick = cands[0];
    c->sweep_tuning.clear();
    int rc = save_dq(c, false);
    for (const Cand& k : cands) {
        for (int rep = 0; rep < 2 && rc == TRANS_OK; ++rep) {      // first run warms up (graph build)
            if ((rc = save_dq(c, true))) break;
            CK(cudaEventRecord(e0, c->stream));
            if ((rc = sweep_once(c, turb, k.mode, k.grid, k.block))) break;
            CK(cudaEventRecord(e1, c->stream));
            CK(cudaEventSynchronize(e1));
            if (k.mode == 1 && c->h_sync->err) { rc = -100; break; }
            float ms = 0;
            CK(cudaEventElapsedTime(&ms, e0, e1));
            if (rep == 1) {
                c->sweep_tuning += (k.mode ? "coop " + std::to_string(k.grid) + "x" + std::to_string(k.block) : std::string("planes"))
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
    c->sweep_mode = pick.mode; c->sweep_grid = pick.grid; c->sweep_block = pick.block;
    return TRANS_OK;
}

int run_sweeps(Ctx* c, int turb) {
    if (c->sweep_mode < 0) {
        int rc = tune_sweeps(c, turb);
        if (rc) return rc;
    }
    return sweep_once(c, turb, c->sweep_mode, c->sweep_grid, c->sweep_block);
}

int run_stage(Ctx* c, int stage, int itr) {
    (void)itr;
    int rc = finalize_geometry(c);
    if (rc) return rc;
    const int turb = turb_on(c);
    const trans_params& p = c->p;
    cudaStream_t s = c->stream;
    int nct = (int)c->cell_tiles.size();
    switch (stage) {
        case TRANS_STAGE_SPECRAD: {
            double CFL_sub = p.CFL_Sub_start + (p.CFL_Sub_end - p.CFL_Sub_start) * (double)(c->KI - p.KI_ini) / (double)p.CFL_Sub_step;
            CFL_sub = std::min(CFL_sub, p.CFL_Sub_end);
            { KScope t(c, K_SPECRAD); launch_specrad(s, c->d_blk, c->d_cell, nct, c->dp, CFL_sub); }
            c->launches++;
            break;
        }
        case TRANS_STAGE_BC_STATE:
            { KScope t(c, K_BC_STATE); launch_bc_state(s, c->d_blk, c->d_bc, (int)c->bc.size(), c->dp, turb); }
            { KScope t(c, K_BC_OUTLET); launch_bc_outlet(s, c->d_blk, c->d_outlet, c->d_lines, (int)c->lines.size(), c->dp, turb); }
            c->launches += 1 + (c->lines.empty() ? 0 : 1);
            break;
        case TRANS_STAGE_GRADIENT:
            { KScope t(c, K_PRIMS); launch_prims(s, c->d_blk, (int)c->blk.size(), c->total_cells, c->d_off); }
            // the FP32 kernels read FP32 copies of this sub-iteration's state, primitives and radii
            if (c->mixed) { KScope t(c, K_MIRROR); mirror(c, {{S_V, 10}, {S_RDS, 4}, {S_PRIM, 5}, {S_RINV, 4}}); }
            { KScope t(c, K_GRADIENT); c->fl->gradient(s, c->d_blk, c->d_cell, nct, turb); }
            { KScope t(c, K_SHOCK_GHOST); c->fl->shock_ghost(s, c->d_blk, c->d_ghost, (int)c->ghost_tiles.size()); }
            c->launches += 3;
            break;
        case TRANS_STAGE_BC_GRAD:
            { KScope t(c, K_BC_GRAD); c->fl->bc_grad(s, c->d_blk, c->d_bc, (int)c->bc.size(), turb); }
            c->launches++;
            break;
        case TRANS_STAGE_RESIDUAL:
            for (int d = 0; d < 3; ++d) {
                KScope t(c, K_FACE);
                c->fl->face_flux[d](s, c->d_blk, c->d_face[d], (int)c->face_tiles[d].size(), c->dp, turb);
            }
            { KScope t(c, K_GATHER); c->fl->gather(s, c->d_blk, c->d_cell, nct, turb); }
            c->launches += 4;
            break;
        case TRANS_STAGE_LUSGS: {
            if (turb && p.Kind_Hybrid == 3) {
                KScope t(c, K_SST_FC1);
                c->fl->sst_fc1(s, c->d_blk, c->d_cell, nct, c->dp);
                c->launches++;
            }
            { KScope t(c, K_PREP); c->fl->prep(s, c->d_blk, c->sv, c->dp, turb); }
            c->launches++;
            {
                int nh = (int)c->plane_off.size() - 1, nl = 0;
                for (int h = 0; h < nh; ++h) nl += (c->plane_off[h + 1] > c->plane_off[h]) ? 2 : 0;
                KScope t(c, K_SWEEP, c->sweep_mode == 1 ? 1 : nl);
                rc = run_sweeps(c, turb);
            }
            if (rc) return rc;
            { KScope t(c, K_SCATTER); c->fl->scatter(s, c->d_blk, c->sv); }
            c->launches++;
            break;
        }
        case TRANS_STAGE_UPDATE: {
            int turb_upd = (p.IF_Euler == 0 && turb == 1 && c->KI >= p.KItm) ? 1 : 0;
            { KScope t(c, K_UPDATE); launch_update(s, c->d_blk, c->d_cell, nct, c->dp, turb_upd, c->d_parts, c->mixed ? 1 : 0); }
            c->launches++;
            CK(cudaMemcpyAsync(c->h_parts.data(), c->d_parts, sizeof(NormPart) * c->h_parts.size(), cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            if (c->sweep_mode == 1 && c->h_sync->err) return fail(c, TRANS_E_TIMEOUT, "LU-SGS sweep grid barrier timed out");
            rc = reduce_norms(c);
            if (rc) return rc;
            break;
        }
        case TRANS_STAGE_UPDATE_U:
            if (p.Kind_Dual != 0) {
                KScope t(c, K_UPDATE_U);
                launch_update_u(s, c->d_blk, c->d_cell, nct, p.Kind_Dual);
                c->launches++;
            }
            break;
        default:
            return fail(c, TRANS_E_ARG, "bad stage");
    }
    CK(cudaGetLastError());
    return TRANS_OK;
}

}  // namespace

extern "C" {

int trans_create(const trans_params* p, int nblocks, const trans_block* blocks, void** out) {
    Ctx* c = nullptr;
    if (!p || !blocks || nblocks <= 0 || !out) return TRANS_E_ARG;
    *out = nullptr;
    // options outside the configurations of this hot path are rejected, never approximated
    if (p->IF_Precondition != 0 || p->Kind_RotMod != 0 || p->Kind_Model != 1 || p->IF_Euler != 0 || p->IF_RK != 0)
        return TRANS_E_ARG;
    if ((p->Kind_Spatial != 2 && p->Kind_Spatial != 3) || (p->Kind_Roe != 1 && p->Kind_Roe != 3)) return TRANS_E_ARG;
    if (p->Kind_Hybrid != 0 && p->Kind_Hybrid != 3) return TRANS_E_ARG;
    if (p->Kind_Hybrid == 3 && (p->Kind_SubHY < 0 || p->Kind_SubHY > 3)) return TRANS_E_ARG;
    if (p->omega[0] != 0.0 || p->omega[1] != 0.0 || p->omega[2] != 0.0) return TRANS_E_ARG;
    if (p->precision != TRANS_FP64 && p->precision != TRANS_MIXED) return TRANS_E_ARG;
    c = new Ctx();
    c->p = *p;
    fill_params(c);
    c->fl = p->precision == TRANS_FP64 ? &flux_launchers_f64() : &flux_launchers_f32();
    c->hb.resize(nblocks);
    c->blk.resize(nblocks);
    size_t total = 0;
    std::vector<long long> off(nblocks);
    for (int n = 0; n < nblocks; ++n) {
        const trans_block& tb = blocks[n];
        if (tb.ni < 4 || tb.nj < 4 || tb.nk < 4 || tb.nconn < 0 || (tb.nconn > 0 && !tb.conn)) { delete c; return TRANS_E_ARG; }
        HostBlock& h = c->hb[n];
        h.NI = tb.ni; h.NJ = tb.nj; h.NK = tb.nk; h.id = tb.id;
        h.conn.assign(tb.conn, tb.conn + tb.nconn);
        int n1[6] = {tb.nj - 1, tb.nj - 1, tb.ni - 1, tb.ni - 1, tb.ni - 1, tb.ni - 1};
        int n2[6] = {tb.nk - 1, tb.nk - 1, tb.nk - 1, tb.nk - 1, tb.nj - 1, tb.nj - 1};
        for (int f = 0; f < 6; ++f)
            if (tb.markwall[f]) h.mw[f].assign(tb.markwall[f], tb.markwall[f] + (size_t)n1[f] * n2[f]);
        DevBlock& b = c->blk[n];
        b.NI = tb.ni; b.NJ = tb.nj; b.NK = tb.nk;
        b.NI1 = b.NI - 1; b.NJ1 = b.NJ - 1; b.NK1 = b.NK - 1;
        b.PI = b.NI + 5; b.PJ = b.NJ + 5; b.PK = b.NK + 5;
        long long ncell = (long long)b.PI * b.PJ * b.PK;
        if (ncell > (1LL << 30)) { delete c; return TRANS_E_ARG; }
        b.ncell = (int)ncell;
        b.nint = b.NI1 * b.NJ1 * b.NK1;
        b.pad_ = 0;
        off[n] = (long long)total / NSLOT;
        total += (size_t)NSLOT * (size_t)ncell;
    }
    c->arena_doubles = total;
    c->mixed = p->precision == TRANS_MIXED;
    cudaError_t e = cudaMalloc(&c->arena, total * sizeof(double));
    if (e != cudaSuccess) { delete c; return TRANS_E_MEMORY; }
    if (cudaMemset(c->arena, 0, total * sizeof(double)) != cudaSuccess) { cudaFree(c->arena); delete c; return TRANS_E_CUDA; }
    if (c->mixed) {
        if (cudaMalloc(&c->farena, total * sizeof(float)) != cudaSuccess) { cudaFree(c->arena); delete c; return TRANS_E_MEMORY; }
        if (cudaMemset(c->farena, 0, total * sizeof(float)) != cudaSuccess) { cudaFree(c->arena); cudaFree(c->farena); delete c; return TRANS_E_CUDA; }
    }
    {
        long long acc = 0;
        size_t pos = 0;
        for (int n = 0; n < nblocks; ++n) {
            c->blk[n].base = c->arena + pos;
            c->blk[n].fbase = c->farena ? c->farena + pos : nullptr;
            pos += (size_t)NSLOT * (size_t)c->blk[n].ncell;
            off[n] = acc;
            acc += c->blk[n].ncell;
        }
        c->total_cells = acc;
    }
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) { trans_destroy(c); return TRANS_E_CUDA; }
    int rc;
    if ((rc = upload_vec(c, c->blk.data(), sizeof(DevBlock) * nblocks, (void**)&c->d_blk))) { trans_destroy(c); return rc; }
    if ((rc = upload_vec(c, off.data(), sizeof(long long) * nblocks, (void**)&c->d_off))) { trans_destroy(c); return rc; }
    // tiles
    std::vector<long long> cnt(nblocks), fcnt[3], gcnt(nblocks);
    for (int d = 0; d < 3; ++d) fcnt[d].resize(nblocks);
    for (int n = 0; n < nblocks; ++n) {
        const DevBlock& b = c->blk[n];
        cnt[n] = b.nint;
        fcnt[0][n] = (long long)b.NI * b.NJ1 * b.NK1;
        fcnt[1][n] = (long long)b.NI1 * b.NJ * b.NK1;
        fcnt[2][n] = (long long)b.NI1 * b.NJ1 * b.NK;
        gcnt[n] = 6LL * ((long long)b.NJ1 * b.NK1 + (long long)b.NI1 * b.NK1 + (long long)b.NI1 * b.NJ1);
    }
    make_tiles(nblocks, cnt, CELL_TILE, c->cell_tiles, &c->cell_tile_blk);
    for (int d = 0; d < 3; ++d) make_tiles(nblocks, fcnt[d], FACE_TILE, c->face_tiles[d], nullptr);
    make_tiles(nblocks, gcnt, CELL_TILE, c->ghost_tiles, nullptr);
    if ((rc = upload_vec(c, c->cell_tiles.data(), sizeof(Tile) * c->cell_tiles.size(), (void**)&c->d_cell))) { trans_destroy(c); return rc; }
    for (int d = 0; d < 3; ++d)
        if ((rc = upload_vec(c, c->face_tiles[d].data(), sizeof(Tile) * c->face_tiles[d].size(), (void**)&c->d_face[d]))) { trans_destroy(c); return rc; }
    if ((rc = upload_vec(c, c->ghost_tiles.data(), sizeof(Tile) * c->ghost_tiles.size(), (void**)&c->d_ghost))) { trans_destroy(c); return rc; }
    // boundary tables
    if ((rc = build_bc(c))) { std::string m = c->err; trans_destroy(c); return rc; }
    if ((rc = upload_vec(c, c->bc.data(), sizeof(BCEntry) * c->bc.size(), (void**)&c->d_bc))) { trans_destroy(c); return rc; }
    if ((rc = upload_vec(c, c->outlet.data(), sizeof(BCEntry) * c->outlet.size(), (void**)&c->d_outlet))) { trans_destroy(c); return rc; }
    if ((rc = upload_vec(c, c->lines.data(), sizeof(OutletLine) * c->lines.size(), (void**)&c->d_lines))) { trans_destroy(c); return rc; }
    // hyperplane order of the LU-SGS sweeps: h = i+j+k = 3 .. max(NI1+NJ1+NK1)
    int hmax = 3;
    for (auto& b : c->blk) hmax = std::max(hmax, b.NI1 + b.NJ1 + b.NK1);
    c->plane_off.assign(1, 0);
    for (int h = 3; h <= hmax; ++h) {
        for (int n = 0; n < nblocks; ++n) {
            const DevBlock& b = c->blk[n];
            for (int k = 1; k <= b.NK1; ++k)
                for (int j = 1; j <= b.NJ1; ++j) {
                    int i = h - j - k;
                    if (i >= 1 && i <= b.NI1) c->sweep.push_back(SweepCell{n, i, j, k});
                }
        }
        c->plane_off.push_back((int)c->sweep.size());
    }
    if ((rc = upload_vec(c, c->sweep.data(), sizeof(SweepCell) * c->sweep.size(), (void**)&c->d_sweep))) { trans_destroy(c); return rc; }
    if ((rc = upload_vec(c, c->plane_off.data(), sizeof(int) * c->plane_off.size(), (void**)&c->d_plane_off))) { trans_destroy(c); return rc; }
    {   // neighbour positions in sweep order: lower i,j,k (0..2) and upper (3..5), -1 = none
        const long long N = (long long)c->sweep.size();
        std::vector<std::vector<int>> pos(nblocks);
        for (int n = 0; n < nblocks; ++n) pos[n].assign((size_t)c->blk[n].nint, -1);
        for (long long q = 0; q < N; ++q) {
            const SweepCell& sc = c->sweep[q];
            const DevBlock& b = c->blk[sc.blk];
            pos[sc.blk][(size_t)(sc.i - 1) + (size_t)b.NI1 * ((sc.j - 1) + (size_t)b.NJ1 * (sc.k - 1))] = (int)q;
        }
        const long long Np = (N + 31) / 32 * 32;           // whole tiles of 32 positions
        std::vector<int> nbp((size_t)6 * Np, -1);
        for (long long q = 0; q < N; ++q) {
            const SweepCell& sc = c->sweep[q];
            const DevBlock& b = c->blk[sc.blk];
            const int ijk[3] = {sc.i, sc.j, sc.k}, hi[3] = {b.NI1, b.NJ1, b.NK1};
            for (int side = 0; side < 2; ++side)
                for (int d = 0; d < 3; ++d) {
                    int x[3] = {ijk[0], ijk[1], ijk[2]};
                    x[d] += side == 0 ? -1 : 1;
                    if (x[d] < 1 || x[d] > hi[d]) continue;
                    nbp[sw_at(q, 3 * side + d, 6)] =
                        pos[sc.blk][(size_t)(x[0] - 1) + (size_t)b.NI1 * ((x[1] - 1) + (size_t)b.NJ1 * (x[2] - 1))];
                }
        }
        if ((rc = upload_vec(c, nbp.data(), sizeof(int) * nbp.size(), (void**)&c->d_nbp))) { trans_destroy(c); return rc; }
        if (cudaMalloc(&c->d_rec, (size_t)NREC * Np * c->fl->elem) != cudaSuccess ||
            cudaMalloc(&c->d_dqs, (size_t)DQ_STRIDE * Np * c->fl->elem) != cudaSuccess) { trans_destroy(c); return TRANS_E_MEMORY; }
        c->sv.cells = c->d_sweep; c->sv.nbp = c->d_nbp; c->sv.rec = c->d_rec; c->sv.dq = c->d_dqs; c->sv.n = N;
    }
    if (cudaMalloc(&c->d_sync, sizeof(SweepSync)) != cudaSuccess || cudaMallocHost(&c->h_sync, sizeof(SweepSync)) != cudaSuccess) {
        trans_destroy(c); return TRANS_E_MEMORY;
    }
    std::memset(c->h_sync, 0, sizeof(SweepSync));
    {   // sweep schedule: TRANS_SWEEP=planes | coop forces one (for tests); default: tuned
        const char* m = std::getenv("TRANS_SWEEP");
        if (m && std::string(m) == "planes") c->sweep_mode = 0;
        if (m && std::string(m) == "coop") {
            int dev = 0, nsm = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
            c->sweep_mode = 1; c->sweep_block = 256; c->sweep_grid = nsm * std::max(1, std::min(2, c->fl->sweep_all_occupancy(256)));
        }
    }
    // wall marks on faces (Input/Read_BlockDimensions.F90:240-283)
    for (int n = 0; n < nblocks; ++n) {
        const DevBlock& b = c->blk[n];
        const HostBlock& h = c->hb[n];
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
            if (any && cudaMemcpy(b.base + (size_t)(S_WALL + d) * b.ncell, w.data(), sizeof(double) * b.ncell,
                                  cudaMemcpyHostToDevice) != cudaSuccess) { trans_destroy(c); return TRANS_E_CUDA; }
        }
    }
    {   // staging buffer for the largest Fortran field (DQdxyz: 18 components, lower bound -1)
        size_t mx = 0;
        for (auto& b : c->blk) mx = std::max(mx, (size_t)(b.NI + 4) * (b.NJ + 4) * (b.NK + 4) * 18);
        c->stage_doubles = mx;
        if (cudaMalloc(&c->d_stage, mx * sizeof(double)) != cudaSuccess) { trans_destroy(c); return TRANS_E_MEMORY; }
    }
    c->h_parts.resize(c->cell_tiles.size());
    if (cudaMalloc(&c->d_parts, sizeof(NormPart) * std::max<size_t>(1, c->h_parts.size())) != cudaSuccess) { trans_destroy(c); return TRANS_E_CUDA; }
    c->norms.assign(nblocks, trans_norms{});
    *out = c;
    return TRANS_OK;
}

int trans_destroy(void* ctx) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return TRANS_OK;
    if (c->stream) cudaStreamSynchronize(c->stream);
    cudaFree(c->arena); cudaFree(c->farena); cudaFree(c->d_blk); cudaFree(c->d_off);
    cudaFree(c->d_cell); cudaFree(c->d_ghost);
    for (int d = 0; d < 3; ++d) cudaFree(c->d_face[d]);
    cudaFree(c->d_bc); cudaFree(c->d_outlet); cudaFree(c->d_lines); cudaFree(c->d_sweep); cudaFree(c->d_parts); cudaFree(c->d_stage);
    cudaFree(c->d_plane_off); cudaFree(c->d_sync);
    cudaFree(c->d_nbp); cudaFree(c->d_rec); cudaFree(c->d_dqs); cudaFree(c->d_dq_save);
    if (c->h_sync) cudaFreeHost(c->h_sync);
    for (int q = 0; q < 2; ++q)
        if (c->sweep_exec[q]) cudaGraphExecDestroy(c->sweep_exec[q]);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return TRANS_OK;
}

static int field_io(Ctx* c, int ib, int f, double* host, bool upload) {
    if (!c || ib < 0 || ib >= (int)c->blk.size() || !host) return TRANS_E_ARG;
    FieldMap fm = field_map(f);
    if (fm.slot < 0) return fail(c, TRANS_E_ARG, "bad field id");
    const DevBlock& b = c->blk[ib];
    size_t ncells = (size_t)(b.NI + 3 - fm.lb) * (b.NJ + 3 - fm.lb) * (b.NK + 3 - fm.lb);
    size_t bytes = ncells * fm.ncomp * sizeof(double);
    cudaStream_t s = c->stream;
    int is_sd = f == TRANS_SD ? 1 : 0;
    if (upload) {
        CK(cudaMemcpyAsync(c->d_stage, host, bytes, cudaMemcpyHostToDevice, s));
        launch_field_xfer(s, b, fm.slot, fm.ncomp, fm.lb, is_sd, c->d_stage, 1);
        c->launches++;
        if (f == TRANS_THTC) {      // sin/cos of the outlet recurrence, evaluated once on the host
            std::vector<double> sn(ncells), cs(ncells);
            for (size_t q = 0; q < ncells; ++q) { sn[q] = std::sin(host[q]); cs[q] = std::cos(host[q]); }
            CK(cudaMemcpyAsync(c->d_stage, sn.data(), ncells * sizeof(double), cudaMemcpyHostToDevice, s));
            launch_field_xfer(s, b, S_SINT, 1, fm.lb, 0, c->d_stage, 1);
            CK(cudaMemcpyAsync(c->d_stage, cs.data(), ncells * sizeof(double), cudaMemcpyHostToDevice, s));
            launch_field_xfer(s, b, S_COST, 1, fm.lb, 0, c->d_stage, 1);
            CK(cudaStreamSynchronize(s));
        }
        if (is_geometry(f)) c->geom_dirty = true;
        if (c->mixed && f == TRANS_D) mirror(c, {{S_D, 7}});
        if (c->mixed && f == TRANS_DQDXYZ) mirror(c, {{S_DQ, 18}});
        if (c->mixed && f == TRANS_SHOCK) mirror(c, {{S_SHOCK, 1}});
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
    CK(cudaStreamSynchronize(s));
    return TRANS_OK;
}

int trans_set_field(void* ctx, int ib, int f, const double* a) {
    return field_io(static_cast<Ctx*>(ctx), ib, f, const_cast<double*>(a), true);
}
int trans_get_field(void* ctx, int ib, int f, double* a) { return field_io(static_cast<Ctx*>(ctx), ib, f, a, false); }

int trans_run_stage(void* ctx, int stage, int ki, int itr_chld) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return TRANS_E_ARG;
    c->KI = ki;
    return run_stage(c, stage, itr_chld);
}

int trans_iterate(void* ctx, int ki, trans_norms* norms) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return TRANS_E_ARG;
    c->KI = ki;
    int nsub = c->p.Kind_Dual != 0 ? c->p.Kchld : 1;
    for (int it = 1; it <= nsub; ++it)
        for (int s = TRANS_STAGE_SPECRAD; s <= TRANS_STAGE_UPDATE; ++s) {
            int rc = run_stage(c, s, it);
            if (rc) return rc;
        }
    int rc = run_stage(c, TRANS_STAGE_UPDATE_U, nsub);
    if (rc) return rc;
    if (norms) std::copy(c->norms.begin(), c->norms.end(), norms);
    return TRANS_OK;
}

int trans_stage_times(void* ctx, int ki, double* ms) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !ms) return TRANS_E_ARG;
    c->KI = ki;
    cudaEvent_t ev[TRANS_NSTAGES + 1];
    for (int q = 0; q <= TRANS_NSTAGES; ++q) CK(cudaEventCreate(&ev[q]));
    for (int q = 0; q < TRANS_NSTAGES; ++q) ms[q] = 0.0;
    int nsub = c->p.Kind_Dual != 0 ? c->p.Kchld : 1;
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

int trans_time_iterations(void* ctx, int ki_first, int n, double* ms, trans_norms* norms) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !ms || n < 0) return TRANS_E_ARG;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaEventRecord(e0, c->stream));
    int rc = TRANS_OK;
    for (int q = 0; q < n && rc == TRANS_OK; ++q) rc = trans_iterate(ctx, ki_first + q, norms);
    CK(cudaEventRecord(e1, c->stream));
    CK(cudaEventSynchronize(e1));
    float t = 0;
    CK(cudaEventElapsedTime(&t, e0, e1));
    *ms = t;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

int trans_get_norms(void* ctx, trans_norms* norms) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !norms) return TRANS_E_ARG;
    std::copy(c->norms.begin(), c->norms.end(), norms);
    return TRANS_OK;
}

int trans_sync(void* ctx) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return TRANS_E_ARG;
    CK(cudaStreamSynchronize(c->stream));
    return TRANS_OK;
}

long long trans_device_bytes(void* ctx) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return 0;
    long long b = (long long)(c->arena_doubles * sizeof(double));
    if (c->farena) b += (long long)(c->arena_doubles * sizeof(float));
    b += (c->sv.n + 31) / 32 * 32 * ((long long)(NREC + DQ_STRIDE) * (long long)c->fl->elem + 6LL * (long long)sizeof(int));
    return b;
}

long long trans_kernel_launches(void* ctx) {
    Ctx* c = static_cast<Ctx*>(ctx);
    return c ? c->launches : 0;
}

// ---------------------------------------------------------------------------------------
// TIME_Update_V with its per-tile norm partials in a fixed device buffer.
//
// The buffer is a file-scope __device__ array, part of the loaded library image: the call
// makes no device allocation of any kind.  Its address is taken once per device with
// cudaGetSymbolAddress, with that device current, on the first call made on it (so that first
// call should come before any stream capture), and handed to the kernel as a plain pointer.
// All contexts and calls share the array and it keeps the last call's contents; every entry a
// call reads is written earlier in the same call, so nothing needs clearing.  Calls that
// overlap (two host threads, or two contexts whose streams run concurrently) race on it.
// ---------------------------------------------------------------------------------------
}  // extern "C"

namespace {
constexpr int kStaticNormTiles = 65536;              // 16,777,216 interior cells; 4 MiB
static __device__ __align__(256) NormPart g_norm_scratch[kStaticNormTiles];
constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
NormPart* g_scratch_ptr[kMaxDevices] = {};

int static_norm_scratch(Ctx* c, NormPart** out) {
    int dev = -1;
    CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(c, TRANS_E_ARG, "device ordinal beyond the static scratch table");
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_norm_scratch);
        if (e != cudaSuccess)
            return fail(c, TRANS_E_CUDA, std::string("cudaGetSymbolAddress(static norm scratch): ") + cudaGetErrorString(e));
        g_scratch_ptr[dev] = static_cast<NormPart*>(ptr);
    }
    *out = g_scratch_ptr[dev];
    return TRANS_OK;
}
}  // namespace

extern "C" {

int trans_update_static_scratch(void* ctx, int ki, trans_norms* norms) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return TRANS_E_ARG;
    if (c->cell_tiles.size() > (size_t)kStaticNormTiles)
        return fail(c, TRANS_E_ARG, "trans_update_static_scratch: " + std::to_string(c->cell_tiles.size()) +
                    " cell tiles exceed the static scratch of 65536 tiles (16,777,216 interior cells)");
    NormPart* scratch = nullptr;
    int rc = static_norm_scratch(c, &scratch);
    if (rc) return rc;
    c->KI = ki;
    rc = finalize_geometry(c);
    if (rc) return rc;
    const trans_params& p = c->p;
    const int turb = turb_on(c);
    const int turb_upd = (p.IF_Euler == 0 && turb == 1 && c->KI >= p.KItm) ? 1 : 0;
    launch_update(c->stream, c->d_blk, c->d_cell, (int)c->cell_tiles.size(), c->dp, turb_upd, scratch, c->mixed ? 1 : 0);
    c->launches++;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(c->h_parts.data(), scratch, sizeof(NormPart) * c->h_parts.size(), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    rc = reduce_norms(c);
    if (norms) std::copy(c->norms.begin(), c->norms.end(), norms);
    return rc;
}

int trans_kernel_times(void* ctx, int ki, double* ms, int* launches, int n) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || !ms || !launches || n < NKCLASS) return TRANS_E_ARG;
    for (int k = 0; k < n; ++k) { ms[k] = 0.0; launches[k] = 0; }
    if (c->sweep_mode < 0) {                   // tune outside the timed iteration
        int rc = trans_iterate(ctx, ki, nullptr);
        if (rc) return rc;
        ++ki;
    }
    c->ktime_on = true;
    c->kev.clear();
    int rc = trans_iterate(ctx, ki, nullptr);
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

const char* trans_kernel_class(int k) { return (k >= 0 && k < NKCLASS) ? kclass_name[k] : ""; }

const char* trans_tuning(void* ctx) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c) return "no context";
    static thread_local std::string out;
    out = "sweep=" + std::string(c->sweep_mode == 1 ? "coop " + std::to_string(c->sweep_grid) + "x" + std::to_string(c->sweep_block)
                                 : c->sweep_mode == 0 ? "planes" : "untuned")
          + "; measured: " + c->sweep_tuning;
    return out.c_str();
}

const char* trans_last_error(void* ctx) {
    Ctx* c = static_cast<Ctx*>(ctx);
    return c ? c->err.c_str() : "no context";
}

}  // extern "C"
