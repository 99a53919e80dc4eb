// worklist.cu -- the work lists of a context, rebuilt whenever its set of cases changes:
// tiles of interior cells and faces, the boundary gather tables built from the reference's
// ConnectivityStruct, outlet lines, the i+j+k hyperplane order of the LU-SGS sweeps with the
// neighbour positions, and the per-case parameter array the kernels read.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "engine.h"
#include <cuda.h>
#include <cudaTypedefs.h>

namespace tg {
namespace eng {

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

int block_index(const CaseRec* cs, int id) {
    for (size_t n = 0; n < cs->hb.size(); ++n)
        if (cs->hb[n].id == id) return (int)n;
    return -1;
}

namespace {

int upload_vec(Ctx* c, const void* h, size_t bytes, void** d) {
    if (*d) { cudaFree(*d); *d = nullptr; }
    if (bytes == 0) return TRANS_OK;
    CK(cudaMalloc(d, bytes));
    CK(cudaMemcpy(*d, h, bytes, cudaMemcpyHostToDevice));
    return TRANS_OK;
}

// Gather tables of BC_Boundarys (BC/Boundary.F90:22-47) for one case: one entry per boundary
// face cell, in block / connection / (k,j,i) order; outlets in a separate table ordered line by
// line.  Block indices are the context's (case's first block + local index).
int build_bc(Ctx* c, const CaseRec* cs) {
    const int g0 = cs->blk0;
    for (size_t nb = 0; nb < cs->hb.size(); ++nb) {
        const HostBlock& h = cs->hb[nb];
        const DevBlock& b = cs->blk[nb];
        for (size_t ic = 0; ic < h.conn.size(); ++ic) {
            const trans_conn& a = h.conn[ic];
            int kind = a.BCType;
            if (kind != 1 && kind != 2 && kind != 3 && kind != 5 && kind != 7 && kind != 9)
                return fail(c, TRANS_E_ARG, "unsupported BC kind " + std::to_string(kind));
            int tb = -1;
            const trans_conn* ta = nullptr;
            if (kind == 9) {
                tb = block_index(cs, a.TargetBlock);
                // a target block outside the case: a cross-rank interface, which the caller
                // exchanges with trans_halo_pack / trans_halo_unpack (PARALLEL_BCs)
                if (tb < 0) continue;
                if (a.TargetConn < 1 || a.TargetConn > (int)cs->hb[tb].conn.size())
                    return fail(c, TRANS_E_ARG, "bad 1-to-1 target");
                ta = &cs->hb[tb].conn[a.TargetConn - 1];
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
                E.kind = kind; E.blk = g0 + (int)nb; E.conn = (int)ic; E.i = I; E.j = J; E.k = K;
                E.dir = a.IJKDirect; E.lor = a.LeftOrRight; E.kindsub = a.SubBCType;
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
                    const DevBlock& r = cs->blk[tb];
                    for (int L = 0; L < 3; ++L) {
                        int ii = ib + S3[L][0], jj = jb + S3[L][1], kk = kb + S3[L][2];
                        if (ii < 1 || ii > r.NI1 || jj < 1 || jj > r.NJ1 || kk < 1 || kk > r.NK1)
                            return fail(c, TRANS_E_ARG, "1-to-1 source cell outside the target block");
                        E.s[L] = cidx(r, ii, jj, kk);
                    }
                    E.src_blk = g0 + tb;
                    E.cost = std::cos(a.rotateAngle);
                    E.sint = std::sin(a.rotateAngle);
                } else {
                    const int* S3[3] = {a.CIJKAdd, a.CIJKAdd1, a.CIJKAdd2};
                    for (int L = 0; L < 3; ++L) E.s[L] = cidx(b, I + S3[L][0], J + S3[L][1], K + S3[L][2]);
                    E.src_blk = g0 + (int)nb;
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
                    L.blk = g0 + (int)nb; L.first = (int)(c->outlet.size() + q); L.n = (int)(r - q); L.pad_ = 0;
                    c->lines.push_back(L);
                    q = r;
                }
                c->outlet.insert(c->outlet.end(), seg.begin(), seg.end());
            }
        }
    }
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

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link against libcuda)
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static bool looked = false;
    if (!looked) {
        looked = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
        else
            cudaGetLastError();
    }
    return fn;
}

// The mixed path's TMA-staged residual: brick tiles per face direction and NRMAP tensor maps
// per block over its FP32 slots, a 4-D tensor (i, j, k, slot) with strides PI, PI*PJ, ncell
// floats (multiples of 16 bytes because PI is a multiple of 4).  Box shapes: direction 1
// 36 x 8 x 1 x 1; directions 2 and 3 a stencil box of 14 and a two-point box of 10 cells along
// the direction, 32 along i.  Returns false (the context then uses k_face_flux + k_gather) if
// the driver cannot encode a map.
bool build_resid_tma(Ctx* c) {
    const int nblk = (int)c->blk.size();
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc) return false;
    std::vector<CUtensorMap> maps((size_t)nblk * NRMAP);
    const cuuint32_t boxes[NRMAP][4] = {{RT_W1, RT_R1, 1, 1}, {RT_X, RT_WIDE, 1, 1}, {RT_X, RT_NARROW, 1, 1},
                                        {RT_X, 1, RT_WIDE, 1}, {RT_X, 1, RT_NARROW, 1}};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    for (int n = 0; n < nblk; ++n) {
        const DevBlock& b = c->blk[n];
        if (!b.fbase || (b.PI & 3) || ((uintptr_t)b.fbase & 15)) return false;
        const cuuint64_t dims[4] = {(cuuint64_t)b.PI, (cuuint64_t)b.PJ, (cuuint64_t)b.PK,
                                    (cuuint64_t)case_slots(c->cases[b.cs]->p)};
        const cuuint64_t strides[3] = {(cuuint64_t)b.PI * 4, (cuuint64_t)b.PI * b.PJ * 4, (cuuint64_t)b.ncell * 4};
        for (int q = 0; q < NRMAP; ++q)
            if (enc(&maps[(size_t)n * NRMAP + q], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, (void*)b.fbase, dims, strides, boxes[q], estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
                return false;
    }
    // bricks: interior cells are array indices 3..N+1; origins along i are multiples of 32
    // (directions 2, 3) or 28 (direction 1), so every box starts on a 16-byte boundary
    std::vector<ResidTile> t[3];
    for (int n = 0; n < nblk; ++n) {
        const DevBlock& b = c->blk[n];
        for (int k = 3; k <= b.NK + 1; ++k)
            for (int j = 3; j <= b.NJ + 1; j += RT_R1)
                for (int i = 0; i <= b.NI + 1; i += RT_X1) t[0].push_back({n, i, j, k});
        for (int k = 3; k <= b.NK + 1; ++k)
            for (int j = 3; j <= b.NJ + 1; j += RT_D)
                for (int i = 0; i <= b.NI + 1; i += RT_X) t[1].push_back({n, i, j, k});
        for (int k = 3; k <= b.NK + 1; k += RT_D)
            for (int j = 3; j <= b.NJ + 1; ++j)
                for (int i = 0; i <= b.NI + 1; i += RT_X) t[2].push_back({n, i, j, k});
    }
    if (upload_vec(c, maps.data(), sizeof(CUtensorMap) * maps.size(), &c->d_rmaps)) return false;
    for (int d = 0; d < 3; ++d) {
        if (upload_vec(c, t[d].data(), sizeof(ResidTile) * t[d].size(), (void**)&c->d_rtiles[d])) return false;
        c->n_rtiles[d] = (int)t[d].size();
    }
    return prepare_resid_tma() == cudaSuccess;
}

}  // namespace

int rebuild(Ctx* c) {
    CK(cudaStreamSynchronize(c->stream));
    free_worklists(c);
    c->blk.clear(); c->cell_tiles.clear(); c->cell_tile_blk.clear(); c->ghost_tiles.clear();
    for (int d = 0; d < 3; ++d) c->face_tiles[d].clear();
    c->bc.clear(); c->bc_first.clear(); c->outlet.clear(); c->lines.clear(); c->sweep.clear(); c->plane_off.clear();
    c->cdev_last.clear();
    if (c->cases.empty()) return TRANS_OK;
    // Runge-Kutta cases sweep only k and omega (TURBTWO_TIME_LUSGS_SST; the mean flow is explicit)
    c->sweep_lanes = c->cases[0]->p.IF_RK == 1 ? 2 : 1;
    // blocks of all cases, in case order
    for (size_t k = 0; k < c->cases.size(); ++k) {
        CaseRec* cs = c->cases[k];
        cs->blk0 = (int)c->blk.size();
        for (DevBlock b : cs->blk) {
            b.cs = (int)k;
            c->blk.push_back(b);
        }
    }
    const int nblk = (int)c->blk.size();
    std::vector<long long> off(nblk);
    long long acc = 0;
    for (int n = 0; n < nblk; ++n) { off[n] = acc; acc += c->blk[n].ncell; }
    c->total_cells = acc;
    int rc;
    if ((rc = upload_vec(c, c->blk.data(), sizeof(DevBlock) * nblk, (void**)&c->d_blk))) return rc;
    if ((rc = upload_vec(c, off.data(), sizeof(long long) * nblk, (void**)&c->d_off))) return rc;
    // tiles of interior cells, faces of each direction and face ghosts (shock extrapolation)
    std::vector<long long> cnt(nblk), fcnt[3], gcnt(nblk);
    for (int d = 0; d < 3; ++d) fcnt[d].resize(nblk);
    for (int n = 0; n < nblk; ++n) {
        const DevBlock& b = c->blk[n];
        cnt[n] = b.nint;
        fcnt[0][n] = (long long)b.NI * b.NJ1 * b.NK1;
        fcnt[1][n] = (long long)b.NI1 * b.NJ * b.NK1;
        fcnt[2][n] = (long long)b.NI1 * b.NJ1 * b.NK;
        gcnt[n] = 6LL * ((long long)b.NJ1 * b.NK1 + (long long)b.NI1 * b.NK1 + (long long)b.NI1 * b.NJ1);
    }
    make_tiles(nblk, cnt, CELL_TILE, c->cell_tiles, &c->cell_tile_blk);
    for (int d = 0; d < 3; ++d) make_tiles(nblk, fcnt[d], FACE_TILE, c->face_tiles[d], nullptr);
    make_tiles(nblk, gcnt, CELL_TILE, c->ghost_tiles, nullptr);
    if ((rc = upload_vec(c, c->cell_tiles.data(), sizeof(Tile) * c->cell_tiles.size(), (void**)&c->d_cell))) return rc;
    for (int d = 0; d < 3; ++d)
        if ((rc = upload_vec(c, c->face_tiles[d].data(), sizeof(Tile) * c->face_tiles[d].size(), (void**)&c->d_face[d]))) return rc;
    if ((rc = upload_vec(c, c->ghost_tiles.data(), sizeof(Tile) * c->ghost_tiles.size(), (void**)&c->d_ghost))) return rc;
    if (c->mixed && c->resid_tma != 0 && !build_resid_tma(c)) c->resid_tma = 0;
    // boundary tables
    c->bc_first.clear();
    for (CaseRec* cs : c->cases) {
        c->bc_first.push_back((int)c->bc.size());
        if ((rc = build_bc(c, cs))) return rc;
    }
    c->bc_first.push_back((int)c->bc.size());
    if ((rc = upload_vec(c, c->bc_first.data(), sizeof(int) * c->bc_first.size(), (void**)&c->d_bc_first))) return rc;
    CK(cudaMalloc(&c->d_intg, sizeof(double) * NINTG * c->cases.size()));
    if ((rc = upload_vec(c, c->bc.data(), sizeof(BCEntry) * c->bc.size(), (void**)&c->d_bc))) return rc;
    if ((rc = upload_vec(c, c->outlet.data(), sizeof(BCEntry) * c->outlet.size(), (void**)&c->d_outlet))) return rc;
    if ((rc = upload_vec(c, c->lines.data(), sizeof(OutletLine) * c->lines.size(), (void**)&c->d_lines))) return rc;
    // hyperplane order of the LU-SGS sweeps over all blocks of all cases: h = i+j+k = 3 ..
    int hmax = 3;
    for (auto& b : c->blk) hmax = std::max(hmax, b.NI1 + b.NJ1 + b.NK1);
    c->plane_off.assign(1, 0);
    std::vector<int> pb_off;
    for (int h = 3; h <= hmax; ++h) {
        for (int n = 0; n < nblk; ++n) {
            const DevBlock& b = c->blk[n];
            pb_off.push_back((int)c->sweep.size());
            for (int k = 1; k <= b.NK1; ++k)
                for (int j = 1; j <= b.NJ1; ++j) {
                    int i = h - j - k;
                    if (i >= 1 && i <= b.NI1) c->sweep.push_back(SweepCell{n, i, j, k});
                }
        }
        pb_off.push_back((int)c->sweep.size());
        c->plane_off.push_back((int)c->sweep.size());
    }
    if ((rc = upload_vec(c, pb_off.data(), sizeof(int) * pb_off.size(), (void**)&c->d_pb_off))) return rc;
    if ((rc = upload_vec(c, c->sweep.data(), sizeof(SweepCell) * c->sweep.size(), (void**)&c->d_sweep))) return rc;
    if ((rc = upload_vec(c, c->plane_off.data(), sizeof(int) * c->plane_off.size(), (void**)&c->d_plane_off))) return rc;
    {   // neighbour positions in sweep order: lower i,j,k (0..2) and upper (3..5), -1 = none
        const long long N = (long long)c->sweep.size();
        const long long Np = (N + 31) / 32 * 32;
        std::vector<std::vector<int>> pos(nblk);
        for (int n = 0; n < nblk; ++n) pos[n].assign((size_t)c->blk[n].nint, -1);
        for (long long q = 0; q < N; ++q) {
            const SweepCell& sc = c->sweep[q];
            const DevBlock& b = c->blk[sc.blk];
            pos[sc.blk][(size_t)(sc.i - 1) + (size_t)b.NI1 * ((sc.j - 1) + (size_t)b.NJ1 * (sc.k - 1))] = (int)q;
        }
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
        if ((rc = upload_vec(c, nbp.data(), sizeof(int) * nbp.size(), (void**)&c->d_nbp))) return rc;
        // sweep position of every slot of every cell tile (tiles hold consecutive interior cells)
        std::vector<int> qpos(c->cell_tiles.size() * (size_t)CELL_TILE, -1);
        for (size_t t = 0; t < c->cell_tiles.size(); ++t) {
            const Tile& tl = c->cell_tiles[t];
            for (int r = 0; r < tl.count; ++r) qpos[t * CELL_TILE + r] = pos[tl.blk][(size_t)tl.start + r];
        }
        if ((rc = upload_vec(c, qpos.data(), sizeof(int) * qpos.size(), (void**)&c->d_qpos))) return rc;
        CK(cudaMalloc(&c->d_rec, (size_t)c->fl->rec_width * Np * c->fl->elem));
        CK(cudaMalloc(&c->d_dqs, (size_t)DQ_STRIDE * Np * c->fl->elem));
        if (c->fl->sweep_pair) {
            // two-plane schedule: the second DeltaQ array, and per launch the first plane's
            // positions that no neighbour on the second plane computes (block corners)
            CK(cudaMalloc(&c->d_dq2, (size_t)DQ_STRIDE * Np * c->fl->elem));
            const int nh = (int)c->plane_off.size() - 1;
            std::vector<int> orph;
            auto add = [&](std::vector<Ctx::SweepPair>& out, int h, int h1, int side) {
                Ctx::SweepPair sp{0, 0, (int)orph.size(), 0};
                if (h1 >= 0 && h1 < nh) { sp.p_first = c->plane_off[h1]; sp.p_count = c->plane_off[h1 + 1] - c->plane_off[h1]; }
                for (int q = c->plane_off[h]; q < c->plane_off[h + 1]; ++q) {
                    bool reached = false;
                    for (int d = 0; d < 3; ++d) reached |= nbp[sw_at(q, side + d, 6)] >= 0;
                    if (!reached || sp.p_count == 0) orph.push_back(q);
                }
                sp.o_count = (int)orph.size() - sp.o_off;
                out.push_back(sp);
            };
            c->pair_lo.clear();
            c->pair_up.clear();
            for (int h = 0; h < nh; h += 2) add(c->pair_lo, h, h + 1, 3);        // reached from its upper neighbours
            for (int h = nh - 1; h >= 0; h -= 2) add(c->pair_up, h, h - 1, 0);   // from its lower neighbours
            if (orph.empty()) orph.push_back(0);
            if ((rc = upload_vec(c, orph.data(), sizeof(int) * orph.size(), (void**)&c->d_orph))) return rc;
        }
        CK(cudaMalloc(&c->d_flags, (size_t)2 * Np * sizeof(int)));
        c->sv.cells = c->d_sweep; c->sv.nbp = c->d_nbp; c->sv.rec = c->d_rec; c->sv.dq = c->d_dqs; c->sv.n = N;
        c->sv.pc = nullptr;
        if (c->cases[0]->p.IF_Precondition == 1) {      // the neighbours' PrecondDW coefficients (FP64 path)
            CK(cudaMalloc(&c->d_pc, (size_t)6 * NPC * Np * sizeof(double)));
            c->sv.pc = c->d_pc;
        }
    }
    {   // staging buffer for the largest Fortran field (DQdxyz: 18 components, lower bound -1)
        size_t mx = 0;
        for (auto& b : c->blk) mx = std::max(mx, (size_t)(b.NI + 4) * (b.NJ + 4) * (b.NK + 4) * 18);
        c->stage_doubles = mx;
        CK(cudaMalloc(&c->d_stage, mx * sizeof(double)));
    }
    {   // first cell tile of every block (tiles are made block by block)
        std::vector<int> tf(nblk + 1, 0);
        for (size_t t = 0; t < c->cell_tile_blk.size(); ++t) tf[c->cell_tile_blk[t] + 1]++;
        for (int n = 0; n < nblk; ++n) tf[n + 1] += tf[n];
        if ((rc = upload_vec(c, tf.data(), sizeof(int) * tf.size(), (void**)&c->d_tile_first))) return rc;
        CK(cudaMalloc(&c->d_norms, sizeof(BlockNorms) * (size_t)nblk * NORM_HIST));
        CK(cudaMallocHost(&c->h_norms, sizeof(BlockNorms) * (size_t)nblk * NORM_HIST));
    }
    c->h_parts.assign(c->cell_tiles.size(), NormPart{});
    CK(cudaMalloc(&c->d_parts, sizeof(NormPart) * std::max<size_t>(1, c->h_parts.size())));
    c->norms.assign(nblk, trans_norms{});
    CK(cudaMalloc(&c->d_cdev, sizeof(CaseDev) * c->cases.size()));
    CK(cudaMallocHost(&c->h_cdev, sizeof(CaseDev) * c->cases.size()));
    // re-tune the sweep schedule when the sweep work has changed by more than a factor 2 since
    // it was tuned (a serving loop adds and removes cases every few iterations, and a tuning run
    // times ~40 candidate sweeps); the schedule kept is re-captured for the new work lists
    const long long npos = (long long)c->sweep.size();
    if (!c->sweep_forced && (c->tuned_positions <= 0 || npos > 2 * c->tuned_positions || 2 * npos < c->tuned_positions))
        c->sweep_mode = -1;
    c->built = true;
    return TRANS_OK;
}

// Tiles of TIxTJxTK cells for the tiled-wavefront sweep schedule (TileView, types.cuh):
// numbered by tile hyperplane ti+tj+tk (then block, tk, tj, ti), cells of a tile listed by
// the tile's own i+j+k planes.
int build_tiles(Ctx* c, int TI, int TJ, int TK) {
    if (c->tile_shape[0] == TI && c->tile_shape[1] == TJ && c->tile_shape[2] == TK && c->d_tiles) return TRANS_OK;
    if (c->d_tiles) { cudaFree(c->d_tiles); c->d_tiles = nullptr; }
    if (c->d_tflags) { cudaFree(c->d_tflags); c->d_tflags = nullptr; }
    c->tv = TileView{};
    c->tile_shape[0] = c->tile_shape[1] = c->tile_shape[2] = 0;
    const int nblk = (int)c->blk.size();
    std::vector<std::vector<int>> pos(nblk);
    for (int n = 0; n < nblk; ++n) pos[n].assign((size_t)c->blk[n].nint, -1);
    for (size_t q = 0; q < c->sweep.size(); ++q) {
        const SweepCell& sc = c->sweep[q];
        const DevBlock& b = c->blk[sc.blk];
        pos[sc.blk][(size_t)(sc.i - 1) + (size_t)b.NI1 * ((sc.j - 1) + (size_t)b.NJ1 * (sc.k - 1))] = (int)q;
    }
    struct TileKey { int h, n, tk, tj, ti; };
    std::vector<TileKey> keys;
    std::vector<int> nti(nblk), ntj(nblk), ntk(nblk);
    for (int n = 0; n < nblk; ++n) {
        const DevBlock& b = c->blk[n];
        nti[n] = (b.NI1 + TI - 1) / TI; ntj[n] = (b.NJ1 + TJ - 1) / TJ; ntk[n] = (b.NK1 + TK - 1) / TK;
        for (int tk = 0; tk < ntk[n]; ++tk)
            for (int tj = 0; tj < ntj[n]; ++tj)
                for (int ti = 0; ti < nti[n]; ++ti) keys.push_back(TileKey{ti + tj + tk, n, tk, tj, ti});
    }
    std::stable_sort(keys.begin(), keys.end(), [](const TileKey& a, const TileKey& b) {
        if (a.h != b.h) return a.h < b.h;
        if (a.n != b.n) return a.n < b.n;
        if (a.tk != b.tk) return a.tk < b.tk;
        if (a.tj != b.tj) return a.tj < b.tj;
        return a.ti < b.ti;
    });
    const int nt = (int)keys.size();
    std::vector<std::vector<int>> tid(nblk);           // tile number of (block, ti, tj, tk)
    for (int n = 0; n < nblk; ++n) tid[n].assign((size_t)nti[n] * ntj[n] * ntk[n], -1);
    for (int t = 0; t < nt; ++t) {
        const TileKey& k = keys[t];
        tid[k.n][(size_t)k.ti + (size_t)nti[k.n] * ((size_t)k.tj + (size_t)ntj[k.n] * k.tk)] = t;
    }
    std::vector<int> plane0, pitem, item, dep((size_t)6 * nt, -1);
    item.reserve(c->sweep.size());
    for (int t = 0; t < nt; ++t) {
        const TileKey& k = keys[t];
        const DevBlock& b = c->blk[k.n];
        const int i0 = k.ti * TI + 1, j0 = k.tj * TJ + 1, k0 = k.tk * TK + 1;
        const int i1 = std::min(i0 + TI - 1, b.NI1), j1 = std::min(j0 + TJ - 1, b.NJ1), k1 = std::min(k0 + TK - 1, b.NK1);
        plane0.push_back((int)pitem.size());
        for (int h = 0; h <= (i1 - i0) + (j1 - j0) + (k1 - k0); ++h) {
            pitem.push_back((int)item.size());
            for (int kk = k0; kk <= k1; ++kk)
                for (int jj = j0; jj <= j1; ++jj) {
                    const int ii = i0 + h - (jj - j0) - (kk - k0);
                    if (ii >= i0 && ii <= i1)
                        item.push_back(pos[k.n][(size_t)(ii - 1) + (size_t)b.NI1 * ((jj - 1) + (size_t)b.NJ1 * (kk - 1))]);
                }
        }
        const int tc[3] = {k.ti, k.tj, k.tk}, tn[3] = {nti[k.n], ntj[k.n], ntk[k.n]};
        for (int side = 0; side < 2; ++side)
            for (int d = 0; d < 3; ++d) {
                int x[3] = {tc[0], tc[1], tc[2]};
                x[d] += side == 0 ? -1 : 1;
                if (x[d] < 0 || x[d] >= tn[d]) continue;
                dep[(size_t)6 * t + 3 * side + d] = tid[k.n][(size_t)x[0] + (size_t)nti[k.n] * ((size_t)x[1] + (size_t)ntj[k.n] * x[2])];
            }
    }
    plane0.push_back((int)pitem.size());
    pitem.push_back((int)item.size());
    if (item.size() != c->sweep.size()) return fail(c, TRANS_E_CUDA, "tile lists do not cover the sweep positions");
    std::vector<int> all;                               // one device array: plane0 | pitem | item | dep
    all.reserve(plane0.size() + pitem.size() + item.size() + dep.size());
    all.insert(all.end(), plane0.begin(), plane0.end());
    all.insert(all.end(), pitem.begin(), pitem.end());
    all.insert(all.end(), item.begin(), item.end());
    all.insert(all.end(), dep.begin(), dep.end());
    int rc;
    if ((rc = upload_vec(c, all.data(), sizeof(int) * all.size(), (void**)&c->d_tiles))) return rc;
    CK(cudaMalloc(&c->d_tflags, sizeof(int) * ((size_t)2 * nt + 1)));
    c->tv.ntiles = nt;
    c->tv.plane0 = c->d_tiles;
    c->tv.pitem = c->d_tiles + plane0.size();
    c->tv.item = c->tv.pitem + pitem.size();
    c->tv.dep = c->tv.item + item.size();
    c->tile_shape[0] = TI; c->tile_shape[1] = TJ; c->tile_shape[2] = TK;
    return TRANS_OK;
}

}  // namespace eng
}  // namespace tg
