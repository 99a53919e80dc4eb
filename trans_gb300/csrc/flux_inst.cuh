// flux_inst.cuh -- instantiation of the templated flux/source/sweep kernels for one type R.
// Included once per precision translation unit with TG_R and TG_NAME defined.
#include <algorithm>

#include "kernels.cuh"
#include "launch.h"

namespace tg {
namespace {
void grd(cudaStream_t s, const DevBlock* b, const Tile* t, int nt, const CaseDev* cd) {
    if (nt > 0) k_gradient<TG_R><<<nt, CELL_TILE, 0, s>>>(b, t, cd);
}
void shg(cudaStream_t s, const DevBlock* b, const Tile* t, int nt) {
    if (nt > 0) k_shock_ghost<TG_R><<<nt, CELL_TILE, 0, s>>>(b, t);
}
void bcg(cudaStream_t s, const DevBlock* b, const BCEntry* e, int n) {
    if (n > 0) k_bc_grad<TG_R><<<(n + 127) / 128, 128, 0, s>>>(b, e, n);
}
template <int DIR>
void ff(cudaStream_t s, const DevBlock* b, const Tile* t, int nt, const CaseDev* cd) {
    if (nt <= 0) return;
    // viscous, then convective fluxes (two register budgets)
    k_face_flux<TG_R, DIR, 1><<<nt, FACE_TILE, 0, s>>>(b, t, cd);
    k_face_flux<TG_R, DIR, 2><<<nt, FACE_TILE, 0, s>>>(b, t, cd);
}
void ga(cudaStream_t s, const DevBlock* b, const Tile* t, int nt, const CaseDev* cd) {
    if (nt > 0) k_gather<TG_R><<<nt, CELL_TILE, 0, s>>>(b, t, cd);
}
void hu(cudaStream_t s, const DevBlock& b, const int* tab, int n, int sweep, double cost, double sint, const double* in) {
    if (n > 0) k_halo_unpack<TG_R><<<(n + 127) / 128, 128, 0, s>>>(b, tab, n, sweep, cost, sint, in);
}
void fc(cudaStream_t s, const DevBlock* b, const Tile* t, int nt, const CaseDev* cd) {
    if (nt > 0) k_sst_fc1<TG_R><<<nt, CELL_TILE, 0, s>>>(b, t, cd);
}
void prep(cudaStream_t s, const DevBlock* b, const Tile* tiles, int nt, const int* qpos, const SweepView& v, const CaseDev* cd) {
    if (nt > 0) k_lusgs_prep<TG_R><<<nt, CELL_TILE, 0, s>>>(b, tiles, qpos, (TG_R*)v.rec, (TG_R*)v.dq, cd);
}
// the FP64 path's neighbour Jacobian terms; the mixed path rebuilds them in the sweep from the
// compact records k_lusgs_prep writes, so it has no such pass
void jac(cudaStream_t s, const DevBlock* b, const SweepView& v, const CaseDev* cd) {
    if constexpr (sizeof(TG_R) == 8) {
        if (v.n > 0)
            k_lusgs_jac<TG_R><<<(unsigned)((v.n + 31) / 32), 6 * 32, 0, s>>>(b, v.cells, v.nbp, (TG_R*)v.rec, v.n);
        if (v.n > 0 && v.pc)        // low-Mach preconditioning: the neighbours' PrecondDW coefficients
            k_lusgs_jac_pc<<<(unsigned)((6 * v.n + 127) / 128), 128, 0, s>>>(b, v.cells, v.nbp, cd, (double*)v.pc, v.n);
    }
}
// one hyperplane; chained = launched with programmatic stream serialisation, so that this
// hyperplane's independent loads overlap the previous one (the kernel waits before its
// dependent part)
template <bool LOWER>
void swp(cudaStream_t s, const SweepView& v, int first, int count, int turb, int chained, int pf_first, int pf_count, int cta) {
    if (count <= 0) return;
    if constexpr (sizeof(TG_R) == 4) {      // mixed path: one thread per position (k_sweep_c)
        const int CTA = cta > 0 ? cta : SWEEP_CTA;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((count + CTA - 1) / CTA);
        cfg.blockDim = dim3(CTA);
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = chained ? 1 : 0;
        cudaLaunchKernelEx(&cfg, k_sweep_c<LOWER>, (const int*)v.nbp, (const float*)v.rec, (float*)v.dq, first, count, turb & 3,
                           chained, pf_first, pf_count);
        return;
    }
    const int* nbp = v.nbp;
    const TG_R* rec = (const TG_R*)v.rec;
    TG_R* dq = (TG_R*)v.dq;
    long long n = v.n;
    cudaLaunchConfig_t cfg = {};
    // FP64: one-warp CTAs spread a hyperplane's warps over the most SMs, hence over the most
    // FP64 units (measured on the cascade: 4.51 ms of sweeps per iteration at 32 threads, 4.76 at
    // 64, 5.13 at 128); FP32 is indifferent between 32 and 128
    constexpr int CTA = sizeof(TG_R) == 8 ? 32 : SWEEP_CTA;
    cfg.gridDim = dim3((sweep_items(count, turb) + CTA - 1) / CTA);
    cfg.blockDim = dim3(CTA);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = chained ? 1 : 0;
    const TG_R* pc = (const TG_R*)v.pc;
    cudaLaunchKernelEx(&cfg, k_sweep<TG_R, LOWER>, nbp, rec, dq, n, first, count, turb, chained, pf_first, pf_count, pc);
}
void swl(cudaStream_t s, const SweepView& v, int first, int count, int turb, int chained, int pf_first, int pf_count, int cta) {
    swp<true>(s, v, first, count, turb, chained, pf_first, pf_count, cta);
}
void swu(cudaStream_t s, const SweepView& v, int first, int count, int turb, int chained, int pf_first, int pf_count, int cta) {
    swp<false>(s, v, first, count, turb, chained, pf_first, pf_count, cta);
}
cudaError_t swa(cudaStream_t s, const SweepView& v, const int* po, int nplanes, int turb, SweepSync* sy, int grid, int block,
                unsigned limit) {
    const int* nbp = v.nbp;
    const TG_R* rec = (const TG_R*)v.rec;
    TG_R* dq = (TG_R*)v.dq;
    long long n = v.n;
    const TG_R* pc = (const TG_R*)v.pc;
    void* args[] = {(void*)&nbp, (void*)&rec, (void*)&dq, (void*)&n, (void*)&po, (void*)&nplanes, (void*)&turb,
                    (void*)&sy, (void*)&limit, (void*)&pc};
    return cudaLaunchCooperativeKernel((const void*)k_sweep_all<TG_R>, dim3(grid), dim3(block), args, 0, s);
}
int swa_occ(int block) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_sweep_all<TG_R>, block, 0) != cudaSuccess) return 0;
    return n;
}
cudaError_t swf(cudaStream_t s, const SweepView& v, int* flagL, int* flagU, int turb, SweepSync* sy, int grid, int block,
                unsigned limit) {
    const int* nbp = v.nbp;
    const TG_R* rec = (const TG_R*)v.rec;
    TG_R* dq = (TG_R*)v.dq;
    long long n = v.n;
    const TG_R* pc = (const TG_R*)v.pc;
    void* args[] = {(void*)&nbp, (void*)&rec, (void*)&dq, (void*)&n, (void*)&flagL, (void*)&flagU, (void*)&turb, (void*)&sy,
                    (void*)&limit, (void*)&pc};
    return cudaLaunchCooperativeKernel((const void*)k_sweep_flow<TG_R>, dim3(grid), dim3(block), args, 0, s);
}
int swf_occ(int block) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_sweep_flow<TG_R>, block, 0) != cudaSuccess) return 0;
    return n;
}
cudaError_t swt(cudaStream_t s, const SweepView& v, const TileView& tv, int lanes, int* flags, int* counter, SweepSync* sy,
                int grid, int block, unsigned limit) {
    if (v.n <= 0 || tv.ntiles <= 0) return cudaSuccess;
    // cooperative: the CTAs wait on one another, so the whole grid must be resident
    const int* nbp = v.nbp;
    const TG_R* rec = (const TG_R*)v.rec;
    TG_R* dq = (TG_R*)v.dq;
    long long n = v.n;
    TileView t = tv;
    const TG_R* pc = (const TG_R*)v.pc;
    void* args[] = {(void*)&nbp, (void*)&rec, (void*)&dq, (void*)&n, (void*)&t, (void*)&lanes, (void*)&flags, (void*)&counter,
                    (void*)&sy, (void*)&limit, (void*)&pc};
    return cudaLaunchCooperativeKernel((const void*)k_sweep_tiles<TG_R>, dim3(grid), dim3(block), args, 0, s);
}
int swt_occ(int block) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_sweep_tiles<TG_R>, block, 0) != cudaSuccess) return 0;
    return n;
}
void swpair(cudaStream_t s, const SweepView& v, void* y, bool lower, int p_first, int p_count, const int* orph, int o_count,
            int turb, int chained, int pf_first, int pf_count, int cta) {
    if constexpr (sizeof(TG_R) == 4) {
        const int n = 4 * (p_count + o_count);                        // four lanes per item
        if (n <= 0) return;
        const int CTA = std::min(cta > 0 ? cta : SWEEP_CTA, 128);      // the kernel's launch bound
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((n + CTA - 1) / CTA);
        cfg.blockDim = dim3(CTA);
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = chained ? 1 : 0;
        float* X = (float*)v.dq;
        float* Y = (float*)y;
        if (lower)
            cudaLaunchKernelEx(&cfg, k_sweep_pair<true>, (const int*)v.nbp, (const float*)v.rec, X, Y, p_first, p_count, orph,
                               o_count, turb & 3, chained, pf_first, pf_count);
        else
            cudaLaunchKernelEx(&cfg, k_sweep_pair<false>, (const int*)v.nbp, (const float*)v.rec, X, Y, p_first, p_count, orph,
                               o_count, turb & 3, chained, pf_first, pf_count);
    }
}
void scat(cudaStream_t s, const DevBlock* b, const Tile* tiles, int nt, const int* qpos, const SweepView& v, int l0) {
    if (nt > 0 && v.n > 0) k_sweep_scatter<TG_R><<<nt, CELL_TILE, 0, s>>>(b, tiles, qpos, (const TG_R*)v.dq, l0);
}
}  // namespace

const FluxLaunchers& TG_NAME() {
    static const FluxLaunchers L = {grd, shg, bcg, {ff<1>, ff<2>, ff<3>}, ga, fc, hu, prep, jac, swl, swu, swa, swa_occ, swf, swf_occ,
                                    swt, swt_occ, scat, sizeof(TG_R) == 4 ? swpair : nullptr, sizeof(TG_R),
                                    sizeof(TG_R) == 4 ? (int)NCREC : (int)NREC};
    return L;
}
}  // namespace tg
