// launch.h -- host-side launchers of the hot-path kernels (defined in k_fp64.cu / k_mixed.cu).
#pragma once
#include <cuda_runtime.h>
#include "dev.cuh"

namespace tg {
struct BCEntry;
struct OutletLine;
struct SweepCell;
struct NormPart;
struct SweepSync;
struct SweepView;
struct TileView;
struct BlockNorms;

// FP64 kernels shared by both precision modes
void launch_specrad(cudaStream_t s, const DevBlock* blks, const Tile* tiles, int nt, const CaseDev* cdev);
void launch_bc_state(cudaStream_t s, const DevBlock* blks, const BCEntry* ent, int n, const CaseDev* cdev);
void launch_bc_outlet(cudaStream_t s, const DevBlock* blks, const BCEntry* ent, const OutletLine* lines, int nl,
                      const CaseDev* cdev);
void launch_prims(cudaStream_t s, const DevBlock* blks, int nblk, long long total, const long long* off);
void launch_update(cudaStream_t s, const DevBlock* blks, const Tile* tiles, int nt, const CaseDev* cdev, NormPart* parts,
                   int d_fp32);
void launch_block_norms(cudaStream_t s, const DevBlock* blks, int nblk, const NormPart* parts, const int* tile_first,
                        BlockNorms* out);
void launch_mirror(cudaStream_t s, const DevBlock* blks, int nblk, long long total, const long long* off, const MirrorList& ml);
void launch_update_u(cudaStream_t s, const DevBlock* blks, const Tile* tiles, int nt, const CaseDev* cdev);
// the mixed path's reduced-operation forms of the spectral radius and the update (k_mixed.cu)
void launch_bc_outlet_mixed(cudaStream_t s, const DevBlock* blks, const BCEntry* ent, const OutletLine* lines, int nl,
                            const CaseDev* cdev);
void launch_prims_mixed(cudaStream_t s, const DevBlock* blks, int nblk, long long total, const long long* off);
void launch_specrad_mixed(cudaStream_t s, const DevBlock* blks, const Tile* tiles, int nt, const CaseDev* cdev);
void launch_update_mixed(cudaStream_t s, const DevBlock* blks, const Tile* tiles, int nt, const CaseDev* cdev, NormPart* parts);
// Runge-Kutta marching: stage update of V(1:5) with the |D1/V1| norm partials (itr = stage 1..3),
// then p, T and the SST update with the k and omega norm partials
void launch_rk_update(cudaStream_t s, const DevBlock* blks, const Tile* tiles, int nt, NormPart* parts, int d_fp32, int itr);
void launch_rk_vupdate(cudaStream_t s, const DevBlock* blks, const Tile* tiles, int nt, const CaseDev* cdev, NormPart* parts,
                       int d_fp32);
void launch_field_xfer(cudaStream_t s, const DevBlock& b, int slot0, int ncomp, int lb, int is_sd, double* stage, int to_slots);
// the words of a cross-rank 1-to-1 segment's face cells (k_halo_pack)
void launch_halo_pack(cudaStream_t s, const DevBlock& b, const int* cells, int n, int sweep, int dq_fp32, double* out);
// several page-locked Fortran-layout arrays <-> slots in one launch (total = chunks of `chunk`
// consecutive elements)
void launch_fields_xfer(cudaStream_t s, const XferBatch& x, long long total, int to_slots, int chunk);
double probe_fma_gflops(int fp64);
double probe_chain_us(int chained, int grid);   // floor of one dependent sweep step (k_mixed.cu)
void launch_geom_static(cudaStream_t s, const DevBlock* blks, int nblk, long long total, const long long* off);
// integrated quantities (k_integrals.cu): NINTG sums per case, Cp of one wall segment
constexpr int NINTG = 12;    // inlet m, m p0, m p | outlet m, m p0, m p | pressure force xyz | viscous force xyz
void launch_integrals(cudaStream_t s, const DevBlock* blks, const BCEntry* ent, const int* first, int ncase,
                      const CaseDev* cdev, double* out);
void launch_wall_cp(cudaStream_t s, const DevBlock* blks, const BCEntry* ent, int e0, int n, const CaseDev* cdev,
                    double* cp);
void launch_wall_forces(cudaStream_t s, const DevBlock* blks, const BCEntry* ent, int e0, int n, const CaseDev* cdev,
                        double* f);

// the mixed path's residual from TMA-staged shared-memory tiles (resid_tma.cuh, k_mixed.cu)
constexpr int RT_X = 32;                  // cells along i of a direction-2/3 tile
constexpr int RT_X1 = 28;                 // cells along i of a direction-1 tile
constexpr int RT_D = 8;                   // cells along the direction of a direction-2/3 tile
constexpr int RT_R1 = 8;                  // rows along j of a direction-1 tile (one warp each)
constexpr int RT_W1 = RT_X1 + 8;          // staged extent along i, direction 1 (x0-4 .. x0+31)
constexpr int RT_WIDE = RT_D + 6;         // staged extent along the direction of the stencil fields
constexpr int RT_NARROW = RT_D + 2;       // ... of the two-point fields
constexpr int NRMAP = 5;                  // tensor maps per block: direction 1; 2 stencil, two-point; 3 stencil, two-point
constexpr unsigned RT_WAIT_LIMIT = 1u << 20;   // polls of the tile's mbarrier before the kernel gives up
cudaError_t prepare_resid_tma();          // the kernels' dynamic shared-memory opt-in
// the integer-pipe double <-> float conversions against the hardware ones on n patterns
// (mismatches[0]: double -> float, [1]: float -> double)
cudaError_t check_conversions(long long n, unsigned long long seed, long long* mismatches);
void launch_resid_tma(int dir, cudaStream_t s, const DevBlock* blks, const ResidTile* tiles, int nt, const CaseDev* cdev,
                      const void* maps, int* err, unsigned limit);

// the mixed path's sweeps with one thread-block cluster of cs CTAs x bs threads per solver
// block and cluster barriers between hyperplanes (k_mixed.cu); pb_off: nh x (nblk+1) first
// positions of each block in each hyperplane; sweep_cluster_fits: clusters that fit at once
// (0: this shape cannot launch)
cudaError_t launch_sweep_cluster(cudaStream_t s, const SweepView& v, const int* pb_off, int nh, int nblk, int turb, int cs, int bs,
                                 int pf);
int sweep_cluster_fits(int cs, int bs);

// flux, source and sweep kernels, instantiated per arithmetic type
struct FluxLaunchers {
    void (*gradient)(cudaStream_t, const DevBlock*, const Tile*, int, const CaseDev*);
    void (*shock_ghost)(cudaStream_t, const DevBlock*, const Tile*, int);
    void (*bc_grad)(cudaStream_t, const DevBlock*, const BCEntry*, int);
    void (*face_flux[3])(cudaStream_t, const DevBlock*, const Tile*, int, const CaseDev*);
    void (*gather)(cudaStream_t, const DevBlock*, const Tile*, int, const CaseDev*);
    void (*sst_fc1)(cudaStream_t, const DevBlock*, const Tile*, int, const CaseDev*);
    // cross-rank 1-to-1 segment: words (host-built table, device staging) into the ghost layers
    void (*halo_unpack)(cudaStream_t, const DevBlock&, const int* tab, int n, int sweep, double cost, double sint,
                        const double* in);
    // LU-SGS right-hand sides + neighbour Jacobian terms into the sweep-order arrays
    // (cell order over the cell tiles; qpos = sweep position of each tile slot)
    void (*prep)(cudaStream_t, const DevBlock*, const Tile*, int nt, const int* qpos, const SweepView&, const CaseDev*);
    void (*jac)(cudaStream_t, const DevBlock*, const SweepView&, const CaseDev*);   // neighbours' Jacobian terms (sweep order)
    // lanes: components swept (bits 0-1: 0 mean flow, 1 all, 2 k-omega) | SWEEP_WPC thread mapping
    // (pf_first, pf_count: a later hyperplane prefetched into L2, count 0 = none; chained: 0 plain
    // launch, 1 programmatic dependent launch released after the wait, 2 released at entry (mixed
    // path); cta: threads per CTA of the mixed path's one-thread-per-position launches, 0 = default)
    void (*sweep_lower)(cudaStream_t, const SweepView&, int first, int count, int lanes, int chained, int pf_first, int pf_count,
                        int cta);
    void (*sweep_upper)(cudaStream_t, const SweepView&, int first, int count, int lanes, int chained, int pf_first, int pf_count,
                        int cta);
    // both sweeps in one cooperative launch (grid must be co-resident: grid <= SMs x occupancy)
    // (limit: polls of one wait before the kernel gives up, records the error and returns)
    cudaError_t (*sweep_all)(cudaStream_t, const SweepView&, const int* plane_off, int nplanes, int lanes, SweepSync*,
                             int grid, int block, unsigned limit);
    int (*sweep_all_occupancy)(int block);          // resident blocks per SM
    // both sweeps as a dataflow over per-position ready flags (one cooperative launch)
    cudaError_t (*sweep_flow)(cudaStream_t, const SweepView&, int* flagL, int* flagU, int turb, SweepSync*, int grid, int block,
                              unsigned limit);
    int (*sweep_flow_occupancy)(int block);
    // both sweeps as a tiled wavefront (one cooperative launch, tiles taken from a counter)
    cudaError_t (*sweep_tiles)(cudaStream_t, const SweepView&, const TileView&, int lanes, int* flags, int* counter, SweepSync*,
                               int grid, int block, unsigned limit);
    int (*sweep_tiles_occupancy)(int block);
    // DeltaQ l0..6 back to cell order, one thread per interior cell of the cell tiles
    void (*scatter)(cudaStream_t, const DevBlock*, const Tile*, int nt, const int* qpos, const SweepView&, int l0);
    // two hyperplanes per launch (mixed path only; null in FP64): the lower sweep reads v.dq and
    // writes y, the upper reads y and writes v.dq; p_first/p_count: the second plane, orph/o_count:
    // the first plane's positions with no neighbour on the second
    void (*sweep_pair)(cudaStream_t, const SweepView&, void* y, bool lower, int p_first, int p_count, const int* orph,
                       int o_count, int lanes, int chained, int pf_first, int pf_count, int cta);
    size_t elem;                                    // bytes of the sweep arithmetic type
    int rec_width;                                  // sweep record entries per position (NREC, or NCREC in FP32)
};
const FluxLaunchers& flux_launchers_f64();
const FluxLaunchers& flux_launchers_f32();

constexpr int FACE_TILE = 128;
#ifndef TG_SWEEP_CTA
#define TG_SWEEP_CTA 128
#endif
constexpr int SWEEP_CTA = TG_SWEEP_CTA;    // threads per CTA of the hyperplane sweep launches
constexpr unsigned SWEEP_SPIN_LIMIT = 1u << 22;     // default polls of one wait before it gives up (~1 s)
}  // namespace tg
