// engine.h -- host side of the GB300 hot path: contexts holding one or many cases (batches),
// their device memory, work lists and the stage sequence of main.F90:54-197.
//
// A context owns a set of cases.  Each case is one independent solve (its own blocks, module
// globals, iteration counter and norms) with its blocks in its own device arena.  All cases
// of a context are advanced together: the work lists (cell/face tiles, boundary gathers,
// sweep hyperplanes) cover every block of every case, so each kernel is one launch for the
// whole batch.  Adding or removing a case rebuilds the work lists; the arenas stay put.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/trans_gpu.h"
#include "launch.h"
#include "types.cuh"

namespace tg {
extern thread_local std::string g_stateless_err;   // the message stateless_error() returns
namespace eng {

struct HostBlock {
    int NI, NJ, NK, id;
    std::vector<trans_conn> conn;
    std::vector<int> mw[6];
};

struct CaseRec {
    int id = 0;                          // handle of the batch API
    trans_params p{};
    Params dp{};
    std::vector<HostBlock> hb;
    std::vector<DevBlock> blk;           // base pointers into this case's arena; cs set at rebuild
    double* arena = nullptr;
    float* farena = nullptr;             // FP32 copies of the slots (mixed path only)
    size_t arena_doubles = 0;
    long long bytes = 0;                 // device bytes charged to the budget
    int KI = 0;                          // outer iteration of the next/last call
    int iters = 0;                       // iterations done since the case was added
    int blk0 = 0;                        // index of its first block in the context's block list
    bool geom_dirty = true;
    std::vector<trans_norms> norms, first_norms;
};

// kernel classes of trans_kernel_times
enum KClass { K_SPECRAD, K_BC_STATE, K_BC_OUTLET, K_PRIMS, K_MIRROR, K_GRADIENT, K_SHOCK_GHOST, K_BC_GRAD,
              K_FACE, K_GATHER, K_SST_FC1, K_PREP, K_SWEEP, K_SCATTER, K_UPDATE, K_UPDATE_U, K_RESID_TMA, NKCLASS };
extern const char* const kclass_name[NKCLASS];

constexpr int GRAPH_ITERS = 8;            // outer iterations per replay of the iteration graph
constexpr int NORM_HIST = GRAPH_ITERS;    // norm history depth (one entry per replayed iteration)

struct Ctx {
    int precision = TRANS_FP64;
    bool mixed = false;
    const FluxLaunchers* fl = nullptr;
    long long budget = 0;                // device bytes the cases may take (0 = no limit)
    long long in_use = 0;
    int next_id = 0;
    std::vector<CaseRec*> cases;
    cudaStream_t stream = nullptr;
    long long launches = 0;
    std::string err;
    // ---- rebuilt when the set of cases changes ----
    std::vector<DevBlock> blk;           // all blocks of all cases
    DevBlock* d_blk = nullptr;
    long long* d_off = nullptr;          // padded-cell offsets of the blocks (for flat kernels)
    long long total_cells = 0;
    std::vector<Tile> cell_tiles, face_tiles[3], ghost_tiles;
    Tile *d_cell = nullptr, *d_face[3] = {nullptr, nullptr, nullptr}, *d_ghost = nullptr;
    std::vector<int> cell_tile_blk;      // block of each cell tile (norm reduction)
    // mixed path: the residual from TMA-staged tiles (one tile list per face direction, NRMAP
    // tensor maps per block over its FP32 slots) when 1; 0 (the default) uses k_face_flux +
    // k_gather; -1 times both on the first residual and keeps the faster.  The two forms sum a
    // cell's fluxes in different orders, so a timed choice can differ between contexts and
    // their results then only agree to FP32 rounding; the fixed default keeps a case's result
    // the same alone and in any batch.
    int resid_tma = 0;
    bool xfer_batch = true;              // trans_set/get_fields: page-locked arrays in one launch
    bool xfer_mapped = true;             // page-locked arrays read in place (false: copied by DMA through the staging buffer)
    std::string resid_tuning;
    ResidTile* d_rtiles[3] = {nullptr, nullptr, nullptr};
    int n_rtiles[3] = {0, 0, 0};
    void* d_rmaps = nullptr;
    unsigned resid_spin = RT_WAIT_LIMIT; // polls of a tile's staging wait (TRANS_RESID_SPIN overrides)
    void* d_halo = nullptr;              // staging of the cross-rank interface exchange
    size_t halo_bytes = 0;
    int* d_kerr = nullptr;               // set by a kernel whose bounded wait gave up
    int* h_kerr = nullptr;               // pinned
    std::vector<BCEntry> bc, outlet;
    std::vector<OutletLine> lines;
    BCEntry *d_bc = nullptr, *d_outlet = nullptr;
    std::vector<int> bc_first;           // entries of case k in bc: [bc_first[k], bc_first[k+1])
    int* d_bc_first = nullptr;
    double* d_intg = nullptr;            // NINTG integrated-quantity sums per case
    OutletLine* d_lines = nullptr;
    std::vector<SweepCell> sweep;
    std::vector<int> plane_off;          // sweep positions of hyperplane h: [plane_off[h], plane_off[h+1])
    SweepCell* d_sweep = nullptr;
    int* d_plane_off = nullptr;
    int* d_pb_off = nullptr;             // nh x (nblk+1): first position of block b in hyperplane h
    SweepView sv{};
    int* d_nbp = nullptr;
    int* d_qpos = nullptr;               // sweep position of every cell-tile slot (-1: past the tile's end)
    int* d_flags = nullptr;
    void* d_rec = nullptr;
    void* d_dqs = nullptr;
    void* d_dq2 = nullptr;               // the lower sweep's results in the two-plane schedule (mixed path)
    void* d_dq_save = nullptr;
    // two-plane schedule (sweep_mode 5): per launch the second plane's positions and the first
    // plane's positions that no position of the second plane reaches (offsets into d_orph)
    struct SweepPair { int p_first, p_count, o_off, o_count; };
    std::vector<SweepPair> pair_lo, pair_up;
    int* d_orph = nullptr;
    double* d_pc = nullptr;              // PrecondDW coefficients of the sweep neighbours (IF_Precondition = 1)
    NormPart* d_parts = nullptr;
    std::vector<NormPart> h_parts;
    int* d_tile_first = nullptr;         // first cell tile of each block (+ end)
    BlockNorms* d_norms = nullptr;       // per block, NORM_HIST iterations deep
    BlockNorms* h_norms = nullptr;       // pinned
    // whole iterations replayed as one CUDA graph (trans_batch_iterate, trans_time_iterations)
    cudaGraphExec_t iter_exec = nullptr;
    int iter_n = 0;
    long long iter_launches = 0;
    cudaGraphExec_t iter1_exec = nullptr;  // one iteration (trans_iterate, and the rest of a run)
    long long iter1_launches = 0;
    bool graphs = true;
    std::vector<trans_norms> norms;      // per block of the context
    CaseDev* d_cdev = nullptr;           // per case slot
    CaseDev* h_cdev = nullptr;           // pinned
    std::vector<CaseDev> cdev_last;      // what was last uploaded
    double* d_stage = nullptr;           // Fortran-layout staging buffer of trans_set/get_field
    cudaEvent_t copy_done = nullptr;     // the last upload's host-to-device copy
    size_t stage_doubles = 0;
    bool built = false;
    // ---- sweep schedule ----
    cudaGraphExec_t sweep_exec = nullptr;
    // 0 = one launch per hyperplane (graph), 1 = one cooperative launch with grid barriers,
    // 2 = dataflow over ready flags, 3 = tiled wavefront, 4 = one thread-block cluster per
    // block with cluster barriers between hyperplanes (mixed path; sweep_grid = CTAs per
    // cluster), 5 = two hyperplanes per launch (mixed path, graph); -1 = pick the fastest on
    // first use
    // (all bit-identical)
    int sweep_mode = -1, sweep_grid = 0, sweep_block = 0;
    int tile_shape[3] = {0, 0, 0};       // tiles of the tiled wavefront (built for this shape)
    int tile_default[3] = {8, 8, 8};     // shape when the schedule is forced (TRANS_TILE=AxBxC)
    int* d_tiles = nullptr;              // plane0 | pitem | item | dep arrays of the TileView
    int* d_tflags = nullptr;             // 2 x ntiles publish flags + the tile counter
    TileView tv{};
    bool sweep_forced = false;
    long long tuned_positions = 0;       // sweep positions the schedule was tuned on (0: never tuned)
    int pdl = 1;                         // chain hyperplane launches (programmatic dependent launch;
                                         // 2 = the mixed path's release of the next launch at entry)
    int pdl_allowed = 1;                 // chaining may be picked by the tuner (TRANS_PDL=0 forbids it)
    int sweep_exec_pdl = -1;             // chaining the sweep graph was captured with
    int sweep_exec_mode = -1;            // schedule (0 or 5) the sweep graph was captured with
    int sweep_wpc = 0;                   // SWEEP_WPC: warp-per-component thread mapping (0: lane-major)
    int sweep_exec_wpc = -1;             // mapping the sweep graph was captured with
    int sweep_pf = 0;                    // L2 prefetch distance of the hyperplane launches (0 = none)
    int sweep_exec_pf = -1;              // prefetch distance the sweep graph was captured with
    int sweep_cta = 0;                   // CTA size of the mixed path's hyperplane launches (0 = default)
    int sweep_exec_cta = -1;             // CTA size the sweep graph was captured with
    int sweep_lanes = 1;                 // DeltaQ components swept: 1 = all, 2 = k and omega only (Runge-Kutta)
    SweepSync* d_sync = nullptr;
    SweepSync* h_sync = nullptr;         // pinned
    unsigned spin_limit = SWEEP_SPIN_LIMIT;   // polls of one device-side wait before it gives up
    std::string sweep_tuning;
    // ---- instrumentation ----
    bool ktime_on = false;
    struct KEv { int k, n; cudaEvent_t a, b; };
    std::vector<KEv> kev;
};

int fail(Ctx* c, int code, const std::string& msg);
const char* stateless_error();          // message of the last failed context-free call on this thread

#define CK(call)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) return fail(c, TRANS_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// times the launches issued in its lifetime as kernel class k (n launches) when enabled
struct KScope {
    Ctx* c; int k, n; cudaEvent_t a = nullptr, b = nullptr;
    KScope(Ctx* c_, int k_, int n_ = 1);
    ~KScope();
};

bool params_supported(const trans_params* p);
int validate_case(const trans_params* p, int nblocks, const trans_block* blocks);
int ctx_init(Ctx* c, int precision, long long budget);
void ctx_free(Ctx* c);
long long case_bytes(const trans_params* p, int nblocks, const trans_block* blocks);
// sub-iterations of one outer iteration: 3 SSP-RK3 stages, Kchld dual-time steps or 1 (main.F90:54-56)
inline int sub_iterations(const trans_params& p) { return p.IF_RK == 1 ? 3 : (p.Kind_Dual != 0 ? p.Kchld : 1); }
// slots per padded cell of a case's blocks (Runge-Kutta cases keep the stage-1 state as well)
inline int case_slots(const trans_params& p) { return p.IF_RK == 1 ? NSLOT_RK : NSLOT; }
int case_add(Ctx* c, const trans_params* p, int nblocks, const trans_block* blocks, CaseRec** out);
int case_remove(Ctx* c, int id);
CaseRec* case_find(Ctx* c, int id);
int rebuild(Ctx* c);
int build_tiles(Ctx* c, int TI, int TJ, int TK);   // tiles of the tiled-wavefront sweep schedule
void free_worklists(Ctx* c);
// one Fortran array in or out; sync = false leaves the copy in flight (the caller synchronises
// the stream before it reuses the array)
int field_io(Ctx* c, CaseRec* cs, int ib, int f, double* host, bool upload, bool sync = true);
// n arrays in or out with one synchronisation at the end
int fields_io(Ctx* c, CaseRec* cs, int n, const int* ib, const int* f, double* const* host, bool upload);
int run_stage(Ctx* c, int stage, int itr);
int upload_cdev(Ctx* c);
// integrated quantities of one case from its current state (k_integrals.cu kernels)
int integrals(Ctx* c, CaseRec* cs, trans_integrals* out);
int all_integrals(Ctx* c, std::vector<trans_integrals>& out);     // every case, in c->cases order
// Cp of each face of a wall segment, or (forces) its pressure and viscous force, 6 per face
int wall_cp(Ctx* c, CaseRec* cs, int ib, int iconn, double* cp, bool forces = false);
// the words of a cross-rank 1-to-1 segment out of (pack) or into (unpack) the context
int halo_io(Ctx* c, CaseRec* cs, int sweep, int ib, int iconn, const trans_conn* partner, double* buf, bool pack);
int block_index(const CaseRec* cs, int id);
// Geom/startup.F90:1-25: the target face cell of a 1-to-1 interface's local face cell
void ijk_start_end(int I, int J, int K, int& Is, int& Js, int& Ks, const int* TL, const int* TT, int lcross);
int finalize_geometry(Ctx* c);
int reduce_norms(Ctx* c);
int run_iteration(Ctx* c);               // one outer iteration of every case at its KI
// n outer iterations of every case, the first at each case's KI, KI advancing by one; whole
// iterations are replayed as one CUDA graph where the cases' switches stay fixed
int run_iterations(Ctx* c, int n);
// everything an iteration needs before it runs, without running one: work lists, geometry
// terms, the sweep schedule (tuned on a right-hand side of the current state) and the
// iteration graph.  The state (interior cells) is unchanged.
int prepare(Ctx* c);
int kernel_times(Ctx* c, double* ms, int* launches);

}  // namespace eng
}  // namespace tg
