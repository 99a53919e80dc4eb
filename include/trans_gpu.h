/*
 * trans_gpu.h -- C ABI of the GB300 implementation of the TRANS per-iteration hot path.
 *
 * The reference (TRANS, Fortran 90) has no plugin API: its hot path is a set of argument-less
 * subroutines that act on the block selected by GLOBAL_SetPointers(iBlock)
 * (Module_Global.F90:274-392) and read module globals.  This header replaces that driver loop
 * body (main.F90:54-197) and the subroutine calls inside it with plain C entry points that a
 * Fortran caller binds through ISO_C_BINDING (BIND(C) interfaces over these prototypes):
 *
 *   trans_create            replaces the per-block allocation of Input/Read_BlockDimensions.F90:306-478
 *                           and takes the connectivity built by Input/PLOT3DReadInit.F90:123-348
 *   trans_set_field         takes one Fortran array of the block (geometry from Geom/CalcDst.F90 +
 *                           Geom/startup.F90:396-755, state from Input/Init.F90) in its allocated layout
 *   trans_get_field         returns one Fortran array in the same layout (Output/OUTPUT_SaveField.F90:8-32
 *                           writes V and Rmiu from it)
 *   trans_iterate           one outer iteration = main.F90:54-171 (+ :192-197 TIME_Update_U)
 *   trans_run_stage         one hot-path subroutine over all blocks, for subroutine-granular drop-in
 *   trans_get_norms         per-block DRSa/DUa/DRSk/DRSo of Time/TIME_Update_V.F90:106-294
 *   trans_destroy
 *
 * Conventions
 *   - All arrays are FP64 in Fortran column-major order, exactly as allocated by the reference
 *     (Input/Read_BlockDimensions.F90:306-478); the lower bounds are listed per field below.
 *   - Return value 0 = OK, negative = error (see TRANS_E_*).  The library never aborts or exits.
 *   - A context owns one CUDA stream; calls on one context are not re-entrant.
 *   - Node counts NI,NJ,NK follow the reference (cells are 1..NI-1 etc., 3 ghost layers per side).
 */
#ifndef TRANS_GPU_H
#define TRANS_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define TRANS_OK 0
#define TRANS_E_ARG (-1)        /* invalid argument or unsupported option                 */
#define TRANS_E_CUDA (-2)       /* CUDA runtime error                                      */
#define TRANS_E_NAN (-3)        /* NaN in the density increment (TIME_Update_V.F90:124-131) */
#define TRANS_E_TIMEOUT (-4)    /* a bounded device-side wait expired                      */
#define TRANS_E_MEMORY (-5)     /* device memory budget exhausted                          */

/* Precision modes */
#define TRANS_FP64 0            /* all-FP64 path, drop-in for the reference subroutines    */
#define TRANS_MIXED 1           /* FP32 reconstruction/flux/SST/sweeps, FP64 update/metrics
                                   (not with Kind_Roe = 2, the rotated Roe scheme)          */

/*
 * Module globals read by the hot path (Module_Global.F90:39-148), with the values they hold
 * after INPUT_ReadOrg, ParameterSet and NonDimensionlization (Input/ReadOrg.F90:12-62,
 * Input/ParameterSet.F90:1-96).
 */
typedef struct trans_params {
    double XM, RXM2, PPF, Csthlnd, Csth1, Ref, Tiny;
    double VxF, VyF, VzF;
    double omega[3];
    double P0in, T0in, Pouthub;
    double VisRatio, FSTI, Rkf, Rof, Rmiuf;
    double A1, Beta_star, Sigk1, Sigo1, Beta1, Gama1, Sigk2, Sigo2, Beta2, Gama2;
    double Prod_Lmt;
    double F_limiter1, F_limiter2, gama_max, gama_min;
    double DT_LUSGS_Main, DT_LUSGS_Sub, CFL_Main, CFL_Sub_start, CFL_Sub_end;
    double Trans_location, Alscale;
    int CFL_Sub_step, IF_Local_Main, IF_Local_Sub;
    int Kind_Spatial, Kind_Roe, Kind_Model, Kind_Hybrid, Kind_SubHY;
    int Kind_Dual, Kchld, IF_RK;
    int IF_Euler, IF_Turb_org, KItm, IF_Comppress, IF_Precondition, Kind_RotMod;
    int If_fix_Transition, KI_ini;
    int precision;                 /* TRANS_FP64 or TRANS_MIXED (not a reference global) */
    int pad_;
} trans_params;

/*
 * One entry of AConnectivity (Module_Block.F90:4-23) after PLOT3D_Read_And_Init
 * (Input/PLOT3DReadInit.F90:135-348).  Index fields keep the reference's 1-based values.
 */
typedef struct trans_conn {
    int BCType, SubBCType, PerType, lcross;
    int pointStart[3], pointEnd[3];
    int IJKDirect, LeftOrRight;
    int IJKAdd[3], CIJKAdd[3], CIJKAdd1[3], CIJKAdd2[3];
    int CEIJKAdd[3], CEIJKAdd1[3], CEIJKAdd2[3];
    int Transform[3], TransformT[3], revMatrix[3];
    int TargetBlock, TargetConn;       /* global block id (1-based), segment index (1-based) */
    double rotateAngle;                /* rotateAngle(1) */
} trans_conn;

/*
 * One block.  ni,nj,nk are node counts (Block%NI etc.), id = NBlockGlobal.  The six MARKWALL
 * arrays (Input/Read_BlockDimensions.F90:146-283) are Fortran arrays MARKWALLi0(NJ1,NK1),
 * MARKWALLim(NJ1,NK1), MARKWALLj0(NI1,NK1), MARKWALLjm(NI1,NK1), MARKWALLk0(NI1,NJ1),
 * MARKWALLkm(NI1,NJ1); NULL means all zero.
 */
typedef struct trans_block {
    int ni, nj, nk, id;
    int nconn, pad_;
    const trans_conn* conn;
    const int* markwall[6];
} trans_block;

/* Per-block residual norms of TIME_Update_V (Time/TIME_Update_V.F90:106-294, 892-908). */
typedef struct trans_norms {
    double DRSa, DUa, DRSk, DUk, DRSo, DUo;
    int Ima, Jma, Kma, nan_flag;
} trans_norms;

/*
 * Integrated quantities of one case's current state (trans_get_integrals), summed on the device
 * over every face of its inlet (kind 5), outlet (kind 7) and wall (kind 1) segments.  Mass flow
 * and momentum follow Output/OUTPUT_Residual_NS.F90:37-75 (face value = volume-weighted average
 * of the two cells with the weights crossed, dotted with SD of the face); total pressure
 * p (1 + 0.2 M^2)^3.5 follows Output/Average_Field.F90:66,157; the wall forces follow
 * Output/OUTPUT_ClCdCm.F90:114-264 before its 2/Area_Ref scaling.  Nondimensional units.
 */
typedef struct trans_integrals {
    double mass_in, p0_in, p_in;     /* inlet faces: mass flow into the domain; mass-averaged p0 and p */
    double mass_out, p0_out, p_out;  /* outlet faces: mass flow out of the domain; mass-averaged p0 and p */
    double loss;                     /* (p0_in - p0_out) / (p0_in - p_in); 0 when p0_in == p_in */
    double force_p[3];               /* wall faces: sum of (PP - PPF) SD Sgn, Sgn = -1 on min faces   */
    double force_v[3];               /* wall faces: sum of mu_w/(Dst Ref) (u |S| - (u.S) S/|S|)       */
} trans_integrals;

/*
 * Field ids for trans_set_field / trans_get_field, with the Fortran allocation each pointer
 * must have (Input/Read_BlockDimensions.F90:306-478; NIp2 = NI+2):
 */
enum trans_field {
    TRANS_V = 0,      /* V(7,-2:NIp2,-2:NJp2,-2:NKp2)          conserved variables            */
    TRANS_PP = 1,     /* PP(-2:NIp2,-2:NJp2,-2:NKp2)           pressure                       */
    TRANS_T = 2,      /* T(-2:NIp2,-2:NJp2,-2:NKp2)            temperature                    */
    TRANS_RMIU = 3,   /* Rmiu(-2:NIp2,-2:NJp2,-2:NKp2)         eddy viscosity                 */
    TRANS_WT0 = 4,    /* Wt0(7,NIp2,NJp2,NKp2)                 time level n                   */
    TRANS_WT1 = 5,    /* Wt1(7,NIp2,NJp2,NKp2)                 time level n-1                 */
    TRANS_SD = 6,     /* SD(3,3,-2:NIp2,-2:NJp2,-2:NKp2)       face area vectors (dir,comp)   */
    TRANS_GRAD = 7,   /* Grad(3,-2:NIp2,-2:NJp2,-2:NKp2)       face areas                     */
    TRANS_VOL = 8,    /* Vol(-2:NIp2,-2:NJp2,-2:NKp2)                                         */
    TRANS_ALAGM = 9,  /* Alagm(3,-2:NIp2,-2:NJp2,-2:NKp2)      face-centre spacing            */
    TRANS_DST = 10,   /* Dst(-2:NIp2,-2:NJp2,-2:NKp2)          wall distance                  */
    TRANS_ALENG = 11, /* ALeng(-2:NIp2,-2:NJp2,-2:NKp2)        DES length scale               */
    TRANS_ASENG = 12, /* ASeng(NIp2,NJp2,NKp2)                                                */
    TRANS_XC = 13,    /* Xc(0:NIp2,0:NJp2,0:NKp2)                                             */
    TRANS_YC = 14,    /* Yc(0:NIp2,0:NJp2,0:NKp2)                                             */
    TRANS_ZC = 15,    /* Zc(0:NIp2,0:NJp2,0:NKp2)                                             */
    TRANS_RAD = 16,   /* rad(-2:NIp2,-2:NJp2,-2:NKp2)                                         */
    TRANS_THTC = 17,  /* thtc(-2:NIp2,-2:NJp2,-2:NKp2)                                        */
    /* work arrays, readable for subroutine-granular parity */
    TRANS_D = 18,     /* D(7,0:NIp2,0:NJp2,0:NKp2)             residual / increment           */
    TRANS_RDS = 19,   /* Rds(3,0:NIp2,0:NJp2,0:NKp2)           spectral radii                 */
    TRANS_DTM = 20,   /* Dtm(NIp2,NJp2,NKp2)                   local time step                */
    TRANS_DQDXYZ = 21,/* DQdxyz(18,-1:NIp2,-1:NJp2,-1:NKp2)    cell gradients                 */
    TRANS_SHOCK = 22, /* shock(-2:NIp2,-2:NJp2,-2:NKp2)        shock sensor                   */
    TRANS_WT2 = 23,   /* Wt2(7,NIp2,NJp2,NKp2)                 Runge-Kutta stage-1 state      */
                      /*   (IF_RK = 1 cases only; Time/TIME_RK_Save.F90:16-28)                */
    TRANS_NFIELDS = 24
};

/* Hot-path stages for trans_run_stage (each acts on all blocks, as main.F90 does).  With
 * IF_RK = 1 an outer iteration has 3 sub-iterations (the SSP-RK3 stages, main.F90:54-56) and
 * two stages change meaning (main.F90:152-161):
 *   TRANS_STAGE_LUSGS  = TIME_RK_Save (stage 1) + TIME_RK + TURBTWO_TIME_LUSGS_SST
 *   TRANS_STAGE_UPDATE = TIME_RK_V_Update_New
 * (Time/TIME_RK_Save.F90:16-28, Time/TIME_RK.F90:27-86, Time/TIME_RK_V_Update_New.F90:66-320). */
enum trans_stage {
    TRANS_STAGE_SPECRAD = 0,   /* TIME_SpectralRadius                         main.F90:66-69   */
    TRANS_STAGE_BC_STATE = 1,  /* BC_Boundarys(-1) (+ PARALLEL_BCs(-1))       main.F90:72-73   */
    TRANS_STAGE_GRADIENT = 2,  /* SPACEINTERP + DIFF_DqDxyz                   main.F90:74-83   */
    TRANS_STAGE_BC_GRAD = 3,   /* BC_Boundarys(0) (+ PARALLEL_BCs(0))         main.F90:84-85   */
    TRANS_STAGE_RESIDUAL = 4,  /* D=0, diffusion, reconstruction, fluxes      main.F90:92-133  */
    TRANS_STAGE_LUSGS = 5,     /* TIME_LUSGS + TURBTWO_TIME_LUSGS_SST         main.F90:139-142 */
    TRANS_STAGE_UPDATE = 6,    /* TIME_Update_V                               main.F90:143     */
    TRANS_STAGE_UPDATE_U = 7,  /* TIME_Update_U                               main.F90:192-197 */
    TRANS_NSTAGES = 8
};

int trans_create(const trans_params* p, int nblocks, const trans_block* blocks, void** ctx);
int trans_destroy(void* ctx);         /* NULL is a no-op returning TRANS_OK */
/* trans_set_field returns once the caller's array has been copied (it may be reused at once); the
 * transpose into the device layout completes in order before any later call's device work. */
int trans_set_field(void* ctx, int ib, int field, const double* fortran_array);
/* n trans_set_field / trans_get_field calls in one, (ib[q], field[q], arrays[q]) for q < n,
 * with one synchronisation at the end: trans_set_fields returns once every array is copied,
 * trans_get_fields once every array is filled.  Page-locked arrays (cudaHostAlloc,
 * cudaHostRegister) are transposed in place over the host link, others through a device
 * staging buffer; either way the layout is the Fortran one above. */
int trans_set_fields(void* ctx, int n, const int* ib, const int* field, const double* const* arrays);
int trans_get_fields(void* ctx, int n, const int* ib, const int* field, double* const* arrays);
int trans_get_field(void* ctx, int ib, int field, double* fortran_array);
/* One outer iteration KI (main.F90:48-197).  norms: array of nblocks entries, may be NULL. */
int trans_iterate(void* ctx, int ki, trans_norms* norms);
/* One stage of one sub-iteration for all blocks; itr_chld is the sub-iteration index (1-based). */
int trans_run_stage(void* ctx, int stage, int ki, int itr_chld);
int trans_get_norms(void* ctx, trans_norms* norms);
/* Prepares the context for iteration KI (KI < 0: each case's next iteration) without running it
 * (no reference counterpart): builds
 * the work lists and geometry terms, tunes the LU-SGS sweep schedule on a right-hand side of
 * the current state and captures the iteration graph that trans_time_iterations and
 * trans_batch_iterate replay (8 outer iterations per replay).  The interior state is unchanged. */
int trans_prepare(void* ctx, int ki);
/* One outer iteration with CUDA events around every stage on the context's stream; ms receives
 * TRANS_NSTAGES elapsed times (no reference counterpart: instrumentation). */
int trans_stage_times(void* ctx, int ki, double* ms);
/* Measured fused multiply-add throughput of the FP64 (fp64=1) or FP32 pipe in GFLOP/s (no
 * reference counterpart: the compute roof the FP64 kernels are reported against). */
double trans_probe_fma_gflops(int fp64);
/* Measured time in microseconds of one dependent step of a chain of launches of `grid` CTAs (each
 * thread reads through L2 what the previous launch wrote, then writes), replayed as a CUDA
 * graph, with programmatic dependent launch when `chained` (no reference counterpart: the
 * latency floor the per-hyperplane sweep launches are reported against). */
double trans_probe_chain_us(int chained, int grid);
/* n outer iterations KI = ki_first.. timed with CUDA events on the context's stream (ms: total).
 * norms as for trans_iterate (last iteration).  No reference counterpart: benchmarking. */
int trans_time_iterations(void* ctx, int ki_first, int n, double* ms, trans_norms* norms);
int trans_sync(void* ctx);
/*
 * Cross-rank 1-to-1 interfaces (BC/PARALLEL_BC_P2P.F90:1-257, PARALLEL_BC_sendrecv_blk, as
 * Common/PARALLEL_Funcs.F90:57-87 calls it after BC_Boundarys): a kind-9 connection whose target
 * block is not in the context is left out of the context's boundary pass; the caller exchanges
 * it after TRANS_STAGE_BC_STATE (sweep -1) and TRANS_STAGE_BC_GRAD (sweep 0).
 * trans_halo_pack writes segment iconn of block ib's words into buf (host memory), face cells in
 * the segment's K, J, I order: sweep -1 36 words per face cell (layer 0: V(1:7), PP, T, Rmiu,
 * Rds(1:3), shock; layers 1 and 2: V(1:7), PP, T, Rmiu, shock), sweep 0 18 (DqDxyz of layer 0),
 * in FP64 (the reference sends MPI_REAL).  trans_halo_unpack fills the segment's ghost layers
 * from the partner segment's words (partner = the target block's connection TargetConn) through
 * the same index transform and rotation as the same-rank copy, so a split case iterates as the
 * whole case does.  Synchronous; TRANS_E_ARG for a connection that is not of kind 9.
 */
int trans_halo_pack(void* ctx, int sweep, int ib, int iconn, double* buf);
int trans_halo_unpack(void* ctx, int sweep, int ib, int iconn, const trans_conn* partner, const double* buf);
/* Integrated quantities of the current state (after the last iteration's update; ghost cells
 * as the last boundary pass left them, as the reference's output routines see them). */
int trans_get_integrals(void* ctx, trans_integrals* out);
/* Pressure coefficient 2 (PP - PPF) of the wall cells of wall segment iconn (1-based, a kind-1
 * connection) of block ib (Output/OUTPUT_Surfaces.F90:303-305): one value per face of the
 * segment, I fastest, then J, then K, over pointStart..pointEnd of the segment's face indices. */
int trans_get_wall_cp(void* ctx, int ib, int iconn, double* cp);
/* Pressure and viscous force of each face of wall segment iconn of block ib, the per-face terms
 * of the force and moment sums of Output/OUTPUT_ClCdCm.F90:199-264 (before its 2/Area_Ref
 * scaling): forces[6r .. 6r+5] = pressure x, y, z and viscous x, y, z of face r, the faces in
 * the order of trans_get_wall_cp.  The moment sums (:250-252) weight them with the face centres,
 * the mean of the face's four nodes, which the caller holds. */
int trans_get_wall_forces(void* ctx, int ib, int iconn, double* forces);
/*
 * Wall distance of GEOM_CalcDST (Geom/CalcDst.F90:127-164) on the device, for any set of points
 * (no context).  xyz: n points, x y z interleaved (the cell centres Xc, Yc, Zc of the interior
 * cells).  nsurf wall surfaces (AllSurfs): dims[2s], dims[2s+1] = NSur, MSur nodes of surface s;
 * nodes: for each surface in turn, its X(NSur,MSur), then Y, then Z, Fortran order.  dst[q] =
 * sqrt of the minimum over the panels of the reference's DDD, the surfaces combined in order
 * with the reference's tiny floor: bit-identical to the reference's loop.  Allocates and frees
 * its own device memory and stream; call with the wanted device current.  Errors:
 * TRANS_E_ARG (non-finite coordinates, bad sizes), TRANS_E_CUDA; message in
 * trans_last_error(NULL).
 */
int trans_wall_distance(long long n, const double* xyz, int nsurf, const int* dims, const double* nodes,
                        double tiny, double* dst);
/*
 * GEOM_CalcDST (Geom/CalcDst.F90:95-521) of one block on the device (no context): from the
 * block's nodes (xyz: X(ni,nj,nk), then Y, then Z, Fortran order) and the wall surfaces (as for
 * trans_wall_distance), the cell centres Xc/Yc/Zc with the boundary face centres in the first
 * ghost layer, thtc and rad, the wall distance Dst, SD and Grad of every face (face 0 = face 1),
 * Alagm, aLeng/aSeng and Vol of every interior cell.  out: 24 arrays of (ni+5)(nj+5)(nk+5)
 * doubles (index -2..n+2 per direction, i fastest), zero where not computed, in the order Xc,
 * Yc, Zc, Dst, aLeng, aSeng, Vol, rad, thtc, SD(dir 1..3, comp 1..3), Grad(1..3),
 * Alagm(1..3).  The corner centres and ghost copies of :530-640 are left to the caller.  Every
 * value equals a CPU evaluation of the reference's expressions (no contraction).
 * TRANS_E_ARG for a negative volume (message in trans_last_error(NULL)).
 */
int trans_block_metrics(int ni, int nj, int nk, const double* xyz, int nsurf, const int* dims, const double* nodes,
                        double tiny, double* out);
/* Device bytes held by the context. */
long long trans_device_bytes(void* ctx);
/* Kernel launches issued since the context was created (all kernels of this library). */
long long trans_kernel_launches(void* ctx);
/*
 * Batches (no reference counterpart: the batching and serving layer).  A batch context holds
 * independent cases -- each with its own blocks, module globals, iteration counter and norms --
 * that are advanced together: every kernel launch covers the blocks of all cases.  Cases are
 * added and removed while the context runs (continuous batching); a case is admitted only if
 * its device bytes fit the context's budget (TRANS_E_MEMORY otherwise, nothing allocated).
 * All cases of one context share the precision mode, the time integrator (IF_RK) and the
 * sub-iteration count (Kchld).
 * A case's KI starts at its KI_ini and advances by one per trans_batch_iterate step, so its
 * results do not depend on which other cases share the context.
 */
int trans_batch_create(int precision, long long device_budget_bytes /* 0 = no limit */, void** ctx);
/* Device bytes a case would take in a batch context (-1: the case is not supported). */
long long trans_batch_case_bytes(const trans_params* p, int nblocks, const trans_block* blocks);
int trans_batch_add(void* ctx, const trans_params* p, int nblocks, const trans_block* blocks, int* case_id);
int trans_batch_remove(void* ctx, int case_id);
/* As trans_set_field / trans_get_field for block ib of one case. */
int trans_batch_set_field(void* ctx, int case_id, int ib, int field, const double* fortran_array);
int trans_batch_get_field(void* ctx, int case_id, int ib, int field, double* fortran_array);
int trans_batch_set_fields(void* ctx, int case_id, int n, const int* ib, const int* field, const double* const* arrays);
int trans_batch_get_fields(void* ctx, int case_id, int n, const int* ib, const int* field, double* const* arrays);
/* n outer iterations of every case.  TRANS_E_NAN: some case produced a NaN (its norms carry
 * nan_flag); the iteration is complete and the caller removes that case. */
int trans_batch_iterate(void* ctx, int n);
/* trans_batch_iterate timed with CUDA events on the context's stream (ms: total). */
int trans_batch_time_iterations(void* ctx, int n, double* ms);
/* Iterations done by a case, its per-block norms of its first and of its last iteration
 * (arrays of nblocks entries, either may be NULL). */
int trans_batch_case_norms(void* ctx, int case_id, int* iterations, trans_norms* first, trans_norms* last);
long long trans_batch_bytes_in_use(void* ctx);
/* As trans_get_integrals / trans_get_wall_cp for one case; one launch covers all cases, so a
 * serving loop reads every case's integrals at once with trans_batch_integrals (ids[k] and
 * out[k] for the first n cases in trans_batch_cases order; returns the number written). */
int trans_batch_get_integrals(void* ctx, int case_id, trans_integrals* out);
int trans_batch_integrals(void* ctx, int* ids, trans_integrals* out, int n);
int trans_batch_get_wall_cp(void* ctx, int case_id, int ib, int iconn, double* cp);
/* Number of cases; their ids in ids[0..max-1]. */
int trans_batch_cases(void* ctx, int* ids, int max);

/*
 * TIME_Update_V (Time/TIME_Update_V.F90:91-908) over all blocks, as trans_run_stage(ctx,
 * TRANS_STAGE_UPDATE, ki, ...), but with the per-tile residual-norm partials kept in a fixed
 * 4 MiB buffer that is part of the library image instead of the context's own buffer.  No
 * counterpart in the reference.  It is for callers that cannot allocate device memory at this
 * point -- for instance a serving loop that has committed its whole device-memory budget to
 * resident solves -- and it allocates nothing: no cudaMalloc, no page-locked host memory, no
 * allocating library routine.  The context must already be built (by trans_prepare,
 * trans_run_stage or trans_iterate), because building it allocates its work lists: an
 * unbuilt context gets TRANS_E_ARG and nothing is allocated.
 * Limit: 65536 cell tiles (16,777,216 interior cells per context); larger contexts get
 * TRANS_E_ARG with a message in trans_last_error.  Call it with the context's device current.
 * The first call on a device looks the buffer up (cudaGetSymbolAddress, which may load the
 * library's device code on that device) and should come before any stream capture.  The
 * buffer is shared by every context and call on a device and keeps the last call's contents;
 * concurrent calls race on it and must be serialised by the caller.  norms: nblocks entries,
 * may be NULL.  TRANS_E_TIMEOUT when the LU-SGS sweep of this iteration gave up on a bounded
 * device-side wait, as the UPDATE stage reports it.  Runge-Kutta contexts (IF_RK = 1), whose
 * update is TIME_RK_V_Update_New, get TRANS_E_ARG.
 */
int trans_update_static_scratch(void* ctx, int ki, trans_norms* norms);
/* One outer iteration KI with CUDA events around every kernel launch on the context's stream:
 * ms[k] and launches[k] per kernel class k (n >= TRANS_NKCLASS entries); names from
 * trans_kernel_class(k).  No reference counterpart: instrumentation. */
#define TRANS_NKCLASS 17
int trans_kernel_times(void* ctx, int ki, double* ms, int* launches, int n);
const char* trans_kernel_class(int k);
/* The schedule the context's tuner picked for the LU-SGS sweeps and what it measured (no
 * reference counterpart).  The string lives until the next call on this thread. */
const char* trans_tuning(void* ctx);
/* Diagnostic, no reference counterpart: checks on the current device the integer-pipe
 * double <-> float conversions the mixed-precision kernels use against the hardware
 * conversions, on n bit patterns (1..2^32) drawn from seed plus a fixed set of edge cases
 * (signed zeros, infinities, NaN, the float range limits, rounding ties).  mismatches[0]
 * counts double -> float results that differ in any bit, mismatches[1] float -> double (NaN
 * equals NaN); both are 0 on a correct build.  Errors: TRANS_E_ARG, TRANS_E_CUDA (message in
 * trans_last_error(NULL)). */
int trans_check_conversions(long long n, unsigned long long seed, long long* mismatches);
/* Message of the last failed call on ctx; with ctx = NULL, of the last failed context-free call
 * (trans_wall_distance) on this thread. */
const char* trans_last_error(void* ctx);

#ifdef __cplusplus
}
#endif
#endif
