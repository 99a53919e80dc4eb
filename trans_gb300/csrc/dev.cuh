// dev.cuh -- device data layout and per-face / per-cell physics of the TRANS hot path.
//
// Layout: every block of every case lives in one device arena.  A block owns NSLOT scalar
// arrays ("slots") of ncell = PI*PJ*PK doubles each, i fastest, covering the full ghost extent
// -2..N+2 of the reference's arrays: PJ = NJ+5, PK = NK+5, and PI = NI+5 rounded up to a
// multiple of 4, so that every row of the FP32 copies starts on a 16-byte boundary and a slot
// range forms a 4-D tensor (i, j, k, slot) that the tensor-memory-access unit can tile.  The
// cells i >= NI+5 of a row are padding that no stencil reads.  Cell-centred and face-centred quantities
// share the index: face i of direction d is stored at cell i (the cell on its +d side).
//
// The physics functions below restate the reference's expressions operation by operation
// (same association, same divisions).  In the FP64 path they are compiled without fused
// multiply-add, so they reproduce a CPU evaluation of the same expressions bit for bit,
// except where a libm function (exp, tanh, pow) is evaluated.  They are templated on the
// arithmetic type R so that the mixed-precision path reuses them in FP32.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "tmath.cuh"

namespace tg {

enum Slot {
    S_V = 0,            // 7
    S_PP = 7, S_T = 8, S_RMIU = 9,
    S_WT0 = 10,         // 7
    S_WT1 = 17,         // 7
    S_SD = 24,          // 9: (dir-1)*3 + (comp-1)
    S_GRAD = 33,        // 3
    S_VOL = 36,
    S_ALAGM = 37,       // 3
    S_DST = 40, S_ALENG = 41, S_ASENG = 42,
    S_XC = 43, S_YC = 44, S_ZC = 45,
    S_RAD = 46, S_THTC = 47, S_SINT = 48, S_COST = 49,
    S_AINV = 50,        // 3: 1/(Alagm(d,i)+Alagm(d,i-1)) on faces
    S_VINV = 53,        // 3: 1/(Vol(i)+Vol(i-1)) on faces
    S_ASD = 56,         // 9: 0.5*(SD(d,c,i)+SD(d,c,i+1)) per cell
    S_WALL = 65,        // 3: MARKWALL flag on faces
    S_D = 68,           // 7
    S_RDS = 75,         // 3
    S_DTM = 78, S_STEPT = 79, S_CVS = 80,
    S_DQ = 81,          // 18
    S_SHOCK = 99,
    S_FM = 100, S_FT = 101,
    S_PRIM = 102,       // 5: u, v, w, k/rho, omega/rho
    S_FX = 107,         // 39: face fluxes, (dir-1)*13 + m
    S_FC1 = 146,        // SST F1 per cell (for the DES length scale of the next cell)
    S_RINV = 147,       // 1/rho
    S_SVEL = 148,       // 3: rho*u * (1/rho) etc., the velocities of the LU-SGS Jacobians
    S_FSCH = 151,       // hybrid blend Fscheme of the rotated Roe scheme (Kind_Roe = 2)
    NSLOT = 152,
    // Runge-Kutta cases (IF_RK = 1) only: their blocks are allocated with NSLOT_RK slots
    S_WT2 = 152,        // 7: the stage-1 state of the SSP-RK3 stages
    NSLOT_RK = 159
};

// The DeltaQ-independent parts of A(Q)*DeltaQ (Time/TIME_LUSGS.F90:696-768) of one cell and
// one direction:
//   row L of A*dQ = AinRo*c[L][0] + AinRx*c[L][1] + AinRy*c[L][2] + AinRz*c[L][3] + AinRe*c[L][4]
// row 0 is the unit normal (0, aSDx, aSDy, aSDz, 0); rows 1..3 are stored whole; row 4 keeps
// (AinRo*VP)*GEt1 as two factors; VPT is the contravariant speed of the k-omega sweep.
enum JacTerm { JC_R0 = 0, JC_R1 = 3, JC_R2 = 8, JC_R3 = 13, JC_VP = 18, JC_GET1 = 19, JC_R4 = 20, JC_VPT = 24, NJAC = 25 };

// Per-cell record of the sweeps, in sweep (hyperplane) order: the Jacobian terms and spectral
// radii of the three lower (L sweep) and three upper (U sweep) neighbours, and the cell's own
// diagonal terms.
// Neighbour k (0..2 lower i,j,k; 3..5 upper) occupies NBREC entries from NBREC*k: its NJAC
// Jacobian terms, then its spectral radius in that direction.
enum SweepRec { NBREC = NJAC + 1, REC_STEPT = 6 * NBREC, REC_CVS = REC_STEPT + 1, REC_FM = REC_STEPT + 2,
                REC_FT = REC_STEPT + 3, NREC = REC_STEPT + 4 };
// The mixed path's (FP32) record is compact: per sweep position the cell's own values from
// which its neighbours rebuild the Jacobian rows, and its diagonal terms, as float4 groups:
// direction d (0..2): face-averaged metric s = 0.5 (SD(d,c) + SD(d,c+1)) and Rds(d); then the
// velocity and total enthalpy H = |v|^2/2 + gamma p/(rho (gamma-1)); then stept, cvs, 1/fm, 1/ft.
enum CompactRec { CR_DIR = 0, CR_VEL = 12, CR_DIAG = 16, NCREC = 20 };
constexpr int DQ_STRIDE = 8;     // DeltaQ of one sweep position: 7 components + 1 pad
// Sweep-order arrays keep the entries of one position together (element m of position q at
// q*width + m): a hyperplane is one contiguous range, and one cell's record spans a few lines.
__host__ __device__ inline size_t sw_at(long long q, int m, int width) {
    return (size_t)q * (size_t)width + (size_t)m;
}

// face-flux components (per face and direction)
enum FX { FX_VX = 0, FX_VY = 1, FX_VZ = 2, FX_VE = 3, FX_TK = 4, FX_TO = 5,
          FX_C0 = 6, FX_CK = 11, FX_CO = 12, NFX = 13 };

struct DevBlock {
    int NI, NJ, NK, NI1, NJ1, NK1, PI, PJ, PK;
    int ncell;            // PI*PJ*PK
    int nint;             // NI1*NJ1*NK1
    int cs;               // case slot: index of the block's case in the CaseDev array
    double* base;
    float* fbase;         // FP32 copies of the slots read by the FP32 kernels (mixed mode only)
};

constexpr int CELL_TILE = 256;   // interior cells per cell tile (and threads per CTA of the cell kernels)
constexpr int SWEEP_LANES = 8;   // threads per cell in the LU-SGS sweeps (one per DeltaQ component)
constexpr int SWEEP_WPC = 16;    // `lanes` bit of the sweep kernels: warp-per-component thread mapping
// threads a sweep launch needs for n positions
__host__ __device__ inline int sweep_items(int n, int lanes) {
    return (lanes & SWEEP_WPC) ? ((n + 31) / 32) * (32 * SWEEP_LANES) : n * SWEEP_LANES;
}

struct MirrorList {       // slot ranges [first, first+count) copied FP64 -> FP32 (or back if to_fp64)
    int n, to_fp64, first[6], count[6];
};

struct Tile {             // a run of consecutive interior cells (or faces) of one block
    int blk, start, count, pad_;
};

// one page-locked Fortran-layout array of a field transfer and its slots (k_fields_xfer)
struct XferEntry {
    double* base;                 // the block's slot arena
    double* host;                 // device address of the page-locked array
    long long off;                // first chunk within the batch
    long long count;              // elements of the array
    int ncell, PI, PJ, ei, ej, slot0, ncomp, lb, is_sd, pad_;
};
constexpr int XFER_CHUNK = 4;     // consecutive elements per thread
constexpr int XFER_MAX = 56;      // entries per launch (the batch stays under 4 KB of kernel parameters)
struct XferBatch {
    XferEntry e[XFER_MAX];
    int n, pad_;
};

struct ResidTile {        // a brick of cells of one block (array indices of its first cell)
    int blk, x0, y0, z0;
};

#define TG_PARAM_REALS(X) X(XM) X(RXM2) X(PPF) X(Csthlnd) X(Csth1) X(Ref) X(Tiny) X(VxF) X(VyF) X(VzF) \
    X(omega0) X(P0in) X(T0in) X(Pouthub) X(VisRatio) X(FSTI) X(A1) X(Beta_star) X(Sigk1) X(Sigo1)    \
    X(Beta1) X(Gama1) X(Sigk2) X(Sigo2) X(Beta2) X(Gama2) X(Prod_Lmt) X(gama_max) X(gama_min) X(F_limiter1) X(F_limiter2) X(Alscale)        \
    X(DT_LUSGS_Main) X(DT_LUSGS_Sub) X(CFL_Main) X(Trans_location)

template <typename R>
struct ParamsT {          // module globals the kernels read (trans_params + derived), in type R
#define TG_DECL(n) R n;
    TG_PARAM_REALS(TG_DECL)
#undef TG_DECL
    int Kind_Spatial, Kind_Roe, Kind_Hybrid, Kind_SubHY, Kind_Dual, IF_Local_Main, IF_Local_Sub;
    int IF_Comppress, If_fix_Transition, Kind_Model, IF_Precondition, Kind_RotMod;
};
using Params = ParamsT<double>;

template <typename R>
inline ParamsT<R> params_as(const Params& p) {
    ParamsT<R> q;
#define TG_CONV(n) q.n = (R)p.n;
    TG_PARAM_REALS(TG_CONV)
#undef TG_CONV
    q.Kind_Spatial = p.Kind_Spatial; q.Kind_Roe = p.Kind_Roe; q.Kind_Hybrid = p.Kind_Hybrid;
    q.Kind_SubHY = p.Kind_SubHY; q.Kind_Dual = p.Kind_Dual; q.IF_Local_Main = p.IF_Local_Main;
    q.IF_Local_Sub = p.IF_Local_Sub; q.IF_Comppress = p.IF_Comppress; q.If_fix_Transition = p.If_fix_Transition;
    q.Kind_Model = p.Kind_Model; q.IF_Precondition = p.IF_Precondition; q.Kind_RotMod = p.Kind_RotMod;
    return q;
}

// One case of a batch as the kernels see it: its module globals (FP64 and FP32 copies) and the
// switches of the current sub-iteration (CFL ramp, turbulence on, turbulence update on).
struct CaseDev {
    Params p;
    ParamsT<float> pf;
    double CFL_sub;
    int turb, turb_upd;
};
template <typename R> __host__ __device__ inline const ParamsT<R>& cparams(const CaseDev& c);
template <> __host__ __device__ inline const ParamsT<double>& cparams<double>(const CaseDev& c) { return c.p; }
template <> __host__ __device__ inline const ParamsT<float>& cparams<float>(const CaseDev& c) { return c.pf; }

__host__ __device__ inline int cidx(const DevBlock& b, int i, int j, int k) {
    return (i + 2) + b.PI * ((j + 2) + b.PJ * (k + 2));
}
__device__ inline double* slot(const DevBlock& b, int s) { return b.base + (size_t)s * (size_t)b.ncell; }
// row pitch of a block of NI nodes in i (the ghost extent NI+5 rounded up to a multiple of 4)
__host__ __device__ inline int padded_pi(int ni) { return (ni + 5 + 3) & ~3; }

__device__ inline float* fslot(const DevBlock& b, int s) { return b.fbase + (size_t)s * (size_t)b.ncell; }
// slot s in the arithmetic type R: the FP64 arrays, or their FP32 copies in the mixed path
template <typename R> __device__ inline R* rs(const DevBlock& b, int s);
template <> __device__ inline double* rs<double>(const DevBlock& b, int s) { return slot(b, s); }
template <> __device__ inline float* rs<float>(const DevBlock& b, int s) { return fslot(b, s); }

// face average of a cell quantity at the face stored at cell cf (Space/SPACEINTERP_GetSurfCenterVars.F90)
template <typename R>
__device__ inline R favg(const R* q, const R* al, const R* ainv, int cf, int s) {
    return (al[cf] * q[cf - s] + al[cf - s] * q[cf]) * ainv[cf];
}

template <typename R> __device__ inline R dmax(R a, R b) { return (a < b) ? b : a; }   // std::max
template <typename R> __device__ inline R dmin(R a, R b) { return (b < a) ? b : a; }   // std::min
template <typename R> __device__ inline R sgn1(R b) { return b >= R(0) ? R(1) : R(-1); }
template <typename R> __device__ inline R sq(R x) { return x * x; }
template <typename R> __device__ inline R p15(R x) { return x * sqrt(x); }
// tanh: the bit-reproducible FP64 restatement, or the CUDA single-precision function
template <typename R> __device__ inline R ttanh(R x);
template <> __device__ inline double ttanh<double>(double x) { return tmx::tanh_(x); }
template <> __device__ inline float ttanh<float>(float x) { return tanhf(x); }

// atan: the bit-reproducible FP64 restatement, or the CUDA single-precision function
template <typename R> __device__ inline R tatan(R x);
template <> __device__ inline double tatan<double>(double x) { return tmx::atan_(x); }
template <> __device__ inline float tatan<float>(float x) { return atanf(x); }
// exp: the bit-reproducible FP64 restatement, or the CUDA single-precision function
template <typename R> __device__ inline R texp(R x);
template <> __device__ inline double texp<double>(double x) { return tmx::exp_(x); }
template <> __device__ inline float texp<float>(float x) { return expf(x); }
// x**2. of a Fortran real exponent: the product, the correctly rounded power; x**10.: the pow
// of tmath in FP64 (as the oracle), products in FP32
template <typename R> __device__ inline R pow2_real(R x) { return x * x; }
template <typename R> __device__ inline R pow10_real(R x);
template <> __device__ inline double pow10_real<double>(double x) { return tmx::pow_(x, 10.0); }
template <> __device__ inline float pow10_real<float>(float x) {
    const float x2 = x * x, x4 = x2 * x2;
    return x4 * x4 * x2;
}

// Sutherland viscosity (Time/SpectralRadius.F90:59 and every copy of it)
template <typename R> __device__ inline R mu_suth(const ParamsT<R>& p, R TT) {
    return (R(1.0) + R(p.Csthlnd)) / (TT * R(p.Csth1) + R(p.Csthlnd)) * p15(R(p.Csth1) * TT);
}
// the variant without Csth1 (Space/TURBTWO_DIFFUSION_Centered.F90:160)
template <typename R> __device__ inline R mu_suth_nocs(const ParamsT<R>& p, R TT) {
    return (R(1.0) + R(p.Csthlnd)) / (TT + R(p.Csthlnd)) * p15(TT);
}

// x**3. of a Fortran real exponent: the pow of tmath in FP64 (as the oracle), x*x*x in FP32
template <typename R> __device__ inline R cube_pow(R x);
template <> __device__ inline double cube_pow<double>(double x) { return tmx::pow_(x, 3.0); }
template <> __device__ inline float cube_pow<float>(float x) { return x * x * x; }

// x**2.0 of a Fortran real exponent (a base of either sign): the product, the correctly
// rounded power
template <typename R> __device__ inline R pow2r(R x) { return x * x; }

// Low-Mach preconditioning (IF_Precondition = 1), Common/UTIL_Precond_Funcs.F90.
// getPrecondPara (:6-32): the preconditioning parameter ubetac2 of one state
template <typename R>
__device__ inline R get_precond_para(const ParamsT<R>& p, R VM2, R AM2, R RR, R TT, R RMIUT, R ALAGMR) {
    const R K = R(3.0), Kc = R(1.0);
    R ubetac2 = dmin(dmax(VM2 / AM2, K * R(p.XM) * R(p.XM)), R(1.0));
    R RmiuL = mu_suth<R>(p, TT);
    R RmiuAll = RmiuL + RMIUT;
    return dmax(ubetac2, Kc * pow2r(RmiuAll / RR / R(p.Ref) / ALAGMR) / AM2);
}

// The coefficients of PrecondDW (:90-127) for one state, each formed as the reference forms it:
// pVx, pVy, pVz, pE/1.4 - 1.2 |v|^2, a11, a15, b11, b15, pRo, pTT, and PPF
constexpr int NPC = 11;

template <typename R>
__device__ inline void precond_terms(const ParamsT<R>& p, R pRo, R pVx, R pVy, R pVz, R pE, R AAc, R ubetac2, R pTT, R* t) {
    R pU2 = pVx * pVx + pVy * pVy + pVz * pVz;
    R rCp = R(1.4 / 0.4) * R(p.PPF) * pRo;
    t[0] = pVx; t[1] = pVy; t[2] = pVz;
    t[3] = pE / R(1.4) - R(1.2) * (pU2);
    t[4] = AAc * AAc * ubetac2;
    t[5] = R(-0.4) * ubetac2 / rCp;
    t[6] = R(1.0) * t[4] / rCp;
    t[7] = (R(1.0) + R(0.4) * ubetac2) / rCp;
    t[8] = pRo;
    t[9] = pTT;
    t[10] = R(p.PPF);
}

// PrecondDW applied to the increment A[0..4] with the coefficients t of precond_terms
template <typename R>
__device__ inline void precond_apply(R* A, const R* t) {
    R pUAU = t[0] * A[1] + t[1] * A[2] + t[2] * A[3];
    A[4] = A[4] - (pUAU) - (t[3]) * A[0];
    R AinP = t[4] * A[0] + t[5] * A[4];
    R AinT = t[6] * A[0] + t[7] * A[4];
    A[0] = AinP / t[10] / t[9] - t[8] * AinT / t[9];
    A[4] = AinP / R(0.4) + (pUAU);
}

// PrecondDW coefficients of the cell at slot index c (FP64 slots; TIME_LUSGS.F90:113-160 and
// every neighbour of the sweeps, :235-248): ubetac2 from getPrecondPara with the cell's
// Rmiu and its smallest Alagm
__device__ inline void precond_terms_at(const Params& p, const DevBlock& b, int c, double* t) {
    const double pRo = slot(b, S_V)[c];
    const double roinv = 1.0 / pRo;
    const double pVx = slot(b, S_V + 1)[c] * roinv, pVy = slot(b, S_V + 2)[c] * roinv, pVz = slot(b, S_V + 3)[c] * roinv;
    const double pE = slot(b, S_V + 4)[c] * roinv;
    const double pPP = slot(b, S_PP)[c], pTT = slot(b, S_T)[c];
    const double AAc = sqrt(1.4 * pPP * roinv);
    const double UVW2 = pVx * pVx + pVy * pVy + pVz * pVz;
    const double ALL = dmin(dmin(slot(b, S_ALAGM)[c], slot(b, S_ALAGM + 1)[c]), slot(b, S_ALAGM + 2)[c]);
    const double ub = get_precond_para<double>(p, UVW2, AAc * AAc, pRo, pTT, slot(b, S_RMIU)[c], ALL);
    precond_terms<double>(p, pRo, pVx, pVy, pVz, pE, AAc, ub, pTT, t);
}

// Space/UTIL_MUSCL.F90:2-18
template <typename R> __device__ inline R alimiter(R var1, R var2) {
    const R epsm = R(1.0e-7);
    return (var1 * (var2 * var2 + R(2.0) * epsm * epsm) + var2 * (R(2.0) * var1 * var1 + epsm * epsm)) /
           (R(2.0) * var1 * var1 - var1 * var2 + R(2.0) * var2 * var2 + R(3.0) * epsm * epsm) * R(0.5) *
           fabs(sgn1(var1) + sgn1(var2));
}

// Space/UTIL_MUSCL.F90:21-35: the limiter of CONVECT_MUSCL2 (Kind_Spatial = 1)
template <typename R> __device__ inline R muscl2_limiter(R var1, R var2) {
    const R epsm = R(1.0e-6);
    R smooth = (R(2.0) * var1 * var2 + epsm) / (var1 * var1 + var2 * var2 + epsm);
    return ((R(1.0) + smooth) * var1 + (R(1.0) - smooth) * var2) * smooth / R(2.0);
}

// Space/CONVECT_MDCD.F90:62-120: left (ql) and right (qr) face states from six cells
template <typename R> __device__ inline void mdcd_pair(const R* s6, R gama, R& ql, R& qr) {
    const R beta = R(sqrt(13.0 / 12.0));
    const R epsm = R(1.0e-6);
    R aw0 = R(1.5) * (R(0.0463783) + gama);
    R aw1 = R(0.5 - 1.5 * 0.0463783) + R(4.5) * gama;
    R aw2 = R(0.5 - 1.5 * 0.0463783) - R(4.5) * gama;
    R aw3 = R(1.5) * (R(0.0463783) - gama);
    const R c26 = R(2. / 6.), c76 = R(7. / 6.), c116 = R(11. / 6.), c16 = R(1. / 6.), c56 = R(5. / 6.), c13 = R(1. / 3.);
    {
        R v_2 = s6[0], v_1 = s6[1], v0 = s6[2], v1 = s6[3], v2 = s6[4], v3 = s6[5];
        R ISK1 = sq(R(0.5) * v_2 - R(2.0) * v_1 + R(1.5) * v0) + sq(beta * v_2 - R(2.0) * beta * v_1 + beta * v0);
        R ISK2 = sq(-(R(0.5) * v_1) + R(0.0) * v0 + R(0.5) * v1) + sq(beta * v_1 - R(2.0) * beta * v0 + beta * v1);
        R ISK3 = sq(-(R(1.5) * v0) + R(2.0) * v1 - R(0.5) * v2) + sq(beta * v0 - R(2.0) * beta * v1 + beta * v2);
        R ISK4 = sq(R(2.5) * v1 - R(4.0) * v2 + R(1.5) * v3) + sq(beta * v1 - R(2.0) * beta * v2 + beta * v3);
        ISK4 = dmax(dmax(dmax(ISK1, ISK2), ISK3), ISK4);
        R ak1 = aw0 / sq(epsm + ISK1), ak2 = aw1 / sq(epsm + ISK2), ak3 = aw2 / sq(epsm + ISK3), ak4 = aw3 / sq(epsm + ISK4);
        R w0 = ak1 / (ak1 + ak2 + ak3 + ak4), w1 = ak2 / (ak1 + ak2 + ak3 + ak4);
        R w2 = ak3 / (ak1 + ak2 + ak3 + ak4), w3 = ak4 / (ak1 + ak2 + ak3 + ak4);
        R qq0 = c26 * v_2 - c76 * v_1 + c116 * v0;
        R qq1 = -(c16 * v_1) + c56 * v0 + c26 * v1;
        R qq2 = c26 * v0 + c56 * v1 - c16 * v2;
        R qq3 = c116 * v1 - c76 * v2 + c13 * v3;
        ql = w0 * qq0 + w1 * qq1 + w2 * qq2 + w3 * qq3;
    }
    {
        R v_3 = s6[0], v_2 = s6[1], v_1 = s6[2], v0 = s6[3], v1 = s6[4], v2 = s6[5];
        R ISK1 = sq(R(0.5) * v2 - R(2.0) * v1 + R(1.5) * v0) + sq(beta * v2 - R(2.0) * beta * v1 + beta * v0);
        R ISK2 = sq(-(R(0.5) * v1) + R(0.0) * v0 + R(0.5) * v_1) + sq(beta * v1 - R(2.0) * beta * v0 + beta * v_1);
        R ISK3 = sq(-(R(1.5) * v0) + R(2.0) * v_1 - R(0.5) * v_2) + sq(beta * v0 - R(2.0) * beta * v_1 + beta * v_2);
        R ISK4 = sq(R(2.5) * v_1 - R(4.0) * v_2 + R(1.5) * v_3) + sq(beta * v_1 - R(2.0) * beta * v_2 + beta * v_3);
        ISK4 = dmax(dmax(dmax(ISK1, ISK2), ISK3), ISK4);
        R ak1 = aw0 / sq(epsm + ISK1), ak2 = aw1 / sq(epsm + ISK2), ak3 = aw2 / sq(epsm + ISK3), ak4 = aw3 / sq(epsm + ISK4);
        R w0 = ak1 / (ak1 + ak2 + ak3 + ak4), w1 = ak2 / (ak1 + ak2 + ak3 + ak4);
        R w2 = ak3 / (ak1 + ak2 + ak3 + ak4), w3 = ak4 / (ak1 + ak2 + ak3 + ak4);
        R qq0 = c26 * v2 - c76 * v1 + c116 * v0;
        R qq1 = -(c16 * v1) + c56 * v0 + c26 * v_1;
        R qq2 = c26 * v0 + c56 * v_1 - c16 * v_2;
        R qq3 = c116 * v_1 - c76 * v_2 + c13 * v_3;
        qr = w0 * qq0 + w1 * qq1 + w2 * qq2 + w3 * qq3;
    }
}

// The mixed path's FP32 form of mdcd_pair (the same states in another association): the left
// and right states of a face use the same four three-cell stencils s0..s3 of the six cells.
// With D_k = s_k - 2 s_{k+1} + s_{k+2} (k = 0..3), the smoothness indicators' second terms
// beta^2 D^2 are shared (left ISK_k and right ISK_(5-k) use D_(k-1)), and of the first terms
// four determine the rest: F3 = -(G2 + D2), F4 = G1 + D3, G3 = -(F2 + D1), G4 = F1 + D0 (F:
// left, G: right); the four candidate values qq0..qq3 of the left state are those of the
// right state in reverse order (1/3 = 2/6); the weights divide by one reciprocal of their sum.
template <> __device__ inline void mdcd_pair<float>(const float* s6, float gama, float& ql, float& qr) {
    const float b2 = 13.0f / 12.0f;                  // beta^2
    const float epsm = 1.0e-6f;
    const float aw0 = 1.5f * (0.0463783f + gama);
    const float aw1 = (0.5f - 1.5f * 0.0463783f) + 4.5f * gama;
    const float aw2 = (0.5f - 1.5f * 0.0463783f) - 4.5f * gama;
    const float aw3 = 1.5f * (0.0463783f - gama);
    const float s0 = s6[0], s1 = s6[1], s2 = s6[2], s3 = s6[3], s4 = s6[4], s5 = s6[5];
    const float D0 = s0 - 2.0f * s1 + s2, D1 = s1 - 2.0f * s2 + s3, D2 = s2 - 2.0f * s3 + s4, D3 = s3 - 2.0f * s4 + s5;
    const float E0 = b2 * D0 * D0, E1 = b2 * D1 * D1, E2 = b2 * D2 * D2, E3 = b2 * D3 * D3;
    const float F1 = 0.5f * s0 - 2.0f * s1 + 1.5f * s2, F2 = 0.5f * (s3 - s1);
    const float G1 = 0.5f * s5 - 2.0f * s4 + 1.5f * s3, G2 = 0.5f * (s2 - s4);
    const float F3 = G2 + D2, F4 = G1 + D3, G3 = F2 + D1, G4 = F1 + D0;      // up to sign, squared next
    const float c13 = 1.0f / 3.0f, c76 = 7.0f / 6.0f, c116 = 11.0f / 6.0f, c16 = 1.0f / 6.0f, c56 = 5.0f / 6.0f;
    const float qq0 = c13 * s0 - c76 * s1 + c116 * s2;
    const float qq1 = -(c16 * s1) + c56 * s2 + c13 * s3;
    const float qq2 = c13 * s2 + c56 * s3 - c16 * s4;
    const float qq3 = c116 * s3 - c76 * s4 + c13 * s5;
    auto state = [&](float I1, float I2, float I3, float I4, float r0, float r1, float r2, float r3) {
        I4 = fmaxf(fmaxf(fmaxf(I1, I2), I3), I4);
        const float a1 = aw0 / sq(epsm + I1), a2 = aw1 / sq(epsm + I2), a3 = aw2 / sq(epsm + I3), a4 = aw3 / sq(epsm + I4);
        const float rs = 1.0f / (a1 + a2 + a3 + a4);
        return (a1 * r0 + a2 * r1 + a3 * r2 + a4 * r3) * rs;
    };
    ql = state(F1 * F1 + E0, F2 * F2 + E1, F3 * F3 + E2, F4 * F4 + E3, qq0, qq1, qq2, qq3);
    qr = state(G1 * G1 + E3, G2 * G2 + E2, G3 * G3 + E1, G4 * G4 + E0, qq3, qq2, qq1, qq0);
}

// Roe_Common of the rotated scheme (Space/CONVECT_Roe_Rotated.F90:597-752), non-preconditioned:
// adds 0.5 |A| dQ along (sav1..3)/sav, times sav and Funscheme, to dr.  rLo, rRo = rccl, rccr
// times omega(1), the frame speeds of the two states.
template <typename R>
__device__ inline void roe_rot_common(const ParamsT<R>& p, R PLo, R PRo, R TLo, R TRo, R ULo, R URo, R VLo, R VRo, R WLo,
                                      R WRo, R sav1, R sav2, R sav3, R sav, R rLo, R rRo, R Funscheme, R* dr) {
    const R rcpcv = R(p.PPF);
    const R DENLo = PLo / (rcpcv * TLo), DENRo = PRo / (rcpcv * TRo);
    const R ga = R(1.4), ga1 = R(0.4);
    const R VAMLo = ULo * ULo + VLo * VLo + WLo * WLo, VAMRo = URo * URo + VRo * VRo + WRo * WRo;
    const R HLo = PLo * ga / (DENLo * ga1) + R(0.5) * VAMLo - R(0.5) * (rLo * rLo);
    const R HRo = PRo * ga / (DENRo * ga1) + R(0.5) * VAMRo - R(0.5) * (rRo * rRo);
    const R rrorl = sqrt(DENRo / DENLo), rrorlp1 = R(1.0) + rrorl;
    const R rm = sqrt(DENRo * DENLo);
    const R um = (ULo + URo * rrorl) / rrorlp1, vm = (VLo + VRo * rrorl) / rrorlp1, wm = (WLo + WRo * rrorl) / rrorlp1;
    const R hm = (HLo + HRo * rrorl) / rrorlp1;
    const R vm2 = um * um + vm * vm + wm * wm;
    const R rccm = (rLo + rRo * rrorl) / rrorlp1;
    const R am2 = ga1 * fabs(hm - R(0.5) * vm2 + R(0.5) * (rccm * rccm));
    const R am = sqrt(am2);
    const R sav1n = sav1 / sav, sav2n = sav2 / sav, sav3n = sav3 / sav;
    const R unormaln = (sav1n * um + sav2n * vm + sav3n * wm);
    const R eig1 = fabs(unormaln), eig2 = fabs(unormaln + am), eig3 = fabs(unormaln - am);
    const R alf = R(0.0), ubetac2 = R(1.0);
    const R dunormaln = (sav1n * (URo - ULo) + sav2n * (VRo - VLo) + sav3n * (WRo - WLo));
    const R astar = (eig2 + eig3) / R(2.0);
    const R Mstar = (eig2 - eig3) / R(2.0) / am;
    const R dW1 = DENRo - DENLo, dU1 = URo - ULo, dU2 = VRo - VLo, dU3 = WRo - WLo, dP1 = PRo - PLo;
    const R dW2 = rm * dU1 + dW1 * um, dW3 = rm * dU2 + dW1 * vm, dW4 = rm * dU3 + dW1 * wm;
    const R dW5 = dP1 / ga1 + R(0.5) * vm2 * dW1 + rm * um * dU1 + rm * vm * dU2 + rm * wm * dU3;
    const R dUroe = Mstar * dunormaln + (astar - (R(1) - R(2.0) * alf) * eig1 - alf * unormaln * Mstar) * (PRo - PLo) / rm / (ubetac2 * am2);
    const R dProe = Mstar * (PRo - PLo) + (astar - eig1 + alf * unormaln * Mstar) * rm * dunormaln;
    const R d1[5] = {eig1 * dW1 + dUroe * rm, eig1 * dW2 + dUroe * rm * um + dProe * sav1n,
                     eig1 * dW3 + dUroe * rm * vm + dProe * sav2n, eig1 * dW4 + dUroe * rm * wm + dProe * sav3n,
                     eig1 * dW5 + dUroe * rm * hm + dProe * unormaln};
    for (int L = 0; L < 5; ++L) dr[L] = dr[L] + R(0.5) * d1[L] * sav * Funscheme;
}

// CONVECT_Roe_Rotated (Space/CONVECT_Roe_Rotated.F90:59-591): central flux along the face
// normal, then the dissipation along the velocity-jump direction and along the rest of the face
// vector (one direction when the jump is below Tiny); dr = the face's contribution (times |S|).
// The grid velocities the reference reads uninitialised (:169, :332, :510) are taken as 0.
template <typename R>
__device__ inline void roe_rotated(const ParamsT<R>& p, R PLo, R PRo, R TLo, R TRo, R ULo, R URo, R VLo, R VRo, R WLo,
                                   R WRo, R sav1, R sav2, R sav3, R sav, R rLo, R rRo, R Funscheme, R* dr) {
    const R rcpcv = R(p.PPF);
    const R DENLo = PLo / (rcpcv * TLo), DENRo = PRo / (rcpcv * TRo);
    const R ga = R(1.4), ga1 = R(0.4);
    const R VAMLo = ULo * ULo + VLo * VLo + WLo * WLo, VAMRo = URo * URo + VRo * VRo + WRo * WRo;
    const R HLo = PLo * ga / (DENLo * ga1) + R(0.5) * VAMLo - R(0.5) * (rLo * rLo);
    const R HRo = PRo * ga / (DENRo * ga1) + R(0.5) * VAMRo - R(0.5) * (rRo * rRo);
    const R sav1n = sav1 / sav, sav2n = sav2 / sav, sav3n = sav3 / sav;
    const R vbc = R(0.0);
    const R ulnormaln = (sav1n * ULo + sav2n * VLo + sav3n * WLo);
    const R urnormaln = (sav1n * URo + sav2n * VRo + sav3n * WRo);
    const R rulnormaln = DENLo * ulnormaln, rurnormaln = DENRo * urnormaln;
    dr[0] = R(-0.5) * (rulnormaln + rurnormaln) * sav;
    dr[1] = R(-0.5) * (rulnormaln * ULo + rurnormaln * URo + sav1n * (PLo + PRo)) * sav;
    dr[2] = R(-0.5) * (rulnormaln * VLo + rurnormaln * VRo + sav2n * (PLo + PRo)) * sav;
    dr[3] = R(-0.5) * (rulnormaln * WLo + rurnormaln * WRo + sav3n * (PLo + PRo)) * sav;
    dr[4] = R(-0.5) * (rulnormaln * HLo + rurnormaln * HRo - vbc * (PLo + PRo)) * sav;
    const R DeltaU = sqrt((URo - ULo) * (URo - ULo) + (VRo - VLo) * (VRo - VLo) + (WRo - WLo) * (WRo - WLo));
    if (DeltaU <= R(p.Tiny)) {
        roe_rot_common<R>(p, PLo, PRo, TLo, TRo, ULo, URo, VLo, VRo, WLo, WRo, sav1, sav2, sav3, sav, rLo, rRo, Funscheme, dr);
        return;
    }
    R n1 = (URo - ULo) / DeltaU, n2 = (VRo - VLo) / DeltaU, n3 = (WRo - WLo) / DeltaU;
    R s = n1 * sav1 + n2 * sav2 + n3 * sav3;
    const R sg = sgn1(s);
    n1 = sg * n1; n2 = sg * n2; n3 = sg * n3;
    s = fabs(s);
    const R a1 = n1 * s, a2 = n2 * s, a3 = n3 * s;
    const R b1 = sav1 - a1, b2 = sav2 - a2, b3 = sav3 - a3;
    const R sa = dmax(sqrt(a1 * a1 + a2 * a2 + a3 * a3), R(p.Tiny));
    roe_rot_common<R>(p, PLo, PRo, TLo, TRo, ULo, URo, VLo, VRo, WLo, WRo, a1, a2, a3, sa, rLo, rRo, Funscheme, dr);
    const R sb = dmax(sqrt(b1 * b1 + b2 * b2 + b3 * b3), R(p.Tiny));
    roe_rot_common<R>(p, PLo, PRo, TLo, TRo, ULo, URo, VLo, VRo, WLo, WRo, b1, b2, b3, sb, rLo, rRo, Funscheme, dr);
}

// Space/CONVECT_Roe_Original.F90:242-407; out = flux / |S|.  rLo, rRo = rccl, rccr times
// omega(1) (:79-80, 138-139, 196-197), the frame speeds of the two states.
template <typename R>
__device__ inline void roe_flux(const ParamsT<R>& p, R PLo, R PRo, R TLo, R TRo, R ULo, R URo, R VLo, R VRo, R WLo, R WRo,
                                R sav1, R sav2, R sav3, R sav, R rLo, R rRo, R* out, R RmiuT = R(0.0), R AlagmR = R(1.0)) {
    R rcpcv = R(p.PPF);
    R DENLo = PLo / (rcpcv * TLo), DENRo = PRo / (rcpcv * TRo);
    const R ga = R(1.4), ga1 = R(1.4 - 1.0);
    R VAMLo = ULo * ULo + VLo * VLo + WLo * WLo;
    R VAMRo = URo * URo + VRo * VRo + WRo * WRo;
    R HLo = PLo * ga / (DENLo * ga1) + R(0.5) * VAMLo - R(0.5) * (rLo * rLo);
    R HRo = PRo * ga / (DENRo * ga1) + R(0.5) * VAMRo - R(0.5) * (rRo * rRo);
    R rrorl = sqrt(DENRo / DENLo);
    R rrorlp1 = R(1.0) + rrorl;
    R rm = sqrt(DENRo * DENLo);
    R um = (ULo + URo * rrorl) / rrorlp1;
    R vm = (VLo + VRo * rrorl) / rrorlp1;
    R wm = (WLo + WRo * rrorl) / rrorlp1;
    R hm = (HLo + HRo * rrorl) / rrorlp1;
    R vm2 = um * um + vm * vm + wm * wm;
    R rccm = (rLo + rrorl * rRo) / rrorlp1;
    R am2 = ga1 * fabs(hm - R(0.5) * vm2 + R(0.5) * (rccm * rccm));
    R am = sqrt(am2);
    R sav1n = sav1 / sav, sav2n = sav2 / sav, sav3n = sav3 / sav;
    R unormaln = (sav1n * um + sav2n * vm + sav3n * wm);
    R eig1, eig2, eig3, alf, ubetac2, amrev;
    if (p.IF_Precondition) {        // Space/CONVECT_Roe_Original.F90:319-331 (RmiuT = VL(d,8), AlagmR = Alagm(d))
        R TTL = am2 / ga / R(p.PPF);
        ubetac2 = get_precond_para<R>(p, vm2, am2, rm, TTL, RmiuT, AlagmR);
        alf = (R(1.0) - ubetac2) / R(2.0);
        R unrev = unormaln * (R(1.0) - alf);
        amrev = sqrt(pow2r<R>(alf * unormaln) + ubetac2 * am2);
        eig1 = fabs(unormaln);
        eig2 = fabs(unrev + amrev);
        eig3 = fabs(unrev - amrev);
    } else {
        eig1 = fabs(unormaln);
        eig2 = fabs(unormaln + am);
        eig3 = fabs(unormaln - am);
        const R e01 = R(0.1), ee = R(0.1 * 0.1), e02 = R(0.2);
        if (eig1 < e01) eig1 = (eig1 * eig1 + ee) / e02;
        if (eig2 < e01) eig2 = (eig2 * eig2 + ee) / e02;
        if (eig3 < e01) eig3 = (eig3 * eig3 + ee) / e02;
        alf = R(0.0);
        ubetac2 = R(1.0);
        amrev = am;
    }
    R dunormaln = (sav1n * (URo - ULo) + sav2n * (VRo - VLo) + sav3n * (WRo - WLo));
    R astar = (eig2 + eig3) / R(2.0);
    R Mstar = (eig2 - eig3) / R(2.0) / amrev;
    R dW1 = DENRo - DENLo;
    R dU1 = URo - ULo, dU2 = VRo - VLo, dU3 = WRo - WLo;
    R dP1 = PRo - PLo;
    R dW2 = rm * dU1 + dW1 * um;
    R dW3 = rm * dU2 + dW1 * vm;
    R dW4 = rm * dU3 + dW1 * wm;
    R dW5 = dP1 / ga1 + R(0.5) * vm2 * dW1 + rm * um * dU1 + rm * vm * dU2 + rm * wm * dU3;
    R dUroe = Mstar * dunormaln + (astar - (R(1) - R(2.0) * alf) * eig1 - alf * unormaln * Mstar) * (PRo - PLo) / rm / (ubetac2 * am2);
    R dProe = Mstar * (PRo - PLo) + (astar - eig1 + alf * unormaln * Mstar) * rm * dunormaln;
    R droR1 = eig1 * dW1 + dUroe * rm;
    R drxR1 = eig1 * dW2 + dUroe * rm * um + dProe * sav1n;
    R dryR1 = eig1 * dW3 + dUroe * rm * vm + dProe * sav2n;
    R drzR1 = eig1 * dW4 + dUroe * rm * wm + dProe * sav3n;
    R dreR1 = eig1 * dW5 + dUroe * rm * hm + dProe * unormaln;
    R ulnormaln = (sav1n * ULo + sav2n * VLo + sav3n * WLo);
    R urnormaln = (sav1n * URo + sav2n * VRo + sav3n * WRo);
    R rulnormaln = DENLo * ulnormaln, rurnormaln = DENRo * urnormaln;
    out[0] = R(-0.5) * (rulnormaln + rurnormaln - droR1);
    out[1] = R(-0.5) * (rulnormaln * ULo + rurnormaln * URo + sav1n * (PLo + PRo) - drxR1);
    out[2] = R(-0.5) * (rulnormaln * VLo + rurnormaln * VRo + sav2n * (PLo + PRo) - dryR1);
    out[3] = R(-0.5) * (rulnormaln * WLo + rurnormaln * WRo + sav3n * (PLo + PRo) - drzR1);
    out[4] = R(-0.5) * (rulnormaln * HLo + rurnormaln * HRo - dreR1);
}

// Space/CONVECT_AUSMPW_Plus.F90:204-317; out = flux / |S|
template <typename R>
__device__ inline void ausmpw_flux(const ParamsT<R>& p, R PLo, R PRo, R TLo, R TRo, R ULo, R URo, R VLo, R VRo, R WLo, R WRo,
                                   R sav1, R sav2, R sav3, R sav, R* out) {
    R rcpcv = R(p.PPF);
    R DENLo = PLo / (rcpcv * TLo), DENRo = PRo / (rcpcv * TRo);
    R sav1n = sav1 / sav, sav2n = sav2 / sav, sav3n = sav3 / sav;
    const R ga = R(1.4), ga1 = R(1.4 - 1.0);
    R VAMLo = ULo * ULo + VLo * VLo + WLo * WLo;
    R VAMRo = URo * URo + VRo * VRo + WRo * WRo;
    R HLo = PLo * ga / (DENLo * ga1) + R(0.5) * VAMLo;
    R HRo = PRo * ga / (DENRo * ga1) + R(0.5) * VAMRo;
    R ULn = (sav1n * ULo + sav2n * VLo + sav3n * WLo);
    R URn = (sav1n * URo + sav2n * VRo + sav3n * WRo);
    R astar_L = sqrt(R(2) * ga1 * HLo / (ga + R(1)));
    R astar_R = sqrt(R(2) * ga1 * HRo / (ga + R(1)));
    R aas_L = astar_L * astar_L / dmax(sqrt(VAMLo), astar_L);
    R aas_R = astar_R * astar_R / dmax(sqrt(VAMRo), astar_R);
    R Acc = dmin(aas_L, aas_R);
    R MaL = ULn / Acc, MaR = URn / Acc;
    const R c316 = R(0.0);    // 3/16 is integer division in the reference (CONVECT_AUSMPW_Plus.F90:274,286)
    const R tiny = R(p.Tiny);
    R MaL_plus, pL_plus, MaR_neg, pR_neg;
    if (fabs(MaL) > R(1.0)) {
        MaL_plus = R(0.5) * (MaL + fabs(MaL));
        pL_plus = R(0.5) * (MaL + fabs(MaL)) / (MaL + tiny);
    } else {
        MaL_plus = R(0.25) * sq(MaL + R(1));
        pL_plus = R(0.25) * sq(MaL + R(1)) * (R(2) - MaL) + c316 * MaL * sq(MaL * MaL - R(1));
    }
    if (fabs(MaR) > R(1.0)) {
        MaR_neg = R(0.5) * (MaR - fabs(MaR));
        pR_neg = R(0.5) * (MaR - fabs(MaR)) / (MaR + tiny);
    } else {
        MaR_neg = R(-1) * R(0.25) * sq(MaR - R(1));
        pR_neg = R(0.25) * sq(MaR - R(1)) * (R(2) + MaR) - c316 * MaR * sq(MaR * MaR - R(1));
    }
    R pS = pL_plus * PLo + pR_neg * PRo;
    R Mas = MaL_plus + MaR_neg;
    R mn = dmin(PLo / PRo, PRo / PLo);
    R wP = R(1.0) - mn * mn * mn;
    R fL = fabs(MaL) < R(1) ? PLo / (pS + tiny) - R(1) : R(0.0);
    R fR = fabs(MaR) < R(1) ? PRo / (pS + tiny) - R(1) : R(0.0);
    R MMaL_plus, MMaR_neg;
    if (Mas >= R(0)) {
        MMaL_plus = MaL_plus + MaR_neg * ((R(1) - wP) * (R(1) + fR) - fL);
        MMaR_neg = MaR_neg * wP * (R(1) + fR);
    } else {
        MMaL_plus = MaL_plus * wP * (R(1) + fL);
        MMaR_neg = MaR_neg + MaL_plus * ((R(1) - wP) * (R(1) + fL) - fR);
    }
    out[0] = R(-1) * MMaL_plus * Acc * DENLo - MMaR_neg * Acc * DENRo;
    out[1] = R(-1) * MMaL_plus * Acc * DENLo * ULo - MMaR_neg * Acc * DENRo * URo - sav1n * (pL_plus * PLo + pR_neg * PRo);
    out[2] = R(-1) * MMaL_plus * Acc * DENLo * VLo - MMaR_neg * Acc * DENRo * VRo - sav2n * (pL_plus * PLo + pR_neg * PRo);
    out[3] = R(-1) * MMaL_plus * Acc * DENLo * WLo - MMaR_neg * Acc * DENRo * WRo - sav3n * (pL_plus * PLo + pR_neg * PRo);
    out[4] = R(-1) * MMaL_plus * Acc * DENLo * HLo - MMaR_neg * Acc * DENRo * HRo;
}

// Time/TIME_LUSGS.F90:696-768 (LUSGS_ADQ) with pGam = 1.4 and zero grid speed, split into
// the DeltaQ-independent terms (jac_terms, once per cell and direction) and the products with
// DeltaQ (jac_row, inside the sweeps).  Every term is the reference's own subexpression, so
// the split rounds exactly as the undivided expression does.
template <typename R>
__device__ inline void jac_terms(R pVx, R pVy, R pVz, R aSDx, R aSDy, R aSDz, R pPP, R roinv, R* J) {
    const R pGam = R(1.4);
    R VP = pVx * aSDx + pVy * aSDy + pVz * aSDz + R(0.0);
    R Ut2 = pVx * pVx + pVy * pVy + pVz * pVz;
    const R aSDt = R(0.0);
    const R Gm1 = R(1.4 - 1.0), Gm2 = R(1.4 - 2.0);
    R AA2 = pGam * pPP * roinv;
    R gUt2 = R(0.5) * Gm1 * Ut2;
    J[JC_R1 + 0] = aSDx * gUt2 - pVx * VP;
    J[JC_R1 + 1] = aSDt + VP - aSDx * Gm2 * pVx;
    J[JC_R1 + 2] = aSDy * pVx - aSDx * Gm1 * pVy;
    J[JC_R1 + 3] = aSDz * pVx - aSDx * Gm1 * pVz;
    J[JC_R1 + 4] = aSDx * Gm1;
    J[JC_R2 + 0] = aSDy * gUt2 - pVy * VP;
    J[JC_R2 + 1] = aSDx * pVy - aSDy * Gm1 * pVx;
    J[JC_R2 + 2] = aSDt + VP - aSDy * Gm2 * pVy;
    J[JC_R2 + 3] = aSDz * pVy - aSDy * Gm1 * pVz;
    J[JC_R2 + 4] = aSDy * Gm1;
    J[JC_R3 + 0] = aSDz * gUt2 - pVz * VP;
    J[JC_R3 + 1] = aSDx * pVz - aSDz * Gm1 * pVx;
    J[JC_R3 + 2] = aSDy * pVz - aSDz * Gm1 * pVy;
    J[JC_R3 + 3] = aSDt + VP - aSDz * Gm2 * pVz;
    J[JC_R3 + 4] = aSDz * Gm1;
    J[JC_R0 + 0] = aSDx;
    J[JC_R0 + 1] = aSDy;
    J[JC_R0 + 2] = aSDz;
    R GEt1 = R(0.5) * Gm2 * Ut2 - AA2 / Gm1;
    R GEt2 = R(0.5) * Ut2 + AA2 / Gm1;
    J[JC_VP] = VP;
    J[JC_GET1] = GEt1;
    J[JC_R4 + 0] = aSDx * GEt2 - Gm1 * pVx * VP;
    J[JC_R4 + 1] = aSDy * GEt2 - Gm1 * pVy * VP;
    J[JC_R4 + 2] = aSDz * GEt2 - Gm1 * pVz * VP;
    J[JC_R4 + 3] = aSDt + pGam * VP;
    // contravariant speed of TURBTWO_TIME_LUSGS_SST (no "+ 0" there)
    J[JC_VPT] = pVx * aSDx + pVy * aSDy + pVz * aSDz;
}

// Time/Hybrid_function.F90:1-39
template <typename R>
__device__ inline R fsst(const ParamsT<R>& p, R Den, R vK, R vOmega, R Dist, R RmiuL, R CDiff) {
    R Ref = R(p.Ref);
    if (p.Kind_SubHY == 1 || p.Kind_SubHY == 3) {
        R arg1 = sqrt(vK) / (R(0.09) * vOmega * Dist * Ref);
        R arg2 = R(500.) * RmiuL / (Den * Dist * Dist * vOmega * Ref * Ref);
        R arga = dmax(arg1, arg2);
        R temp = dmax(Den * CDiff * Ref, R(1.0e-10));
        R argb = R(4.) * Den * R(0.856) * vK / (temp * Dist * Dist);
        R arg = dmin(arga, argb);
        return ttanh(arg * arg * arg * arg);
    }
    if (p.Kind_SubHY == 2) {
        R arg1 = R(2.) * sqrt(vK) / (R(0.09) * vOmega * Dist * Ref);
        R arg2 = R(500.) * RmiuL / (Den * Dist * Dist * vOmega * Ref * Ref);
        R arg = dmax(arg1, arg2);
        return ttanh(arg * arg);
    }
    return R(0.0);      // DES (0); no branch for IDDES (5), whose destruction does not use it
}

// IDDES functions of Time/Hybrid_function.F90:43-105 (Kind_SubHY = 5), constants of
// Module_Global.F90:126 (akapa_iddes 0.41, Cw 0.15, Ct 1.87, Cl 5.00; their squares folded as
// products); g = the nine velocity gradients dudx, dudy, dudz, dvdx, ..., dwdz
template <typename R> __device__ inline R sij_norm(const R* g) {
    R s = g[0] * g[0] + g[1] * g[1] + g[2] * g[2] + g[3] * g[3] + g[4] * g[4] + g[5] * g[5] + g[6] * g[6] + g[7] * g[7] +
          g[8] * g[8];
    s = sqrt(s);
    return dmax(s, R(1.0e-10));
}

template <typename R>
__device__ inline R fd_function(const ParamsT<R>& p, R Den1, R RmiuT1, R aDst1, R aLmax1, const R* g) {
    const R K2 = R(0.41 * 0.41);
    R alpha1 = R(0.25) - aDst1 / aLmax1;
    R fb = dmin(R(2.) * texp(R(-9.0) * alpha1 * alpha1), R(1.));
    R Sij = sij_norm(g);
    R rdt = (RmiuT1 / Den1) / (K2 * pow2_real(aDst1) * Sij * R(p.Ref));
    R fdt = R(1.) - ttanh((R(8.) * rdt) * (R(8.) * rdt) * (R(8.) * rdt));
    return dmax((R(1.) - fdt), fb);
}

template <typename R>
__device__ inline R fe_function(const ParamsT<R>& p, R Den2, R RmiuT2, R RmiuL2, R aDst2, R aLmax2, const R* g) {
    const R K2 = R(0.41 * 0.41), CT2 = R(1.87 * 1.87), CL2 = R(5.00 * 5.00);
    R alpha2 = R(0.25) - aDst2 / aLmax2;
    R fe1 = alpha2 >= R(0.) ? R(2.) * texp(R(-11.09) * alpha2 * alpha2) : R(2.) * texp(R(-9.) * alpha2 * alpha2);
    R Sij = sij_norm(g);
    R rdt = (RmiuT2 / Den2) / (K2 * pow2_real(aDst2) * Sij * R(p.Ref));
    R ft = ttanh((CT2 * rdt) * (CT2 * rdt) * (CT2 * rdt));
    R rdl = (RmiuL2 / Den2) / (K2 * pow2_real(aDst2) * Sij * R(p.Ref));
    R fl = ttanh(pow10_real(CL2 * rdl));
    R fe2 = R(1.) - dmax(ft, fl);
    return fe2 * dmax((fe1 - R(1.)), R(0.));
}

}  // namespace tg
