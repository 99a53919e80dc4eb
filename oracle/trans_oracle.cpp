// trans_oracle.cpp -- CPU FP64 restatement of the TRANS per-iteration hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle the GPU implementation is checked
// against; only tests, the smoke check and the CPU-baseline leg of the benchmark load it.
//
// It restates, loop by loop and in the reference's own (scatter) form, the Fortran
// subroutines of thuGithHub/TRANS BaseVersion (paths below are relative to BaseVersion/),
// with -r8 semantics: every REAL and every unsuffixed literal is double.  Compile with
// -ffp-contract=off so that no multiply-add is fused (the reference was built with
// -fp-model strict).  The reference itself cannot be compiled here (no Fortran compiler, and
// it needs MPI and a prebuilt TecIO archive), and it ships no tests, fixtures or sample cases:
// PARITY UNPINNED by the reference's own vectors.  The restatement is pinned instead by
// analytic invariants (free-stream preservation, limiter and flux identities) in tests/.
//
// Restatement choices, each equal to the reference's mathematics:
//   x**2 -> x*x, x**3 -> (x*x)*x, x**4 -> (x*x)*(x*x)   (integer powers)
//   x**0.5 -> sqrt(x)      x**1.5 -> x*sqrt(x)            (for x >= 0)
//   exp, tanh, x**y -> the functions of tmath.h (published methods in plain IEEE arithmetic,
//   within a few ulp of libm), so that the GPU library, which uses the same methods, can be
//   compared bit for bit
//   SIGN(1,b) -> +1 for b >= 0 (including -0.0), -1 otherwise
// Dead code of the reference is not restated: the residual smoothing of TIME_Update_V
// (its writes to D are commented out), Fscheme (read only by CONVECT_Roe_Rotated), ghost Rds
// and shock copies (never read / overwritten before use), the stray rcc block of CONVECT_MDCD.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/trans_gpu.h"
#include "tmath.h"

namespace {

inline double p15(double x) { return x * std::sqrt(x); }
inline double sgn1(double b) { return b >= 0.0 ? 1.0 : -1.0; }
inline double sq(double x) { return x * x; }
// x**2.0 with a real exponent: the product x*x, the correctly rounded value of the power (a
// compiler may emit it for the whole-number exponent without changing the result)
inline double pow2r(double x) { return x * x; }

// Low-Mach preconditioning (IF_Precondition = 1), Common/UTIL_Precond_Funcs.F90.
// getPrecondPara (:6-32): the preconditioning parameter ubetac2 of one state.
double get_precond_para(const trans_params& p, double VM2, double AM2, double RR, double TT, double RMIUT, double ALAGMR) {
    const double K = 3.0, Kc = 1.0;
    double ubetac2 = std::min(std::max(VM2 / AM2, K * p.XM * p.XM), 1.0);
    double RmiuL = (1.0 + p.Csthlnd) / (TT * p.Csth1 + p.Csthlnd) * p15(p.Csth1 * TT);
    double RmiuAll = RmiuL + RMIUT;
    return std::max(ubetac2, Kc * pow2r(RmiuAll / RR / p.Ref / ALAGMR) / AM2);
}

// PrecondDW (:90-127): the conservative increment (AinRo..AinRe) mapped through the
// preconditioning matrix of the state (pRo, pV, pE, AAc, ubetac2, pTT)
void precond_dw(const trans_params& p, double& AinRo, double& AinRx, double& AinRy, double& AinRz, double& AinRe, double pRo,
                double pVx, double pVy, double pVz, double pE, double AAc, double ubetac2, double pTT) {
    double pU2 = pVx * pVx + pVy * pVy + pVz * pVz;
    double pUAU = pVx * AinRx + pVy * AinRy + pVz * AinRz;
    AinRe = AinRe - (pUAU) - (pE / 1.4 - 1.2 * (pU2)) * AinRo;
    double rCp = 1.4 / 0.4 * p.PPF * pRo;
    double a11 = AAc * AAc * ubetac2;
    double a15 = -0.4 * ubetac2 / rCp;
    double b11 = 1.0 * a11 / rCp;
    double b15 = (1.0 + 0.4 * ubetac2) / rCp;
    double AinP = a11 * AinRo + a15 * AinRe;
    double AinT = b11 * AinRo + b15 * AinRe;
    AinRo = AinP / p.PPF / pTT - pRo * AinT / pTT;
    AinRe = AinP / 0.4 + (pUAU);
    (void)AinRx; (void)AinRy; (void)AinRz;
}

// Fortran-style arrays on the full ghost extent -2..N+2, leading components first.
struct Arr {
    std::vector<double> v;
    int n1 = 1, n2 = 1, pi = 0, pj = 0, pk = 0;
    void alloc(int a, int b, int ni, int nj, int nk) {
        n1 = a; n2 = b; pi = ni + 5; pj = nj + 5; pk = nk + 5;
        v.assign((size_t)n1 * n2 * pi * pj * pk, 0.0);
    }
    inline size_t cell(int i, int j, int k) const {
        return (size_t)(i + 2) + (size_t)pi * ((size_t)(j + 2) + (size_t)pj * (size_t)(k + 2));
    }
    inline double& operator()(int i, int j, int k) { return v[cell(i, j, k)]; }
    inline double& operator()(int a, int i, int j, int k) { return v[(size_t)(a - 1) + (size_t)n1 * cell(i, j, k)]; }
    inline double& operator()(int a, int b, int i, int j, int k) {
        return v[(size_t)(a - 1) + (size_t)n1 * ((size_t)(b - 1) + (size_t)n2 * cell(i, j, k))];
    }
};

struct Blk {
    int NI, NJ, NK, NI1, NJ1, NK1, id;
    std::vector<trans_conn> conn;
    std::vector<int> mw[6];     // MARKWALL arrays, Fortran (n1,n2) column-major
    int mwn1[6];
    Arr V, PP, T, Rmiu, Wt0, Wt1, Wt2, SD, Grad, Vol, Alagm, Dst, ALeng, ASeng, Xc, Yc, Zc, rad, thtc;
    Arr D, Rds, Dtm, DQ, shock, F, VL, VR, rccl, rccr, FunDES, Fsch, Fr1;
    trans_norms nrm;
    int markwall(int face, int a, int b) const {
        if (mw[face].empty()) return 0;
        return mw[face][(size_t)(a - 1) + (size_t)mwn1[face] * (size_t)(b - 1)];
    }
};

struct Ctx {
    trans_params p;
    std::vector<Blk> B;
    int IF_turb = 0;
    int KI = 1;
    int Itr_Chld = 1;
    std::string err;
    int nan_flag = 0;
};

// ---------------------------------------------------------------------------------------
// Time/SpectralRadius.F90:1-180
// ---------------------------------------------------------------------------------------
void spectral_radius(Ctx& c, Blk& b) {
    const trans_params& p = c.p;
    for (int K = 1; K <= b.NK1; ++K)
    for (int J = 1; J <= b.NJ1; ++J)
    for (int I = 1; I <= b.NI1; ++I) {
        double Den = b.V(1, I, J, K);
        double Vxi = b.V(2, I, J, K) / Den;
        double Vyi = b.V(3, I, J, K) / Den;
        double Vzi = b.V(4, I, J, K) / Den;
        double AAc = std::sqrt(1.4 * b.PP(I, J, K) / Den);
        double TT = b.T(I, J, K);
        double RmiuL = (1.0 + p.Csthlnd) / (TT * p.Csth1 + p.Csthlnd) * p15(p.Csth1 * TT);
        double RmiuTL = b.Rmiu(I, J, K);
        double uvmu = (RmiuL + RmiuTL + 1.0e-20) * 4.0 / 3.0;
        double uvmupr = (RmiuL / 0.72 + RmiuTL / 0.9 + 1.0e-20) * 1.4;
        double pruvmu = std::max(uvmu, uvmupr) / Den;
        double ARX1 = 0.5 * (b.SD(1, 1, I, J, K) + b.SD(1, 1, I + 1, J, K));
        double ARY1 = 0.5 * (b.SD(1, 2, I, J, K) + b.SD(1, 2, I + 1, J, K));
        double ARZ1 = 0.5 * (b.SD(1, 3, I, J, K) + b.SD(1, 3, I + 1, J, K));
        double ST1sq = ARX1 * ARX1 + ARY1 * ARY1 + ARZ1 * ARZ1;
        double vibc = 0.0;   // 0.5*(vibn(i)+vibn(i+1)): grid speeds are identically zero
        double ARX2 = 0.5 * (b.SD(2, 1, I, J, K) + b.SD(2, 1, I, J + 1, K));
        double ARY2 = 0.5 * (b.SD(2, 2, I, J, K) + b.SD(2, 2, I, J + 1, K));
        double ARZ2 = 0.5 * (b.SD(2, 3, I, J, K) + b.SD(2, 3, I, J + 1, K));
        double ST2sq = ARX2 * ARX2 + ARY2 * ARY2 + ARZ2 * ARZ2;
        double ARX3 = 0.5 * (b.SD(3, 1, I, J, K) + b.SD(3, 1, I, J, K + 1));
        double ARY3 = 0.5 * (b.SD(3, 2, I, J, K) + b.SD(3, 2, I, J, K + 1));
        double ARZ3 = 0.5 * (b.SD(3, 3, I, J, K) + b.SD(3, 3, I, J, K + 1));
        double ST3sq = ARX3 * ARX3 + ARY3 * ARY3 + ARZ3 * ARZ3;
        double UU = Vxi * ARX1 + Vyi * ARY1 + Vzi * ARZ1 + vibc;
        double VV = Vxi * ARX2 + Vyi * ARY2 + Vzi * ARZ2 + vibc;
        double WW = Vxi * ARX3 + Vyi * ARY3 + Vzi * ARZ3 + vibc;
        double alfu = 0.0, alfv = 0.0, alfw = 0.0;
        double AAcu = AAc, AAcv = AAc, AAcw = AAc;
        if (p.IF_Precondition) {            // Time/SpectralRadius.F90:91-127
            double UVW2 = Vxi * Vxi + Vyi * Vyi + Vzi * Vzi;
            double ubetac2 = get_precond_para(p, UVW2, AAc * AAc, Den, 0.0, 0.0, 1.0);
            double RmiuAll = RmiuL + RmiuTL;
            double ubu = std::max(ubetac2, pow2r(RmiuAll / Den / p.Ref / b.Alagm(1, I, J, K) / AAc));
            alfu = (1.0 - ubu) / 2.0;
            AAcu = std::sqrt(alfu * alfu * UVW2 + ubu * AAc * AAc);
            double ubv = std::max(ubetac2, pow2r(RmiuAll / Den / p.Ref / b.Alagm(2, I, J, K) / AAc));
            alfv = (1.0 - ubv) / 2.0;
            AAcv = std::sqrt(alfv * alfv * UVW2 + ubv * AAc * AAc);
            double ubw = std::max(ubetac2, pow2r(RmiuAll / Den / p.Ref / b.Alagm(3, I, J, K) / AAc));
            alfw = (1.0 - ubw) / 2.0;
            AAcw = std::sqrt(alfw * alfw * UVW2 + ubw * AAc * AAc);
        }
        b.Rds(1, I, J, K) = std::fabs(UU) * (1.0 - alfu) + std::sqrt(ST1sq) * AAcu + 2.0 * ST1sq / b.Vol(I, J, K) * pruvmu / p.Ref;
        b.Rds(2, I, J, K) = std::fabs(VV) * (1.0 - alfv) + std::sqrt(ST2sq) * AAcv + 2.0 * ST2sq / b.Vol(I, J, K) * pruvmu / p.Ref;
        b.Rds(3, I, J, K) = std::fabs(WW) * (1.0 - alfw) + std::sqrt(ST3sq) * AAcw + 2.0 * ST3sq / b.Vol(I, J, K) * pruvmu / p.Ref;
        double Dtm_local = b.Vol(I, J, K) / (b.Rds(1, I, J, K) + b.Rds(2, I, J, K) + b.Rds(3, I, J, K));
        if (p.IF_Local_Main == 1) b.Dtm(I, J, K) = p.CFL_Main * Dtm_local;
        else b.Dtm(I, J, K) = p.DT_LUSGS_Main;
        double CFL_sub = p.CFL_Sub_start + (p.CFL_Sub_end - p.CFL_Sub_start) * (double)(c.KI - p.KI_ini) / (double)p.CFL_Sub_step;
        CFL_sub = std::min(CFL_sub, p.CFL_Sub_end);
        if (p.Kind_Dual != 0) {
            if (p.IF_Local_Sub == 1) b.Dtm(I, J, K) = CFL_sub * Dtm_local;
            else b.Dtm(I, J, K) = p.DT_LUSGS_Sub;
        }
    }
}

// ---------------------------------------------------------------------------------------
// BC/  (sweep -1: cell-centre state, sweep 0: gradients)
// ---------------------------------------------------------------------------------------
struct SegIdx {
    int Ibgn, Jbgn, Kbgn, Iend, Jend, Kend;
    int iadd, jadd, kadd, iadd1, jadd1, kadd1, iadd2, jadd2, kadd2;
    int Eiadd, Ejadd, Ekadd, Eiadd1, Ejadd1, Ekadd1, Eiadd2, Ejadd2, Ekadd2;
    int Siadd, Sjadd, Skadd, IJKDir;
    explicit SegIdx(const trans_conn& a) {
        Ibgn = a.pointStart[0]; Jbgn = a.pointStart[1]; Kbgn = a.pointStart[2];
        Iend = a.pointEnd[0]; Jend = a.pointEnd[1]; Kend = a.pointEnd[2];
        iadd = a.CIJKAdd[0]; jadd = a.CIJKAdd[1]; kadd = a.CIJKAdd[2];
        iadd1 = a.CIJKAdd1[0]; jadd1 = a.CIJKAdd1[1]; kadd1 = a.CIJKAdd1[2];
        iadd2 = a.CIJKAdd2[0]; jadd2 = a.CIJKAdd2[1]; kadd2 = a.CIJKAdd2[2];
        Eiadd = a.CEIJKAdd[0]; Ejadd = a.CEIJKAdd[1]; Ekadd = a.CEIJKAdd[2];
        Eiadd1 = a.CEIJKAdd1[0]; Ejadd1 = a.CEIJKAdd1[1]; Ekadd1 = a.CEIJKAdd1[2];
        Eiadd2 = a.CEIJKAdd2[0]; Ejadd2 = a.CEIJKAdd2[1]; Ekadd2 = a.CEIJKAdd2[2];
        Siadd = a.IJKAdd[0]; Sjadd = a.IJKAdd[1]; Skadd = a.IJKAdd[2];
        IJKDir = a.IJKDirect;
    }
};

// BC/BC_Wall.F90:2-135
void bc_wall(Ctx& c, Blk& b, const trans_conn& a, int sweep) {
    const trans_params& p = c.p;
    SegIdx s(a);
    int Kindsub_BC = a.SubBCType;
    if (sweep == -1) {
        for (int K = s.Kbgn; K <= s.Kend; ++K)
        for (int J = s.Jbgn; J <= s.Jend; ++J)
        for (int I = s.Ibgn; I <= s.Iend; ++I) {
            int is = I + s.iadd, js = J + s.jadd, ks = K + s.kadd;
            int il = I + s.Eiadd, jl = J + s.Ejadd, kl = K + s.Ekadd;
            double ztemp = 0.5 * (b.Zc(is, js, ks) + b.Zc(il, jl, kl));
            double ytemp = 0.5 * (b.Yc(is, js, ks) + b.Yc(il, jl, kl));
            double vibc = 0.0;
            double vjbc = (double)Kindsub_BC * p.omega[0] * ztemp;
            double vkbc = -(double)Kindsub_BC * p.omega[0] * ytemp;
            const int adds[3][6] = {{s.iadd, s.jadd, s.kadd, s.Eiadd, s.Ejadd, s.Ekadd},
                                    {s.iadd1, s.jadd1, s.kadd1, s.Eiadd1, s.Ejadd1, s.Ekadd1},
                                    {s.iadd2, s.jadd2, s.kadd2, s.Eiadd2, s.Ejadd2, s.Ekadd2}};
            for (int L = 0; L < 3; ++L) {
                is = I + adds[L][0]; js = J + adds[L][1]; ks = K + adds[L][2];
                il = I + adds[L][3]; jl = J + adds[L][4]; kl = K + adds[L][5];
                b.PP(il, jl, kl) = b.PP(is, js, ks);
                b.T(il, jl, kl) = b.T(is, js, ks);
                b.V(1, il, jl, kl) = b.PP(il, jl, kl) / (b.T(il, jl, kl) + p.Tiny) * p.RXM2;
                double den = b.V(1, il, jl, kl);
                b.V(2, il, jl, kl) = vibc * den;
                b.V(3, il, jl, kl) = vjbc * den;
                b.V(4, il, jl, kl) = vkbc * den;
            }
            if (c.IF_turb) {
                is = I + s.iadd; js = J + s.jadd; ks = K + s.kadd;
                il = I + s.Eiadd; jl = J + s.Ejadd; kl = K + s.Ekadd;
                double Dn = b.Dst(il, jl, kl);
                double Den = b.V(1, il, jl, kl);
                double TT = b.T(il, jl, kl);
                double Rmiuw = (1.0 + p.Csthlnd) / (TT * p.Csth1 + p.Csthlnd) * p15(p.Csth1 * TT);
                double Omegaw = 60.0 * Rmiuw / (Den * 0.075 * Dn * Dn * p.Ref * p.Ref);
                Rmiuw = b.Rmiu(is, js, ks);
                const int E[3][3] = {{s.Eiadd, s.Ejadd, s.Ekadd}, {s.Eiadd1, s.Ejadd1, s.Ekadd1}, {s.Eiadd2, s.Ejadd2, s.Ekadd2}};
                for (int L = 0; L < 3; ++L) {
                    il = I + E[L][0]; jl = J + E[L][1]; kl = K + E[L][2];
                    b.V(6, il, jl, kl) = 0.0;
                    b.V(7, il, jl, kl) = Omegaw;
                    b.Rmiu(il, jl, kl) = Rmiuw;
                }
            }
        }
    } else {
        for (int K = s.Kbgn; K <= s.Kend; ++K)
        for (int J = s.Jbgn; J <= s.Jend; ++J)
        for (int I = s.Ibgn; I <= s.Iend; ++I) {
            int is = I + s.iadd, js = J + s.jadd, ks = K + s.kadd;
            int il = I + s.Eiadd, jl = J + s.Ejadd, kl = K + s.Ekadd;
            for (int L = 1; L <= 18; ++L) b.DQ(L, il, jl, kl) = b.DQ(L, is, js, ks);
        }
    }
}

// BC/BC_far.F90:135-207
void bc_farbond(double XM, double P2, double RR, double Vxi, double Vyi, double Vzi, double DNx, double DNy,
                double DNz, double VxF, double VyF, double VzF, double& PP0, double& RR0, double& VX0,
                double& VY0, double& VZ0, double& dir) {
    double pGam = 1.4;
    double AF = 1.0 / XM;
    double AE = std::sqrt(pGam * P2 / RR);
    double QNE = Vxi * DNx + Vyi * DNy + Vzi * DNz;
    double QNF = VxF * DNx + VyF * DNy + VzF * DNz;
    double RF = QNF - 5.0 * AF;
    double RE = QNE + 5.0 * AE;
    double QN = 0.5 * (RE + RF);
    double AS = 0.1 * (RE - RF);
    if (QN > -AS && QN < 0.0) {
        double SON = 1.0 / pGam / (XM * XM);
        double QTX = VxF - QNF * DNx, QTY = VyF - QNF * DNy, QTZ = VzF - QNF * DNz;
        VX0 = QTX + QN * DNx; VY0 = QTY + QN * DNy; VZ0 = QTZ + QN * DNz;
        RR0 = otm::pow_(AS * AS / SON / pGam, 2.5);
        PP0 = AS * AS * RR0 / pGam;
        dir = -1.0;
    }
    if (QN >= 0.0 && QN < AS) {
        double SON = P2 / otm::pow_(RR, pGam);
        double QTX = Vxi - QNE * DNx, QTY = Vyi - QNE * DNy, QTZ = Vzi - QNE * DNz;
        VX0 = QTX + QN * DNx; VY0 = QTY + QN * DNy; VZ0 = QTZ + QN * DNz;
        RR0 = otm::pow_(AS * AS / SON / pGam, 2.5);
        PP0 = AS * AS * RR0 / pGam;
        dir = 1.0;
    }
    if (QN <= -AS) {
        VX0 = VxF; VY0 = VyF; VZ0 = VzF;
        RR0 = 1.0;
        PP0 = 1.0 / pGam / XM / XM;
        dir = -1.0;
    }
    if (QN >= AS) {
        VX0 = Vxi; VY0 = Vyi; VZ0 = Vzi;
        RR0 = RR; PP0 = P2;
        dir = 1.0;
    }
}

// BC/BC_far.F90:1-131
void bc_far(Ctx& c, Blk& b, const trans_conn& a, int sweep) {
    const trans_params& p = c.p;
    SegIdx s(a);
    double out_n = (double)(2 * a.LeftOrRight - 4);
    int d = s.IJKDir;
    if (sweep == -1) {
        for (int K = s.Kbgn; K <= s.Kend; ++K)
        for (int J = s.Jbgn; J <= s.Jend; ++J)
        for (int I = s.Ibgn; I <= s.Iend; ++I) {
            int is = I + s.Siadd, js = J + s.Sjadd, ks = K + s.Skadd;
            double Sout1 = b.SD(d, 1, is, js, ks) / b.Grad(d, is, js, ks);
            double Sout2 = b.SD(d, 2, is, js, ks) / b.Grad(d, is, js, ks);
            double Sout3 = b.SD(d, 3, is, js, ks) / b.Grad(d, is, js, ks);
            double Dnx = Sout1 * out_n, Dny = Sout2 * out_n, Dnz = Sout3 * out_n;
            is = I + s.iadd; js = J + s.jadd; ks = K + s.kadd;
            double Den = b.V(1, is, js, ks);
            double Vxi = b.V(2, is, js, ks) / Den;
            double Vyi = b.V(3, is, js, ks) / Den;
            double Vzi = b.V(4, is, js, ks) / Den;
            double P2 = b.PP(is, js, ks);
            double PP0 = 0, Den0 = 0, Vx0 = 0, Vy0 = 0, Vz0 = 0, dir = 0;
            bc_farbond(p.XM, P2, Den, Vxi, Vyi, Vzi, Dnx, Dny, Dnz, p.VxF, p.VyF, p.VzF, PP0, Den0, Vx0, Vy0, Vz0, dir);
            int il = I + s.Eiadd, jl = J + s.Ejadd, kl = K + s.Ekadd;
            b.V(1, il, jl, kl) = 2 * Den0 - b.V(1, is, js, ks);
            double den = b.V(1, il, jl, kl);
            b.V(2, il, jl, kl) = 2.0 * Vx0 - Vxi;
            b.V(3, il, jl, kl) = 2.0 * Vy0 - Vyi;
            b.V(4, il, jl, kl) = 2.0 * Vz0 - Vzi;
            b.PP(il, jl, kl) = 2.0 * PP0 - P2;
            b.T(il, jl, kl) = p.RXM2 * b.PP(il, jl, kl) / den;
            const int E[2][3] = {{s.Eiadd1, s.Ejadd1, s.Ekadd1}, {s.Eiadd2, s.Ejadd2, s.Ekadd2}};
            for (int L = 0; L < 2; ++L) {
                int ig = I + E[L][0], jg = J + E[L][1], kg = K + E[L][2];
                for (int m = 1; m <= 5; ++m) b.V(m, ig, jg, kg) = b.V(m, il, jl, kl);
                b.PP(ig, jg, kg) = b.PP(il, jl, kl);
                b.T(ig, jg, kg) = b.T(il, jl, kl);
            }
            if (c.IF_turb) {
                if (dir > 0.0) {
                    b.V(6, il, jl, kl) = b.V(6, is, js, ks);
                    b.V(7, il, jl, kl) = b.V(7, is, js, ks);
                    b.Rmiu(il, jl, kl) = b.Rmiu(is, js, ks);
                } else {
                    double TT = b.T(il, jl, kl);
                    double Dn = b.V(1, il, jl, kl);
                    double RmiuFar = (1.0 + p.Csthlnd) / (TT * p.Csth1 + p.Csthlnd) * p15(p.Csth1 * TT);
                    b.Rmiu(il, jl, kl) = 2.0 * p.VisRatio * RmiuFar - b.Rmiu(is, js, ks);
                    b.V(6, il, jl, kl) = 2.0 * 1.5 * p.FSTI * p.FSTI * Dn - b.V(6, is, js, ks);
                    b.V(7, il, jl, kl) = b.V(6, il, jl, kl) / (b.Rmiu(il, jl, kl) + p.Tiny) * Dn;
                }
                for (int L = 0; L < 2; ++L) {
                    int ig = I + E[L][0], jg = J + E[L][1], kg = K + E[L][2];
                    b.V(6, ig, jg, kg) = b.V(6, il, jl, kl);
                    b.V(7, ig, jg, kg) = b.V(7, il, jl, kl);
                    b.Rmiu(ig, jg, kg) = b.Rmiu(il, jl, kl);
                }
            }
        }
    } else {
        for (int K = s.Kbgn; K <= s.Kend; ++K)
        for (int J = s.Jbgn; J <= s.Jend; ++J)
        for (int I = s.Ibgn; I <= s.Iend; ++I) {
            int is = I + s.iadd, js = J + s.jadd, ks = K + s.kadd;
            int il = I + s.Eiadd, jl = J + s.Ejadd, kl = K + s.Ekadd;
            for (int L = 1; L <= 18; ++L) b.DQ(L, il, jl, kl) = b.DQ(L, is, js, ks);
        }
    }
}

// BC/BC_Symm.F90:1-131
void bc_symm(Ctx& c, Blk& b, const trans_conn& a, int sweep) {
    SegIdx s(a);
    int d = s.IJKDir;
    if (sweep == -1) {
        for (int K = s.Kbgn; K <= s.Kend; ++K)
        for (int J = s.Jbgn; J <= s.Jend; ++J)
        for (int I = s.Ibgn; I <= s.Iend; ++I) {
            int is = I + s.Siadd, js = J + s.Sjadd, ks = K + s.Skadd;
            double Sout1 = b.SD(d, 1, is, js, ks) / b.Grad(d, is, js, ks);
            double Sout2 = b.SD(d, 2, is, js, ks) / b.Grad(d, is, js, ks);
            double Sout3 = b.SD(d, 3, is, js, ks) / b.Grad(d, is, js, ks);
            is = I + s.iadd; js = J + s.jadd; ks = K + s.kadd;
            double den = b.V(1, is, js, ks);
            double Vxi = b.V(2, is, js, ks) / den, Vyi = b.V(3, is, js, ks) / den, Vzi = b.V(4, is, js, ks) / den;
            double Vc1 = Vxi * Sout1 + Vyi * Sout2 + Vzi * Sout3;
            int il = I + s.Eiadd, jl = J + s.Ejadd, kl = K + s.Ekadd;
            b.V(1, il, jl, kl) = b.V(1, is, js, ks);
            b.V(2, il, jl, kl) = b.V(2, is, js, ks) - 2 * Sout1 * Vc1 * b.V(1, is, js, ks);
            b.V(3, il, jl, kl) = b.V(3, is, js, ks) - 2 * Sout2 * Vc1 * b.V(1, is, js, ks);
            b.V(4, il, jl, kl) = b.V(4, is, js, ks) - 2 * Sout3 * Vc1 * b.V(1, is, js, ks);
            b.V(5, il, jl, kl) = b.V(5, is, js, ks);
            b.PP(il, jl, kl) = b.PP(is, js, ks);
            b.T(il, jl, kl) = b.T(is, js, ks);
            is = I + s.iadd1; js = J + s.jadd1; ks = K + s.kadd1;
            il = I + s.Eiadd1; jl = J + s.Ejadd1; kl = K + s.Ekadd1;
            // the reference does not set V(1) of the second ghost layer (BC/BC_Symm.F90:70-75)
            b.V(2, il, jl, kl) = b.V(2, is, js, ks) - 2 * Sout1 * Vc1 * b.V(1, is, js, ks);
            b.V(3, il, jl, kl) = b.V(3, is, js, ks) - 2 * Sout2 * Vc1 * b.V(1, is, js, ks);
            b.V(4, il, jl, kl) = b.V(4, is, js, ks) - 2 * Sout3 * Vc1 * b.V(1, is, js, ks);
            b.V(5, il, jl, kl) = b.V(5, is, js, ks);
            b.PP(il, jl, kl) = b.PP(is, js, ks);
            b.T(il, jl, kl) = b.T(is, js, ks);
            is = I + s.iadd2; js = J + s.jadd2; ks = K + s.kadd2;
            il = I + s.Eiadd2; jl = J + s.Ejadd2; kl = K + s.Ekadd2;
            b.V(1, il, jl, kl) = b.V(1, is, js, ks);
            b.V(2, il, jl, kl) = b.V(2, is, js, ks) - 2 * Sout1 * Vc1 * b.V(1, is, js, ks);
            b.V(3, il, jl, kl) = b.V(3, is, js, ks) - 2 * Sout2 * Vc1 * b.V(1, is, js, ks);
            b.V(4, il, jl, kl) = b.V(4, is, js, ks) - 2 * Sout3 * Vc1 * b.V(1, is, js, ks);
            b.V(5, il, jl, kl) = b.V(5, is, js, ks);
            b.PP(il, jl, kl) = b.PP(is, js, ks);
            b.T(il, jl, kl) = b.T(is, js, ks);
            if (c.IF_turb) {
                const int A[3][6] = {{s.iadd, s.jadd, s.kadd, s.Eiadd, s.Ejadd, s.Ekadd},
                                     {s.iadd1, s.jadd1, s.kadd1, s.Eiadd1, s.Ejadd1, s.Ekadd1},
                                     {s.iadd2, s.jadd2, s.kadd2, s.Eiadd2, s.Ejadd2, s.Ekadd2}};
                for (int L = 0; L < 3; ++L) {
                    is = I + A[L][0]; js = J + A[L][1]; ks = K + A[L][2];
                    il = I + A[L][3]; jl = J + A[L][4]; kl = K + A[L][5];
                    b.V(6, il, jl, kl) = b.V(6, is, js, ks);
                    b.V(7, il, jl, kl) = b.V(7, is, js, ks);
                    b.Rmiu(il, jl, kl) = b.Rmiu(is, js, ks);
                }
            }
        }
    } else {
        for (int K = s.Kbgn; K <= s.Kend; ++K)
        for (int J = s.Jbgn; J <= s.Jend; ++J)
        for (int I = s.Ibgn; I <= s.Iend; ++I) {
            int is = I + s.iadd, js = J + s.jadd, ks = K + s.kadd;
            int il = I + s.Eiadd, jl = J + s.Ejadd, kl = K + s.Ekadd;
            for (int L = 1; L <= 18; ++L) b.DQ(L, il, jl, kl) = b.DQ(L, is, js, ks);
        }
    }
}

// BC/BC_Inlet.F90:1-125
void bc_inlet(Ctx& c, Blk& b, const trans_conn& a, int sweep) {
    const trans_params& p = c.p;
    SegIdx s(a);
    if (sweep == -1) {
        for (int K = s.Kbgn; K <= s.Kend; ++K)
        for (int J = s.Jbgn; J <= s.Jend; ++J)
        for (int I = s.Ibgn; I <= s.Iend; ++I) {
            int is = I + s.iadd, js = J + s.jadd, ks = K + s.kadd;
            int il = I + s.Eiadd, jl = J + s.Ejadd, kl = K + s.Ekadd;
            double PsIn = b.PP(is, js, ks);
            PsIn = std::min(PsIn, 0.999 * p.P0in);
            double comm = std::max(1.0, otm::pow_(p.P0in / PsIn, 1.0 / 3.5));
            double mach = std::sqrt((comm - 1.0) * 2 / 0.4);
            double TsIn = p.T0in / comm;
            double Roin = p.RXM2 * PsIn / TsIn;
            double asonic = std::sqrt(1.4 * PsIn / Roin);
            double Vabs = mach * asonic;
            double VxInlet = Vabs;
            double VyInlet = p.omega[0] * (b.Zc(is, js, ks));
            double VzInlet = -p.omega[0] * b.Yc(is, js, ks);
            b.V(1, il, jl, kl) = Roin;
            b.V(2, il, jl, kl) = Roin * VxInlet;
            b.V(3, il, jl, kl) = Roin * VyInlet;
            b.V(4, il, jl, kl) = Roin * VzInlet;
            b.V(5, il, jl, kl) = PsIn / 0.4 + 0.5 * (sq(b.V(2, il, jl, kl)) + sq(b.V(3, il, jl, kl)) + sq(b.V(4, il, jl, kl))) / Roin
                                 - 0.5 * sq(p.omega[0] * b.rad(il, jl, kl)) * Roin;
            b.PP(il, jl, kl) = PsIn;
            b.T(il, jl, kl) = TsIn;
            int i0 = il, j0 = jl, k0 = kl;
            const int E[2][3] = {{s.Eiadd1, s.Ejadd1, s.Ekadd1}, {s.Eiadd2, s.Ejadd2, s.Ekadd2}};
            for (int L = 0; L < 2; ++L) {
                int ig = I + E[L][0], jg = J + E[L][1], kg = K + E[L][2];
                for (int m = 1; m <= 5; ++m) b.V(m, ig, jg, kg) = b.V(m, i0, j0, k0);
                b.PP(ig, jg, kg) = PsIn;
                b.T(ig, jg, kg) = TsIn;
            }
            if (c.IF_turb) {
                double TT = b.T(il, jl, kl);
                double RmiuIn = (1.0 + p.Csthlnd) / (TT * p.Csth1 + p.Csthlnd) * p15(p.Csth1 * TT);
                b.Rmiu(il, jl, kl) = p.VisRatio * RmiuIn;
                double Den = b.V(1, il, jl, kl);
                b.V(6, il, jl, kl) = 1.5 * p.FSTI * p.FSTI * Den;
                b.V(7, il, jl, kl) = b.V(6, il, jl, kl) / (b.Rmiu(il, jl, kl) + p.Tiny) * Den;
                for (int L = 0; L < 2; ++L) {
                    int ig = I + E[L][0], jg = J + E[L][1], kg = K + E[L][2];
                    b.V(6, ig, jg, kg) = b.V(6, i0, j0, k0);
                    b.V(7, ig, jg, kg) = b.V(7, i0, j0, k0);
                    b.Rmiu(ig, jg, kg) = b.Rmiu(i0, j0, k0);
                }
            }
        }
    } else {
        for (int K = s.Kbgn; K <= s.Kend; ++K)
        for (int J = s.Jbgn; J <= s.Jend; ++J)
        for (int I = s.Ibgn; I <= s.Iend; ++I) {
            int is = I + s.iadd, js = J + s.jadd, ks = K + s.kadd;
            int il = I + s.Eiadd, jl = J + s.Ejadd, kl = K + s.Ekadd;
            for (int L = 1; L <= 18; ++L) b.DQ(L, il, jl, kl) = b.DQ(L, is, js, ks);
        }
    }
}

// BC/BC_Outlet.F90:1-109
void bc_outlet(Ctx& c, Blk& b, const trans_conn& a, int sweep) {
    const trans_params& p = c.p;
    SegIdx s(a);
    if (sweep == 0) {
        for (int K = s.Kbgn; K <= s.Kend; ++K)
        for (int J = s.Jbgn; J <= s.Jend; ++J)
        for (int I = s.Ibgn; I <= s.Iend; ++I) {
            int is = I + s.iadd, js = J + s.jadd, ks = K + s.kadd;
            int il = I + s.Eiadd, jl = J + s.Ejadd, kl = K + s.Ekadd;
            for (int L = 1; L <= 18; ++L) b.DQ(L, il, jl, kl) = b.DQ(L, is, js, ks);
        }
        return;
    }
    for (int K = s.Kbgn; K <= s.Kend; ++K)
    for (int J = s.Jbgn; J <= s.Jend; ++J)
    for (int I = s.Ibgn; I <= s.Iend; ++I) {
        int is = I + s.iadd, js = J + s.jadd, ks = K + s.kadd;
        int il = I + s.Eiadd, jl = J + s.Ejadd, kl = K + s.Ekadd;
        b.T(il, jl, kl) = b.T(is, js, ks);
        if (J == s.Jbgn) {
            b.PP(il, jl, kl) = p.Pouthub;
        } else {
            double rcs1 = b.rad(il, jl, kl);
            double rcs2 = b.rad(il, jl - 1, kl);
            double sinr = std::sin(b.thtc(il, jl - 1, kl));
            double cosr = std::cos(b.thtc(il, jl - 1, kl));
            double den = b.V(1, il, jl - 1, kl);
            double RoVr2 = sq(b.V(4, il, jl - 1, kl) / den * cosr - sinr * b.V(3, il, jl - 1, kl) / den + p.omega[0] * rcs2);
            b.PP(il, jl, kl) = b.PP(il, jl - 1, kl) + std::fabs((rcs1 - rcs2) * den * RoVr2) / (rcs2 + p.Tiny);
        }
        b.V(1, il, jl, kl) = b.PP(il, jl, kl) / b.T(il, jl, kl) * p.RXM2;
        double den_ratio = b.V(1, il, jl, kl) / b.V(1, is, js, ks);
        b.V(2, il, jl, kl) = b.V(2, is, js, ks) * den_ratio;
        b.V(3, il, jl, kl) = b.V(3, is, js, ks) * den_ratio;
        b.V(4, il, jl, kl) = b.V(4, is, js, ks) * den_ratio;
        const int E[2][3] = {{s.Eiadd1, s.Ejadd1, s.Ekadd1}, {s.Eiadd2, s.Ejadd2, s.Ekadd2}};
        for (int L = 0; L < 2; ++L) {
            int ig = I + E[L][0], jg = J + E[L][1], kg = K + E[L][2];
            for (int m = 1; m <= 4; ++m) b.V(m, ig, jg, kg) = b.V(m, il, jl, kl);
            b.PP(ig, jg, kg) = b.PP(il, jl, kl);
            b.T(ig, jg, kg) = b.T(il, jl, kl);
        }
        if (c.IF_turb) {
            b.V(6, il, jl, kl) = b.V(6, is, js, ks);
            b.V(7, il, jl, kl) = b.V(7, is, js, ks);
            b.Rmiu(il, jl, kl) = b.Rmiu(is, js, ks);
            for (int L = 0; L < 2; ++L) {
                int ig = I + E[L][0], jg = J + E[L][1], kg = K + E[L][2];
                b.V(6, ig, jg, kg) = b.V(6, il, jl, kl);
                b.V(7, ig, jg, kg) = b.V(7, il, jl, kl);
                b.Rmiu(ig, jg, kg) = b.Rmiu(il, jl, kl);
            }
        }
    }
}

// Geom/startup.F90:1-25
void ijk_start_end(int I, int J, int K, int& Is, int& Js, int& Ks, const int* TL, const int* TT, int lcross) {
    int ft1 = TL[0], ft2 = TL[1], ft3 = TL[2];
    int gt1 = TT[0], gt2 = TT[1], gt3 = TT[2];
    int lcross1 = 1 - lcross;
    int temp1 = ft1 * I + ft2 * J + ft3 * K;
    int temp2 = ft1 * (J * lcross1 + K * lcross) + ft2 * (I * lcross1 + K * lcross) + ft3 * (I * lcross1 + J * lcross);
    int temp3 = ft1 * (J * lcross + K * lcross1) + ft2 * (I * lcross + K * lcross1) + ft3 * (I * lcross + J * lcross1);
    Is = gt1 * temp1 + (gt2 + gt3) * temp2;
    Js = gt2 * temp1 + gt1 * temp2 + gt3 * temp3;
    Ks = gt3 * temp1 + (gt1 + gt2) * temp3;
}

// BC/BC_P2P.F90:1-186 (same-rank interface at full precision)
void bc_p2p(Ctx& c, Blk& b, const trans_conn& a, Blk& r, int sweep) {
    SegIdx s(a);
    const trans_conn& bc = r.conn[a.TargetConn - 1];
    SegIdx t(bc);
    int IIadd = s.Iend - s.Ibgn + 2, JJadd = s.Jend - s.Jbgn + 2, KKadd = s.Kend - s.Kbgn + 2;
    double dstage = a.rotateAngle;
    double sint = std::sin(dstage), cost = std::cos(dstage);
    double cos2t = cost * cost, sin2t = sint * sint, sct = sint * cost;
    for (int K = s.Kbgn; K <= s.Kend; ++K)
    for (int J = s.Jbgn; J <= s.Jend; ++J)
    for (int I = s.Ibgn; I <= s.Iend; ++I) {
        int iL = I - s.Ibgn + 1, jL = J - s.Jbgn + 1, kL = K - s.Kbgn + 1;
        iL = a.revMatrix[0] * IIadd + (1 - 2 * a.revMatrix[0]) * iL;
        jL = a.revMatrix[1] * JJadd + (1 - 2 * a.revMatrix[1]) * jL;
        kL = a.revMatrix[2] * KKadd + (1 - 2 * a.revMatrix[2]) * kL;
        int ib, jb, kb;
        ijk_start_end(iL, jL, kL, ib, jb, kb, a.Transform, a.TransformT, a.lcross);
        ib = ib + t.Ibgn - 1; jb = jb + t.Jbgn - 1; kb = kb + t.Kbgn - 1;
        if (sweep == -1) {
            const int S[3][3] = {{t.iadd, t.jadd, t.kadd}, {t.iadd1, t.jadd1, t.kadd1}, {t.iadd2, t.jadd2, t.kadd2}};
            const int E[3][3] = {{s.Eiadd, s.Ejadd, s.Ekadd}, {s.Eiadd1, s.Ejadd1, s.Ekadd1}, {s.Eiadd2, s.Ejadd2, s.Ekadd2}};
            for (int L = 0; L < 3; ++L) {
                int is = ib + S[L][0], js = jb + S[L][1], ks = kb + S[L][2];
                int il = I + E[L][0], jl = J + E[L][1], kl = K + E[L][2];
                b.V(1, il, jl, kl) = r.V(1, is, js, ks);
                b.V(2, il, jl, kl) = r.V(2, is, js, ks);
                double txy = r.V(3, is, js, ks), txz = r.V(4, is, js, ks);
                b.V(3, il, jl, kl) = cost * txy + sint * txz;
                b.V(4, il, jl, kl) = -sint * txy + cost * txz;
                for (int m = 5; m <= 7; ++m) b.V(m, il, jl, kl) = r.V(m, is, js, ks);
                b.PP(il, jl, kl) = r.PP(is, js, ks);
                b.T(il, jl, kl) = r.T(is, js, ks);
                b.Rmiu(il, jl, kl) = r.Rmiu(is, js, ks);
            }
        } else {
            int is = ib + t.iadd, js = jb + t.jadd, ks = kb + t.kadd;
            int il = I + s.Eiadd, jl = J + s.Ejadd, kl = K + s.Ekadd;
            double ugx = r.DQ(1, is, js, ks), ugy = r.DQ(2, is, js, ks), ugz = r.DQ(3, is, js, ks);
            double vgx = r.DQ(4, is, js, ks), vgy = r.DQ(5, is, js, ks), vgz = r.DQ(6, is, js, ks);
            double wgx = r.DQ(7, is, js, ks), wgy = r.DQ(8, is, js, ks), wgz = r.DQ(9, is, js, ks);
            b.DQ(1, il, jl, kl) = ugx;
            b.DQ(2, il, jl, kl) = cost * ugy + sint * ugz;
            b.DQ(3, il, jl, kl) = -sint * ugy + cost * ugz;
            b.DQ(4, il, jl, kl) = cost * vgx + sint * wgx;
            b.DQ(5, il, jl, kl) = cos2t * vgy + sct * (vgz + wgy) + sin2t * wgz;
            b.DQ(6, il, jl, kl) = cos2t * vgz + sct * (-vgy + wgz) - sin2t * wgy;
            b.DQ(7, il, jl, kl) = -sint * vgx + cost * wgx;
            b.DQ(8, il, jl, kl) = -sin2t * vgz + sct * (-vgy + wgz) + cos2t * wgy;
            b.DQ(9, il, jl, kl) = sin2t * vgy + sct * (vgz + wgy) + cos2t * wgz;
            for (int LL = 4; LL <= 6; ++LL) {
                int L = (LL - 1) * 3 + 1;
                b.DQ(L, il, jl, kl) = r.DQ(L, is, js, ks);
                double gy = r.DQ(L + 1, is, js, ks), gz = r.DQ(L + 2, is, js, ks);
                b.DQ(L + 1, il, jl, kl) = cost * gy + sint * gz;
                b.DQ(L + 2, il, jl, kl) = -sint * gy + cost * gz;
            }
        }
    }
}

// BC/Boundary.F90:1-48
void bc_boundarys(Ctx& c, int sweep) {
    // blocks are independent within one BC pass: a 1-to-1 copy reads interior cells only
#pragma omp parallel for schedule(dynamic)
    for (size_t nb = 0; nb < c.B.size(); ++nb) {
        Blk& b = c.B[nb];
        for (auto& a : b.conn) {
            switch (a.BCType) {
                case 1: bc_wall(c, b, a, sweep); break;
                case 2: bc_far(c, b, a, sweep); break;
                case 3: bc_symm(c, b, a, sweep); break;
                case 5: bc_inlet(c, b, a, sweep); break;
                case 7: bc_outlet(c, b, a, sweep); break;
                case 9:
                    for (auto& r : c.B)
                        if (r.id == a.TargetBlock) { bc_p2p(c, b, a, r, sweep); break; }
                    break;
                default: break;
            }
        }
    }
}

// ---------------------------------------------------------------------------------------
// Space/SPACEINTERP_GetSurfCenterVars.F90:22-226
// ---------------------------------------------------------------------------------------
void spaceinterp(Ctx& c, Blk& b) {
    const int di[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int d = 1; d <= 3; ++d) {
        int i0 = d == 1 ? 0 : 1, i1 = d == 1 ? b.NI + 1 : b.NI1;
        int j0 = d == 2 ? 0 : 1, j1 = d == 2 ? b.NJ + 1 : b.NJ1;
        int k0 = d == 3 ? 0 : 1, k1 = d == 3 ? b.NK + 1 : b.NK1;
        for (int k = k0; k <= k1; ++k)
        for (int j = j0; j <= j1; ++j)
        for (int i = i0; i <= i1; ++i) {
            int im = i - di[d - 1][0], jm = j - di[d - 1][1], km = k - di[d - 1][2];
            double Den1 = b.V(1, im, jm, km);
            double U1 = b.V(2, im, jm, km) / Den1, V1 = b.V(3, im, jm, km) / Den1, W1 = b.V(4, im, jm, km) / Den1;
            double P1 = b.PP(im, jm, km), T1 = b.T(im, jm, km);
            double Den = b.V(1, i, j, k);
            double U = b.V(2, i, j, k) / Den, V = b.V(3, i, j, k) / Den, W = b.V(4, i, j, k) / Den;
            double P = b.PP(i, j, k), T = b.T(i, j, k);
            double a0 = b.Alagm(d, i, j, k), a1 = b.Alagm(d, im, jm, km);
            double alsinv = 1.0 / (a0 + a1);
            b.VL(d, 1, i, j, k) = (a0 * U1 + a1 * U) * alsinv;
            b.VL(d, 2, i, j, k) = (a0 * V1 + a1 * V) * alsinv;
            b.VL(d, 3, i, j, k) = (a0 * W1 + a1 * W) * alsinv;
            b.VL(d, 4, i, j, k) = (a0 * P1 + a1 * P) * alsinv;
            b.VL(d, 5, i, j, k) = (a0 * T1 + a1 * T) * alsinv;
            b.rccl(d, i, j, k) = (a0 * b.rad(im, jm, km) + a1 * b.rad(i, j, k)) * alsinv;
            b.rccr(d, i, j, k) = b.rccl(d, i, j, k);
            for (int L = 1; L <= 5; ++L) b.VR(d, L, i, j, k) = b.VL(d, L, i, j, k);
        }
    }
    if (!c.IF_turb) return;
    for (int d = 1; d <= 3; ++d) {
        int i0 = d == 1 ? 0 : 1, i1 = d == 1 ? b.NI + 1 : b.NI1;
        int j0 = d == 2 ? 0 : 1, j1 = d == 2 ? b.NJ + 1 : b.NJ1;
        int k0 = d == 3 ? 0 : 1, k1 = d == 3 ? b.NK + 1 : b.NK1;
        for (int k = k0; k <= k1; ++k)
        for (int j = j0; j <= j1; ++j)
        for (int i = i0; i <= i1; ++i) {
            int im = i - di[d - 1][0], jm = j - di[d - 1][1], km = k - di[d - 1][2];
            double Den1 = b.V(1, im, jm, km);
            double Tkk1 = b.V(6, im, jm, km) / Den1, TOO1 = b.V(7, im, jm, km) / Den1, RmiuT1 = b.Rmiu(im, jm, km);
            double Den = b.V(1, i, j, k);
            double Tkk = b.V(6, i, j, k) / Den, TOO = b.V(7, i, j, k) / Den, RmiuT = b.Rmiu(i, j, k);
            double a0 = b.Alagm(d, i, j, k), a1 = b.Alagm(d, im, jm, km);
            double alsinv = 1.0 / (a0 + a1);
            b.VL(d, 6, i, j, k) = (a0 * Tkk1 + a1 * Tkk) * alsinv;
            b.VL(d, 7, i, j, k) = (a0 * TOO1 + a1 * TOO) * alsinv;
            b.VL(d, 8, i, j, k) = (a0 * RmiuT1 + a1 * RmiuT) * alsinv;
            for (int L = 6; L <= 8; ++L) b.VR(d, L, i, j, k) = b.VL(d, L, i, j, k);
        }
    }
}

// ---------------------------------------------------------------------------------------
// Space/DIFF_DqDxyz.F90:25-396 (gradients of interior cells, shock sensor and its
// extrapolation; the first-ghost-layer gradients of :77-230 are overwritten by
// BC_Boundarys(0) on every boundary face cell and are not restated)
// ---------------------------------------------------------------------------------------
// The hybrid blend Fscheme of one interior cell (Space/DIFF_DqDxyz.F90:311-380), read only by
// the rotated Roe scheme: CH1 = 3, CH2 = 1, CH3 = 2, cmu = 0.09, tau = 1
// (Module_Global.F90:64,105-106,124); real exponents 2 and 3 are products, 0.5 a square root
double fscheme(const trans_params& p, Blk& b, int I, int J, int K, double W12, double W13, double W23, double Vort) {
    (void)W12; (void)W13; (void)W23;
    double DuDx = b.DQ(1, I, J, K), DuDy = b.DQ(2, I, J, K), DuDz = b.DQ(3, I, J, K);
    double DvDx = b.DQ(4, I, J, K), DvDy = b.DQ(5, I, J, K), DvDz = b.DQ(6, I, J, K);
    double DwDx = b.DQ(7, I, J, K), DwDy = b.DQ(8, I, J, K), DwDz = b.DQ(9, I, J, K);
    double S11 = (DuDx + DuDx) / 2., S22 = (DvDy + DvDy) / 2., S33 = (DwDz + DwDz) / 2.;
    double S12 = (DuDy + DvDx) / 2., S13 = (DuDz + DwDx) / 2., S23 = (DwDy + DvDz) / 2.;
    double Skl = std::sqrt(2. * (1. * S11 * S11 + 1. * S22 * S22 + 1. * S33 * S33 + 2. * S12 * S12 + 2. * S13 * S13 + 2. * S23 * S23));
    double Den = b.V(1, I, J, K), RmiuT = b.Rmiu(I, J, K), TT = b.T(I, J, K);
    double RMIUL = (1. + p.Csthlnd) / (TT * p.Csth1 + p.Csthlnd) * p15(p.Csth1 * TT);
    double vK = b.V(6, I, J, K) / Den, vOmega = b.V(7, I, J, K) / Den;
    double DLTxyz = b.ALeng(I, J, K);
    double dTKO = b.DQ(13, I, J, K) * b.DQ(16, I, J, K) + b.DQ(14, I, J, K) * b.DQ(17, I, J, K) + b.DQ(15, I, J, K) * b.DQ(18, I, J, K);
    double Dist = b.Dst(I, J, K);
    double CDKO = std::max(2.0 * Den * p.Sigo2 / vOmega * (dTKO), 1.0e-10);
    double arg1 = std::max(std::sqrt(vK) / p.Beta_star / vOmega / Dist / p.Ref, 500.0 * RMIUL / Den / Dist / Dist / vOmega / p.Ref / p.Ref);
    arg1 = std::min(arg1, 4.0 * Den * p.Sigo2 * vK / CDKO / Dist / Dist);
    double a2 = arg1 * arg1;
    double FunC1 = otm::tanh_(a2 * a2);
    double aLgrd = ((1. - FunC1) * 0.61 + FunC1 * 0.78) * DLTxyz;
    double B0 = 2. * Vort * std::max(Vort, Skl) / std::max((Vort * Vort + Skl * Skl) / 2., p.Alscale * 0.1);
    double g0 = otm::tanh_(B0 * B0 * B0 * B0);
    double sok = std::max(std::sqrt((Vort * Vort + Skl * Skl) / 2.), 0.1 / 1.0);
    double alturb = std::sqrt((RmiuT + RMIUL) / Den / (p.Ref * sok * p15(0.09)));
    double A0 = 1. * std::max(((aLgrd / alturb / g0) - 0.1), 0.0);
    return std::max(1. * otm::tanh_(A0 * A0 * A0), p.F_limiter1);
}

void diff_dqdxyz(Ctx& c, Blk& b) {
    for (int k = 1; k <= b.NK1; ++k)
    for (int j = 1; j <= b.NJ1; ++j)
    for (int i = 1; i <= b.NI1; ++i) {
        double volinv = 1.0 / b.Vol(i, j, k);
        const int var[4] = {1, 2, 3, 5};
        for (int q = 0; q < 4; ++q) {
            int L = var[q];
            double e = b.VL(1, L, i + 1, j, k), w = b.VL(1, L, i, j, k);
            double n = b.VL(2, L, i, j + 1, k), s = b.VL(2, L, i, j, k);
            double t = b.VL(3, L, i, j, k + 1), bo = b.VL(3, L, i, j, k);
            for (int m = 1; m <= 3; ++m)
                b.DQ(3 * q + m, i, j, k) = volinv * (e * b.SD(1, m, i + 1, j, k) - w * b.SD(1, m, i, j, k) + n * b.SD(2, m, i, j + 1, k)
                                                     - s * b.SD(2, m, i, j, k) + t * b.SD(3, m, i, j, k + 1) - bo * b.SD(3, m, i, j, k));
        }
    }
    if (c.IF_turb) {
        for (int k = 1; k <= b.NK1; ++k)
        for (int j = 1; j <= b.NJ1; ++j)
        for (int i = 1; i <= b.NI1; ++i) {
            double volinv = 1.0 / b.Vol(i, j, k);
            for (int q = 0; q < 2; ++q) {
                int L = 6 + q;
                double e = b.VL(1, L, i + 1, j, k), w = b.VL(1, L, i, j, k);
                double n = b.VL(2, L, i, j + 1, k), s = b.VL(2, L, i, j, k);
                double t = b.VL(3, L, i, j, k + 1), bo = b.VL(3, L, i, j, k);
                for (int m = 1; m <= 3; ++m)
                    b.DQ(12 + 3 * q + m, i, j, k) = volinv * (e * b.SD(1, m, i + 1, j, k) - w * b.SD(1, m, i, j, k) + n * b.SD(2, m, i, j + 1, k)
                                                              - s * b.SD(2, m, i, j, k) + t * b.SD(3, m, i, j, k + 1) - bo * b.SD(3, m, i, j, k));
            }
        }
    }
    for (int K = 1; K <= b.NK1; ++K)
    for (int J = 1; J <= b.NJ1; ++J)
    for (int I = 1; I <= b.NI1; ++I) {
        double DuDx = b.DQ(1, I, J, K), DuDy = b.DQ(2, I, J, K), DuDz = b.DQ(3, I, J, K);
        double DvDx = b.DQ(4, I, J, K), DvDy = b.DQ(5, I, J, K), DvDz = b.DQ(6, I, J, K);
        double DwDx = b.DQ(7, I, J, K), DwDy = b.DQ(8, I, J, K), DwDz = b.DQ(9, I, J, K);
        double W12 = (DuDy - DvDx) / 2.0, W13 = (DuDz - DwDx) / 2.0, W23 = (DvDz - DwDy) / 2.0;
        double Vort = std::sqrt(2.0 * (2.0 * W12 * W12 + 2.0 * W13 * W13 + 2.0 * W23 * W23));
        double DivU = std::sqrt(DuDx * DuDx + DvDy * DvDy + DwDz * DwDz);
        b.shock(I, J, K) = DivU * DivU / std::max(DivU * DivU + Vort * Vort, 1.0);
        if (c.p.Kind_Roe == 2) b.Fsch(I, J, K) = fscheme(c.p, b, I, J, K, W12, W13, W23, Vort);
    }
    if (c.p.Kind_Roe == 2) {    // the face-adjacent ghosts of Fscheme (:399-404)
        for (int k = 1; k <= b.NK1; ++k) for (int j = 1; j <= b.NJ1; ++j) {
            b.Fsch(0, j, k) = b.Fsch(1, j, k); b.Fsch(b.NI, j, k) = b.Fsch(b.NI1, j, k);
        }
        for (int k = 1; k <= b.NK1; ++k) for (int i = 1; i <= b.NI1; ++i) {
            b.Fsch(i, 0, k) = b.Fsch(i, 1, k); b.Fsch(i, b.NJ, k) = b.Fsch(i, b.NJ1, k);
        }
        for (int j = 1; j <= b.NJ1; ++j) for (int i = 1; i <= b.NI1; ++i) {
            b.Fsch(i, j, 0) = b.Fsch(i, j, 1); b.Fsch(i, j, b.NK) = b.Fsch(i, j, b.NK1);
        }
    }
    // shock extrapolation into three ghost layers, whole planes in the reference's order
    int lo = -2, hi_i = b.NI + 2, hi_j = b.NJ + 2, hi_k = b.NK + 2;
    for (int L = 1; L <= 3; ++L) {
        for (int k = lo; k <= hi_k; ++k) for (int j = lo; j <= hi_j; ++j) b.shock(1 - L, j, k) = b.shock(1, j, k);
        for (int k = lo; k <= hi_k; ++k) for (int i = lo; i <= hi_i; ++i) b.shock(i, 1 - L, k) = b.shock(i, 1, k);
        for (int j = lo; j <= hi_j; ++j) for (int i = lo; i <= hi_i; ++i) b.shock(i, j, 1 - L) = b.shock(i, j, 1);
        for (int k = lo; k <= hi_k; ++k) for (int j = lo; j <= hi_j; ++j) b.shock(b.NI1 + L, j, k) = b.shock(b.NI1, j, k);
        for (int k = lo; k <= hi_k; ++k) for (int i = lo; i <= hi_i; ++i) b.shock(i, b.NJ1 + L, k) = b.shock(i, b.NJ1, k);
        for (int j = lo; j <= hi_j; ++j) for (int i = lo; i <= hi_i; ++i) b.shock(i, j, b.NK1 + L) = b.shock(i, j, b.NK1);
    }
}

// ---------------------------------------------------------------------------------------
// Space/DIFFUSION_Centered.F90:64-822
// ---------------------------------------------------------------------------------------
void diffusion_centered(Ctx& c, Blk& b) {
    const trans_params& p = c.p;
    const double NMD = -2.0 / 3.0;
    const double prl = 0.72, prte = 0.9;
    for (int d = 1; d <= 3; ++d) {
        const int e[3] = {d == 1, d == 2, d == 3};
        int nI = d == 1 ? b.NI : b.NI1, nJ = d == 2 ? b.NJ : b.NJ1, nK = d == 3 ? b.NK : b.NK1;
        // reference loop orders: I direction J,K,I; J and K directions K,J,I
        int o1n = d == 1 ? nJ : nK, o2n = d == 1 ? nK : nJ;
        for (int o1 = 1; o1 <= o1n; ++o1)
        for (int o2 = 1; o2 <= o2n; ++o2)
        for (int I = 1; I <= nI; ++I) {
            int J = d == 1 ? o1 : o2, K = d == 1 ? o2 : o1;
            int Im = I - e[0], Jm = J - e[1], Km = K - e[2];
            int Ip = I + e[0], Jp = J + e[1], Kp = K + e[2];
            int idx = d == 1 ? I : (d == 2 ? J : K), nmax = d == 1 ? b.NI : (d == 2 ? b.NJ : b.NK);
            int Iswall0 = 0, Iswallm = 0;
            int face0 = 2 * (d - 1), facem = face0 + 1;
            int ma = d == 1 ? J : I, mb = d == 3 ? J : K;
            if (idx == 1 && b.markwall(face0, ma, mb) == 1) Iswall0 = 1;
            if (idx == nmax && b.markwall(facem, ma, mb) == 1) Iswallm = 1;
            double alsinv = 1.0 / (b.Vol(I, J, K) + b.Vol(Im, Jm, Km));
            double all = b.Vol(Im, Jm, Km) * alsinv;
            double alr = b.Vol(I, J, K) * alsinv;
            if (Iswall0 || Iswallm) alsinv = 0.0;
            double g[4][3];   // face gradients of u, v, w, T
            const int vi[4] = {2, 3, 4, 0};
            const int q0[4] = {1, 4, 7, 10};
            for (int q = 0; q < 4; ++q) {
                double gx1 = b.DQ(q0[q], Im, Jm, Km), gy1 = b.DQ(q0[q] + 1, Im, Jm, Km), gz1 = b.DQ(q0[q] + 2, Im, Jm, Km);
                double gx = b.DQ(q0[q], I, J, K), gy = b.DQ(q0[q] + 1, I, J, K), gz = b.DQ(q0[q] + 2, I, J, K);
                double xL = all * gx1 + alr * gx, yL = all * gy1 + alr * gy, zL = all * gz1 + alr * gz;
                int Lv = q < 3 ? q + 1 : 5;
                double disfpp = b.VL(d, Lv, Ip, Jp, Kp);
                double disfnn = b.VL(d, Lv, Im, Jm, Km);
                double disfp, disfn;
                if (q < 3) {
                    disfp = b.V(vi[q], I, J, K) / b.V(1, I, J, K);
                    disfn = b.V(vi[q], Im, Jm, Km) / b.V(1, Im, Jm, Km);
                } else {
                    disfp = b.T(I, J, K);
                    disfn = b.T(Im, Jm, Km);
                }
                double cm[3];
                for (int m = 1; m <= 3; ++m)
                    cm[m - 1] = alsinv * (-b.SD(d, m, Ip, Jp, Kp) * (disfpp - disfp) - b.SD(d, m, Im, Jm, Km) * (disfn - disfnn)
                                          + b.SD(d, m, I, J, K) * (disfp - disfn));
                g[q][0] = cm[0] + xL; g[q][1] = cm[1] + yL; g[q][2] = cm[2] + zL;
            }
            double a0 = b.Alagm(d, I, J, K), a1 = b.Alagm(d, Im, Jm, Km);
            alsinv = 1.0 / (a0 + a1);
            all = a0 * alsinv;
            alr = a1 * alsinv;
            double TTL = b.VL(d, 5, I, J, K);
            double RmiuL = (1.0 + p.Csthlnd) / (TTL * p.Csth1 + p.Csthlnd) * p15(p.Csth1 * TTL);
            double RmiuT = b.Rmiu(I, J, K), RmiuT1 = b.Rmiu(Im, Jm, Km);
            double RmiuTL = all * RmiuT1 + alr * RmiuT;
            if (Iswall0 || Iswallm) RmiuTL = 0.0;
            double DuDxL = g[0][0], DuDyL = g[0][1], DuDzL = g[0][2];
            double DvDxL = g[1][0], DvDyL = g[1][1], DvDzL = g[1][2];
            double DwDxL = g[2][0], DwDyL = g[2][1], DwDzL = g[2][2];
            double DTDxL = g[3][0], DTDyL = g[3][1], DTDzL = g[3][2];
            double TxxLam = RmiuL * (NMD * (DuDxL + DvDyL + DwDzL) + 2.0 * DuDxL);
            double TyyLam = RmiuL * (NMD * (DuDxL + DvDyL + DwDzL) + 2.0 * DvDyL);
            double TzzLam = RmiuL * (NMD * (DuDxL + DvDyL + DwDzL) + 2.0 * DwDzL);
            double TxyLam = RmiuL * (DuDyL + DvDxL);
            double TyzLam = RmiuL * (DvDzL + DwDyL);
            double TzxLam = RmiuL * (DuDzL + DwDxL);
            double TxxTur = RmiuTL * (NMD * (DuDxL + DvDyL + DwDzL) + 2.0 * DuDxL);
            double TyyTur = RmiuTL * (NMD * (DuDxL + DvDyL + DwDzL) + 2.0 * DvDyL);
            double TzzTur = RmiuTL * (NMD * (DuDxL + DvDyL + DwDzL) + 2.0 * DwDzL);
            double TxyTur = RmiuTL * (DuDyL + DvDxL);
            double TyzTur = RmiuTL * (DvDzL + DwDyL);
            double TzxTur = RmiuTL * (DuDzL + DwDxL);
            double Txx = TxxLam + TxxTur, Tyy = TyyLam + TyyTur, Tzz = TzzLam + TzzTur;
            double Txy = TxyLam + TxyTur, Tyz = TyzLam + TyzTur, Tzx = TzxLam + TzxTur;
            double cp = 1.4 * p.PPF / (1.4 - 1.0);
            double akmu = cp * (RmiuL / prl + RmiuTL / prte);
            double ucc = b.VL(d, 1, I, J, K), vcc = b.VL(d, 2, I, J, K), wcc = b.VL(d, 3, I, J, K);
            double Phix = akmu * DTDxL + ucc * Txx + vcc * Txy + wcc * Tzx;
            double Phiy = akmu * DTDyL + ucc * Txy + vcc * Tyy + wcc * Tyz;
            double Phiz = akmu * DTDzL + ucc * Tzx + vcc * Tyz + wcc * Tzz;
            double Dx = b.SD(d, 1, I, J, K), Dy = b.SD(d, 2, I, J, K), Dz = b.SD(d, 3, I, J, K);
            double DIFFro = 0.0;
            double DIFFX = (Txx * Dx + Txy * Dy + Tzx * Dz) / p.Ref;
            double DIFFY = (Txy * Dx + Tyy * Dy + Tyz * Dz) / p.Ref;
            double DIFFZ = (Tzx * Dx + Tyz * Dy + Tzz * Dz) / p.Ref;
            double DIFFE = (Phix * Dx + Phiy * Dy + Phiz * Dz) / p.Ref;
            const double F[5] = {DIFFro, DIFFX, DIFFY, DIFFZ, DIFFE};
            for (int L = 1; L <= 5; ++L) {
                b.D(L, I, J, K) = b.D(L, I, J, K) - F[L - 1];
                b.D(L, Im, Jm, Km) = b.D(L, Im, Jm, Km) + F[L - 1];
            }
        }
    }
    // rotating-frame source (DIFFUSION_Centered.F90:812-822)
    for (int k = 1; k <= b.NK1; ++k)
    for (int j = 1; j <= b.NJ1; ++j)
    for (int i = 1; i <= b.NI1; ++i) {
        double RoW = p.omega[0];
        double ss3 = 2.0 * RoW * b.V(4, i, j, k) + RoW * b.Yc(i, j, k) * p.omega[0] * b.V(1, i, j, k);
        double ss4 = -2.0 * RoW * b.V(3, i, j, k) + RoW * b.Zc(i, j, k) * p.omega[0] * b.V(1, i, j, k);
        b.D(3, i, j, k) = b.D(3, i, j, k) + ss3 * b.Vol(i, j, k);
        b.D(4, i, j, k) = b.D(4, i, j, k) + ss4 * b.Vol(i, j, k);
    }
}

// Space/TURBTWO_DIFFUSION_Centered.F90:57-553
void turbtwo_diffusion(Ctx& c, Blk& b) {
    const trans_params& p = c.p;
    for (int d = 1; d <= 3; ++d) {
        const int e[3] = {d == 1, d == 2, d == 3};
        int nI = d == 1 ? b.NI : b.NI1, nJ = d == 2 ? b.NJ : b.NJ1, nK = d == 3 ? b.NK : b.NK1;
        int o1n = d == 1 ? nJ : nK, o2n = d == 1 ? nK : nJ;
        for (int o1 = 1; o1 <= o1n; ++o1)
        for (int o2 = 1; o2 <= o2n; ++o2)
        for (int I = 1; I <= nI; ++I) {
            int J = d == 1 ? o1 : o2, K = d == 1 ? o2 : o1;
            int Im = I - e[0], Jm = J - e[1], Km = K - e[2];
            int Ip = I + e[0], Jp = J + e[1], Kp = K + e[2];
            int idx = d == 1 ? I : (d == 2 ? J : K), nmax = d == 1 ? b.NI : (d == 2 ? b.NJ : b.NK);
            int Iswall0 = 0, Iswallm = 0;
            int face0 = 2 * (d - 1), facem = face0 + 1;
            int ma = d == 1 ? J : I, mb = d == 3 ? J : K;
            if (idx == 1 && b.markwall(face0, ma, mb) == 1) Iswall0 = 1;
            if (idx == nmax && b.markwall(facem, ma, mb) == 1) Iswallm = 1;
            double alsinv = 1.0 / (b.Vol(I, J, K) + b.Vol(Im, Jm, Km));
            double all = b.Vol(Im, Jm, Km) * alsinv;
            double alr = b.Vol(I, J, K) * alsinv;
            if (Iswall0 || Iswallm) alsinv = 0.0;
            double g[2][3];
            for (int q = 0; q < 2; ++q) {
                int q0 = 13 + 3 * q;
                double gx1 = b.DQ(q0, Im, Jm, Km), gy1 = b.DQ(q0 + 1, Im, Jm, Km), gz1 = b.DQ(q0 + 2, Im, Jm, Km);
                double gx = b.DQ(q0, I, J, K), gy = b.DQ(q0 + 1, I, J, K), gz = b.DQ(q0 + 2, I, J, K);
                double xL = all * gx1 + alr * gx, yL = all * gy1 + alr * gy, zL = all * gz1 + alr * gz;
                int Lv = 6 + q;
                double disfpp = b.VL(d, Lv, Ip, Jp, Kp);
                double disfnn = b.VL(d, Lv, Im, Jm, Km);
                double disfp = b.V(Lv, I, J, K) / b.V(1, I, J, K);
                double disfn = b.V(Lv, Im, Jm, Km) / b.V(1, Im, Jm, Km);
                double cm[3];
                for (int m = 1; m <= 3; ++m)
                    cm[m - 1] = alsinv * (-b.SD(d, m, Ip, Jp, Kp) * (disfpp - disfp) - b.SD(d, m, Im, Jm, Km) * (disfn - disfnn)
                                          + b.SD(d, m, I, J, K) * (disfp - disfn));
                g[q][0] = cm[0] + xL; g[q][1] = cm[1] + yL; g[q][2] = cm[2] + zL;
            }
            double a0 = b.Alagm(d, I, J, K), a1 = b.Alagm(d, Im, Jm, Km);
            alsinv = 1.0 / (a0 + a1);
            all = a0 * alsinv;
            alr = a1 * alsinv;
            double TT = b.T(I, J, K), TT1 = b.T(Im, Jm, Km);
            double TTL = all * TT1 + alr * TT;
            double RmiuL = (1.0 + p.Csthlnd) / (TTL + p.Csthlnd) * p15(TTL);
            double RmiuT = b.Rmiu(I, J, K), RmiuT1 = b.Rmiu(Im, Jm, Km);
            double RmiuTL = all * RmiuT1 + alr * RmiuT;
            if (Iswall0 || Iswallm) RmiuTL = 0.0;
            double SigkAB, SigoAB;
            if (p.Kind_Model == 2) {        // WD+2006: constant sigma (TURBTWO_DIFFUSION_Centered.F90:168-170)
                SigkAB = p.Sigk1;
                SigoAB = p.Sigo1;
            } else {
            double DEN0 = b.V(1, I, J, K);
            double TKK0 = b.V(6, I, J, K) / DEN0, TOO0 = b.V(7, I, J, K) / DEN0;
            double DEN1 = b.V(1, Im, Jm, Km);
            double TKK1 = b.V(6, Im, Jm, Km) / DEN1, TOO1 = b.V(7, Im, Jm, Km) / DEN1;
            double Den = all * DEN1 + alr * DEN0;
            double TKK = all * TKK1 + alr * TKK0;
            double TOO = all * TOO1 + alr * TOO0;
            double dTKO = g[0][0] * g[1][0] + g[0][1] * g[1][1] + g[0][2] * g[1][2];
            double CDKO = std::max(2.0 * Den * p.Sigo2 / TOO * (dTKO), 1.0e-10);
            double distfc = alr * b.Dst(I, J, K) + all * b.Dst(Im, Jm, Km);
            double arg1 = std::max(std::sqrt(TKK) / p.Beta_star / TOO / distfc / p.Ref,
                                   500.0 * RmiuL / Den / distfc / distfc / TOO / p.Ref / p.Ref);
            arg1 = std::min(arg1, 4.0 * Den * p.Sigo2 * TKK / CDKO / distfc / distfc);
            double a2 = arg1 * arg1;
            double fc1c = otm::tanh_(a2 * a2);
            SigkAB = fc1c * p.Sigk1 + (1.0 - fc1c) * p.Sigk2;
            SigoAB = fc1c * p.Sigo1 + (1.0 - fc1c) * p.Sigo2;
            }
            double vmute = RmiuL + RmiuTL * SigkAB;
            double vmuoq = RmiuL + RmiuTL * SigoAB;
            double Dx = b.SD(d, 1, I, J, K), Dy = b.SD(d, 2, I, J, K), Dz = b.SD(d, 3, I, J, K);
            double DIFFTK = (vmute * (g[0][0] * Dx + g[0][1] * Dy + g[0][2] * Dz)) / p.Ref;
            double DIFFTO = (vmuoq * (g[1][0] * Dx + g[1][1] * Dy + g[1][2] * Dz)) / p.Ref;
            b.D(6, I, J, K) = b.D(6, I, J, K) - DIFFTK;
            b.D(6, Im, Jm, Km) = b.D(6, Im, Jm, Km) + DIFFTK;
            b.D(7, I, J, K) = b.D(7, I, J, K) - DIFFTO;
            b.D(7, Im, Jm, Km) = b.D(7, Im, Jm, Km) + DIFFTO;
        }
    }
}

// ---------------------------------------------------------------------------------------
// Space/UTIL_MUSCL.F90:2-18 and Space/CONVECT_MUSCL.F90:30-281
// ---------------------------------------------------------------------------------------
double alimiter(double var1, double var2) {
    const double one = 1.0, epsm = 1.0e-7;
    return (var1 * (var2 * var2 + 2.0 * epsm * epsm) + var2 * (2.0 * var1 * var1 + epsm * epsm)) /
           (2.0 * var1 * var1 - var1 * var2 + 2.0 * var2 * var2 + 3.0 * epsm * epsm) * 0.5 *
           std::fabs(sgn1(var1) * one + sgn1(var2) * one);
}

// Space/UTIL_MUSCL.F90:21-35 (MUSCL2, the limiter of CONVECT_MUSCL2, Kind_Spatial = 1)
double muscl2_limiter(double var1, double var2) {
    const double epsm = 1.0e-6;
    double smooth = (2.0 * var1 * var2 + epsm) / (var1 * var1 + var2 * var2 + epsm);
    return ((1.0 + smooth) * var1 + (1.0 - smooth) * var2) * smooth / 2.0;
}

// CONVECT_MUSCL (Kind_Spatial = 2, limiter alimiter) and CONVECT_MUSCL2
// (Space/CONVECT_MUSCL2.F90:29-291, Kind_Spatial = 1: the same loops with muscl2_limiter)
void convect_muscl(Ctx& c, Blk& b) {
    double (*lim)(double, double) = c.p.Kind_Spatial == 1 ? muscl2_limiter : alimiter;
    for (int i = 0; i <= b.NI + 1; ++i)
    for (int j = 0; j <= b.NJ + 1; ++j)
    for (int k = 0; k <= b.NK + 1; ++k)
    for (int L = 1; L <= 5; ++L)
        for (int d = 1; d <= 3; ++d) b.VR(d, L, i, j, k) = b.VL(d, L, i, j, k);
    for (int d = 1; d <= 3; ++d) {
        const int e[3] = {d == 1, d == 2, d == 3};
        int i0 = 1, i1 = b.NI1, j0 = 1, j1 = b.NJ1, k0 = 1, k1 = b.NK1;
        if (d == 1) { i0 = 0; i1 = b.NI; }
        if (d == 2) { j0 = 0; j1 = b.NJ; }
        if (d == 3) { k0 = 0; k1 = b.NK; }
        for (int k = k0; k <= k1; ++k)
        for (int j = j0; j <= j1; ++j)
        for (int i = i0; i <= i1; ++i) {
            int ip = i + e[0], jp = j + e[1], kp = k + e[2];
            double q[5];
            q[0] = b.V(2, i, j, k) / b.V(1, i, j, k);
            q[1] = b.V(3, i, j, k) / b.V(1, i, j, k);
            q[2] = b.V(4, i, j, k) / b.V(1, i, j, k);
            q[3] = b.PP(i, j, k);
            q[4] = b.T(i, j, k);
            for (int L = 1; L <= 5; ++L) {
                double DR = b.VL(d, L, ip, jp, kp) - q[L - 1];
                double DL = q[L - 1] - b.VR(d, L, i, j, k);
                b.VL(d, L, ip, jp, kp) = q[L - 1] + lim(DR, DL);
                b.VR(d, L, i, j, k) = q[L - 1] - lim(DL, DR);
            }
            double rrr = b.rad(i, j, k);
            double DR = b.rccl(d, ip, jp, kp) - rrr;
            double DL = rrr - b.rccr(d, i, j, k);
            b.rccl(d, ip, jp, kp) = rrr + lim(DR, DL);
            b.rccr(d, i, j, k) = rrr - lim(DL, DR);
        }
    }
}

// Space/TURBTWO_CONVECT_MUSCL.F90:28-141
void turbtwo_convect_muscl(Ctx& c, Blk& b) {
    for (int i = 0; i <= b.NI + 1; ++i)
    for (int j = 0; j <= b.NJ + 1; ++j)
    for (int k = 0; k <= b.NK + 1; ++k)
    for (int L = 6; L <= 7; ++L)
        for (int d = 1; d <= 3; ++d) b.VR(d, L, i, j, k) = b.VL(d, L, i, j, k);
    for (int d = 1; d <= 3; ++d) {
        const int e[3] = {d == 1, d == 2, d == 3};
        int i0 = 1, i1 = b.NI1, j0 = 1, j1 = b.NJ1, k0 = 1, k1 = b.NK1;
        if (d == 1) { i0 = 0; i1 = b.NI; }
        if (d == 2) { j0 = 0; j1 = b.NJ; }
        if (d == 3) { k0 = 0; k1 = b.NK; }
        for (int k = k0; k <= k1; ++k)
        for (int j = j0; j <= j1; ++j)
        for (int i = i0; i <= i1; ++i) {
            int ip = i + e[0], jp = j + e[1], kp = k + e[2];
            for (int L = 6; L <= 7; ++L) {
                double TKK = b.V(L, i, j, k) / b.V(1, i, j, k);
                double DR = b.VL(d, L, ip, jp, kp) - TKK;
                double DL = TKK - b.VR(d, L, i, j, k);
                b.VL(d, L, ip, jp, kp) = TKK + alimiter(DR, DL);
                b.VR(d, L, i, j, k) = TKK - alimiter(DL, DR);
            }
        }
    }
}

// ---------------------------------------------------------------------------------------
// Space/CONVECT_MDCD.F90:41-658 (the stray K-direction rcc block at :450-521 writes one ghost
// element that nothing reads and is not restated)
// ---------------------------------------------------------------------------------------
void mdcd_pair(const double* s6, double gama, double& ql, double& qr) {
    const double beta = std::sqrt(13.0 / 12.0);
    const double epsm = 1.0e-6;
    double aw0 = 1.5 * (0.0463783 + gama);
    double aw1 = 0.5 - 1.5 * 0.0463783 + 4.5 * gama;
    double aw2 = 0.5 - 1.5 * 0.0463783 - 4.5 * gama;
    double aw3 = 1.5 * (0.0463783 - gama);
    {
        double v_2 = s6[0], v_1 = s6[1], v0 = s6[2], v1 = s6[3], v2 = s6[4], v3 = s6[5];
        double ISK1 = sq(0.5 * v_2 - 2.0 * v_1 + 1.5 * v0) + sq(beta * v_2 - 2.0 * beta * v_1 + beta * v0);
        double ISK2 = sq(-0.5 * v_1 + 0.0 * v0 + 0.5 * v1) + sq(beta * v_1 - 2.0 * beta * v0 + beta * v1);
        double ISK3 = sq(-1.5 * v0 + 2.0 * v1 - 0.5 * v2) + sq(beta * v0 - 2.0 * beta * v1 + beta * v2);
        double ISK4 = sq(2.5 * v1 - 4.0 * v2 + 1.5 * v3) + sq(beta * v1 - 2.0 * beta * v2 + beta * v3);
        ISK4 = std::max(std::max(std::max(ISK1, ISK2), ISK3), ISK4);
        double ak1 = aw0 / sq(epsm + ISK1), ak2 = aw1 / sq(epsm + ISK2), ak3 = aw2 / sq(epsm + ISK3), ak4 = aw3 / sq(epsm + ISK4);
        double w0 = ak1 / (ak1 + ak2 + ak3 + ak4), w1 = ak2 / (ak1 + ak2 + ak3 + ak4);
        double w2 = ak3 / (ak1 + ak2 + ak3 + ak4), w3 = ak4 / (ak1 + ak2 + ak3 + ak4);
        double qq0 = 2. / 6. * v_2 - 7. / 6. * v_1 + 11. / 6. * v0;
        double qq1 = -(1. / 6. * v_1) + 5. / 6. * v0 + 2. / 6. * v1;
        double qq2 = 2. / 6. * v0 + 5. / 6. * v1 - 1. / 6. * v2;
        double qq3 = 11. / 6. * v1 - 7. / 6. * v2 + 1. / 3. * v3;
        ql = w0 * qq0 + w1 * qq1 + w2 * qq2 + w3 * qq3;
    }
    {
        double v_3 = s6[0], v_2 = s6[1], v_1 = s6[2], v0 = s6[3], v1 = s6[4], v2 = s6[5];
        double ISK1 = sq(0.5 * v2 - 2.0 * v1 + 1.5 * v0) + sq(beta * v2 - 2.0 * beta * v1 + beta * v0);
        double ISK2 = sq(-0.5 * v1 + 0.0 * v0 + 0.5 * v_1) + sq(beta * v1 - 2.0 * beta * v0 + beta * v_1);
        double ISK3 = sq(-1.5 * v0 + 2.0 * v_1 - 0.5 * v_2) + sq(beta * v0 - 2.0 * beta * v_1 + beta * v_2);
        double ISK4 = sq(2.5 * v_1 - 4.0 * v_2 + 1.5 * v_3) + sq(beta * v_1 - 2.0 * beta * v_2 + beta * v_3);
        ISK4 = std::max(std::max(std::max(ISK1, ISK2), ISK3), ISK4);
        double ak1 = aw0 / sq(epsm + ISK1), ak2 = aw1 / sq(epsm + ISK2), ak3 = aw2 / sq(epsm + ISK3), ak4 = aw3 / sq(epsm + ISK4);
        double w0 = ak1 / (ak1 + ak2 + ak3 + ak4), w1 = ak2 / (ak1 + ak2 + ak3 + ak4);
        double w2 = ak3 / (ak1 + ak2 + ak3 + ak4), w3 = ak4 / (ak1 + ak2 + ak3 + ak4);
        double qq0 = 2. / 6. * v2 - 7. / 6. * v1 + 11. / 6. * v0;
        double qq1 = -(1. / 6. * v1) + 5. / 6. * v0 + 2. / 6. * v_1;
        double qq2 = 2. / 6. * v0 + 5. / 6. * v_1 - 1. / 6. * v_2;
        double qq3 = 11. / 6. * v_1 - 7. / 6. * v_2 + 1. / 3. * v_3;
        qr = w0 * qq0 + w1 * qq1 + w2 * qq2 + w3 * qq3;
    }
}

// CONVECT_MDCD (Kind_Spatial = 3) and CONVECT_MDCDHYB (Space/CONVECT_MDCDHYB.F90:1-477,
// Kind_Spatial = 4): the same MDCD states, replaced by MUSCL states v0 +- alimiter/2 where the
// sensor reaches F_limiter2 (:118-120, :175-177 and the J, K twins); MDCDHYB has neither the rcc
// reconstruction nor the K-direction clamp of the sensor at 0
void convect_mdcd(Ctx& c, Blk& b) {
    const trans_params& p = c.p;
    const bool hyb = p.Kind_Spatial == 4;
    for (int d = 1; d <= 3; ++d) {
        const int e[3] = {d == 1, d == 2, d == 3};
        int nI = d == 1 ? b.NI : b.NI1, nJ = d == 2 ? b.NJ : b.NJ1, nK = d == 3 ? b.NK : b.NK1;
        for (int k = 1; k <= nK; ++k)
        for (int j = 1; j <= nJ; ++j)
        for (int i = 1; i <= nI; ++i) {
            double s6[5][6];
            double sh[6];
            for (int npt = 1; npt <= 6; ++npt) {
                int o = -4 + npt;
                int ii = i + o * e[0], jj = j + o * e[1], kk = k + o * e[2];
                s6[0][npt - 1] = b.V(2, ii, jj, kk) / b.V(1, ii, jj, kk);
                s6[1][npt - 1] = b.V(3, ii, jj, kk) / b.V(1, ii, jj, kk);
                s6[2][npt - 1] = b.V(4, ii, jj, kk) / b.V(1, ii, jj, kk);
                s6[3][npt - 1] = b.PP(ii, jj, kk);
                s6[4][npt - 1] = b.T(ii, jj, kk);
                sh[npt - 1] = b.shock(ii, jj, kk);
            }
            double sensor = std::max(std::max(std::max(std::max(std::max(sh[0], sh[1]), sh[2]), sh[3]), sh[4]), sh[5]);
            if (d == 3 && !hyb) sensor = std::max(sensor, 0.0);
            double gama = p.gama_min + sensor * (p.gama_max - p.gama_min);
            for (int L = 1; L <= 5; ++L) {
                double ql, qr;
                const double* v = s6[L - 1];
                mdcd_pair(v, gama, ql, qr);
                if (hyb && sensor >= p.F_limiter2) {
                    ql = v[2] + 0.5 * alimiter(v[3] - v[2], v[2] - v[1]);
                    qr = v[3] - 0.5 * alimiter(v[3] - v[2], v[4] - v[3]);
                }
                b.VL(d, L, i, j, k) = ql;
                b.VR(d, L, i, j, k) = qr;
            }
            if (d == 3 || hyb) continue;   // K-direction rcc is left at the face average (stray block, :450-521)
            double r6[6];
            for (int npt = 1; npt <= 6; ++npt) {
                int o = -4 + npt;
                r6[npt - 1] = b.rad(i + o * e[0], j + o * e[1], k + o * e[2]);
            }
            double ql, qr;
            mdcd_pair(r6, gama, ql, qr);
            b.rccl(d, i, j, k) = ql;
            b.rccr(d, i, j, k) = qr;
        }
    }
}

// ---------------------------------------------------------------------------------------
// Space/CONVECT_Roe_Original.F90:59-407 (non-preconditioned branch)
// ---------------------------------------------------------------------------------------
void roe_common(const trans_params& p, double PLo, double PRo, double TLo, double TRo, double ULo, double URo,
                double VLo, double VRo, double WLo, double WRo, double sav1, double sav2, double sav3, double sav,
                double rLo, double rRo, double* out, double RmiuT = 0.0, double AlagmR = 1.0) {
    double rcpcv = p.PPF;
    double DENLo = PLo / (rcpcv * TLo), DENRo = PRo / (rcpcv * TRo);
    double ga = 1.4, ga1 = 1.4 - 1.0;
    double VAMLo = ULo * ULo + VLo * VLo + WLo * WLo;
    double VAMRo = URo * URo + VRo * VRo + WRo * WRo;
    double HLo = PLo * ga / (DENLo * ga1) + 0.5 * VAMLo - 0.5 * (rLo * rLo);
    double HRo = PRo * ga / (DENRo * ga1) + 0.5 * VAMRo - 0.5 * (rRo * rRo);
    double acl = std::sqrt(ga * PLo / DENLo), acr = std::sqrt(ga * PRo / DENRo);
    double rrorl = std::sqrt(DENRo / DENLo);
    double rrorlp1 = 1.0 + rrorl;
    double rm = std::sqrt(DENRo * DENLo);
    double um = (ULo + URo * rrorl) / rrorlp1;
    double vm = (VLo + VRo * rrorl) / rrorlp1;
    double wm = (WLo + WRo * rrorl) / rrorlp1;
    double hm = (HLo + HRo * rrorl) / rrorlp1;
    double vm2 = um * um + vm * vm + wm * wm;
    double rccm = (rLo + rrorl * rRo) / rrorlp1;
    double am2 = ga1 * std::fabs(hm - 0.5 * vm2 + 0.5 * (rccm * rccm));
    double am = std::sqrt(am2);
    double sav1n = sav1 / sav, sav2n = sav2 / sav, sav3n = sav3 / sav;
    double unormaln = (sav1n * um + sav2n * vm + sav3n * wm);
    double anormaln = am;
    double dacou = acr - acl;
    (void)dacou;
    double eig1, eig2, eig3, alf, ubetac2, amrev;
    if (p.IF_Precondition) {        // Space/CONVECT_Roe_Original.F90:319-331
        double TTL = am2 / ga / p.PPF;
        ubetac2 = get_precond_para(p, vm2, am2, rm, TTL, RmiuT, AlagmR);
        alf = (1.0 - ubetac2) / 2.0;
        double unrev = unormaln * (1.0 - alf);
        amrev = std::sqrt(pow2r(alf * unormaln) + ubetac2 * am2);
        eig1 = std::fabs(unormaln);
        eig2 = std::fabs(unrev + amrev);
        eig3 = std::fabs(unrev - amrev);
    } else {
        eig1 = std::fabs(unormaln);
        eig2 = std::fabs(unormaln + anormaln);
        eig3 = std::fabs(unormaln - anormaln);
        if (eig1 < 0.1) eig1 = (eig1 * eig1 + 0.1 * 0.1) / 0.2;
        if (eig2 < 0.1) eig2 = (eig2 * eig2 + 0.1 * 0.1) / 0.2;
        if (eig3 < 0.1) eig3 = (eig3 * eig3 + 0.1 * 0.1) / 0.2;
        alf = 0.0;
        ubetac2 = 1.0;
        amrev = am;
    }
    double dunormaln = (sav1n * (URo - ULo) + sav2n * (VRo - VLo) + sav3n * (WRo - WLo));
    double astar = (eig2 + eig3) / 2.0;
    double Mstar = (eig2 - eig3) / 2.0 / amrev;
    double dW1 = DENRo - DENLo;
    double dU1 = URo - ULo, dU2 = VRo - VLo, dU3 = WRo - WLo;
    double dP1 = PRo - PLo;
    double dW2 = rm * dU1 + dW1 * um;
    double dW3 = rm * dU2 + dW1 * vm;
    double dW4 = rm * dU3 + dW1 * wm;
    double dW5 = dP1 / ga1 + 0.5 * vm2 * dW1 + rm * um * dU1 + rm * vm * dU2 + rm * wm * dU3;
    double dUroe = Mstar * dunormaln + (astar - (1 - 2.0 * alf) * eig1 - alf * unormaln * Mstar) * (PRo - PLo) / rm / (ubetac2 * am2);
    double dProe = Mstar * (PRo - PLo) + (astar - eig1 + alf * unormaln * Mstar) * rm * dunormaln;
    double droR1 = eig1 * dW1 + dUroe * rm;
    double drxR1 = eig1 * dW2 + dUroe * rm * um + dProe * sav1n;
    double dryR1 = eig1 * dW3 + dUroe * rm * vm + dProe * sav2n;
    double drzR1 = eig1 * dW4 + dUroe * rm * wm + dProe * sav3n;
    double dreR1 = eig1 * dW5 + dUroe * rm * hm + dProe * unormaln;
    double ulnormaln = (sav1n * ULo + sav2n * VLo + sav3n * WLo);
    double urnormaln = (sav1n * URo + sav2n * VRo + sav3n * WRo);
    double rulnormaln = DENLo * ulnormaln, rurnormaln = DENRo * urnormaln;
    out[0] = -0.5 * (rulnormaln + rurnormaln - droR1);
    out[1] = -0.5 * (rulnormaln * ULo + rurnormaln * URo + sav1n * (PLo + PRo) - drxR1);
    out[2] = -0.5 * (rulnormaln * VLo + rurnormaln * VRo + sav2n * (PLo + PRo) - dryR1);
    out[3] = -0.5 * (rulnormaln * WLo + rurnormaln * WRo + sav3n * (PLo + PRo) - drzR1);
    out[4] = -0.5 * (rulnormaln * HLo + rurnormaln * HRo - dreR1);
}

// Space/CONVECT_AUSMPW_Plus.F90:204-317
void ausmpw_common(const trans_params& p, double PLo, double PRo, double TLo, double TRo, double ULo, double URo,
                   double VLo, double VRo, double WLo, double WRo, double sav1, double sav2, double sav3, double sav,
                   double* out) {
    double rcpcv = p.PPF;
    double DENLo = PLo / (rcpcv * TLo), DENRo = PRo / (rcpcv * TRo);
    double sav1n = sav1 / sav, sav2n = sav2 / sav, sav3n = sav3 / sav;
    double ga = 1.4, ga1 = 1.4 - 1.0;
    double VAMLo = ULo * ULo + VLo * VLo + WLo * WLo;
    double VAMRo = URo * URo + VRo * VRo + WRo * WRo;
    double HLo = PLo * ga / (DENLo * ga1) + 0.5 * VAMLo;
    double HRo = PRo * ga / (DENRo * ga1) + 0.5 * VAMRo;
    double ULn = (sav1n * ULo + sav2n * VLo + sav3n * WLo);
    double URn = (sav1n * URo + sav2n * VRo + sav3n * WRo);
    double astar_L = std::sqrt(2 * ga1 * HLo / (ga + 1));
    double astar_R = std::sqrt(2 * ga1 * HRo / (ga + 1));
    double aas_L = astar_L * astar_L / std::max(std::sqrt(VAMLo), astar_L);
    double aas_R = astar_R * astar_R / std::max(std::sqrt(VAMRo), astar_R);
    double Acc = std::min(aas_L, aas_R);
    double MaL = ULn / Acc, MaR = URn / Acc;
    const double c316 = (double)(3 / 16);   // integer division in the reference: 0
    double MaL_plus, pL_plus, MaR_neg, pR_neg;
    if (std::fabs(MaL) > 1.0) {
        MaL_plus = 0.5 * (MaL + std::fabs(MaL));
        pL_plus = 0.5 * (MaL + std::fabs(MaL)) / (MaL + p.Tiny);
    } else {
        MaL_plus = 0.25 * sq(MaL + 1);
        pL_plus = 0.25 * sq(MaL + 1) * (2 - MaL) + c316 * MaL * sq(MaL * MaL - 1);
    }
    if (std::fabs(MaR) > 1.0) {
        MaR_neg = 0.5 * (MaR - std::fabs(MaR));
        pR_neg = 0.5 * (MaR - std::fabs(MaR)) / (MaR + p.Tiny);
    } else {
        MaR_neg = (-1) * 0.25 * sq(MaR - 1);
        pR_neg = 0.25 * sq(MaR - 1) * (2 + MaR) - c316 * MaR * sq(MaR * MaR - 1);
    }
    double pS = pL_plus * PLo + pR_neg * PRo;
    double Mas = MaL_plus + MaR_neg;
    double mn = std::min(PLo / PRo, PRo / PLo);
    double wP = 1.0 - mn * mn * mn;
    double fL = std::fabs(MaL) < 1 ? PLo / (pS + p.Tiny) - 1 : 0.0;
    double fR = std::fabs(MaR) < 1 ? PRo / (pS + p.Tiny) - 1 : 0.0;
    double MMaL_plus, MMaR_neg;
    if (Mas >= 0) {
        MMaL_plus = MaL_plus + MaR_neg * ((1 - wP) * (1 + fR) - fL);
        MMaR_neg = MaR_neg * wP * (1 + fR);
    } else {
        MMaL_plus = MaL_plus * wP * (1 + fL);
        MMaR_neg = MaR_neg + MaL_plus * ((1 - wP) * (1 + fL) - fR);
    }
    out[0] = (-1) * MMaL_plus * Acc * DENLo - MMaR_neg * Acc * DENRo;
    out[1] = (-1) * MMaL_plus * Acc * DENLo * ULo - MMaR_neg * Acc * DENRo * URo - sav1n * (pL_plus * PLo + pR_neg * PRo);
    out[2] = (-1) * MMaL_plus * Acc * DENLo * VLo - MMaR_neg * Acc * DENRo * VRo - sav2n * (pL_plus * PLo + pR_neg * PRo);
    out[3] = (-1) * MMaL_plus * Acc * DENLo * WLo - MMaR_neg * Acc * DENRo * WRo - sav3n * (pL_plus * PLo + pR_neg * PRo);
    out[4] = (-1) * MMaL_plus * Acc * DENLo * HLo - MMaR_neg * Acc * DENRo * HRo;
}

// Roe_Common of the rotated scheme (Space/CONVECT_Roe_Rotated.F90:597-752), non-preconditioned:
// adds 0.5 |A| dQ along (sav1..3)/sav, times sav and the face blend Funscheme, to dr[0..4]
void roe_rot_common(const trans_params& p, double PLo, double PRo, double TLo, double TRo, double ULo, double URo,
                    double VLo, double VRo, double WLo, double WRo, double sav1, double sav2, double sav3, double sav,
                    double rLo, double rRo, double Funscheme, double* dr) {
    double rcpcv = p.PPF;
    double DENLo = PLo / (rcpcv * TLo), DENRo = PRo / (rcpcv * TRo);
    const double ga = 1.4, ga1 = 0.4;
    double VAMLo = ULo * ULo + VLo * VLo + WLo * WLo, VAMRo = URo * URo + VRo * VRo + WRo * WRo;
    double HLo = PLo * ga / (DENLo * ga1) + 0.5 * VAMLo - 0.5 * (rLo * rLo);
    double HRo = PRo * ga / (DENRo * ga1) + 0.5 * VAMRo - 0.5 * (rRo * rRo);
    double rrorl = std::sqrt(DENRo / DENLo), rrorlp1 = 1.0 + rrorl;
    double rm = std::sqrt(DENRo * DENLo);
    double um = (ULo + URo * rrorl) / rrorlp1, vm = (VLo + VRo * rrorl) / rrorlp1, wm = (WLo + WRo * rrorl) / rrorlp1;
    double hm = (HLo + HRo * rrorl) / rrorlp1;
    double vm2 = um * um + vm * vm + wm * wm;
    double rccm = (rLo + rRo * rrorl) / rrorlp1;
    double am2 = ga1 * std::fabs(hm - 0.5 * vm2 + 0.5 * (rccm * rccm));
    double am = std::sqrt(am2);
    double sav1n = sav1 / sav, sav2n = sav2 / sav, sav3n = sav3 / sav;
    double unormaln = (sav1n * um + sav2n * vm + sav3n * wm);
    double anormaln = am;
    double eig1 = std::fabs(unormaln), eig2 = std::fabs(unormaln + anormaln), eig3 = std::fabs(unormaln - anormaln);
    const double alf = 0.0, ubetac2 = 1.0;
    double amrev = am;
    double dunormaln = (sav1n * (URo - ULo) + sav2n * (VRo - VLo) + sav3n * (WRo - WLo));
    double astar = (eig2 + eig3) / 2.0;
    double Mstar = (eig2 - eig3) / 2.0 / amrev;
    double dW1 = DENRo - DENLo, dU1 = URo - ULo, dU2 = VRo - VLo, dU3 = WRo - WLo, dP1 = PRo - PLo;
    double dW2 = rm * dU1 + dW1 * um, dW3 = rm * dU2 + dW1 * vm, dW4 = rm * dU3 + dW1 * wm;
    double dW5 = dP1 / ga1 + 0.5 * vm2 * dW1 + rm * um * dU1 + rm * vm * dU2 + rm * wm * dU3;
    double dUroe = Mstar * dunormaln + (astar - (1 - 2.0 * alf) * eig1 - alf * unormaln * Mstar) * (PRo - PLo) / rm / (ubetac2 * am2);
    double dProe = Mstar * (PRo - PLo) + (astar - eig1 + alf * unormaln * Mstar) * rm * dunormaln;
    double d1[5] = {eig1 * dW1 + dUroe * rm, eig1 * dW2 + dUroe * rm * um + dProe * sav1n,
                    eig1 * dW3 + dUroe * rm * vm + dProe * sav2n, eig1 * dW4 + dUroe * rm * wm + dProe * sav3n,
                    eig1 * dW5 + dUroe * rm * hm + dProe * unormaln};
    for (int L = 0; L < 5; ++L) dr[L] = dr[L] + 0.5 * d1[L] * sav * Funscheme;
}

// CONVECT_Roe_Rotated (Space/CONVECT_Roe_Rotated.F90:59-591): central flux along the face
// normal, then Roe dissipation along the velocity-jump direction n1 and along the rest of the
// face vector (one direction when the jump is below Tiny).  The grid velocities vibc, vjbc,
// vkbc that the reference reads uninitialised (:169, :332, :510) are taken as 0.
void roe_rotated(const trans_params& p, double PLo, double PRo, double TLo, double TRo, double ULo, double URo,
                 double VLo, double VRo, double WLo, double WRo, double sav1, double sav2, double sav3, double sav,
                 double rLo, double rRo, double Funscheme, double* dr) {
    double rcpcv = p.PPF;
    double DENLo = PLo / (rcpcv * TLo), DENRo = PRo / (rcpcv * TRo);
    const double ga = 1.4, ga1 = 0.4;
    double VAMLo = ULo * ULo + VLo * VLo + WLo * WLo, VAMRo = URo * URo + VRo * VRo + WRo * WRo;
    double HLo = PLo * ga / (DENLo * ga1) + 0.5 * VAMLo - 0.5 * (rLo * rLo);
    double HRo = PRo * ga / (DENRo * ga1) + 0.5 * VAMRo - 0.5 * (rRo * rRo);
    double sav1n = sav1 / sav, sav2n = sav2 / sav, sav3n = sav3 / sav;
    const double vbc = 0.0;
    double ulnormaln = (sav1n * ULo + sav2n * VLo + sav3n * WLo);
    double urnormaln = (sav1n * URo + sav2n * VRo + sav3n * WRo);
    double rulnormaln = DENLo * ulnormaln, rurnormaln = DENRo * urnormaln;
    dr[0] = -0.5 * (rulnormaln + rurnormaln) * sav;
    dr[1] = -0.5 * (rulnormaln * ULo + rurnormaln * URo + sav1n * (PLo + PRo)) * sav;
    dr[2] = -0.5 * (rulnormaln * VLo + rurnormaln * VRo + sav2n * (PLo + PRo)) * sav;
    dr[3] = -0.5 * (rulnormaln * WLo + rurnormaln * WRo + sav3n * (PLo + PRo)) * sav;
    dr[4] = -0.5 * (rulnormaln * HLo + rurnormaln * HRo - vbc * (PLo + PRo)) * sav;
    double DeltaU = std::sqrt((URo - ULo) * (URo - ULo) + (VRo - VLo) * (VRo - VLo) + (WRo - WLo) * (WRo - WLo));
    if (DeltaU <= p.Tiny) {
        roe_rot_common(p, PLo, PRo, TLo, TRo, ULo, URo, VLo, VRo, WLo, WRo, sav1, sav2, sav3, sav, rLo, rRo, Funscheme, dr);
        return;
    }
    double n1 = (URo - ULo) / DeltaU, n2 = (VRo - VLo) / DeltaU, n3 = (WRo - WLo) / DeltaU;
    double s = n1 * sav1 + n2 * sav2 + n3 * sav3;
    double sg = sgn1(s);
    n1 = sg * n1; n2 = sg * n2; n3 = sg * n3;
    s = std::fabs(s);
    double a1 = n1 * s, a2 = n2 * s, a3 = n3 * s;
    double b1 = sav1 - a1, b2 = sav2 - a2, b3 = sav3 - a3;
    double sa = std::max(std::sqrt(a1 * a1 + a2 * a2 + a3 * a3), p.Tiny);
    roe_rot_common(p, PLo, PRo, TLo, TRo, ULo, URo, VLo, VRo, WLo, WRo, a1, a2, a3, sa, rLo, rRo, Funscheme, dr);
    double sb = std::max(std::sqrt(b1 * b1 + b2 * b2 + b3 * b3), p.Tiny);
    roe_rot_common(p, PLo, PRo, TLo, TRo, ULo, URo, VLo, VRo, WLo, WRo, b1, b2, b3, sb, rLo, rRo, Funscheme, dr);
}

void convect_inviscid(Ctx& c, Blk& b) {
    const trans_params& p = c.p;
    for (int d = 1; d <= 3; ++d) {
        const int e[3] = {d == 1, d == 2, d == 3};
        int nI = d == 1 ? b.NI : b.NI1, nJ = d == 2 ? b.NJ : b.NJ1, nK = d == 3 ? b.NK : b.NK1;
        for (int k = 1; k <= nK; ++k)
        for (int j = 1; j <= nJ; ++j)
        for (int i = 1; i <= nI; ++i) {
            double ULo = b.VL(d, 1, i, j, k), URo = b.VR(d, 1, i, j, k);
            double VLo = b.VL(d, 2, i, j, k), VRo = b.VR(d, 2, i, j, k);
            double WLo = b.VL(d, 3, i, j, k), WRo = b.VR(d, 3, i, j, k);
            double PLo = b.VL(d, 4, i, j, k), PRo = b.VR(d, 4, i, j, k);
            double TLo = b.VL(d, 5, i, j, k), TRo = b.VR(d, 5, i, j, k);
            double sav1 = b.SD(d, 1, i, j, k), sav2 = b.SD(d, 2, i, j, k), sav3 = b.SD(d, 3, i, j, k);
            double sav = b.Grad(d, i, j, k);
            double f[5];
            if (p.Kind_Roe == 2) {          // dr = the face's flux contribution, already times |S|
                int im = i - e[0], jm = j - e[1], km = k - e[2];
                double Funscheme = (b.Fsch(im, jm, km) + b.Fsch(i, j, k)) / 2.;
                double dr[5];
                // rLo, rRo = rccl, rccr * omega(1) (Space/CONVECT_Roe_Rotated.F90:102-103, 274-275, 446-447)
                double rLo = b.rccl(d, i, j, k) * p.omega[0], rRo = b.rccr(d, i, j, k) * p.omega[0];
                roe_rotated(p, PLo, PRo, TLo, TRo, ULo, URo, VLo, VRo, WLo, WRo, sav1, sav2, sav3, sav, rLo, rRo, Funscheme, dr);
                for (int L = 1; L <= 5; ++L) {
                    b.D(L, i, j, k) = b.D(L, i, j, k) - dr[L - 1];
                    b.D(L, im, jm, km) = b.D(L, im, jm, km) + dr[L - 1];
                }
                continue;
            }
            if (p.Kind_Roe == 1) {
                double rLo = b.rccl(d, i, j, k) * p.omega[0], rRo = b.rccr(d, i, j, k) * p.omega[0];
                // RmiuT = VL(d,8), the face-averaged eddy viscosity (0 while turbulence is off);
                // AlagmR = Alagm(d,i,j,k) (CONVECT_Roe_Original.F90:86-87)
                roe_common(p, PLo, PRo, TLo, TRo, ULo, URo, VLo, VRo, WLo, WRo, sav1, sav2, sav3, sav, rLo, rRo, f,
                           b.VL(d, 8, i, j, k), b.Alagm(d, i, j, k));
            } else {
                ausmpw_common(p, PLo, PRo, TLo, TRo, ULo, URo, VLo, VRo, WLo, WRo, sav1, sav2, sav3, sav, f);
            }
            int im = i - e[0], jm = j - e[1], km = k - e[2];
            for (int L = 1; L <= 5; ++L) {
                b.D(L, i, j, k) = b.D(L, i, j, k) - f[L - 1] * sav;
                b.D(L, im, jm, km) = b.D(L, im, jm, km) + f[L - 1] * sav;
            }
        }
    }
}

// Space/TURBTWO_CONVECT_Upwind.F90:37-122
void turbtwo_convect_upwind(Ctx& c, Blk& b) {
    const trans_params& p = c.p;
    for (int d = 1; d <= 3; ++d) {
        const int e[3] = {d == 1, d == 2, d == 3};
        int nI = d == 1 ? b.NI : b.NI1, nJ = d == 2 ? b.NJ : b.NJ1, nK = d == 3 ? b.NK : b.NK1;
        for (int K = 1; K <= nK; ++K)
        for (int J = 1; J <= nJ; ++J)
        for (int I = 1; I <= nI; ++I) {
            double UL = b.VL(d, 1, I, J, K), UR = b.VR(d, 1, I, J, K);
            double VLl = b.VL(d, 2, I, J, K), VRr = b.VR(d, 2, I, J, K);
            double WL = b.VL(d, 3, I, J, K), WR = b.VR(d, 3, I, J, K);
            double PL = b.VL(d, 4, I, J, K), PR = b.VR(d, 4, I, J, K);
            double TL = b.VL(d, 5, I, J, K), TR = b.VR(d, 5, I, J, K);
            double rcpcv = p.PPF;
            double DENL = PL / (rcpcv * TL), DENR = PR / (rcpcv * TR);
            double sav1 = b.SD(d, 1, I, J, K), sav2 = b.SD(d, 2, I, J, K), sav3 = b.SD(d, 3, I, J, K);
            double ulnormal = (sav1 * UL + sav2 * VLl + sav3 * WL);
            double urnormal = (sav1 * UR + sav2 * VRr + sav3 * WR);
            double rulnormal = DENL * ulnormal, rurnormal = DENR * urnormal;
            double small = 1.e-10;
            double eigTKO = 0.5 * std::max(std::fabs(ulnormal), std::fabs(urnormal));
            double TKL = std::max(b.VL(d, 6, I, J, K), small), TKR = std::max(b.VR(d, 6, I, J, K), small);
            double dTK = -0.5 * (rulnormal * TKL + rurnormal * TKR - eigTKO * (DENR * TKR - DENL * TKL));
            double TOL = std::max(b.VL(d, 7, I, J, K), small), TOR = std::max(b.VR(d, 7, I, J, K), small);
            double dTO = -0.5 * (rulnormal * TOL + rurnormal * TOR - eigTKO * (DENR * TOR - DENL * TOL));
            int Im = I - e[0], Jm = J - e[1], Km = K - e[2];
            b.D(6, I, J, K) = b.D(6, I, J, K) - dTK;
            b.D(6, Im, Jm, Km) = b.D(6, Im, Jm, Km) + dTK;
            b.D(7, I, J, K) = b.D(7, I, J, K) - dTO;
            b.D(7, Im, Jm, Km) = b.D(7, Im, Jm, Km) + dTO;
        }
    }
}

// ---------------------------------------------------------------------------------------
// Space/RC_Correction.F90:19-124 (Kind_RotMod = 1): the rotation/curvature factor f_r1 of the
// SST production, as the reference's build evaluates it (-O2 without -auto: the local arrays
// St2 and Wij are static, zero at load, and the entries the routine never writes -- St2(3,3)
// and the diagonal of Wij -- stay 0).  omega(M) (:107) reads an index M that the routine never
// sets (the loop variable is MM, which runs over 1 only); with the static zero M it would read
// outside omega(1:3).  The restatement reads omega(1), the loop's evident intent; the term is 0
// whenever omega(1) is 0.
// VL(d,v) is what SPACEINTERP_GetSurfCenterVars wrote in this iteration, 0 where it writes
// nothing (the reference zeroes VL at allocation, Input/Read_BlockDimensions.F90:418, and no
// routine writes those entries).  Kind_RotMod = 2 computes f_r2 (:126-171), which no routine
// of the path reads, so it leaves every result unchanged and is not evaluated.
// ---------------------------------------------------------------------------------------
void rc_correction(Ctx& c, Blk& b) {
    const trans_params& p = c.p;
    const double cr1 = 1.0, cr2 = 2.0, cr3 = 1.0;
    for (int K = 1; K <= b.NK1; ++K)
    for (int J = 1; J <= b.NJ1; ++J)
    for (int I = 1; I <= b.NI1; ++I) {
        double St2[4][4] = {}, Wij[4][4] = {};          // 1-based, as the reference indexes them
        double DuDx = b.DQ(1, I, J, K), DuDy = b.DQ(2, I, J, K), DuDz = b.DQ(3, I, J, K);
        double DvDx = b.DQ(4, I, J, K), DvDy = b.DQ(5, I, J, K), DvDz = b.DQ(6, I, J, K);
        double DwDx = b.DQ(7, I, J, K), DwDy = b.DQ(8, I, J, K);
        St2[1][1] = DuDx;
        St2[1][2] = 0.5 * (DuDy + DvDx);
        St2[1][3] = 0.5 * (DuDz + DwDx);
        St2[2][1] = St2[1][2];
        St2[2][2] = DvDy;
        St2[2][3] = 0.5 * (DvDz + DwDy);
        St2[3][1] = St2[1][3];
        St2[3][2] = St2[2][3];
        Wij[1][2] = 0.5 * (DuDy - DvDx);
        Wij[1][3] = 0.5 * (DuDz - DwDx);
        Wij[2][3] = 0.5 * (DvDz - DwDy) - p.omega[0];
        Wij[2][1] = -Wij[1][2];
        Wij[3][1] = -Wij[1][3];
        Wij[3][2] = -Wij[2][3];
        double SSum = 0.0, WSum = 0.0;
        for (int JJ = 1; JJ <= 3; ++JJ)
            for (int II = 1; II <= 3; ++II) {
                SSum = SSum + St2[II][JJ] * St2[II][JJ];
                WSum = WSum + Wij[II][JJ] * Wij[II][JJ];
            }
        SSum = SSum * 2.0;
        WSum = WSum * 2.0;
        double r_bar = 0.0;
        for (int JJ = 1; JJ <= 3; ++JJ)
            for (int II = 1; II <= 3; ++II) {
                int LL1 = (II - 1) * 3 + JJ, LL2 = (JJ - 1) * 3 + II;
                double Sij = b.DQ(LL1, I, J, K) + b.DQ(LL2, I, J, K);
                auto face = [&](int i, int j, int k) {
                    double vol1 = b.Vol(i, j, k) / (b.Vol(i, j, k) + b.Vol(I, J, K));
                    return vol1 * (b.DQ(LL1, i, j, k) + b.DQ(LL2, i, j, k)) + (1.0 - vol1) * Sij;
                };
                double Sijf1 = face(I - 1, J, K), Sijf2 = face(I + 1, J, K);
                double Sijf3 = face(I, J - 1, K), Sijf4 = face(I, J + 1, K);
                double Sijf5 = face(I, J, K - 1), Sijf6 = face(I, J, K + 1);
                double volinv = 1.0 / b.Vol(I, J, K);
                auto U = [&](int v, int i, int j, int k) {     // the VL*SD sum of RC_Correction.F90:95-100
                    return b.VL(1, v, i, j, k) * b.SD(1, v, i, j, k) + b.VL(2, v, i, j, k) * b.SD(2, v, i, j, k) +
                           b.VL(3, v, i, j, k) * b.SD(3, v, i, j, k);
                };
                double DsijDt = U(1, I + 1, J, K) * Sijf2 - U(1, I, J, K) * Sijf1 + U(2, I, J + 1, K) * Sijf4 -
                                U(2, I, J, K) * Sijf3 + U(3, I, J, K + 1) * Sijf6 - U(3, I, J, K) * Sijf5;
                double DsDt = DsijDt * 0.5 * volinv;
                double DsDt2 = 0.0;
                for (int MM = 1; MM <= 1; ++MM)
                    for (int NN = 1; NN <= 3; ++NN) {
                        double epsIMN = 0.5 * (II - MM) * (MM - NN) * (NN - II);
                        double epsJMN = 0.5 * (JJ - MM) * (MM - NN) * (NN - JJ);
                        DsDt2 = DsDt2 + (epsIMN * St2[JJ][NN] + epsJMN * St2[II][NN]) * p.omega[0];
                    }
                DsDt = DsDt + DsDt2;
                for (int KK = 1; KK <= 3; ++KK) r_bar = r_bar + Wij[II][KK] * St2[JJ][KK] * DsDt;
            }
        double Dsum = std::max(SSum, 0.09 * sq(b.V(7, I, J, K) / b.V(1, I, J, K)));
        double r_star = std::sqrt(SSum / WSum);
        r_bar = 2.0 * r_bar / (std::sqrt(WSum) * p15(Dsum));
        double f_rot = (1 + cr1) * 2.0 * r_star / (1.0 + r_star) * (1 - cr3 * otm::atan_(cr2 * r_bar)) - cr1;
        b.Fr1(I, J, K) = std::max(std::min(f_rot, 1.25), 0.0);
    }
}

// ---------------------------------------------------------------------------------------
// Time/TIME_LUSGS.F90:60-768 (non-preconditioned)
// ---------------------------------------------------------------------------------------
void lusgs_adq(double pGam, double pVx, double pVy, double pVz, double aSDx, double aSDy, double aSDz, double pPP,
               double roinv, double AinRo, double AinRx, double AinRy, double AinRz, double AinRe, double* Dif, double vbcc) {
    double VP = pVx * aSDx + pVy * aSDy + pVz * aSDz + vbcc;
    double Ut2 = pVx * pVx + pVy * pVy + pVz * pVz;
    double aSDt = 0.0;
    double Gm1 = pGam - 1.0, Gm2 = pGam - 2.0;
    double AA2 = pGam * pPP * roinv;
    double gUt2 = 0.5 * Gm1 * Ut2;
    Dif[0] = AinRo * aSDt + AinRx * aSDx + AinRy * aSDy + AinRz * aSDz + AinRe * 0.0;
    Dif[1] = AinRo * (aSDx * gUt2 - pVx * VP) + AinRx * (aSDt + VP - aSDx * Gm2 * pVx) + AinRy * (aSDy * pVx - aSDx * Gm1 * pVy)
             + AinRz * (aSDz * pVx - aSDx * Gm1 * pVz) + AinRe * (aSDx * Gm1);
    Dif[2] = AinRo * (aSDy * gUt2 - pVy * VP) + AinRx * (aSDx * pVy - aSDy * Gm1 * pVx) + AinRy * (aSDt + VP - aSDy * Gm2 * pVy)
             + AinRz * (aSDz * pVy - aSDy * Gm1 * pVz) + AinRe * (aSDy * Gm1);
    Dif[3] = AinRo * (aSDz * gUt2 - pVz * VP) + AinRx * (aSDx * pVz - aSDz * Gm1 * pVx) + AinRy * (aSDy * pVz - aSDz * Gm1 * pVy)
             + AinRz * (aSDt + VP - aSDz * Gm2 * pVz) + AinRe * (aSDz * Gm1);
    double GEt1 = 0.5 * Gm2 * Ut2 - AA2 / Gm1;
    double GEt2 = 0.5 * Ut2 + AA2 / Gm1;
    Dif[4] = AinRo * VP * GEt1 + AinRx * (aSDx * GEt2 - Gm1 * pVx * VP) + AinRy * (aSDy * GEt2 - Gm1 * pVy * VP)
             + AinRz * (aSDz * GEt2 - Gm1 * pVz * VP) + AinRe * (aSDt + pGam * VP);
}

// neighbour term of the L (sgn=+1) and U (sgn=-1) sweeps for direction d at neighbour cell (ni,nj,nk);
// (fi,fj,fk)/(gi,gj,gk) are the two faces of the neighbour cell whose metrics are averaged
void lusgs_nb(const trans_params& p, Blk& b, int d, int ni, int nj, int nk, int fi, int fj, int fk, int gi, int gj, int gk,
              double sgn, double* out) {
    double AinRo = b.D(1, ni, nj, nk), AinRx = b.D(2, ni, nj, nk), AinRy = b.D(3, ni, nj, nk);
    double AinRz = b.D(4, ni, nj, nk), AinRe = b.D(5, ni, nj, nk);
    double pRo = b.V(1, ni, nj, nk);
    double roinv = 1.0 / pRo;
    double pVx = b.V(2, ni, nj, nk) * roinv, pVy = b.V(3, ni, nj, nk) * roinv, pVz = b.V(4, ni, nj, nk) * roinv;
    double aSDx = 0.5 * (b.SD(d, 1, fi, fj, fk) + b.SD(d, 1, gi, gj, gk));
    double aSDy = 0.5 * (b.SD(d, 2, fi, fj, fk) + b.SD(d, 2, gi, gj, gk));
    double aSDz = 0.5 * (b.SD(d, 3, fi, fj, fk) + b.SD(d, 3, gi, gj, gk));
    double vbc = 0.5 * (0.0 + 0.0);
    double pPP = b.PP(ni, nj, nk);
    double Dif[5];
    lusgs_adq(1.4, pVx, pVy, pVz, aSDx, aSDy, aSDz, pPP, roinv, AinRo, AinRx, AinRy, AinRz, AinRe, Dif, vbc);
    if (p.IF_Precondition) {        // TIME_LUSGS.F90:235-248 (and every neighbour of both sweeps)
        double pE = b.V(5, ni, nj, nk) * roinv;
        double pTT = b.T(ni, nj, nk);
        double AAc = std::sqrt(1.4 * pPP * roinv);
        double UVW2 = pVx * pVx + pVy * pVy + pVz * pVz;
        double ALL = std::min(std::min(b.Alagm(1, ni, nj, nk), b.Alagm(2, ni, nj, nk)), b.Alagm(3, ni, nj, nk));
        double ubetac2 = get_precond_para(p, UVW2, AAc * AAc, pRo, pTT, b.Rmiu(ni, nj, nk), ALL);
        precond_dw(p, Dif[0], Dif[1], Dif[2], Dif[3], Dif[4], pRo, pVx, pVy, pVz, pE, AAc, ubetac2, pTT);
    }
    double RDSt = b.Rds(d, ni, nj, nk);
    for (int L = 0; L < 5; ++L) {
        if (sgn > 0) out[L] = 0.5 * (Dif[L] + RDSt * b.D(L + 1, ni, nj, nk));
        else out[L] = 0.5 * (Dif[L] - RDSt * b.D(L + 1, ni, nj, nk));
    }
}

void time_lusgs(Ctx& c, Blk& b) {
    const trans_params& p = c.p;
    for (int K = 1; K <= b.NK1; ++K)
    for (int J = 1; J <= b.NJ1; ++J)
    for (int I = 1; I <= b.NI1; ++I)
        for (int L = 1; L <= 5; ++L)
            b.D(L, I, J, K) = b.D(L, I, J, K) / b.Vol(I, J, K) -
                              (3.0 * b.V(L, I, J, K) - 4.0 * b.Wt0(L, I, J, K) + b.Wt1(L, I, J, K)) * 0.5 / p.DT_LUSGS_Main;
    for (int K = 1; K <= b.NK1; ++K)
    for (int J = 1; J <= b.NJ1; ++J)
    for (int I = 1; I <= b.NI1; ++I) {
        double stept = 2.0 * b.Dtm(I, J, K) / (3.0 * b.Dtm(I, J, K) / p.DT_LUSGS_Main + 2.0);
        b.F(1, I, J, K) = 1.0 + (b.Rds(1, I, J, K) + b.Rds(2, I, J, K) + b.Rds(3, I, J, K)) * (stept / b.Vol(I, J, K));
    }
    if (p.IF_Precondition) {        // TIME_LUSGS.F90:113-160: the right-hand side preconditioned
        for (int K = 1; K <= b.NK1; ++K)
        for (int J = 1; J <= b.NJ1; ++J)
        for (int I = 1; I <= b.NI1; ++I) {
            double pRo = b.V(1, I, J, K);
            double roinv = 1.0 / pRo;
            double pVx = b.V(2, I, J, K) * roinv, pVy = b.V(3, I, J, K) * roinv, pVz = b.V(4, I, J, K) * roinv;
            double pE = b.V(5, I, J, K) * roinv;
            double pPP = b.PP(I, J, K), pTT = b.T(I, J, K);
            double AAc = std::sqrt(1.4 * pPP * roinv);
            double UVW2 = pVx * pVx + pVy * pVy + pVz * pVz;
            double ALL = std::min(std::min(b.Alagm(1, I, J, K), b.Alagm(2, I, J, K)), b.Alagm(3, I, J, K));
            double ubetac2 = get_precond_para(p, UVW2, AAc * AAc, pRo, pTT, b.Rmiu(I, J, K), ALL);
            precond_dw(p, b.D(1, I, J, K), b.D(2, I, J, K), b.D(3, I, J, K), b.D(4, I, J, K), b.D(5, I, J, K), pRo, pVx, pVy,
                       pVz, pE, AAc, ubetac2, pTT);
        }
    }
    // L sweep
    for (int K = 1; K <= b.NK1; ++K)
    for (int J = 1; J <= b.NJ1; ++J)
    for (int I = 1; I <= b.NI1; ++I) {
        double stept = 2.0 * b.Dtm(I, J, K) / (3.0 * b.Dtm(I, J, K) / p.DT_LUSGS_Main + 2.0);
        double cvs = stept / b.Vol(I, J, K);
        double Di[5] = {0, 0, 0, 0, 0}, Dj[5] = {0, 0, 0, 0, 0}, Dk[5] = {0, 0, 0, 0, 0};
        if (I != 1) lusgs_nb(p, b, 1, I - 1, J, K, I, J, K, I - 1, J, K, +1, Di);
        if (J != 1) lusgs_nb(p, b, 2, I, J - 1, K, I, J, K, I, J - 1, K, +1, Dj);
        if (K != 1) lusgs_nb(p, b, 3, I, J, K - 1, I, J, K, I, J, K - 1, +1, Dk);
        stept = 2.0 * b.Dtm(I, J, K) / (3.0 * b.Dtm(I, J, K) / p.DT_LUSGS_Main + 2.0);
        for (int L = 1; L <= 5; ++L)
            b.D(L, I, J, K) = (b.D(L, I, J, K) * stept + (Di[L - 1] + Dj[L - 1] + Dk[L - 1]) * cvs) / b.F(1, I, J, K);
    }
    // U sweep
    for (int K = b.NK1; K >= 1; --K)
    for (int J = b.NJ1; J >= 1; --J)
    for (int I = b.NI1; I >= 1; --I) {
        double stept = 2.0 * b.Dtm(I, J, K) / (3.0 * b.Dtm(I, J, K) / p.DT_LUSGS_Main + 2.0);
        double cvs = stept / b.Vol(I, J, K);
        double Di[5] = {0, 0, 0, 0, 0}, Dj[5] = {0, 0, 0, 0, 0}, Dk[5] = {0, 0, 0, 0, 0};
        if (I != b.NI1) lusgs_nb(p, b, 1, I + 1, J, K, I + 2, J, K, I + 1, J, K, -1, Di);
        if (J != b.NJ1) lusgs_nb(p, b, 2, I, J + 1, K, I, J + 2, K, I, J + 1, K, -1, Dj);
        if (K != b.NK1) lusgs_nb(p, b, 3, I, J, K + 1, I, J, K + 2, I, J, K + 1, -1, Dk);
        for (int L = 1; L <= 5; ++L)
            b.D(L, I, J, K) = b.D(L, I, J, K) - (Di[L - 1] + Dj[L - 1] + Dk[L - 1]) * cvs / b.F(1, I, J, K);
    }
}

// ---------------------------------------------------------------------------------------
// Time/TURBTWO_TIME_LUSGS_SST.F90:118-766 and Time/Hybrid_function.F90:1-105 (SST only)
// ---------------------------------------------------------------------------------------
double fsst(const trans_params& p, double Den, double vK, double vOmega, double Dist, double RmiuL, double CDiff) {
    if (p.Kind_SubHY == 0) return 0.0;
    if (p.Kind_SubHY == 1 || p.Kind_SubHY == 3) {
        double arg1 = std::sqrt(vK) / (0.09 * vOmega * Dist * p.Ref);
        double arg2 = 500. * RmiuL / (Den * Dist * Dist * vOmega * p.Ref * p.Ref);
        double arga = std::max(arg1, arg2);
        double temp = std::max(Den * CDiff * p.Ref, 1.0e-10);
        double argb = 4. * Den * 0.856 * vK / (temp * Dist * Dist);
        double arg = std::min(arga, argb);
        return otm::tanh_(arg * arg * arg * arg);
    }
    if (p.Kind_SubHY == 2) {
        double arg1 = 2. * std::sqrt(vK) / (0.09 * vOmega * Dist * p.Ref);
        double arg2 = 500. * RmiuL / (Den * Dist * Dist * vOmega * p.Ref * p.Ref);
        double arg = std::max(arg1, arg2);
        return otm::tanh_(arg * arg);
    }
    return 0.0;
}

// IDDES functions of Time/Hybrid_function.F90:43-105 (Kind_SubHY = 5).  The constants
// akapa_iddes, Cw, Ct, Cl are Module_Global.F90:126; a square (0.41**2., aDst**2.) is the
// product, the correctly rounded power; (Cl**2.*rdl)**10. is the pow of tmath.
// g: the nine velocity gradients dudx, dudy, dudz, dvdx, ..., dwdz.
constexpr double KAPPA_IDDES2 = 0.41 * 0.41, CT_IDDES2 = 1.87 * 1.87, CL_IDDES2 = 5.00 * 5.00, CW_IDDES = 0.15;

double sij_norm(const double* g) {
    double s = g[0] * g[0] + g[1] * g[1] + g[2] * g[2] + g[3] * g[3] + g[4] * g[4] + g[5] * g[5] + g[6] * g[6] +
               g[7] * g[7] + g[8] * g[8];
    s = std::sqrt(s);
    return std::max(s, 1.0e-10);
}

double fd_function(const trans_params& p, double Den1, double RmiuT1, double aDst1, double aLmax1, const double* g) {
    double alpha1 = 0.25 - aDst1 / aLmax1;
    double fb = std::min(2. * otm::exp_(-9.0 * alpha1 * alpha1), 1.);
    double Sij = sij_norm(g);
    double rdt = (RmiuT1 / Den1) / (KAPPA_IDDES2 * (aDst1 * aDst1) * Sij * p.Ref);
    double fdt = 1. - otm::tanh_((8. * rdt) * (8. * rdt) * (8. * rdt));
    return std::max((1. - fdt), fb);
}

double fe_function(const trans_params& p, double Den2, double RmiuT2, double RmiuL2, double aDst2, double aLmax2,
                   const double* g) {
    double alpha2 = 0.25 - aDst2 / aLmax2;
    double fe1 = alpha2 >= 0. ? 2. * otm::exp_(-11.09 * alpha2 * alpha2) : 2. * otm::exp_(-9. * alpha2 * alpha2);
    double Sij = sij_norm(g);
    double rdt = (RmiuT2 / Den2) / (KAPPA_IDDES2 * (aDst2 * aDst2) * Sij * p.Ref);
    double ft = otm::tanh_((CT_IDDES2 * rdt) * (CT_IDDES2 * rdt) * (CT_IDDES2 * rdt));
    double rdl = (RmiuL2 / Den2) / (KAPPA_IDDES2 * (aDst2 * aDst2) * Sij * p.Ref);
    double fl = otm::tanh_(otm::pow_(CL_IDDES2 * rdl, 10.));
    double fe2 = 1. - std::max(ft, fl);
    return fe2 * std::max((fe1 - 1.), 0.);
}

// Wilcox 2006 k-omega sources and diagonal of one cell (Kind_Model = 2,
// Time/TURBTWO_TIME_LUSGS_SST.F90:418-547)
void wd2006_sources(Ctx& c, Blk& b, int I, int J, int K) {
    const trans_params& p = c.p;
    double dudx = b.DQ(1, I, J, K), dudy = b.DQ(2, I, J, K), dudz = b.DQ(3, I, J, K);
    double dvdx = b.DQ(4, I, J, K), dvdy = b.DQ(5, I, J, K), dvdz = b.DQ(6, I, J, K);
    double dwdx = b.DQ(7, I, J, K), dwdy = b.DQ(8, I, J, K), dwdz = b.DQ(9, I, J, K);
    double dtkdx = b.DQ(13, I, J, K), dtkdy = b.DQ(14, I, J, K), dtkdz = b.DQ(15, I, J, K);
    double dtodx = b.DQ(16, I, J, K), dtody = b.DQ(17, I, J, K), dtodz = b.DQ(18, I, J, K);
    double W[3][3], S[3][3];
    W[0][0] = 0.; W[1][1] = 0.; W[2][2] = 0.;
    W[0][1] = 0.5 * (dudy - dvdx); W[0][2] = 0.5 * (dudz - dwdx); W[1][2] = 0.5 * (dvdz - dwdy);
    W[1][0] = -W[0][1]; W[2][0] = -W[0][2]; W[2][1] = -W[1][2];
    S[0][0] = 0.5 * (dudx + dudx); S[1][1] = 0.5 * (dvdy + dvdy); S[2][2] = 0.5 * (dwdz + dwdz);
    S[0][1] = 0.5 * (dudy + dvdx); S[0][2] = 0.5 * (dudz + dwdx); S[1][2] = 0.5 * (dvdz + dwdy);
    S[1][0] = S[0][1]; S[2][0] = S[0][2]; S[2][1] = S[1][2];
    double Div = dudx + dvdy + dwdz;
    double Votg = sq(dudy - dvdx) + sq(dvdz - dwdy) + sq(dwdx - dudz);
    double prod = (2.0 * (dudx * dudx + dvdy * dvdy + dwdz * dwdz) + sq(dudy + dvdx) + sq(dvdz + dwdy) + sq(dwdx + dudz)
                   - 2.0 / 3.0 * Div * Div);
    double tprod = std::min(prod, Votg) * b.Rmiu(I, J, K) / p.Ref;
    double ARo = b.V(1, I, J, K), ARTk = b.V(6, I, J, K), ARTO = b.V(7, I, J, K);
    double tprodl1 = p.Prod_Lmt * p.Beta_star * ARTk * ARTO / ARo * p.Ref;
    tprod = std::min(tprod, tprodl1);
    double SourceP = tprod - 2.0 / 3.0 * std::min(Div, 0.0) * ARTk;
    double SourceN1 = -2.0 / 3.0 * std::max(Div, 0.0) - p.Beta_star * ARTO / ARo * p.Ref;
    double Source = SourceP + SourceN1 * ARTk;
    double CnegTk = std::fabs(SourceN1);
    b.D(6, I, J, K) = b.D(6, I, J, K) + Source;
    tprod = std::min(prod, Votg) / p.Ref;
    double WWSg = 0.;
    for (int ii = 0; ii < 3; ++ii)
        for (int jj = 0; jj < 3; ++jj)
            for (int kk = 0; kk < 3; ++kk) WWSg = WWSg + W[ii][jj] * W[jj][kk] * S[kk][ii];
    double aK_omg = std::fabs(WWSg / otm::pow_(0.09 * ARTO / ARo * p.Ref, 3.));
    double FBeta = (1. + 85. * aK_omg) / (1. + 100. * aK_omg);
    double Beta_06 = p.Beta1 * FBeta;
    double cdif = dtkdx * dtodx + dtkdy * dtody + dtkdz * dtodz;
    double dltCD = cdif <= 0. ? 0. : 0.125;
    SourceP = p.Gama1 * ARo * tprod - 2.0 / 3.0 * p.Gama1 * std::min(Div, 0.0) * ARTO;
    SourceN1 = -2.0 / 3.0 * p.Gama1 * std::max(Div, 0.0) - Beta_06 * ARTO / ARo * p.Ref;
    Source = SourceP + SourceN1 * ARTO;
    double SourceCross = dltCD * ARo * ARo / ARTO / p.Ref * cdif;
    Source = Source + SourceCross;
    double CnegTO = 2.0 * std::fabs(SourceN1);
    b.D(7, I, J, K) = b.D(7, I, J, K) + Source;
    double stept = 2.0 * b.Dtm(I, J, K) / (3.0 * b.Dtm(I, J, K) / p.DT_LUSGS_Main + 2.0);
    b.F(1, I, J, K) = 1. + (b.Rds(1, I, J, K) + b.Rds(2, I, J, K) + b.Rds(3, I, J, K)) * (stept / b.Vol(I, J, K)) + (CnegTk + CnegTO) * stept;
    b.F(2, I, J, K) = b.F(1, I, J, K);
}

// Wilcox 2006 limits and eddy viscosity of the k-omega update (Kind_Model = 2,
// Time/TIME_Update_V.F90:821-858, Time/TIME_RK_V_Update_New.F90:195-232); prod as the caller
// computed it
void wd2006_update(const trans_params& p, Blk& b, int I, int J, int K, double ARTk, double ARTO, double pRo,
                   double RmiuL, double prod) {
    double Dudx = b.DQ(1, I, J, K), Dudy = b.DQ(2, I, J, K), Dudz = b.DQ(3, I, J, K);
    double Dvdx = b.DQ(4, I, J, K), Dvdy = b.DQ(5, I, J, K), Dvdz = b.DQ(6, I, J, K);
    double Dwdx = b.DQ(7, I, J, K), Dwdy = b.DQ(8, I, J, K), Dwdz = b.DQ(9, I, J, K);
    double Sii = Dudx - (Dudx + Dvdy + Dwdz) / 3.;
    double Sjj = Dvdy - (Dudx + Dvdy + Dwdz) / 3.;
    double Skk = Dwdz - (Dudx + Dvdy + Dwdz) / 3.;
    double Sij = (Dudy + Dvdx) / 2.0, Sik = (Dudz + Dwdx) / 2.0, Sjk = (Dvdz + Dwdy) / 2.0;
    double Skl = std::sqrt(1.0 * Sii * Sii + 1.0 * Sjj * Sjj + 1.0 * Skk * Skk + 2.0 * Sij * Sij + 2.0 * Sik * Sik + 2.0 * Sjk * Sjk);
    ARTO = std::max(ARTO, std::sqrt(pRo * std::fabs(prod) / (p.Prod_Lmt * p.Beta_star)) / p.Ref);
    ARTk = std::min(ARTk, 100000.0 * RmiuL * ARTO / pRo);
    b.V(6, I, J, K) = ARTk;
    b.V(7, I, J, K) = ARTO;
    ARTO = std::max(ARTO, 7. / 8. * pRo * std::sqrt(Skl * Skl * 2. / 0.09) / p.Ref);
    b.Rmiu(I, J, K) = ARTk / ARTO * pRo;
}

void turbtwo_lusgs_sst(Ctx& c, Blk& b) {
    const trans_params& p = c.p;
    for (int K = 1; K <= b.NK1; ++K)
    for (int J = 1; J <= b.NJ1; ++J)
    for (int I = 1; I <= b.NI1; ++I)
        for (int L = 6; L <= 7; ++L)
            b.D(L, I, J, K) = b.D(L, I, J, K) / b.Vol(I, J, K) -
                              (3.0 * b.V(L, I, J, K) - 4.0 * b.Wt0(L, I, J, K) + b.Wt1(L, I, J, K)) * 0.5 / p.DT_LUSGS_Main;
    // loop-carried values of the previous interior cell read by the DES length scale
    // (TURBTWO_TIME_LUSGS_SST.F90:198,209); the first cell of the block uses fc1 = 0 and its own omega
    double arg1_prev = 0.0, Vomega_prev = b.V(7, 1, 1, 1) / b.V(1, 1, 1, 1);
    for (int K = 1; K <= b.NK1; ++K)
    for (int J = 1; J <= b.NJ1; ++J)
    for (int I = 1; I <= b.NI1; ++I) {
        if (p.Kind_Model == 2) { wd2006_sources(c, b, I, J, K); continue; }
        double dudx = b.DQ(1, I, J, K), dudy = b.DQ(2, I, J, K), dudz = b.DQ(3, I, J, K);
        double dvdx = b.DQ(4, I, J, K), dvdy = b.DQ(5, I, J, K), dvdz = b.DQ(6, I, J, K);
        double dwdx = b.DQ(7, I, J, K), dwdy = b.DQ(8, I, J, K), dwdz = b.DQ(9, I, J, K);
        double dtkdx = b.DQ(13, I, J, K), dtkdy = b.DQ(14, I, J, K), dtkdz = b.DQ(15, I, J, K);
        double dtodx = b.DQ(16, I, J, K), dtody = b.DQ(17, I, J, K), dtodz = b.DQ(18, I, J, K);
        double Div = dudx + dvdy + dwdz;
        double Votg = sq(dudy - dvdx) + sq(dvdz - dwdy) + sq(dwdx - dudz);
        double prod = (2.0 * (dudx * dudx + dvdy * dvdy + dwdz * dwdz) + sq(dudy + dvdx) + sq(dvdz + dwdy) + sq(dwdx + dudz)
                       - 2.0 / 3.0 * Div * Div);
        double cdif = dtkdx * dtodx + dtkdy * dtody + dtkdz * dtodz;
        double tprod = std::min(prod, Votg) * b.Rmiu(I, J, K) / p.Ref;
        double ARo = b.V(1, I, J, K), ARTk = b.V(6, I, J, K), ARTO = b.V(7, I, J, K);
        double tprodl1 = p.Prod_Lmt * p.Beta_star * ARTk * ARTO / ARo * p.Ref;
        tprod = std::min(tprod, tprodl1);
        double TT = b.T(I, J, K);
        double RmiuL = (1.0 + p.Csthlnd) / (TT * p.Csth1 + p.Csthlnd) * p15(p.Csth1 * TT);
        double Fdes = 1.0;
        double alIDDES = 1.0;
        const bool iddes = p.Kind_Hybrid == 3 && p.Kind_SubHY == 5;
        if (p.Kind_Hybrid == 3) {
            double aLt = std::sqrt(ARTk / ARo) / (p.Beta_star * ARTO / ARo * p.Ref);
            double Cdiff_DDES_S = (2. * 0.856 / Vomega_prev) / p.Ref * cdif;
            double Den = ARo, vk = ARTk / ARo;
            double vOmega = ARTO / ARo;
            Vomega_prev = vOmega;
            double aDst = b.Dst(I, J, K);
            // FSST has no branch for Kind_SubHY = 5 (its result is undefined there); with IDDES the
            // Fdes it feeds is overwritten below before it is used, so 0 stands in for it
            double Fsst_DES = fsst(p, Den, vk, vOmega, aDst, RmiuL, Cdiff_DDES_S);
            double aLgrd = ((1. - arg1_prev) * 0.61 + arg1_prev * 0.78) * b.ALeng(I, J, K);
            Fdes = std::max(aLt * (1. - Fsst_DES) / aLgrd, 1.0);
            b.FunDES(I, J, K) = aLt * (1. - Fsst_DES) / aLgrd;
            if (iddes) {            // Time/TURBTWO_TIME_LUSGS_SST.F90:218-252
                double aLmax = b.ALeng(I, J, K), aLmin = b.ASeng(I, J, K);
                double Cdes = (1. - arg1_prev) * 0.61 + arg1_prev * 0.78;     // Ciddes_epsi, Ciddes_omeg
                double dlt_IDDES = std::min(std::max(std::max(CW_IDDES * aLmax, CW_IDDES * aDst), aLmin), aLmax);
                aLgrd = Cdes * dlt_IDDES;
                const double g[9] = {dudx, dudy, dudz, dvdx, dvdy, dvdz, dwdx, dwdy, dwdz};
                double RmiuT = b.Rmiu(I, J, K);
                double fd = fd_function(p, Den, RmiuT, aDst, aLmax, g);
                double fe = fe_function(p, Den, RmiuT, RmiuL, aDst, aLmax, g);
                alIDDES = (1. + fe) * fd * aLt + (1. - fd) * aLgrd;
                b.FunDES(I, J, K) = aLt / alIDDES;
            }
        }
        double DistN = b.Dst(I, J, K);
        double CDKO = std::max(2.0 * ARo * p.Sigo2 / (ARTO / ARo) * cdif, 1.0e-10);
        double arg1 = std::max(std::sqrt(ARTk / ARo) / p.Beta_star / (ARTO / ARo) / DistN / p.Ref,
                               500.0 * RmiuL / DistN / DistN / ARTO / p.Ref / p.Ref);
        arg1 = std::min(arg1, 4.0 * p.Sigo2 * ARTk / CDKO / DistN / DistN);
        double a2 = arg1 * arg1;
        arg1 = otm::tanh_(a2 * a2);
        arg1_prev = arg1;
        double AA = std::sqrt(1.4 * b.PP(I, J, K) / ARo);
        double Mt = std::sqrt(ARTk / ARo) / AA;
        double Alf1 = 1.0, Alf2 = 0.4, Alf3 = 0.2;
        double f_r1 = b.Fr1(I, J, K);       // 1 unless RCCorrection set it (Kind_RotMod = 1)
        double Source, SourceP, SourceN1, SourceNc, CnegTk, CnegTO;
        double fixsrc = (p.If_fix_Transition && b.Xc(I, J, K) < p.Trans_location) ? 1.0 : 0.0;
        if (p.IF_Comppress == 0) {
            SourceP = tprod - 2.0 / 3.0 * std::min(Div, 0.0) * ARTk;
            SourceP = SourceP * f_r1;
            SourceN1 = -2.0 / 3.0 * std::max(Div, 0.0) - p.Beta_star * ARTO / ARo * p.Ref * Fdes;
            SourceNc = ARTk;
            Source = SourceP + SourceN1 * SourceNc;
            CnegTk = std::fabs(SourceN1);
        } else {
            SourceP = (1. - (1. - arg1) * Alf2 * Mt * Mt) * tprod - 2.0 / 3.0 * std::min(Div, 0.0) * ARTk;
            SourceP = SourceP * f_r1;
            SourceN1 = -2.0 / 3.0 * std::max(Div, 0.0) - (1. + (1. - arg1) * (Alf1 - Alf3) * Mt * Mt) * p.Beta_star * ARTO / ARo * p.Ref * Fdes;
            SourceNc = ARTk;
            Source = SourceP + SourceN1 * SourceNc;
            CnegTk = std::fabs(SourceN1);
        }
        if (fixsrc != 0.0) Source = 0.0;
        if (iddes) {        // the IDDES destruction (TURBTWO_TIME_LUSGS_SST.F90:299-310, 354-366)
            if (p.IF_Comppress == 0)
                SourceN1 = -2.0 / 3.0 * std::max(Div, 0.0) - std::sqrt(ARTk / ARo) / alIDDES;
            else
                SourceN1 = -2.0 / 3.0 * std::max(Div, 0.0) - (1. + (1. - arg1) * (Alf1 - Alf3) * Mt * Mt) * std::sqrt(ARTk / ARo) / alIDDES;
            Source = SourceP + SourceN1 * ARTk;
            CnegTk = std::fabs(-2.0 / 3.0 * std::max(Div, 0.0) - 1.5 * std::sqrt(ARTk / ARo) / alIDDES);
            if (fixsrc != 0.0) Source = 0.0;
        }
        b.D(6, I, J, K) = b.D(6, I, J, K) + Source;
        tprod = std::min(prod, Votg) / p.Ref;
        double GamaAB = p.Gama1 * arg1 + p.Gama2 * (1.0 - arg1);
        double BetaAB = p.Beta1 * arg1 + p.Beta2 * (1.0 - arg1);
        if (p.IF_Comppress == 0) {
            SourceP = GamaAB * ARo * tprod - 2.0 / 3.0 * GamaAB * std::min(Div, 0.0) * ARTO;
            SourceP = SourceP * f_r1;
            SourceN1 = -2.0 / 3.0 * GamaAB * std::max(Div, 0.0) - BetaAB * ARTO / ARo * p.Ref;
        } else {
            SourceP = (GamaAB + (1. - arg1) * Alf2 * Mt * Mt) * ARo * tprod - 2.0 / 3.0 * GamaAB * std::min(Div, 0.0) * ARTO;
            SourceP = SourceP * f_r1;
            SourceN1 = -2.0 / 3.0 * GamaAB * std::max(Div, 0.0) - (1. - (1. - arg1) * (Alf1 - Alf3) * Mt * Mt) * BetaAB * ARTO / ARo * p.Ref;
        }
        SourceNc = ARTO;
        Source = SourceP + SourceN1 * SourceNc;
        double SourceCross = 2.0 * (1 - arg1) * ARo * p.Sigo2 / (ARTO / ARo) * cdif / p.Ref;
        SourceCross = sgn1(SourceCross) * std::min(std::fabs(SourceCross), std::fabs(SourceP) * 0.5);
        Source = Source + SourceCross;
        b.D(7, I, J, K) = b.D(7, I, J, K) + Source;
        CnegTO = 2.0 * std::fabs(SourceN1);
        double stept = 2.0 * b.Dtm(I, J, K) / (3.0 * b.Dtm(I, J, K) / p.DT_LUSGS_Main + 2.0);
        b.F(1, I, J, K) = 1. + (b.Rds(1, I, J, K) + b.Rds(2, I, J, K) + b.Rds(3, I, J, K)) * (stept / b.Vol(I, J, K)) + (CnegTk + CnegTO) * stept;
        b.F(2, I, J, K) = b.F(1, I, J, K);
    }
    auto nb = [&](int d, int ni, int nj, int nk, int fi, int fj, int fk, int gi, int gj, int gk, double sgn, double* out) {
        double pRo = b.V(1, ni, nj, nk);
        double roinv = 1.0 / pRo;
        double pVx = b.V(2, ni, nj, nk) * roinv, pVy = b.V(3, ni, nj, nk) * roinv, pVz = b.V(4, ni, nj, nk) * roinv;
        double aSDx = 0.5 * (b.SD(d, 1, fi, fj, fk) + b.SD(d, 1, gi, gj, gk));
        double aSDy = 0.5 * (b.SD(d, 2, fi, fj, fk) + b.SD(d, 2, gi, gj, gk));
        double aSDz = 0.5 * (b.SD(d, 3, fi, fj, fk) + b.SD(d, 3, gi, gj, gk));
        double VP = pVx * aSDx + pVy * aSDy + pVz * aSDz;
        double DifRTk = b.D(6, ni, nj, nk) * VP, DifRTO = b.D(7, ni, nj, nk) * VP;
        double RDSt = b.Rds(d, ni, nj, nk);
        if (sgn > 0) {
            out[0] = 0.5 * (DifRTk + RDSt * b.D(6, ni, nj, nk));
            out[1] = 0.5 * (DifRTO + RDSt * b.D(7, ni, nj, nk));
        } else {
            out[0] = 0.5 * (DifRTk - RDSt * b.D(6, ni, nj, nk));
            out[1] = 0.5 * (DifRTO - RDSt * b.D(7, ni, nj, nk));
        }
    };
    for (int K = 1; K <= b.NK1; ++K)
    for (int J = 1; J <= b.NJ1; ++J)
    for (int I = 1; I <= b.NI1; ++I) {
        double stept = 2.0 * b.Dtm(I, J, K) / (3.0 * b.Dtm(I, J, K) / p.DT_LUSGS_Main + 2.0);
        double cvs = stept / b.Vol(I, J, K);
        double Di[2] = {0, 0}, Dj[2] = {0, 0}, Dk[2] = {0, 0};
        if (I != 1) nb(1, I - 1, J, K, I, J, K, I - 1, J, K, +1, Di);
        if (J != 1) nb(2, I, J - 1, K, I, J, K, I, J - 1, K, +1, Dj);
        if (K != 1) nb(3, I, J, K - 1, I, J, K, I, J, K - 1, +1, Dk);
        b.D(6, I, J, K) = (b.D(6, I, J, K) * stept + (Di[0] + Dj[0] + Dk[0]) * cvs) / b.F(1, I, J, K);
        b.D(7, I, J, K) = (b.D(7, I, J, K) * stept + (Di[1] + Dj[1] + Dk[1]) * cvs) / b.F(2, I, J, K);
    }
    for (int K = b.NK1; K >= 1; --K)
    for (int J = b.NJ1; J >= 1; --J)
    for (int I = b.NI1; I >= 1; --I) {
        double stept = 2.0 * b.Dtm(I, J, K) / (3.0 * b.Dtm(I, J, K) / p.DT_LUSGS_Main + 2.0);
        double cvs = stept / b.Vol(I, J, K);
        double Di[2] = {0, 0}, Dj[2] = {0, 0}, Dk[2] = {0, 0};
        if (I != b.NI1) nb(1, I + 1, J, K, I + 2, J, K, I + 1, J, K, -1, Di);
        if (J != b.NJ1) nb(2, I, J + 1, K, I, J + 2, K, I, J + 1, K, -1, Dj);
        if (K != b.NK1) nb(3, I, J, K + 1, I, J, K + 2, I, J, K + 1, -1, Dk);
        b.D(6, I, J, K) = b.D(6, I, J, K) - (Di[0] + Dj[0] + Dk[0]) * cvs / b.F(1, I, J, K);
        b.D(7, I, J, K) = b.D(7, I, J, K) - (Di[1] + Dj[1] + Dk[1]) * cvs / b.F(2, I, J, K);
    }
}

// ---------------------------------------------------------------------------------------
// Time/TIME_Update_V.F90:91-908 (norms, non-preconditioned update, SST update)
// ---------------------------------------------------------------------------------------
void time_update_v(Ctx& c, Blk& b) {
    const trans_params& p = c.p;
    b.nrm.nan_flag = 0;
    double DRSa = 0.0, DUa = 0.0;
    int Ima = 0, Jma = 0, Kma = 0;
    for (int K = 1; K <= b.NK1; ++K)
    for (int J = 1; J <= b.NJ1; ++J)
    for (int I = 1; I <= b.NI1; ++I) {
        double DR = std::fabs(b.D(1, I, J, K) / b.V(1, I, J, K));
        if (std::isnan(b.D(1, I, J, K))) b.nrm.nan_flag = 1;
        if (DUa <= DR) { DUa = DR; Ima = I; Jma = J; Kma = K; }
        DRSa = DRSa + DR * DR;
    }
    DRSa = std::sqrt(DRSa / b.NI1 / b.NJ1 / b.NK1);
    double DRSk = 0, DUk = 0, DRSo = 0, DUo = 0;
    for (int K = 1; K <= b.NK1; ++K)
    for (int J = 1; J <= b.NJ1; ++J)
    for (int I = 1; I <= b.NI1; ++I) {
        double DRk = std::fabs(b.D(6, I, J, K) / b.V(1, I, J, K));
        if (DUk <= DRk) DUk = DRk;
        DRSk = DRSk + DRk * DRk;
    }
    DRSk = std::sqrt(DRSk / b.NI1 / b.NJ1 / b.NK1);
    for (int K = 1; K <= b.NK1; ++K)
    for (int J = 1; J <= b.NJ1; ++J)
    for (int I = 1; I <= b.NI1; ++I) {
        double DRo = std::fabs(b.D(7, I, J, K) / b.V(1, I, J, K));
        if (DUo <= DRo) DUo = DRo;
        DRSo = DRSo + DRo * DRo;
    }
    DRSo = std::sqrt(DRSo / b.NI1 / b.NJ1 / b.NK1);
    bool turb_upd = (p.IF_Euler == 0 && c.IF_turb == 1 && c.KI >= p.KItm);
    for (int K = 1; K <= b.NK1; ++K)
    for (int J = 1; J <= b.NJ1; ++J)
    for (int I = 1; I <= b.NI1; ++I) {
        double AinRo = b.D(1, I, J, K), AinRx = b.D(2, I, J, K), AinRy = b.D(3, I, J, K);
        double AinRz = b.D(4, I, J, K), AinRe = b.D(5, I, J, K);
        double pRo = b.V(1, I, J, K);
        double roinv = 1.0 / pRo;
        if (p.IF_Precondition) {
            // TIME_Update_V.F90:580-607: conservative increments; the kinetic energy takes the
            // new momenta with the old 1/rho, and T the old pressure with the new density
            double pRx = b.V(2, I, J, K), pRy = b.V(3, I, J, K), pRz = b.V(4, I, J, K), pRe = b.V(5, I, J, K);
            pRo = pRo + AinRo;
            pRo = std::fabs(pRo);
            pRx = pRx + AinRx; pRy = pRy + AinRy; pRz = pRz + AinRz;
            pRe = pRe + AinRe;
            pRe = std::fabs(pRe);
            double DV = 0.5 * (pRx * pRx + pRy * pRy + pRz * pRz) * roinv;
            double pPP = (pRe - DV) * (1.4 - 1.0);
            if (pPP <= 0.0) {
                pPP = std::fabs(pPP);
                pRe = pPP / (1.4 - 1.0) + DV;
            }
            double pTT = p.RXM2 * b.PP(I, J, K) / pRo;
            b.V(1, I, J, K) = pRo; b.V(2, I, J, K) = pRx; b.V(3, I, J, K) = pRy; b.V(4, I, J, K) = pRz; b.V(5, I, J, K) = pRe;
            b.PP(I, J, K) = pPP;
            b.T(I, J, K) = pTT;
        } else {
        double pVx = b.V(2, I, J, K) * roinv, pVy = b.V(3, I, J, K) * roinv, pVz = b.V(4, I, J, K) * roinv;
        double AinX = (AinRx - pVx * AinRo) * roinv;
        double AinY = (AinRy - pVy * AinRo) * roinv;
        double AinZ = (AinRz - pVz * AinRo) * roinv;
        double AinP = (1.4 - 1.0) * (AinRe - 0.5 * AinRo * (pVx * pVx + pVy * pVy + pVz * pVz) - pRo * (AinX * pVx + AinY * pVy + AinZ * pVz));
        if (AinRo >= 0.) pRo = pRo + AinRo;
        else pRo = pRo * otm::exp_(AinRo / (pRo + 1.e-10));
        pRo = std::fabs(pRo);
        if (AinP >= 0.) b.PP(I, J, K) = b.PP(I, J, K) + AinP;
        else b.PP(I, J, K) = b.PP(I, J, K) * otm::exp_(AinP / (b.PP(I, J, K) + 1.e-10));
        b.PP(I, J, K) = std::fabs(b.PP(I, J, K));
        b.T(I, J, K) = p.RXM2 * b.PP(I, J, K) / pRo;
        pVx = pVx + AinX; pVy = pVy + AinY; pVz = pVz + AinZ;
        b.V(1, I, J, K) = pRo;
        b.V(2, I, J, K) = pRo * pVx;
        b.V(3, I, J, K) = pRo * pVy;
        b.V(4, I, J, K) = pRo * pVz;
        double DV = 0.5 * (pVx * pVx + pVy * pVy + pVz * pVz);
        b.V(5, I, J, K) = b.PP(I, J, K) / (1.4 - 1.0) + DV * pRo - 0.5 * sq(p.omega[0] * b.rad(I, J, K)) * pRo;
        }
        if (!turb_upd) continue;
        double AinRTk = b.D(6, I, J, K), AinRTO = b.D(7, I, J, K);
        double ARTk = b.V(6, I, J, K), ARTO = b.V(7, I, J, K);
        if (AinRTk >= 0.0) ARTk = ARTk + AinRTk;
        else ARTk = ARTk * otm::exp_(AinRTk / (ARTk + 1.e-10));
        ARTk = std::max(ARTk, 1.0e-10);
        if (AinRTO >= 0.0) ARTO = ARTO + AinRTO;
        else ARTO = ARTO * otm::exp_(AinRTO / (ARTO + 1.e-10));
        ARTO = std::max(ARTO, 1.0e-10);
        pRo = b.V(1, I, J, K);
        double VV = sq(b.V(2, I, J, K)) + sq(b.V(3, I, J, K)) + sq(b.V(4, I, J, K));
        double PPP = (1.4 - 1.0) * b.V(5, I, J, K) - 0.5 * (1.4 - 1.0) * (VV / pRo - sq(p.omega[0] * b.rad(I, J, K)) * pRo);
        double TT = p.RXM2 * PPP / pRo;
        double RmiuL = (1.0 + p.Csthlnd) / (TT * p.Csth1 + p.Csthlnd) * p15(p.Csth1 * TT);
        double DistN = b.Dst(I, J, K);
        double Dudx = b.DQ(1, I, J, K), Dudy = b.DQ(2, I, J, K), Dudz = b.DQ(3, I, J, K);
        double Dvdx = b.DQ(4, I, J, K), Dvdy = b.DQ(5, I, J, K), Dvdz = b.DQ(6, I, J, K);
        double Dwdx = b.DQ(7, I, J, K), Dwdy = b.DQ(8, I, J, K), Dwdz = b.DQ(9, I, J, K);
        double Div = Dudx + Dvdy + Dwdz;
        double prod = (2.0 * (Dudx * Dudx + Dvdy * Dvdy + Dwdz * Dwdz) + sq(Dudy + Dvdx) + sq(Dvdz + Dwdy) + sq(Dwdx + Dudz)
                       - 2.0 / 3.0 * Div * Div);
        if (p.Kind_Model == 2) { wd2006_update(p, b, I, J, K, ARTk, ARTO, pRo, RmiuL, prod); continue; }
        double arg2 = 2.0 * std::sqrt(ARTk / pRo) / p.Beta_star / (ARTO / pRo) / DistN / p.Ref;
        arg2 = std::max(arg2, 500.0 * RmiuL / DistN / DistN / ARTO / p.Ref / p.Ref);
        arg2 = otm::tanh_(arg2 * arg2);
        double Sii = Dudx, Sjj = Dvdy, Skk = Dwdz;
        double Sij = (Dudy + Dvdx) / 2.0, Sik = (Dudz + Dwdx) / 2.0, Sjk = (Dvdz + Dwdy) / 2.0;
        double Skl = std::sqrt(2.0 * (1.0 * Sii * Sii + 1.0 * Sjj * Sjj + 1.0 * Skk * Skk + 2.0 * Sij * Sij + 2.0 * Sik * Sik + 2.0 * Sjk * Sjk));
        double Cmua = std::min(1.0, p.A1 * ARTO / pRo / ((Skl) * arg2 + 1.e-10) * p.Ref);
        ARTO = std::max(ARTO, std::sqrt(pRo * Cmua * std::fabs(prod) / (p.Prod_Lmt * p.Beta_star)) / p.Ref);
        ARTk = std::min(ARTk, 100000.0 * RmiuL * ARTO / pRo / Cmua);
        b.V(6, I, J, K) = ARTk;
        b.V(7, I, J, K) = ARTO;
        b.Rmiu(I, J, K) = Cmua * ARTk / ARTO * pRo;
    }
    b.nrm.DRSa = DRSa; b.nrm.DUa = DUa; b.nrm.Ima = Ima; b.nrm.Jma = Jma; b.nrm.Kma = Kma;
    b.nrm.DRSk = DRSk; b.nrm.DUk = DUk; b.nrm.DRSo = DRSo; b.nrm.DUo = DUo;
}

// Time/TIME_Update_U.F90:16-44
void time_update_u(Ctx& c, Blk& b) {
    for (int L = 1; L <= 7; ++L)
    for (int J = 1; J <= b.NJ1; ++J)
    for (int K = 1; K <= b.NK1; ++K)
    for (int I = 1; I <= b.NI1; ++I) {
        if (c.p.Kind_Dual == 1) b.Wt0(L, I, J, K) = b.V(L, I, J, K);
        else if (c.p.Kind_Dual == 2) {
            b.Wt1(L, I, J, K) = b.Wt0(L, I, J, K);
            b.Wt0(L, I, J, K) = b.V(L, I, J, K);
        }
    }
}

// ---------------------------------------------------------------------------------------
// Runge-Kutta marching (IF_RK = 1, main.F90:152-161)
// ---------------------------------------------------------------------------------------
// Time/TIME_RK_Save.F90:16-28: the stage-1 state, all ML = 7 components
void time_rk_save(Ctx& c, Blk& b) {
    if (c.Itr_Chld != 1) return;
    for (int L = 1; L <= 7; ++L)
    for (int J = 1; J <= b.NJ1; ++J)
    for (int K = 1; K <= b.NK1; ++K)
    for (int I = 1; I <= b.NI1; ++I) b.Wt2(L, I, J, K) = b.V(L, I, J, K);
}

// Time/TIME_RK.F90:27-86: norms of |D1/V1| on the residual, then the SSP-RK3 stage on V(1:5)
void time_rk(Ctx& c, Blk& b) {
    b.nrm.nan_flag = 0;
    double DRSa = 0.0, DUa = 0.0;
    int Ima = 0, Jma = 0, Kma = 0;
    for (int K = 1; K <= b.NK1; ++K)
    for (int J = 1; J <= b.NJ1; ++J)
    for (int I = 1; I <= b.NI1; ++I) {
        double DR = std::fabs(b.D(1, I, J, K) / b.V(1, I, J, K));
        if (std::isnan(b.D(1, I, J, K))) b.nrm.nan_flag = 1;
        if (DUa <= DR) { DUa = DR; Ima = I; Jma = J; Kma = K; }
        DRSa = DRSa + DR * DR;
    }
    DRSa = std::sqrt(DRSa / b.NI1 / b.NJ1 / b.NK1);
    for (int K = 1; K <= b.NK1; ++K)
    for (int J = 1; J <= b.NJ1; ++J)
    for (int I = 1; I <= b.NI1; ++I)
        for (int L = 1; L <= 5; ++L) {
            const double dtm = b.Dtm(I, J, K), d = b.D(L, I, J, K), vol = b.Vol(I, J, K);
            if (c.Itr_Chld == 1)
                b.V(L, I, J, K) = b.V(L, I, J, K) + dtm * d / vol;
            else if (c.Itr_Chld == 2)
                b.V(L, I, J, K) = 0.75 * b.Wt2(L, I, J, K) + 0.25 * b.V(L, I, J, K) + 0.25 * dtm * d / vol;
            else if (c.Itr_Chld == 3)
                b.V(L, I, J, K) = 1.0 / 3.0 * b.Wt2(L, I, J, K) + 2.0 / 3.0 * b.V(L, I, J, K) + 2.0 / 3.0 * dtm * d / vol;
        }
    b.nrm.DRSa = DRSa; b.nrm.DUa = DUa; b.nrm.Ima = Ima; b.nrm.Jma = Jma; b.nrm.Kma = Kma;
}

// Time/TIME_RK_V_Update_New.F90:66-320: p and T from the new V (no rotation term), the SST
// update of k and omega from the k-omega LU-SGS increments (Sutherland without Csth1), then
// the k and omega norms on the updated density
void time_rk_v_update(Ctx& c, Blk& b) {
    const trans_params& p = c.p;
    bool turb_upd = (p.IF_Euler == 0 && c.IF_turb == 1 && c.KI >= p.KItm);
    for (int K = 1; K <= b.NK1; ++K)
    for (int J = 1; J <= b.NJ1; ++J)
    for (int I = 1; I <= b.NI1; ++I) {
        double VV = b.V(2, I, J, K) * b.V(2, I, J, K) + b.V(3, I, J, K) * b.V(3, I, J, K) + b.V(4, I, J, K) * b.V(4, I, J, K);
        b.PP(I, J, K) = (1.4 - 1.0) * b.V(5, I, J, K) - 0.5 * (1.4 - 1.0) * VV / b.V(1, I, J, K);
        b.T(I, J, K) = p.RXM2 * b.PP(I, J, K) / b.V(1, I, J, K);
        if (!turb_upd) continue;
        double AinRTk = b.D(6, I, J, K), AinRTO = b.D(7, I, J, K);
        double ARTk = b.V(6, I, J, K), ARTO = b.V(7, I, J, K);
        if (AinRTk >= 0.0) ARTk = ARTk + AinRTk;
        else ARTk = ARTk * otm::exp_(AinRTk / (ARTk + 1.e-10));
        ARTk = std::max(ARTk, 1.0e-10);
        if (AinRTO >= 0.0) ARTO = ARTO + AinRTO;
        else ARTO = ARTO * otm::exp_(AinRTO / (ARTO + 1.e-10));
        ARTO = std::max(ARTO, 1.0e-10);
        double pRo = b.V(1, I, J, K);
        VV = sq(b.V(2, I, J, K)) + sq(b.V(3, I, J, K)) + sq(b.V(4, I, J, K));
        double PPP = 0.4 * b.V(5, I, J, K) - 0.2 * VV / pRo;
        double TT = p.RXM2 * PPP / pRo;
        double RmiuL = (1.0 + p.Csthlnd) / (TT + p.Csthlnd) * p15(TT);
        double DistN = b.Dst(I, J, K);
        double Dudx = b.DQ(1, I, J, K), Dudy = b.DQ(2, I, J, K), Dudz = b.DQ(3, I, J, K);
        double Dvdx = b.DQ(4, I, J, K), Dvdy = b.DQ(5, I, J, K), Dvdz = b.DQ(6, I, J, K);
        double Dwdx = b.DQ(7, I, J, K), Dwdy = b.DQ(8, I, J, K), Dwdz = b.DQ(9, I, J, K);
        double Div = Dudx + Dvdy + Dwdz;
        double prod = (2.0 * (Dudx * Dudx + Dvdy * Dvdy + Dwdz * Dwdz) + sq(Dudy + Dvdx) + sq(Dvdz + Dwdy) + sq(Dwdx + Dudz)
                       - 2.0 / 3.0 * Div * Div);
        if (p.Kind_Model == 2) { wd2006_update(p, b, I, J, K, ARTk, ARTO, pRo, RmiuL, prod); continue; }
        double arg2 = 2.0 * std::sqrt(ARTk / pRo) / p.Beta_star / (ARTO / pRo) / DistN / p.Ref;
        arg2 = std::max(arg2, 500.0 * RmiuL / DistN / DistN / ARTO / p.Ref / p.Ref);
        arg2 = otm::tanh_(arg2 * arg2);
        double Sii = Dudx, Sjj = Dvdy, Skk = Dwdz;
        double Sij = (Dudy + Dvdx) / 2.0, Sik = (Dudz + Dwdx) / 2.0, Sjk = (Dvdz + Dwdy) / 2.0;
        double Skl = std::sqrt(2.0 * (1.0 * Sii * Sii + 1.0 * Sjj * Sjj + 1.0 * Skk * Skk + 2.0 * Sij * Sij + 2.0 * Sik * Sik + 2.0 * Sjk * Sjk));
        double Cmua = std::min(1.0, p.A1 * ARTO / pRo / ((Skl) * arg2 + 1.e-10) * p.Ref);
        ARTO = std::max(ARTO, std::sqrt(pRo * Cmua * std::fabs(prod) / (p.Prod_Lmt * p.Beta_star)) / p.Ref);
        ARTk = std::min(ARTk, 100000.0 * RmiuL * ARTO / pRo / Cmua);
        b.V(6, I, J, K) = ARTk;
        b.V(7, I, J, K) = ARTO;
        b.Rmiu(I, J, K) = Cmua * ARTk / ARTO * pRo;
    }
    double DRSk = 0, DUk = 0, DRSo = 0, DUo = 0;
    for (int K = 1; K <= b.NK1; ++K)
    for (int J = 1; J <= b.NJ1; ++J)
    for (int I = 1; I <= b.NI1; ++I) {
        double DRk = std::fabs(b.D(6, I, J, K) / b.V(1, I, J, K));
        if (DUk <= DRk) DUk = DRk;
        DRSk = DRSk + DRk * DRk;
    }
    DRSk = std::sqrt(DRSk / b.NI1 / b.NJ1 / b.NK1);
    for (int K = 1; K <= b.NK1; ++K)
    for (int J = 1; J <= b.NJ1; ++J)
    for (int I = 1; I <= b.NI1; ++I) {
        double DRo = std::fabs(b.D(7, I, J, K) / b.V(1, I, J, K));
        if (DUo <= DRo) DUo = DRo;
        DRSo = DRSo + DRo * DRo;
    }
    DRSo = std::sqrt(DRSo / b.NI1 / b.NJ1 / b.NK1);
    b.nrm.DRSk = DRSk; b.nrm.DUk = DUk; b.nrm.DRSo = DRSo; b.nrm.DUo = DUo;
}

// ---------------------------------------------------------------------------------------
// main.F90:54-171 stage by stage
// ---------------------------------------------------------------------------------------
void set_turb(Ctx& c) {
    const trans_params& p = c.p;
    c.IF_turb = (p.IF_Euler == 0 && p.IF_Turb_org == 1 && (c.KI >= p.KItm || p.Kind_Hybrid > 0)) ? 1 : 0;
}

int run_stage(Ctx& c, int stage) {
    switch (stage) {
        case TRANS_STAGE_SPECRAD:
#pragma omp parallel for schedule(dynamic)
            for (size_t n = 0; n < c.B.size(); ++n) spectral_radius(c, c.B[n]);
            break;
        case TRANS_STAGE_BC_STATE:
            bc_boundarys(c, -1);
            break;
        case TRANS_STAGE_GRADIENT:
#pragma omp parallel for schedule(dynamic)
            for (size_t n = 0; n < c.B.size(); ++n) {
                spaceinterp(c, c.B[n]);
                if (c.p.IF_Euler == 0) diff_dqdxyz(c, c.B[n]);
            }
            break;
        case TRANS_STAGE_BC_GRAD:
            bc_boundarys(c, 0);
            break;
        case TRANS_STAGE_RESIDUAL:
            // per block: RCCorrection (main.F90:89) and the three loops of main.F90:92-133 touch
            // only the block's own arrays
#pragma omp parallel for schedule(dynamic)
            for (size_t n = 0; n < c.B.size(); ++n) {
                Blk& b = c.B[n];
                if (c.p.Kind_RotMod == 1) rc_correction(c, b);
                std::fill(b.D.v.begin(), b.D.v.end(), 0.0);
                if (c.p.IF_Euler == 0) diffusion_centered(c, b);
                if (c.IF_turb) turbtwo_diffusion(c, b);
                if (c.p.Kind_Spatial <= 2) convect_muscl(c, b);
                else convect_mdcd(c, b);
                if (c.IF_turb) turbtwo_convect_muscl(c, b);
                convect_inviscid(c, b);
                if (c.IF_turb) turbtwo_convect_upwind(c, b);
            }
            break;
        case TRANS_STAGE_LUSGS:
#pragma omp parallel for schedule(dynamic)
            for (size_t n = 0; n < c.B.size(); ++n) {
                if (c.p.IF_RK == 1) {
                    time_rk_save(c, c.B[n]);
                    time_rk(c, c.B[n]);
                } else {
                    time_lusgs(c, c.B[n]);
                }
                if (c.IF_turb) turbtwo_lusgs_sst(c, c.B[n]);
            }
            break;
        case TRANS_STAGE_UPDATE:
#pragma omp parallel for schedule(dynamic)
            for (size_t n = 0; n < c.B.size(); ++n) {
                if (c.p.IF_RK == 1) time_rk_v_update(c, c.B[n]);
                else time_update_v(c, c.B[n]);
            }
            for (auto& b : c.B) c.nan_flag |= b.nrm.nan_flag;
            break;
        case TRANS_STAGE_UPDATE_U:
            if (c.p.Kind_Dual != 0) {
#pragma omp parallel for schedule(dynamic)
                for (size_t n = 0; n < c.B.size(); ++n) time_update_u(c, c.B[n]);
            }
            break;
        default:
            return TRANS_E_ARG;
    }
    return TRANS_OK;
}

struct FieldDesc { Arr Blk::*arr; int ncomp; int lb; };

FieldDesc field_desc(int f) {
    switch (f) {
        case TRANS_V: return {&Blk::V, 7, -2};
        case TRANS_PP: return {&Blk::PP, 1, -2};
        case TRANS_T: return {&Blk::T, 1, -2};
        case TRANS_RMIU: return {&Blk::Rmiu, 1, -2};
        case TRANS_WT0: return {&Blk::Wt0, 7, 1};
        case TRANS_WT1: return {&Blk::Wt1, 7, 1};
        case TRANS_SD: return {&Blk::SD, 9, -2};
        case TRANS_GRAD: return {&Blk::Grad, 3, -2};
        case TRANS_VOL: return {&Blk::Vol, 1, -2};
        case TRANS_ALAGM: return {&Blk::Alagm, 3, -2};
        case TRANS_DST: return {&Blk::Dst, 1, -2};
        case TRANS_ALENG: return {&Blk::ALeng, 1, -2};
        case TRANS_ASENG: return {&Blk::ASeng, 1, 1};
        case TRANS_XC: return {&Blk::Xc, 1, 0};
        case TRANS_YC: return {&Blk::Yc, 1, 0};
        case TRANS_ZC: return {&Blk::Zc, 1, 0};
        case TRANS_RAD: return {&Blk::rad, 1, -2};
        case TRANS_THTC: return {&Blk::thtc, 1, -2};
        case TRANS_D: return {&Blk::D, 7, 0};
        case TRANS_RDS: return {&Blk::Rds, 3, 0};
        case TRANS_DTM: return {&Blk::Dtm, 1, 1};
        case TRANS_DQDXYZ: return {&Blk::DQ, 18, -1};
        case TRANS_SHOCK: return {&Blk::shock, 1, -2};
        case TRANS_WT2: return {&Blk::Wt2, 7, 1};
        default: return {nullptr, 0, 0};
    }
}

}  // namespace

extern "C" {

int oracle_create(const trans_params* p, int nblocks, const trans_block* blocks, void** out) {
    if (!p || !blocks || nblocks <= 0 || !out) return TRANS_E_ARG;
    if ((p->IF_Precondition != 0 && p->IF_Precondition != 1) || p->Kind_RotMod < 0 || p->Kind_RotMod > 2 ||
        (p->Kind_Model != 1 && p->Kind_Model != 2))
        return TRANS_E_ARG;
    if (p->IF_Precondition == 1 && p->IF_RK != 0) return TRANS_E_ARG;     // preconditioning with LU-SGS only
    if (p->Kind_Spatial < 1 || p->Kind_Spatial > 4) return TRANS_E_ARG;
    if (p->Kind_Roe < 1 || p->Kind_Roe > 3) return TRANS_E_ARG;
    if (p->Kind_Hybrid != 0 && p->Kind_Hybrid != 3) return TRANS_E_ARG;
    // DES (0), the DDES shielding functions (1-3) and IDDES (5); FSST is undefined for 4
    if (p->Kind_Hybrid == 3 && (p->Kind_SubHY < 0 || p->Kind_SubHY > 5 || p->Kind_SubHY == 4)) return TRANS_E_ARG;
    // rotation about the x axis at omega(1); omega(2) and omega(3) are read by no routine of the path
    if (!std::isfinite(p->omega[0])) return TRANS_E_ARG;
    if (p->IF_RK != 0 && p->IF_RK != 1) return TRANS_E_ARG;
    Ctx* c = new Ctx();
    c->p = *p;
    c->B.resize(nblocks);
    for (int n = 0; n < nblocks; ++n) {
        const trans_block& tb = blocks[n];
        Blk& b = c->B[n];
        b.NI = tb.ni; b.NJ = tb.nj; b.NK = tb.nk; b.id = tb.id;
        b.NI1 = b.NI - 1; b.NJ1 = b.NJ - 1; b.NK1 = b.NK - 1;
        b.conn.assign(tb.conn, tb.conn + tb.nconn);
        const int n1[6] = {b.NJ1, b.NJ1, b.NI1, b.NI1, b.NI1, b.NI1};
        const int n2[6] = {b.NK1, b.NK1, b.NK1, b.NK1, b.NJ1, b.NJ1};
        for (int f = 0; f < 6; ++f) {
            b.mwn1[f] = n1[f];
            if (tb.markwall[f]) b.mw[f].assign(tb.markwall[f], tb.markwall[f] + (size_t)n1[f] * n2[f]);
        }
        int ni = b.NI, nj = b.NJ, nk = b.NK;
        b.V.alloc(7, 1, ni, nj, nk); b.PP.alloc(1, 1, ni, nj, nk); b.T.alloc(1, 1, ni, nj, nk);
        b.Rmiu.alloc(1, 1, ni, nj, nk); b.Wt0.alloc(7, 1, ni, nj, nk); b.Wt1.alloc(7, 1, ni, nj, nk);
        b.Wt2.alloc(7, 1, ni, nj, nk);
        b.SD.alloc(3, 3, ni, nj, nk); b.Grad.alloc(3, 1, ni, nj, nk); b.Vol.alloc(1, 1, ni, nj, nk);
        b.Alagm.alloc(3, 1, ni, nj, nk); b.Dst.alloc(1, 1, ni, nj, nk); b.ALeng.alloc(1, 1, ni, nj, nk);
        b.ASeng.alloc(1, 1, ni, nj, nk); b.Xc.alloc(1, 1, ni, nj, nk); b.Yc.alloc(1, 1, ni, nj, nk);
        b.Zc.alloc(1, 1, ni, nj, nk); b.rad.alloc(1, 1, ni, nj, nk); b.thtc.alloc(1, 1, ni, nj, nk);
        b.D.alloc(7, 1, ni, nj, nk); b.Rds.alloc(3, 1, ni, nj, nk); b.Dtm.alloc(1, 1, ni, nj, nk);
        b.DQ.alloc(18, 1, ni, nj, nk); b.shock.alloc(1, 1, ni, nj, nk); b.F.alloc(2, 1, ni, nj, nk);
        b.VL.alloc(3, 8, ni, nj, nk); b.VR.alloc(3, 8, ni, nj, nk);
        b.rccl.alloc(3, 1, ni, nj, nk); b.rccr.alloc(3, 1, ni, nj, nk); b.FunDES.alloc(1, 1, ni, nj, nk);
        b.Fsch.alloc(1, 1, ni, nj, nk);
        b.Fr1.alloc(1, 1, ni, nj, nk);
        std::fill(b.Fr1.v.begin(), b.Fr1.v.end(), 1.0);       // f_r1 = 1 (Input/Read_BlockDimensions.F90:426)
        std::memset(&b.nrm, 0, sizeof(b.nrm));
    }
    *out = c;
    return TRANS_OK;
}

int oracle_destroy(void* ctx) {
    delete static_cast<Ctx*>(ctx);
    return TRANS_OK;
}

static int field_copy(void* ctx, int ib, int f, double* host, bool to_host) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || ib < 0 || ib >= (int)c->B.size()) return TRANS_E_ARG;
    FieldDesc fd = field_desc(f);
    if (!fd.arr) return TRANS_E_ARG;
    Blk& b = c->B[ib];
    Arr& a = b.*(fd.arr);
    int ei = b.NI + 2 - fd.lb + 1, ej = b.NJ + 2 - fd.lb + 1, ek = b.NK + 2 - fd.lb + 1;
    size_t n = 0;
    for (int k = 0; k < ek; ++k)
    for (int j = 0; j < ej; ++j)
    for (int i = 0; i < ei; ++i) {
        size_t cell = a.cell(i + fd.lb, j + fd.lb, k + fd.lb);
        for (int m = 0; m < fd.ncomp; ++m, ++n) {
            if (to_host) host[n] = a.v[(size_t)m + (size_t)fd.ncomp * cell];
            else a.v[(size_t)m + (size_t)fd.ncomp * cell] = host[n];
        }
    }
    return TRANS_OK;
}

int oracle_set_field(void* ctx, int ib, int f, const double* host) {
    return field_copy(ctx, ib, f, const_cast<double*>(host), false);
}
int oracle_get_field(void* ctx, int ib, int f, double* host) { return field_copy(ctx, ib, f, host, true); }

int oracle_run_stage(void* ctx, int stage, int ki, int itr_chld) {
    Ctx* c = static_cast<Ctx*>(ctx);
    c->KI = ki;
    c->Itr_Chld = itr_chld;
    set_turb(*c);
    return run_stage(*c, stage);
}

int oracle_iterate(void* ctx, int ki, trans_norms* norms) {
    Ctx* c = static_cast<Ctx*>(ctx);
    c->KI = ki;
    set_turb(*c);
    int nsub = c->p.IF_RK == 1 ? 3 : (c->p.Kind_Dual != 0 ? c->p.Kchld : 1);      // main.F90:54-56
    c->nan_flag = 0;
    for (int it = 1; it <= nsub; ++it) {
        c->Itr_Chld = it;
        for (int s = TRANS_STAGE_SPECRAD; s <= TRANS_STAGE_UPDATE; ++s) run_stage(*c, s);
    }
    run_stage(*c, TRANS_STAGE_UPDATE_U);
    if (norms)
        for (size_t n = 0; n < c->B.size(); ++n) norms[n] = c->B[n].nrm;
    return c->nan_flag ? TRANS_E_NAN : TRANS_OK;
}

// host threads of the per-block loops (the reference runs one MPI rank per block); returns the
// number in use after the call
int oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

int oracle_get_norms(void* ctx, trans_norms* norms) {
    Ctx* c = static_cast<Ctx*>(ctx);
    for (size_t n = 0; n < c->B.size(); ++n) norms[n] = c->B[n].nrm;
    return TRANS_OK;
}

// Cross-rank 1-to-1 interfaces (BC/PARALLEL_BC_P2P.F90:1-257).  A kind-9 connection whose
// target block is not in this context is left out of BC_Boundarys (bc_boundarys finds no
// target) and exchanged by the caller between BC_STATE / BC_GRAD and the next stage:
// oracle_halo_pack fills the segment's send buffer from this block's interior layers, face
// cells in the segment's K, J, I order, in the reference's buffer layout (sweep -1: 36 words
// per face cell -- layer 0: V(1:7), PP, T, Rmiu, Rds(1:3), shock; layers 1 and 2: V(1:7), PP,
// T, Rmiu, shock; sweep 0: DqDxyz(1:18) of layer 0), at full precision (the reference sends
// FP32).  oracle_halo_unpack fills this segment's ghost layers from the partner segment's
// buffer through the same index transform and rotation as the same-rank copy (bc_p2p), and
// applies what that copy applies (Rds and shock travel but are not written: the ghost shock is
// overwritten by the extrapolation of DIFF_DqDxyz, the ghost Rds is not read by the path).
int halo_words(int sweep) { return sweep == -1 ? 36 : 18; }

int oracle_halo_pack(void* ctx, int sweep, int ib, int iconn, double* buf) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || ib < 0 || ib >= (int)c->B.size() || !buf || (sweep != -1 && sweep != 0)) return TRANS_E_ARG;
    Blk& b = c->B[ib];
    if (iconn < 1 || iconn > (int)b.conn.size() || b.conn[iconn - 1].BCType != 9) return TRANS_E_ARG;
    SegIdx s(b.conn[iconn - 1]);
    const int S[3][3] = {{s.iadd, s.jadd, s.kadd}, {s.iadd1, s.jadd1, s.kadd1}, {s.iadd2, s.jadd2, s.kadd2}};
    size_t n = 0;
    for (int K = s.Kbgn; K <= s.Kend; ++K)
    for (int J = s.Jbgn; J <= s.Jend; ++J)
    for (int I = s.Ibgn; I <= s.Iend; ++I) {
        if (sweep == -1) {
            for (int L = 0; L < 3; ++L) {
                int is = I + S[L][0], js = J + S[L][1], ks = K + S[L][2];
                for (int m = 1; m <= 7; ++m) buf[n++] = b.V(m, is, js, ks);
                buf[n++] = b.PP(is, js, ks);
                buf[n++] = b.T(is, js, ks);
                buf[n++] = b.Rmiu(is, js, ks);
                if (L == 0)
                    for (int d = 1; d <= 3; ++d) buf[n++] = b.Rds(d, is, js, ks);
                buf[n++] = b.shock(is, js, ks);
            }
        } else {
            int is = I + s.iadd, js = J + s.jadd, ks = K + s.kadd;
            for (int m = 1; m <= 18; ++m) buf[n++] = b.DQ(m, is, js, ks);
        }
    }
    return TRANS_OK;
}

int oracle_halo_unpack(void* ctx, int sweep, int ib, int iconn, const trans_conn* partner, const double* buf) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || ib < 0 || ib >= (int)c->B.size() || !buf || !partner || (sweep != -1 && sweep != 0)) return TRANS_E_ARG;
    Blk& b = c->B[ib];
    if (iconn < 1 || iconn > (int)b.conn.size() || b.conn[iconn - 1].BCType != 9) return TRANS_E_ARG;
    const trans_conn& a = b.conn[iconn - 1];
    SegIdx s(a), t(*partner);
    const int ti = t.Iend - t.Ibgn + 1, tj = t.Jend - t.Jbgn + 1, tk = t.Kend - t.Kbgn + 1;
    int IIadd = s.Iend - s.Ibgn + 2, JJadd = s.Jend - s.Jbgn + 2, KKadd = s.Kend - s.Kbgn + 2;
    double dstage = a.rotateAngle;
    double sint = std::sin(dstage), cost = std::cos(dstage);
    double cos2t = cost * cost, sin2t = sint * sint, sct = sint * cost;
    const int W = halo_words(sweep);
    for (int K = s.Kbgn; K <= s.Kend; ++K)
    for (int J = s.Jbgn; J <= s.Jend; ++J)
    for (int I = s.Ibgn; I <= s.Iend; ++I) {
        int iL = I - s.Ibgn + 1, jL = J - s.Jbgn + 1, kL = K - s.Kbgn + 1;
        iL = a.revMatrix[0] * IIadd + (1 - 2 * a.revMatrix[0]) * iL;
        jL = a.revMatrix[1] * JJadd + (1 - 2 * a.revMatrix[1]) * jL;
        kL = a.revMatrix[2] * KKadd + (1 - 2 * a.revMatrix[2]) * kL;
        int pb, pj, pk;
        ijk_start_end(iL, jL, kL, pb, pj, pk, a.Transform, a.TransformT, a.lcross);     // partner face cell
        pb -= 1; pj -= 1; pk -= 1;
        if (pb < 0 || pb >= ti || pj < 0 || pj >= tj || pk < 0 || pk >= tk) return TRANS_E_ARG;
        const double* w = buf + ((size_t)pb + (size_t)ti * ((size_t)pj + (size_t)tj * (size_t)pk)) * W;
        if (sweep == -1) {
            const int E[3][3] = {{s.Eiadd, s.Ejadd, s.Ekadd}, {s.Eiadd1, s.Ejadd1, s.Ekadd1}, {s.Eiadd2, s.Ejadd2, s.Ekadd2}};
            const int off[3] = {0, 14, 25};
            for (int L = 0; L < 3; ++L) {
                const double* x = w + off[L];
                int il = I + E[L][0], jl = J + E[L][1], kl = K + E[L][2];
                b.V(1, il, jl, kl) = x[0];
                b.V(2, il, jl, kl) = x[1];
                double txy = x[2], txz = x[3];
                b.V(3, il, jl, kl) = cost * txy + sint * txz;
                b.V(4, il, jl, kl) = -sint * txy + cost * txz;
                for (int m = 5; m <= 7; ++m) b.V(m, il, jl, kl) = x[m - 1];
                b.PP(il, jl, kl) = x[7];
                b.T(il, jl, kl) = x[8];
                b.Rmiu(il, jl, kl) = x[9];
            }
        } else {
            int il = I + s.Eiadd, jl = J + s.Ejadd, kl = K + s.Ekadd;
            double ugx = w[0], ugy = w[1], ugz = w[2];
            double vgx = w[3], vgy = w[4], vgz = w[5];
            double wgx = w[6], wgy = w[7], wgz = w[8];
            b.DQ(1, il, jl, kl) = ugx;
            b.DQ(2, il, jl, kl) = cost * ugy + sint * ugz;
            b.DQ(3, il, jl, kl) = -sint * ugy + cost * ugz;
            b.DQ(4, il, jl, kl) = cost * vgx + sint * wgx;
            b.DQ(5, il, jl, kl) = cos2t * vgy + sct * (vgz + wgy) + sin2t * wgz;
            b.DQ(6, il, jl, kl) = cos2t * vgz + sct * (-vgy + wgz) - sin2t * wgy;
            b.DQ(7, il, jl, kl) = -sint * vgx + cost * wgx;
            b.DQ(8, il, jl, kl) = -sin2t * vgz + sct * (-vgy + wgz) + cos2t * wgy;
            b.DQ(9, il, jl, kl) = sin2t * vgy + sct * (vgz + wgy) + cos2t * wgz;
            for (int LL = 4; LL <= 6; ++LL) {
                int L = (LL - 1) * 3 + 1;
                b.DQ(L, il, jl, kl) = w[L - 1];
                double gy = w[L], gz = w[L + 1];
                b.DQ(L + 1, il, jl, kl) = cost * gy + sint * gz;
                b.DQ(L + 2, il, jl, kl) = -sint * gy + cost * gz;
            }
        }
    }
    return TRANS_OK;
}

// scalar entry points for known-answer tests of the flux and limiter formulas
double oracle_alimiter(double a, double b) { return alimiter(a, b); }
double oracle_muscl2_limiter(double a, double b) { return muscl2_limiter(a, b); }
void oracle_ausmpw(const trans_params* p, const double* in, double* out) {
    ausmpw_common(*p, in[0], in[1], in[2], in[3], in[4], in[5], in[6], in[7], in[8], in[9], in[10], in[11], in[12], in[13], out);
}
void oracle_roe(const trans_params* p, const double* in, double* out) {
    roe_common(*p, in[0], in[1], in[2], in[3], in[4], in[5], in[6], in[7], in[8], in[9], in[10], in[11], in[12], in[13], 0.0, 0.0, out);
}
void oracle_mdcd(const double* s6, double gama, double* out) { mdcd_pair(s6, gama, out[0], out[1]); }

}  // extern "C"

extern "C" {
double oracle_tm_exp(double x) { return otm::exp_(x); }
double oracle_tm_expm1(double x) { return otm::expm1_(x); }
double oracle_tm_tanh(double x) { return otm::tanh_(x); }
double oracle_tm_log(double x) { return otm::log_(x); }
double oracle_tm_pow(double x, double y) { return otm::pow_(x, y); }
double oracle_tm_atan(double x) { return otm::atan_(x); }
}
