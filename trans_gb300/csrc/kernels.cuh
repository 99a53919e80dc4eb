// kernels.cuh -- CUDA kernels of the TRANS hot path, templated on the flux arithmetic type R.
//
// One thread per interior cell, face or boundary face cell; blocks of every case are covered
// by tile lists (a tile never straddles two blocks).  Kernel order within one sub-iteration:
//   specrad -> bc_state (+ outlet lines) -> prims -> gradient -> shock_ghost -> bc_grad
//   -> face_flux(i,j,k) -> gather -> lusgs_rhs -> sweep_L(h ascending) -> sweep_U(h descending)
//   -> update (+ norms)
// which is the order of main.F90:65-151.
#pragma once
#include "dev.cuh"
#include "types.cuh"

namespace tg {

// ---------------------------------------------------------------------------------------
// Residual-norm partials (Time/TIME_Update_V.F90:106-146, 892-908): sums of |D/V|^2, maxima of
// |D/V| and the NaN flag.  A CTA reduces them by warp shuffles -- lane l takes lane l+w for
// w = 16, 8, 4, 2, 1 -- then warp 0 over the warps' results, a fixed order.  The maximum of
// |D1/V1| keeps the later cell on ties (IF(DUa<=DR), :135).
// ---------------------------------------------------------------------------------------
__device__ inline NormPart norm_identity() {
    NormPart a;
    a.sa = 0; a.ma = -1; a.sk = 0; a.mk = 0; a.so = 0; a.mo = 0; a.ia = -1; a.nan = 0; a.pad_ = 0;
    return a;
}
__device__ inline void norm_join(NormPart& a, const NormPart& b) {
    a.sa += b.sa; a.sk += b.sk; a.so += b.so;
    if (b.ma > a.ma || (b.ma == a.ma && b.ia > a.ia)) { a.ma = b.ma; a.ia = b.ia; }
    a.mk = dmax(a.mk, b.mk); a.mo = dmax(a.mo, b.mo);
    a.nan |= b.nan;
}
__device__ inline NormPart norm_shfl_down(const NormPart& a, int w) {
    const unsigned full = 0xffffffffu;
    NormPart b;
    b.sa = __shfl_down_sync(full, a.sa, w); b.ma = __shfl_down_sync(full, a.ma, w);
    b.sk = __shfl_down_sync(full, a.sk, w); b.mk = __shfl_down_sync(full, a.mk, w);
    b.so = __shfl_down_sync(full, a.so, w); b.mo = __shfl_down_sync(full, a.mo, w);
    b.ia = __shfl_down_sync(full, a.ia, w); b.nan = __shfl_down_sync(full, a.nan, w);
    b.pad_ = 0;
    return b;
}
__device__ inline NormPart norm_reduce_warp(NormPart a) {
    for (int w = 16; w > 0; w >>= 1) {
        const NormPart o = norm_shfl_down(a, w);
        if ((int)(threadIdx.x & 31) + w < 32) norm_join(a, o);
    }
    return a;
}
// the CTA's reduction, valid in thread 0 (blockDim a multiple of 32); every thread calls it
__device__ inline NormPart norm_reduce_cta(NormPart a) {
    __shared__ NormPart s_warp[32];
    a = norm_reduce_warp(a);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) s_warp[wid] = a;
    __syncthreads();
    if (wid == 0) a = norm_reduce_warp(lane < (int)(blockDim.x >> 5) ? s_warp[lane] : norm_identity());
    return a;
}

#ifdef TG_COMMON_KERNELS
// ---------------------------------------------------------------------------------------
// Time/SpectralRadius.F90:47-180
// ---------------------------------------------------------------------------------------
__global__ void k_specrad(const DevBlock* __restrict__ blks, const Tile* __restrict__ tiles, const CaseDev* __restrict__ cdev) {
    const Tile t = tiles[blockIdx.x];
    if ((int)threadIdx.x >= t.count) return;
    const DevBlock b = blks[t.blk];
    const Params p = cdev[b.cs].p;
    const double CFL_sub = cdev[b.cs].CFL_sub;
    int n = t.start + threadIdx.x;
    int I = n % b.NI1 + 1, J = (n / b.NI1) % b.NJ1 + 1, K = n / (b.NI1 * b.NJ1) + 1;
    int c = cidx(b, I, J, K);
    const double* V = slot(b, S_V);
    double Den = V[c];
    double Vxi = slot(b, S_V + 1)[c] / Den;
    double Vyi = slot(b, S_V + 2)[c] / Den;
    double Vzi = slot(b, S_V + 3)[c] / Den;
    double AAc = sqrt(1.4 * slot(b, S_PP)[c] / Den);
    double TT = slot(b, S_T)[c];
    double RmiuL = mu_suth<double>(p, TT);
    double RmiuTL = slot(b, S_RMIU)[c];
    double uvmu = (RmiuL + RmiuTL + 1.0e-20) * 4.0 / 3.0;
    double uvmupr = (RmiuL / 0.72 + RmiuTL / 0.9 + 1.0e-20) * 1.4;
    double pruvmu = dmax(uvmu, uvmupr) / Den;
    double vol = slot(b, S_VOL)[c];
    double rs = 0.0;
    double Rd[3];
    // low-Mach preconditioning (Time/SpectralRadius.F90:91-127): the acoustic speed and the
    // convective weight of each direction from ubetac2 and its viscous limit
    double UVW2 = 0.0, ubetac2 = 1.0, RmiuAll = 0.0;
    if (p.IF_Precondition) {
        UVW2 = Vxi * Vxi + Vyi * Vyi + Vzi * Vzi;
        ubetac2 = get_precond_para<double>(p, UVW2, AAc * AAc, Den, 0.0, 0.0, 1.0);
        RmiuAll = RmiuL + RmiuTL;
    }
    for (int d = 0; d < 3; ++d) {
        double ARX = slot(b, S_ASD + 3 * d)[c], ARY = slot(b, S_ASD + 3 * d + 1)[c], ARZ = slot(b, S_ASD + 3 * d + 2)[c];
        double STsq = ARX * ARX + ARY * ARY + ARZ * ARZ;
        double UU = Vxi * ARX + Vyi * ARY + Vzi * ARZ + 0.0;
        double alf = 0.0, AAcd = AAc;
        if (p.IF_Precondition) {
            double ubd = dmax(ubetac2, pow2r<double>(RmiuAll / Den / p.Ref / slot(b, S_ALAGM + d)[c] / AAc));
            alf = (1.0 - ubd) / 2.0;
            AAcd = sqrt(alf * alf * UVW2 + ubd * AAc * AAc);
        }
        Rd[d] = fabs(UU) * (1.0 - alf) + sqrt(STsq) * AAcd + 2.0 * STsq / vol * pruvmu / p.Ref;
        slot(b, S_RDS + d)[c] = Rd[d];
    }
    rs = Rd[0] + Rd[1] + Rd[2];
    double Dtm_local = vol / rs;
    double dtm = p.IF_Local_Main == 1 ? p.CFL_Main * Dtm_local : p.DT_LUSGS_Main;
    if (p.Kind_Dual != 0) dtm = p.IF_Local_Sub == 1 ? CFL_sub * Dtm_local : p.DT_LUSGS_Sub;
    slot(b, S_DTM)[c] = dtm;
}

// ---------------------------------------------------------------------------------------
// BC/BC_Wall.F90, BC/BC_far.F90, BC/BC_Symm.F90, BC/BC_Inlet.F90, BC/BC_P2P.F90 (sweep -1)
// ---------------------------------------------------------------------------------------
__device__ inline void farbond(double XM, double P2, double RR, double Vxi, double Vyi, double Vzi, double DNx, double DNy,
                               double DNz, double VxF, double VyF, double VzF, double& PP0, double& RR0, double& VX0,
                               double& VY0, double& VZ0, double& dir) {
    const double pGam = 1.4;
    double AF = 1.0 / XM;
    double AE = sqrt(pGam * P2 / RR);
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
        RR0 = tmx::pow_(AS * AS / SON / pGam, 2.5);
        PP0 = AS * AS * RR0 / pGam;
        dir = -1.0;
    }
    if (QN >= 0.0 && QN < AS) {
        double SON = P2 / tmx::pow_(RR, pGam);
        double QTX = Vxi - QNE * DNx, QTY = Vyi - QNE * DNy, QTZ = Vzi - QNE * DNz;
        VX0 = QTX + QN * DNx; VY0 = QTY + QN * DNy; VZ0 = QTZ + QN * DNz;
        RR0 = tmx::pow_(AS * AS / SON / pGam, 2.5);
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

__global__ void k_bc_state(const DevBlock* __restrict__ blks, const BCEntry* __restrict__ ent, int n,
                           const CaseDev* __restrict__ cdev) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const BCEntry E = ent[e];
    if (E.kind == 7) return;                       // outlets run line by line in k_bc_outlet
    const DevBlock b = blks[E.blk];
    const Params p = cdev[b.cs].p;
    const int turb = cdev[b.cs].turb;
    double* V[7];
    for (int m = 0; m < 7; ++m) V[m] = slot(b, S_V + m);
    double* PP = slot(b, S_PP);
    double* T = slot(b, S_T);
    double* Rm = slot(b, S_RMIU);
    const int s0 = E.s[0], l0 = E.l[0];
    if (E.kind == 1) {                              // BC/BC_Wall.F90:42-117
        // wall velocity of the frame Kindsub_BC * omega (BC_Wall.F90:46-52), as the reference
        // evaluates it (its sign of zero included)
        const double ztemp = 0.5 * (slot(b, S_ZC)[s0] + slot(b, S_ZC)[l0]);
        const double ytemp = 0.5 * (slot(b, S_YC)[s0] + slot(b, S_YC)[l0]);
        const double vibc = 0.0;
        const double vjbc = (double)E.kindsub * p.omega0 * ztemp;
        const double vkbc = -(double)E.kindsub * p.omega0 * ytemp;
        for (int L = 0; L < 3; ++L) {
            int is = E.s[L], il = E.l[L];
            PP[il] = PP[is];
            T[il] = T[is];
            V[0][il] = PP[il] / (T[il] + p.Tiny) * p.RXM2;
            double den = V[0][il];
            V[1][il] = vibc * den;
            V[2][il] = vjbc * den;
            V[3][il] = vkbc * den;
        }
        if (turb) {
            double Dn = slot(b, S_DST)[l0];
            double Den = V[0][l0];
            double TT = T[l0];
            double Rmiuw = mu_suth<double>(p, TT);
            double Omegaw = 60.0 * Rmiuw / (Den * 0.075 * Dn * Dn * p.Ref * p.Ref);
            Rmiuw = Rm[s0];
            for (int L = 0; L < 3; ++L) {
                int il = E.l[L];
                V[5][il] = 0.0;
                V[6][il] = Omegaw;
                Rm[il] = Rmiuw;
            }
        }
    } else if (E.kind == 2) {                       // BC/BC_far.F90:40-118
        int d = E.dir - 1;
        double out_n = (double)(2 * E.lor - 4);
        double grad = slot(b, S_GRAD + d)[E.face];
        double Sout1 = slot(b, S_SD + 3 * d)[E.face] / grad;
        double Sout2 = slot(b, S_SD + 3 * d + 1)[E.face] / grad;
        double Sout3 = slot(b, S_SD + 3 * d + 2)[E.face] / grad;
        double Dnx = Sout1 * out_n, Dny = Sout2 * out_n, Dnz = Sout3 * out_n;
        double Den = V[0][s0];
        double Vxi = V[1][s0] / Den, Vyi = V[2][s0] / Den, Vzi = V[3][s0] / Den;
        double P2 = PP[s0];
        double PP0 = 0, Den0 = 0, Vx0 = 0, Vy0 = 0, Vz0 = 0, dir = 0;
        farbond(p.XM, P2, Den, Vxi, Vyi, Vzi, Dnx, Dny, Dnz, p.VxF, p.VyF, p.VzF, PP0, Den0, Vx0, Vy0, Vz0, dir);
        V[0][l0] = 2 * Den0 - V[0][s0];
        double den = V[0][l0];
        V[1][l0] = 2.0 * Vx0 - Vxi;
        V[2][l0] = 2.0 * Vy0 - Vyi;
        V[3][l0] = 2.0 * Vz0 - Vzi;
        PP[l0] = 2.0 * PP0 - P2;
        T[l0] = p.RXM2 * PP[l0] / den;
        for (int L = 1; L < 3; ++L) {
            int ig = E.l[L];
            for (int m = 0; m < 5; ++m) V[m][ig] = V[m][l0];
            PP[ig] = PP[l0];
            T[ig] = T[l0];
        }
        if (turb) {
            if (dir > 0.0) {
                V[5][l0] = V[5][s0];
                V[6][l0] = V[6][s0];
                Rm[l0] = Rm[s0];
            } else {
                double TT = T[l0];
                double Dn = V[0][l0];
                double RmiuFar = mu_suth<double>(p, TT);
                Rm[l0] = 2.0 * p.VisRatio * RmiuFar - Rm[s0];
                V[5][l0] = 2.0 * 1.5 * p.FSTI * p.FSTI * Dn - V[5][s0];
                V[6][l0] = V[5][l0] / (Rm[l0] + p.Tiny) * Dn;
            }
            for (int L = 1; L < 3; ++L) {
                int ig = E.l[L];
                V[5][ig] = V[5][l0];
                V[6][ig] = V[6][l0];
                Rm[ig] = Rm[l0];
            }
        }
    } else if (E.kind == 3) {                       // BC/BC_Symm.F90:42-110
        int d = E.dir - 1;
        double grad = slot(b, S_GRAD + d)[E.face];
        double Sout1 = slot(b, S_SD + 3 * d)[E.face] / grad;
        double Sout2 = slot(b, S_SD + 3 * d + 1)[E.face] / grad;
        double Sout3 = slot(b, S_SD + 3 * d + 2)[E.face] / grad;
        double den = V[0][s0];
        double Vxi = V[1][s0] / den, Vyi = V[2][s0] / den, Vzi = V[3][s0] / den;
        double Vc1 = Vxi * Sout1 + Vyi * Sout2 + Vzi * Sout3;
        for (int L = 0; L < 3; ++L) {
            int is = E.s[L], il = E.l[L];
            if (L != 1) V[0][il] = V[0][is];       // the second ghost layer keeps its density (BC_Symm.F90:70-75)
            V[1][il] = V[1][is] - 2 * Sout1 * Vc1 * V[0][is];
            V[2][il] = V[2][is] - 2 * Sout2 * Vc1 * V[0][is];
            V[3][il] = V[3][is] - 2 * Sout3 * Vc1 * V[0][is];
            V[4][il] = V[4][is];
            PP[il] = PP[is];
            T[il] = T[is];
        }
        if (turb)
            for (int L = 0; L < 3; ++L) {
                int is = E.s[L], il = E.l[L];
                V[5][il] = V[5][is];
                V[6][il] = V[6][is];
                Rm[il] = Rm[is];
            }
    } else if (E.kind == 5) {                       // BC/BC_Inlet.F90:38-110
        double PsIn = PP[s0];
        PsIn = dmin(PsIn, 0.999 * p.P0in);
        double comm = dmax(1.0, tmx::pow_(p.P0in / PsIn, 1.0 / 3.5));
        double mach = sqrt((comm - 1.0) * 2 / 0.4);
        double TsIn = p.T0in / comm;
        double Roin = p.RXM2 * PsIn / TsIn;
        double asonic = sqrt(1.4 * PsIn / Roin);
        double Vabs = mach * asonic;
        V[0][l0] = Roin;
        V[1][l0] = Roin * Vabs;
        V[2][l0] = Roin * (p.omega0 * slot(b, S_ZC)[s0]);
        V[3][l0] = Roin * (-p.omega0 * slot(b, S_YC)[s0]);
        double rr = p.omega0 * slot(b, S_RAD)[l0];
        V[4][l0] = PsIn / 0.4 + 0.5 * (sq(V[1][l0]) + sq(V[2][l0]) + sq(V[3][l0])) / Roin - 0.5 * sq(rr) * Roin;
        PP[l0] = PsIn;
        T[l0] = TsIn;
        for (int L = 1; L < 3; ++L) {
            int ig = E.l[L];
            for (int m = 0; m < 5; ++m) V[m][ig] = V[m][l0];
            PP[ig] = PsIn;
            T[ig] = TsIn;
        }
        if (turb) {
            double TT = T[l0];
            double RmiuIn = mu_suth<double>(p, TT);
            Rm[l0] = p.VisRatio * RmiuIn;
            double Den = V[0][l0];
            V[5][l0] = 1.5 * p.FSTI * p.FSTI * Den;
            V[6][l0] = V[5][l0] / (Rm[l0] + p.Tiny) * Den;
            for (int L = 1; L < 3; ++L) {
                int ig = E.l[L];
                V[5][ig] = V[5][l0];
                V[6][ig] = V[6][l0];
                Rm[ig] = Rm[l0];
            }
        }
    } else if (E.kind == 9) {                       // BC/BC_P2P.F90:76-139
        const DevBlock r = blks[E.src_blk];
        const double cost = E.cost, sint = E.sint;
        for (int L = 0; L < 3; ++L) {
            int is = E.s[L], il = E.l[L];
            V[0][il] = slot(r, S_V)[is];
            V[1][il] = slot(r, S_V + 1)[is];
            double txy = slot(r, S_V + 2)[is], txz = slot(r, S_V + 3)[is];
            V[2][il] = cost * txy + sint * txz;
            V[3][il] = -sint * txy + cost * txz;
            for (int m = 4; m < 7; ++m) V[m][il] = slot(r, S_V + m)[is];
            PP[il] = slot(r, S_PP)[is];
            T[il] = slot(r, S_T)[is];
            Rm[il] = slot(r, S_RMIU)[is];
        }
    }
}

// BC/BC_Outlet.F90:50-106: the static pressure recurrence runs along j, one warp per line.
// Each pass loads 32 entries at once (their interior values, radii and angles) and forms the
// terms that do not depend on the previous j (rcs1 - rcs2, rcs2 + tiny, omega * rcs2: the same
// operations the sequential loop does, issued earlier); the recurrence itself then runs entry
// by entry in the sequential loop's operation order, every lane repeating it on the entry's
// operands taken by shuffle, so the result is bit for bit the sequential one; the ghost writes
// are parallel again.
__global__ void k_bc_outlet(const DevBlock* __restrict__ blks, const BCEntry* __restrict__ ent,
                            const OutletLine* __restrict__ lines, int nl, const CaseDev* __restrict__ cdev) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= nl) return;                                   // whole warps leave together
    const OutletLine Ln = lines[w];
    const DevBlock b = blks[Ln.blk];
    const Params& p = cdev[b.cs].p;
    const int turb = cdev[b.cs].turb;
    double* V[7];
    for (int m = 0; m < 7; ++m) V[m] = slot(b, S_V + m);
    double* PP = slot(b, S_PP);
    double* T = slot(b, S_T);
    double* Rm = slot(b, S_RMIU);
    const double* rad = slot(b, S_RAD);
    const double* sint = slot(b, S_SINT);
    const double* cost = slot(b, S_COST);
    // the previous j's ghost values (PP, rho, rho*v, rho*w of the first ghost layer)
    double pp_prev = 0.0, den_prev = 1.0, v3_prev = 0.0, v4_prev = 0.0;
    for (int j0 = 0; j0 < Ln.n; j0 += 32) {
        const bool act = j0 + lane < Ln.n;
        BCEntry E;
        int first = 1;
        double Tl = 1.0, v1s = 1.0, v3s = 0.0, v4s = 0.0, dr = 0.0, rt = 1.0, wr = 0.0, sinr = 0.0, cosr = 0.0;
        if (act) {
            E = ent[Ln.first + j0 + lane];
            const int s0 = E.s[0];
            Tl = T[s0];
            v1s = V[0][s0];
            v3s = V[2][s0];
            v4s = V[3][s0];
            first = E.sub == 1;
            if (!first) {
                const int lm = E.l[0] - b.PI;              // (il, jl-1, kl)
                const double rcs1 = rad[E.l[0]], rcs2 = rad[lm];
                dr = rcs1 - rcs2;
                rt = rcs2 + p.Tiny;
                wr = p.omega0 * rcs2;
                sinr = sint[lm];
                cosr = cost[lm];
            }
        }
        const int cnt = min(32, Ln.n - j0);
        double pp = 0.0, den = 0.0, ratio = 0.0;
        for (int i = 0; i < cnt; ++i) {
            const int fi = __shfl_sync(0xffffffffu, first, i);
            const double tli = __shfl_sync(0xffffffffu, Tl, i), v1i = __shfl_sync(0xffffffffu, v1s, i);
            const double v3i = __shfl_sync(0xffffffffu, v3s, i), v4i = __shfl_sync(0xffffffffu, v4s, i);
            const double dri = __shfl_sync(0xffffffffu, dr, i), rti = __shfl_sync(0xffffffffu, rt, i);
            const double wri = __shfl_sync(0xffffffffu, wr, i);
            const double si = __shfl_sync(0xffffffffu, sinr, i), ci = __shfl_sync(0xffffffffu, cosr, i);
            double ppi;
            if (fi) {                                       // j == Jbgn
                ppi = p.Pouthub;
            } else {
                const double RoVr2 = sq(v4_prev / den_prev * ci - si * v3_prev / den_prev + wri);
                ppi = pp_prev + fabs(dri * den_prev * RoVr2) / rti;
            }
            const double deni = ppi / tli * p.RXM2;
            const double ri = deni / v1i;
            if (lane == i) { pp = ppi; den = deni; ratio = ri; }
            pp_prev = ppi;
            den_prev = deni;
            v3_prev = v3i * ri;
            v4_prev = v4i * ri;
        }
        if (!act) continue;
        const int s0 = E.s[0];
        const double v2 = V[1][s0] * ratio, v3 = v3s * ratio, v4 = v4s * ratio;
        for (int L = 0; L < 3; ++L) {
            const int ig = E.l[L];
            V[0][ig] = den; V[1][ig] = v2; V[2][ig] = v3; V[3][ig] = v4;
            PP[ig] = pp;
            T[ig] = Tl;
        }
        if (turb) {
            const double k6 = V[5][s0], k7 = V[6][s0], rm = Rm[s0];
            for (int L = 0; L < 3; ++L) {
                const int ig = E.l[L];
                V[5][ig] = k6; V[6][ig] = k7; Rm[ig] = rm;
            }
        }
    }
}

// ---------------------------------------------------------------------------------------
// primitives used by every stencil: u=V2/V1, v, w, k=V6/V1, omega=V7/V1, 1/V1 and V*(1/V1)
// ---------------------------------------------------------------------------------------
__global__ void k_prims(const DevBlock* __restrict__ blks, int nblk, long long total, const long long* __restrict__ off) {
    long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total) return;
    int lo = 0, hi = nblk - 1;
    while (lo < hi) { int mid = (lo + hi + 1) >> 1; if (off[mid] <= g) lo = mid; else hi = mid - 1; }
    const DevBlock b = blks[lo];
    int c = (int)(g - off[lo]);
    double v1 = slot(b, S_V)[c];
    slot(b, S_PRIM)[c] = slot(b, S_V + 1)[c] / v1;
    slot(b, S_PRIM + 1)[c] = slot(b, S_V + 2)[c] / v1;
    slot(b, S_PRIM + 2)[c] = slot(b, S_V + 3)[c] / v1;
    slot(b, S_PRIM + 3)[c] = slot(b, S_V + 5)[c] / v1;
    slot(b, S_PRIM + 4)[c] = slot(b, S_V + 6)[c] / v1;
    double ri = 1.0 / v1;
    slot(b, S_RINV)[c] = ri;
    slot(b, S_SVEL)[c] = slot(b, S_V + 1)[c] * ri;
    slot(b, S_SVEL + 1)[c] = slot(b, S_V + 2)[c] * ri;
    slot(b, S_SVEL + 2)[c] = slot(b, S_V + 3)[c] * ri;
}

// FP32 copies of FP64 slot ranges over every padded cell (mixed path)
__global__ void k_mirror(const DevBlock* __restrict__ blks, int nblk, long long total, const long long* __restrict__ off,
                         MirrorList ml) {
    long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total) return;
    int lo = 0, hi = nblk - 1;
    while (lo < hi) { int mid = (lo + hi + 1) >> 1; if (off[mid] <= g) lo = mid; else hi = mid - 1; }
    const DevBlock b = blks[lo];
    int c = (int)(g - off[lo]);
    for (int r = 0; r < ml.n; ++r)
        for (int q = ml.first[r]; q < ml.first[r] + ml.count[r]; ++q) {
            if (ml.to_fp64) slot(b, q)[c] = (double)fslot(b, q)[c];
            else fslot(b, q)[c] = (float)slot(b, q)[c];
        }
}

#endif  // TG_COMMON_KERNELS


// ---------------------------------------------------------------------------------------
// ---------------------------------------------------------------------------------------
// Space/DIFF_DqDxyz.F90:25-74, 232-265, 300-381 (gradients and shock sensor, interior cells)
// ---------------------------------------------------------------------------------------
template <typename R>
__global__ void k_gradient(const DevBlock* __restrict__ blks, const Tile* __restrict__ tiles, const CaseDev* __restrict__ cdev) {
    const Tile t = tiles[blockIdx.x];
    if ((int)threadIdx.x >= t.count) return;
    const DevBlock b = blks[t.blk];
    const int turb = cdev[b.cs].turb;
    int n = t.start + threadIdx.x;
    int I = n % b.NI1 + 1, J = (n / b.NI1) % b.NJ1 + 1, K = n / (b.NI1 * b.NJ1) + 1;
    int c = cidx(b, I, J, K);
    const int st[3] = {1, b.PI, b.PI * b.PJ};
    R volinv = R(1.0) / rs<R>(b, S_VOL)[c];
    const R* qs[6] = {rs<R>(b, S_PRIM), rs<R>(b, S_PRIM + 1), rs<R>(b, S_PRIM + 2), rs<R>(b, S_T),
                      rs<R>(b, S_PRIM + 3), rs<R>(b, S_PRIM + 4)};
    int nq = turb ? 6 : 4;
    const R* SD = rs<R>(b, S_SD);
    // FP32: the gradients stay in registers until every stencil load is issued (a load after a
    // store to the same arena would wait for the previous round trip), then go out together;
    // FP64: stored as they come (holding them raised the FP64 kernel from 128 to 158 registers,
    // and it is bound by the FP64 pipe, not by load latency)
    R gq[6][3];
    for (int q = 0; q < nq; ++q) {
        R fw[3], fe[3];
        for (int d = 0; d < 3; ++d) {
            const R* al = rs<R>(b, S_ALAGM + d);
            const R* ai = rs<R>(b, S_AINV + d);
            fw[d] = favg(qs[q], al, ai, c, st[d]);
            fe[d] = favg(qs[q], al, ai, c + st[d], st[d]);
        }
        for (int m = 0; m < 3; ++m) {
            const R* S1 = SD + (size_t)(0 * 3 + m) * b.ncell;
            const R* S2 = SD + (size_t)(1 * 3 + m) * b.ncell;
            const R* S3 = SD + (size_t)(2 * 3 + m) * b.ncell;
            R g = volinv * (fe[0] * S1[c + st[0]] - fw[0] * S1[c] + fe[1] * S2[c + st[1]] - fw[1] * S2[c]
                                 + fe[2] * S3[c + st[2]] - fw[2] * S3[c]);
            gq[q][m] = g;
            if constexpr (sizeof(R) == 8) rs<R>(b, S_DQ + 3 * q + m)[c] = g;
        }
    }
    if constexpr (sizeof(R) == 4)
        for (int q = 0; q < nq; ++q)
            for (int m = 0; m < 3; ++m) rs<R>(b, S_DQ + 3 * q + m)[c] = gq[q][m];
    R DuDx = gq[0][0], DuDy = gq[0][1], DuDz = gq[0][2];
    R DvDx = gq[1][0], DvDy = gq[1][1], DvDz = gq[1][2];
    R DwDx = gq[2][0], DwDy = gq[2][1], DwDz = gq[2][2];
    R W12 = (DuDy - DvDx) / R(2.0), W13 = (DuDz - DwDx) / R(2.0), W23 = (DvDz - DwDy) / R(2.0);
    R Vort = sqrt(R(2.0) * (R(2.0) * W12 * W12 + R(2.0) * W13 * W13 + R(2.0) * W23 * W23));
    R DivU = sqrt(DuDx * DuDx + DvDy * DvDy + DwDz * DwDz);
    rs<R>(b, S_SHOCK)[c] = DivU * DivU / dmax(DivU * DivU + Vort * Vort, R(1.0));
    const ParamsT<R>& p = cparams<R>(cdev[b.cs]);
    if (p.Kind_Roe == 2) {
        // the hybrid blend Fscheme (Space/DIFF_DqDxyz.F90:311-380), read only by the rotated Roe
        // scheme: CH1 = 3, CH2 = 1, CH3 = 2, cmu = 0.09, tau = 1; real exponents 2 and 3 as
        // products, 0.5 as a square root
        R S11 = (DuDx + DuDx) / R(2.), S22 = (DvDy + DvDy) / R(2.), S33 = (DwDz + DwDz) / R(2.);
        R S12 = (DuDy + DvDx) / R(2.), S13 = (DuDz + DwDx) / R(2.), S23 = (DwDy + DvDz) / R(2.);
        R Skl = sqrt(R(2.) * (R(1.) * S11 * S11 + R(1.) * S22 * S22 + R(1.) * S33 * S33 + R(2.) * S12 * S12 +
                              R(2.) * S13 * S13 + R(2.) * S23 * S23));
        R Den = rs<R>(b, S_V)[c], RmiuT = rs<R>(b, S_RMIU)[c], TT = rs<R>(b, S_T)[c];
        R RMIUL = mu_suth<R>(p, TT);
        R vK = rs<R>(b, S_V + 5)[c] / Den, vOmega = rs<R>(b, S_V + 6)[c] / Den;
        R DLTxyz = rs<R>(b, S_ALENG)[c];
        auto G = [&](int q) { return rs<R>(b, S_DQ + q)[c]; };
        R dTKO = G(12) * G(15) + G(13) * G(16) + G(14) * G(17);
        R Dist = rs<R>(b, S_DST)[c];
        const R Sigo2 = R(p.Sigo2), Bs = R(p.Beta_star), Ref = R(p.Ref);
        R CDKO = dmax(R(2.0) * Den * Sigo2 / vOmega * (dTKO), R(1.0e-10));
        R arg1 = dmax(sqrt(vK) / Bs / vOmega / Dist / Ref, R(500.0) * RMIUL / Den / Dist / Dist / vOmega / Ref / Ref);
        arg1 = dmin(arg1, R(4.0) * Den * Sigo2 * vK / CDKO / Dist / Dist);
        R a2 = arg1 * arg1;
        R FunC1 = ttanh(a2 * a2);
        R aLgrd = ((R(1.) - FunC1) * R(0.61) + FunC1 * R(0.78)) * DLTxyz;
        R B0 = R(2.) * Vort * dmax(Vort, Skl) / dmax((Vort * Vort + Skl * Skl) / R(2.), R(p.Alscale) * R(0.1));
        R g0 = ttanh(B0 * B0 * B0 * B0);
        R sok = dmax(sqrt((Vort * Vort + Skl * Skl) / R(2.)), R(0.1) / R(1.0));
        R alturb = sqrt((RmiuT + RMIUL) / Den / (Ref * sok * p15(R(0.09))));
        R A0 = R(1.) * dmax(((aLgrd / alturb / g0) - R(0.1)), R(0.0));
        rs<R>(b, S_FSCH)[c] = dmax(R(1.) * ttanh(A0 * A0 * A0), R(p.F_limiter1));
    }
}

// shock of the three ghost layers of every face = shock of the adjacent interior cell
// (Space/DIFF_DqDxyz.F90:388-396 restricted to the face ghosts the stencils read)
template <typename R>
__global__ void k_shock_ghost(const DevBlock* __restrict__ blks, const Tile* __restrict__ tiles) {
    const Tile t = tiles[blockIdx.x];
    if ((int)threadIdx.x >= t.count) return;
    const DevBlock b = blks[t.blk];
    int n = t.start + threadIdx.x;
    // enumerate 6 faces x 3 layers of face cells
    int nf[3] = {b.NJ1 * b.NK1, b.NI1 * b.NK1, b.NI1 * b.NJ1};
    int d = 0;
    while (n >= 6 * nf[d]) { n -= 6 * nf[d]; ++d; }
    int side = n / (3 * nf[d]); n -= side * 3 * nf[d];
    int L = n / nf[d] + 1; n -= (L - 1) * nf[d];
    int i, j, k, ii, jj, kk;
    if (d == 0) { j = n % b.NJ1 + 1; k = n / b.NJ1 + 1; i = side ? b.NI1 + L : 1 - L; ii = side ? b.NI1 : 1; jj = j; kk = k; }
    else if (d == 1) { i = n % b.NI1 + 1; k = n / b.NI1 + 1; j = side ? b.NJ1 + L : 1 - L; jj = side ? b.NJ1 : 1; ii = i; kk = k; }
    else { i = n % b.NI1 + 1; j = n / b.NI1 + 1; k = side ? b.NK1 + L : 1 - L; kk = side ? b.NK1 : 1; ii = i; jj = j; }
    R* sh = rs<R>(b, S_SHOCK);
    sh[cidx(b, i, j, k)] = sh[cidx(b, ii, jj, kk)];
    if (L == 1) {       // Fscheme's face-adjacent ghosts (Space/DIFF_DqDxyz.F90:399-404)
        R* fs = rs<R>(b, S_FSCH);
        fs[cidx(b, i, j, k)] = fs[cidx(b, ii, jj, kk)];
    }
}

// BC_Boundarys(0): gradients of the first ghost layer (BC/*.F90 sweep 0, BC/BC_P2P.F90:140-184)
// the 18 gradient components of a ghost cell across a 1-to-1 interface rotated by the
// interface's angle (BC/BC_P2P.F90:140-181): g = the source cell's, o = the ghost's
template <typename R>
__device__ inline void p2p_grad_rotate(const R* g, R cost, R sint, R* o) {
    const R cos2t = cost * cost, sin2t = sint * sint, sct = sint * cost;
    const R ugx = g[0], ugy = g[1], ugz = g[2];
    const R vgx = g[3], vgy = g[4], vgz = g[5];
    const R wgx = g[6], wgy = g[7], wgz = g[8];
    o[0] = ugx;
    o[1] = cost * ugy + sint * ugz;
    o[2] = -sint * ugy + cost * ugz;
    o[3] = cost * vgx + sint * wgx;
    o[4] = cos2t * vgy + sct * (vgz + wgy) + sin2t * wgz;
    o[5] = cos2t * vgz + sct * (-vgy + wgz) - sin2t * wgy;
    o[6] = -sint * vgx + cost * wgx;
    o[7] = -sin2t * vgz + sct * (-vgy + wgz) + cos2t * wgy;
    o[8] = sin2t * vgy + sct * (vgz + wgy) + cos2t * wgz;
    for (int LL = 4; LL <= 6; ++LL) {
        const int L = (LL - 1) * 3;            // 0-based first component of the group
        o[L] = g[L];
        const R gy = g[L + 1], gz = g[L + 2];
        o[L + 1] = cost * gy + sint * gz;
        o[L + 2] = -sint * gy + cost * gz;
    }
}

// unpack of a cross-rank 1-to-1 segment (see k_halo_pack): sweep -1 writes the FP64 state with
// R = double; sweep 0 the gradients in R (the FP32 copies in the mixed path), so each runs in
// the translation unit, and with the contraction, of the same-rank copy it stands in for
template <typename R>
__global__ void k_halo_unpack(DevBlock b, const int* __restrict__ tab, int n, int sweep, double cost, double sint,
                              const double* __restrict__ in) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    if (sweep == -1) {
        const double* w = in + (size_t)36 * tab[4 * q];
        const int off[3] = {0, 14, 25};
        for (int L = 0; L < 3; ++L) {
            const double* x = w + off[L];
            const int il = tab[4 * q + 1 + L];
            slot(b, S_V)[il] = x[0];
            slot(b, S_V + 1)[il] = x[1];
            const double txy = x[2], txz = x[3];
            slot(b, S_V + 2)[il] = cost * txy + sint * txz;
            slot(b, S_V + 3)[il] = -sint * txy + cost * txz;
            for (int m = 4; m < 7; ++m) slot(b, S_V + m)[il] = x[m];
            slot(b, S_PP)[il] = x[7];
            slot(b, S_T)[il] = x[8];
            slot(b, S_RMIU)[il] = x[9];
        }
    } else {
        const double* w = in + (size_t)18 * tab[4 * q];
        const int il = tab[4 * q + 1];
        R g[18], o[18];
        for (int m = 0; m < 18; ++m) g[m] = R(w[m]);
        p2p_grad_rotate<R>(g, R(cost), R(sint), o);
        for (int m = 0; m < 18; ++m) rs<R>(b, S_DQ + m)[il] = o[m];
    }
}

template <typename R>
__global__ void k_bc_grad(const DevBlock* __restrict__ blks, const BCEntry* __restrict__ ent, int n) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const BCEntry E = ent[e];
    const DevBlock b = blks[E.blk];
    const int il = E.l[0], is = E.s[0];
    if (E.kind != 9) {
        for (int L = 0; L < 18; ++L) rs<R>(b, S_DQ + L)[il] = rs<R>(b, S_DQ + L)[is];
        return;
    }
    const DevBlock r = blks[E.src_blk];
    R g[18], o[18];
    for (int L = 0; L < 18; ++L) g[L] = rs<R>(r, S_DQ + L)[is];
    p2p_grad_rotate<R>(g, R(E.cost), R(E.sint), o);
    for (int L = 0; L < 18; ++L) rs<R>(b, S_DQ + L)[il] = o[L];
}

// ---------------------------------------------------------------------------------------
// Face fluxes of direction DIR (faces 1..N along DIR, interior in the other two):
//   Space/DIFFUSION_Centered.F90, Space/TURBTWO_DIFFUSION_Centered.F90,
//   Space/CONVECT_MUSCL.F90 | Space/CONVECT_MDCD.F90, Space/TURBTWO_CONVECT_MUSCL.F90,
//   Space/CONVECT_Roe_Original.F90 | Space/CONVECT_AUSMPW_Plus.F90, Space/TURBTWO_CONVECT_Upwind.F90
//
// face_flux_body computes the NFX fluxes of one face from an accessor q: q.v(slot, o) is the
// slot's value at the cell o steps along DIR from the face's cell c (o = -1 is the cell on the
// face's minus side).  The kernels differ only in where the values come from: FaceGlobal reads
// the slot arrays (k_face_flux); the shared-memory tiles of the mixed path read a staged copy.
// ---------------------------------------------------------------------------------------
template <typename R>
struct FaceGlobal {
    const DevBlock& b;
    int c, s;
    __device__ R v(int slot, int o) const { return R(rs<R>(b, slot)[c + o * s]); }
};

// PART 0: every flux; 1: the viscous and k-omega diffusion fluxes only; 2: the convective ones
template <typename R, int DIR, int PART = 0, class A>
__device__ __forceinline__ void face_flux_body(const ParamsT<R>& p, int turb, const A& q, R* F) {
    constexpr int d = DIR - 1;
    constexpr int AL = S_ALAGM + d, AIN = S_AINV + d, SDD = S_SD + 3 * d;
    // face average of a slot at the face o steps from this one (SPACEINTERP_GetSurfCenterVars)
    auto fa = [&](int slot, int o) { return (q.v(AL, o) * q.v(slot, o - 1) + q.v(AL, o - 1) * q.v(slot, o)) * q.v(AIN, o); };
    if constexpr (PART != 2) {
    // ---------------- viscous flux (DIFFUSION_Centered) ----------------
    const bool wall = q.v(S_WALL + d, 0) != R(0.0);
    const R vinv = q.v(S_VINV + d, 0);
    const R vall = q.v(S_VOL, -1) * vinv;
    const R valr = q.v(S_VOL, 0) * vinv;
    const R alsinv = wall ? R(0.0) : R(vinv);
    constexpr int qv[4] = {S_PRIM, S_PRIM + 1, S_PRIM + 2, S_T};
    R g[4][3];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int Q = qv[k];
        R disfpp = fa(Q, 1);
        R disfnn = fa(Q, -1);
        R disfp = q.v(Q, 0), disfn = q.v(Q, -1);
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            const int G = S_DQ + 3 * k + m;
            R xL = vall * q.v(G, -1) + valr * q.v(G, 0);
            R cmv = alsinv * (-q.v(SDD + m, 1) * (disfpp - disfp) - q.v(SDD + m, -1) * (disfn - disfnn) +
                              q.v(SDD + m, 0) * (disfp - disfn));
            g[k][m] = cmv + xL;
        }
    }
    const R a0 = q.v(AL, 0), a1 = q.v(AL, -1);
    const R ai = q.v(AIN, 0);
    const R all = a0 * ai, alr = a1 * ai;
    const R TTL = fa(S_T, 0);
    const R RmiuL = mu_suth<R>(p, TTL);
    R RmiuTL = all * q.v(S_RMIU, -1) + alr * q.v(S_RMIU, 0);
    if (wall) RmiuTL = R(0.0);
    {
        const R NMD = R(-2.0 / 3.0);
        R DuDxL = g[0][0], DuDyL = g[0][1], DuDzL = g[0][2];
        R DvDxL = g[1][0], DvDyL = g[1][1], DvDzL = g[1][2];
        R DwDxL = g[2][0], DwDyL = g[2][1], DwDzL = g[2][2];
        R DTDxL = g[3][0], DTDyL = g[3][1], DTDzL = g[3][2];
        R div = DuDxL + DvDyL + DwDzL;
        R Txx = RmiuL * (NMD * div + R(2.0) * DuDxL) + RmiuTL * (NMD * div + R(2.0) * DuDxL);
        R Tyy = RmiuL * (NMD * div + R(2.0) * DvDyL) + RmiuTL * (NMD * div + R(2.0) * DvDyL);
        R Tzz = RmiuL * (NMD * div + R(2.0) * DwDzL) + RmiuTL * (NMD * div + R(2.0) * DwDzL);
        R Txy = RmiuL * (DuDyL + DvDxL) + RmiuTL * (DuDyL + DvDxL);
        R Tyz = RmiuL * (DvDzL + DwDyL) + RmiuTL * (DvDzL + DwDyL);
        R Tzx = RmiuL * (DuDzL + DwDxL) + RmiuTL * (DuDzL + DwDxL);
        R cp_ = R(1.4) * R(p.PPF) / R(1.4 - 1.0);
        R akmu = cp_ * (RmiuL / R(0.72) + RmiuTL / R(0.9));
        R ucc = fa(S_PRIM, 0), vcc = fa(S_PRIM + 1, 0), wcc = fa(S_PRIM + 2, 0);
        R Phix = akmu * DTDxL + ucc * Txx + vcc * Txy + wcc * Tzx;
        R Phiy = akmu * DTDyL + ucc * Txy + vcc * Tyy + wcc * Tyz;
        R Phiz = akmu * DTDzL + ucc * Tzx + vcc * Tyz + wcc * Tzz;
        R Dx = q.v(SDD, 0), Dy = q.v(SDD + 1, 0), Dz = q.v(SDD + 2, 0);
        R Ref = R(p.Ref);
        F[FX_VX] = (Txx * Dx + Txy * Dy + Tzx * Dz) / Ref;
        F[FX_VY] = (Txy * Dx + Tyy * Dy + Tyz * Dz) / Ref;
        F[FX_VZ] = (Tzx * Dx + Tyz * Dy + Tzz * Dz) / Ref;
        F[FX_VE] = (Phix * Dx + Phiy * Dy + Phiz * Dz) / Ref;
    }
    // ---------------- k-omega diffusion (TURBTWO_DIFFUSION_Centered) ----------------
    if (turb) {
        R gt[2][3];
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const int Q = S_PRIM + 3 + k;
            R disfpp = fa(Q, 1);
            R disfnn = fa(Q, -1);
            R disfp = q.v(Q, 0), disfn = q.v(Q, -1);
#pragma unroll
            for (int m = 0; m < 3; ++m) {
                const int G = S_DQ + 12 + 3 * k + m;
                R xL = vall * q.v(G, -1) + valr * q.v(G, 0);
                R cmv = alsinv * (-q.v(SDD + m, 1) * (disfpp - disfp) - q.v(SDD + m, -1) * (disfn - disfnn) +
                                  q.v(SDD + m, 0) * (disfp - disfn));
                gt[k][m] = cmv + xL;
            }
        }
        R TTLt = all * q.v(S_T, -1) + alr * q.v(S_T, 0);
        R RmiuLt = mu_suth_nocs<R>(p, TTLt);
        const R Ref = R(p.Ref);
        R SigkAB, SigoAB;
        if (p.Kind_Model == 2) {         // WD+2006: constant sigma (TURBTWO_DIFFUSION_Centered.F90:168-170)
            SigkAB = R(p.Sigk1);
            SigoAB = R(p.Sigo1);
        } else {
            R DEN0 = q.v(S_V, 0), TKK0 = q.v(S_PRIM + 3, 0), TOO0 = q.v(S_PRIM + 4, 0);
            R DEN1 = q.v(S_V, -1), TKK1 = q.v(S_PRIM + 3, -1), TOO1 = q.v(S_PRIM + 4, -1);
            R Den = all * DEN1 + alr * DEN0;
            R TKK = all * TKK1 + alr * TKK0;
            R TOO = all * TOO1 + alr * TOO0;
            R dTKO = gt[0][0] * gt[1][0] + gt[0][1] * gt[1][1] + gt[0][2] * gt[1][2];
            R Sigo2 = R(p.Sigo2), Bs = R(p.Beta_star);
            R CDKO = dmax(R(2.0) * Den * Sigo2 / TOO * (dTKO), R(1.0e-10));
            R distfc = alr * q.v(S_DST, 0) + all * q.v(S_DST, -1);
            R arg1 = dmax(sqrt(TKK) / Bs / TOO / distfc / Ref, R(500.0) * RmiuLt / Den / distfc / distfc / TOO / Ref / Ref);
            arg1 = dmin(arg1, R(4.0) * Den * Sigo2 * TKK / CDKO / distfc / distfc);
            R a2 = arg1 * arg1;
            R fc1c = ttanh(a2 * a2);
            SigkAB = fc1c * R(p.Sigk1) + (R(1.0) - fc1c) * R(p.Sigk2);
            SigoAB = fc1c * R(p.Sigo1) + (R(1.0) - fc1c) * Sigo2;
        }
        R vmute = RmiuLt + RmiuTL * SigkAB;
        R vmuoq = RmiuLt + RmiuTL * SigoAB;
        R Dx = q.v(SDD, 0), Dy = q.v(SDD + 1, 0), Dz = q.v(SDD + 2, 0);
        F[FX_TK] = (vmute * (gt[0][0] * Dx + gt[0][1] * Dy + gt[0][2] * Dz)) / Ref;
        F[FX_TO] = (vmuoq * (gt[1][0] * Dx + gt[1][1] * Dy + gt[1][2] * Dz)) / Ref;
    }
    }   // PART != 2
    if constexpr (PART == 1) return;
    // ---------------- reconstruction ----------------
    R qL[7], qR[7];
    constexpr int qc[5] = {S_PRIM, S_PRIM + 1, S_PRIM + 2, S_PP, S_T};
    R gama = R(0.0);
    if (p.Kind_Spatial <= 2) {     // CONVECT_MUSCL (2) or CONVECT_MUSCL2 (1): the limiter differs
        const bool m2 = p.Kind_Spatial == 1;
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            const int Q = qc[k];
            R fm = fa(Q, -1), f0 = fa(Q, 0), fp = fa(Q, 1);
            R q1 = q.v(Q, -1), q0 = q.v(Q, 0);
            R DR = f0 - q1, DL = q1 - fm;
            qL[k] = q1 + (m2 ? muscl2_limiter(DR, DL) : alimiter(DR, DL));
            DR = fp - q0; DL = q0 - f0;
            qR[k] = q0 - (m2 ? muscl2_limiter(DL, DR) : alimiter(DL, DR));
        }
    } else {                       // CONVECT_MDCD (3) or CONVECT_MDCDHYB (4)
        const bool hyb = p.Kind_Spatial == 4;
        R sensor = q.v(S_SHOCK, -3);
        sensor = dmax(sensor, q.v(S_SHOCK, -2));
        sensor = dmax(sensor, q.v(S_SHOCK, -1));
        sensor = dmax(sensor, q.v(S_SHOCK, 0));
        sensor = dmax(sensor, q.v(S_SHOCK, 1));
        sensor = dmax(sensor, q.v(S_SHOCK, 2));
        if (DIR == 3 && !hyb) sensor = dmax(sensor, R(0.0));
        gama = R(p.gama_min) + sensor * (R(p.gama_max) - R(p.gama_min));
        // MDCDHYB: MUSCL states where the sensor reaches F_limiter2 (Space/CONVECT_MDCDHYB.F90:118-120, 175-177)
        const bool muscl = hyb && sensor >= R(p.F_limiter2);
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            const int Q = qc[k];
            R s6[6];
#pragma unroll
            for (int o = 0; o < 6; ++o) s6[o] = q.v(Q, o - 3);
            if (muscl) {
                qL[k] = s6[2] + R(0.5) * alimiter(s6[3] - s6[2], s6[2] - s6[1]);
                qR[k] = s6[3] - R(0.5) * alimiter(s6[3] - s6[2], s6[4] - s6[3]);
            } else {
                mdcd_pair(s6, gama, qL[k], qR[k]);
            }
        }
    }
    if (turb) {
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const int Q = S_PRIM + 3 + k;
            R fm = fa(Q, -1), f0 = fa(Q, 0), fp = fa(Q, 1);
            R q1 = q.v(Q, -1), q0 = q.v(Q, 0);
            R DR = f0 - q1, DL = q1 - fm;
            qL[5 + k] = q1 + alimiter(DR, DL);
            DR = fp - q0; DL = q0 - f0;
            qR[5 + k] = q0 - alimiter(DL, DR);
        }
    }
    // ---------------- frame speeds of the two states (rotating frame) ----------------
    // rLo, rRo = rccl, rccr * omega(1), read by the Roe schemes only.  rccl/rccr start as the
    // face average of rad (SPACEINTERP_GetSurfCenterVars); CONVECT_MUSCL / CONVECT_MUSCL2 limit
    // them like the primitives (CONVECT_MUSCL.F90:111-116, CONVECT_MUSCL2.F90:114-118); CONVECT_MDCD
    // replaces them in I and J by the MDCD states of rad with the cell's weights
    // (CONVECT_MDCD.F90:51-120, 259-328) and leaves the K faces at the average (its K block sits
    // outside the face loops, :450-521); CONVECT_MDCDHYB leaves every face at the average.
    R rLo = R(0.0), rRo = R(0.0);
    if (p.omega0 != R(0.0) && p.Kind_Roe != 3) {
        R rl, rr;
        if (p.Kind_Spatial <= 2) {
            const bool m2 = p.Kind_Spatial == 1;
            R fm = fa(S_RAD, -1), f0 = fa(S_RAD, 0), fp = fa(S_RAD, 1);
            R q1 = q.v(S_RAD, -1), q0 = q.v(S_RAD, 0);
            R DR = f0 - q1, DL = q1 - fm;
            rl = q1 + (m2 ? muscl2_limiter(DR, DL) : alimiter(DR, DL));
            DR = fp - q0; DL = q0 - f0;
            rr = q0 - (m2 ? muscl2_limiter(DL, DR) : alimiter(DL, DR));
        } else if (p.Kind_Spatial == 3 && DIR != 3) {
            R s6[6];
#pragma unroll
            for (int o = 0; o < 6; ++o) s6[o] = q.v(S_RAD, o - 3);
            mdcd_pair(s6, gama, rl, rr);
        } else {
            rl = fa(S_RAD, 0);
            rr = rl;
        }
        rLo = rl * R(p.omega0);
        rRo = rr * R(p.omega0);
    }
    // ---------------- inviscid flux ----------------
    R sav1 = q.v(SDD, 0), sav2 = q.v(SDD + 1, 0), sav3 = q.v(SDD + 2, 0);
    R sav = q.v(S_GRAD + d, 0);
    R f[5];
    if (p.Kind_Roe == 2) {          // rotated Roe: the contribution already carries |S|
        const R Funscheme = (q.v(S_FSCH, -1) + q.v(S_FSCH, 0)) / R(2.);
        roe_rotated<R>(p, qL[3], qR[3], qL[4], qR[4], qL[0], qR[0], qL[1], qR[1], qL[2], qR[2], sav1, sav2, sav3, sav,
                       rLo, rRo, Funscheme, f);
#pragma unroll
        for (int L = 0; L < 5; ++L) F[FX_C0 + L] = f[L];
    } else {
        if (p.Kind_Roe == 1) {
            // preconditioning reads VL(d,8), the face-averaged eddy viscosity (0 while turbulence
            // is off), and Alagm(d) of the face's cell (Space/CONVECT_Roe_Original.F90:86-87)
            const R RmiuTf = (p.IF_Precondition && turb) ? fa(S_RMIU, 0) : R(0.0);
            roe_flux<R>(p, qL[3], qR[3], qL[4], qR[4], qL[0], qR[0], qL[1], qR[1], qL[2], qR[2], sav1, sav2, sav3, sav, rLo, rRo,
                        f, RmiuTf, q.v(AL, 0));
        } else
            ausmpw_flux<R>(p, qL[3], qR[3], qL[4], qR[4], qL[0], qR[0], qL[1], qR[1], qL[2], qR[2], sav1, sav2, sav3, sav, f);
#pragma unroll
        for (int L = 0; L < 5; ++L) F[FX_C0 + L] = f[L] * sav;
    }
    if (turb) {
        R rcpcv = R(p.PPF);
        R DENL = qL[3] / (rcpcv * qL[4]), DENR = qR[3] / (rcpcv * qR[4]);
        R ulnormal = (sav1 * qL[0] + sav2 * qL[1] + sav3 * qL[2]);
        R urnormal = (sav1 * qR[0] + sav2 * qR[1] + sav3 * qR[2]);
        R rulnormal = DENL * ulnormal, rurnormal = DENR * urnormal;
        const R small = R(1.e-10);
        R eigTKO = R(0.5) * dmax(fabs(ulnormal), fabs(urnormal));
        R TKL = dmax(qL[5], small), TKR = dmax(qR[5], small);
        F[FX_CK] = R(-0.5) * (rulnormal * TKL + rurnormal * TKR - eigTKO * (DENR * TKR - DENL * TKL));
        R TOL = dmax(qL[6], small), TOR = dmax(qR[6], small);
        F[FX_CO] = R(-0.5) * (rulnormal * TOL + rurnormal * TOR - eigTKO * (DENR * TOR - DENL * TOL));
    }
}

#ifndef TG_FACE_MINB
#define TG_FACE_MINB 8      // resident CTAs per SM asked of the FP32 convective-flux kernels (64 registers)
#endif
#ifndef TG_FACE_MINB_VISC
#define TG_FACE_MINB_VISC 6 // ... of the FP32 viscous-flux kernels (80 registers)
#endif
// one thread per face; the fluxes go to the FX slots, k_gather sums them per cell.  PART 0: all
// of them in one kernel; both paths launch the viscous and k-omega diffusion fluxes (PART 1)
// and the convective ones (PART 2) as two kernels, which share few inputs and write disjoint
// FX words, so that each gets its own register budget (the same arithmetic, so the FP64
// fluxes stay bit-identical): as one kernel the FP32 fluxes needed 96 registers (five CTAs per
// SM) and were issue-latency bound, split 80 and 64 (six and eight); the FP64 ones 250 (two),
// split at most 168 and 142 (three each)
template <typename R, int DIR, int PART = 0>
__global__ void __launch_bounds__(128, sizeof(R) == 4 ? (PART == 1 ? TG_FACE_MINB_VISC : TG_FACE_MINB) : (PART == 0 ? 1 : 3)) k_face_flux(const DevBlock* __restrict__ blks, const Tile* __restrict__ tiles,
                                                          const CaseDev* __restrict__ cdev) {
    const Tile t = tiles[blockIdx.x];
    if ((int)threadIdx.x >= t.count) return;
    const DevBlock b = blks[t.blk];
    const ParamsT<R> p = cparams<R>(cdev[b.cs]);
    const int turb = cdev[b.cs].turb;
    int n = t.start + threadIdx.x;
    const int ni = DIR == 1 ? b.NI : b.NI1, nj = DIR == 2 ? b.NJ : b.NJ1;
    int i = n % ni + 1, j = (n / ni) % nj + 1, k = n / (ni * nj) + 1;
    const int s = DIR == 1 ? 1 : (DIR == 2 ? b.PI : b.PI * b.PJ);
    const int c = cidx(b, i, j, k);
    const FaceGlobal<R> q{b, c, s};
    R F[NFX];
    face_flux_body<R, DIR, PART>(p, turb, q, F);
    const size_t nc = (size_t)b.ncell;
    R* FX = rs<R>(b, S_FX + NFX * (DIR - 1));
    if constexpr (PART != 2) {
#pragma unroll
        for (int m = 0; m < FX_TK; ++m) FX[(size_t)m * nc + c] = F[m];
        if (turb) {
            FX[(size_t)FX_TK * nc + c] = F[FX_TK];
            FX[(size_t)FX_TO * nc + c] = F[FX_TO];
        }
    }
    if constexpr (PART != 1) {
#pragma unroll
        for (int m = FX_C0; m < FX_CK; ++m) FX[(size_t)m * nc + c] = F[m];
        if (turb) {
            FX[(size_t)FX_CK * nc + c] = F[FX_CK];
            FX[(size_t)FX_CO * nc + c] = F[FX_CO];
        }
    }
}

// ---------------------------------------------------------------------------------------
// D of every interior cell in the reference's accumulation order (main.F90:92-133):
//   D = 0 - Fv(i) + Fv(i+1) - Fv(j) + Fv(j+1) - Fv(k) + Fv(k+1) - Fc(i) + Fc(i+1) - ...
// ---------------------------------------------------------------------------------------
template <typename R>
__global__ void k_gather(const DevBlock* __restrict__ blks, const Tile* __restrict__ tiles, const CaseDev* __restrict__ cdev) {
    const Tile t = tiles[blockIdx.x];
    if ((int)threadIdx.x >= t.count) return;
    const DevBlock b = blks[t.blk];
    const int turb = cdev[b.cs].turb;
    int n = t.start + threadIdx.x;
    int I = n % b.NI1 + 1, J = (n / b.NI1) % b.NJ1 + 1, K = n / (b.NI1 * b.NJ1) + 1;
    int c = cidx(b, I, J, K);
    const int st[3] = {1, b.PI, b.PI * b.PJ};
    const size_t nc = (size_t)b.ncell;
    const R* FX = rs<R>(b, S_FX);
    auto fx = [&](int d, int m, int cc) { return R(FX[(size_t)(NFX * d + m) * nc + cc]); };
    {   // rho: no viscous flux
        R acc = R(0.0);
        for (int d = 0; d < 3; ++d) { acc = acc - fx(d, FX_C0, c); acc = acc + fx(d, FX_C0, c + st[d]); }
        rs<R>(b, S_D)[c] = acc;
    }
    // rotating-frame source of DIFFUSION_Centered (:812-822), after its viscous terms: Coriolis
    // and centrifugal force on y and z momentum times the cell volume.  With omega(1) = 0 it adds
    // a signed zero, which leaves a sum that started at +0 unchanged, so it is skipped.
    const R om = cparams<R>(cdev[b.cs]).omega0;
    for (int L = 1; L < 5; ++L) {
        R acc = R(0.0);
        for (int d = 0; d < 3; ++d) { acc = acc - fx(d, FX_VX + L - 1, c); acc = acc + fx(d, FX_VX + L - 1, c + st[d]); }
        if ((L == 2 || L == 3) && om != R(0.0)) {
            const R* V = rs<R>(b, S_V);
            const R V1 = R(V[c]);
            const R ss = L == 2 ? R(2.0) * om * R(V[3 * nc + c]) + om * R(rs<R>(b, S_YC)[c]) * om * V1
                                : R(-2.0) * om * R(V[2 * nc + c]) + om * R(rs<R>(b, S_ZC)[c]) * om * V1;
            acc = acc + ss * R(rs<R>(b, S_VOL)[c]);
        }
        for (int d = 0; d < 3; ++d) { acc = acc - fx(d, FX_C0 + L, c); acc = acc + fx(d, FX_C0 + L, c + st[d]); }
        rs<R>(b, S_D + L)[c] = acc;
    }
    if (turb) {
        for (int q = 0; q < 2; ++q) {
            R acc = R(0.0);
            for (int d = 0; d < 3; ++d) { acc = acc - fx(d, FX_TK + q, c); acc = acc + fx(d, FX_TK + q, c + st[d]); }
            for (int d = 0; d < 3; ++d) { acc = acc - fx(d, FX_CK + q, c); acc = acc + fx(d, FX_CK + q, c + st[d]); }
            rs<R>(b, S_D + 5 + q)[c] = acc;
        }
    } else {
        rs<R>(b, S_D + 5)[c] = R(0.0);
        rs<R>(b, S_D + 6)[c] = R(0.0);
    }
}

// ---------------------------------------------------------------------------------------
// F1 of SST per cell (Time/TURBTWO_TIME_LUSGS_SST.F90:265-273), read by the DES length scale
// of the lexicographically next cell
// ---------------------------------------------------------------------------------------
template <typename R>
__device__ inline R sst_fc1(const ParamsT<R>& p, const DevBlock& b, int c) {
    R ARo = (rs<R>(b, S_V)[c]), ARTk = (rs<R>(b, S_V + 5)[c]), ARTO = (rs<R>(b, S_V + 6)[c]);
    R cdif = (rs<R>(b, S_DQ + 12)[c]) * (rs<R>(b, S_DQ + 15)[c]) + (rs<R>(b, S_DQ + 13)[c]) * (rs<R>(b, S_DQ + 16)[c])
             + (rs<R>(b, S_DQ + 14)[c]) * (rs<R>(b, S_DQ + 17)[c]);
    R TT = (rs<R>(b, S_T)[c]);
    R RmiuL = mu_suth<R>(p, TT);
    R DistN = (rs<R>(b, S_DST)[c]);
    R Ref = R(p.Ref), Sigo2 = R(p.Sigo2), Bs = R(p.Beta_star);
    R CDKO = dmax(R(2.0) * ARo * Sigo2 / (ARTO / ARo) * cdif, R(1.0e-10));
    R arg1 = dmax(sqrt(ARTk / ARo) / Bs / (ARTO / ARo) / DistN / Ref, R(500.0) * RmiuL / DistN / DistN / ARTO / Ref / Ref);
    arg1 = dmin(arg1, R(4.0) * Sigo2 * ARTk / CDKO / DistN / DistN);
    R a2 = arg1 * arg1;
    return ttanh(a2 * a2);
}

template <typename R>
__global__ void k_sst_fc1(const DevBlock* __restrict__ blks, const Tile* __restrict__ tiles, const CaseDev* __restrict__ cdev) {
    const Tile t = tiles[blockIdx.x];
    if ((int)threadIdx.x >= t.count) return;
    const DevBlock b = blks[t.blk];
    if (!cdev[b.cs].turb || cdev[b.cs].p.Kind_Hybrid != 3) return;     // only the DES cases need F1
    const ParamsT<R> p = cparams<R>(cdev[b.cs]);
    int n = t.start + threadIdx.x;
    int I = n % b.NI1 + 1, J = (n / b.NI1) % b.NJ1 + 1, K = n / (b.NI1 * b.NJ1) + 1;
    int c = cidx(b, I, J, K);
    rs<R>(b, S_FC1)[c] = sst_fc1<R>(p, b, c);
}

// ---------------------------------------------------------------------------------------
// Time/TIME_LUSGS.F90:60-108 and Time/TURBTWO_TIME_LUSGS_SST.F90:118-411: right-hand sides,
// SST sources and the two diagonals, one thread per interior cell in cell order (coalesced
// reads of the cell's slots); the results go to the cell's sweep position q (qpos) together
// with the neighbours' Jacobian terms and spectral radii (k_lusgs_jac).
// ---------------------------------------------------------------------------------------
// Space/RC_Correction.F90:19-124 (Kind_RotMod = 1): the rotation/curvature factor f_r1 of the
// SST production of one interior cell (I,J,K), slot index c, evaluated as the reference's build
// evaluates it: the static local arrays' entries it never writes (St2(3,3), the diagonal of
// Wij) are 0; omega(M), whose index the routine never sets, is read as omega(1) (the term is
// 0 whenever omega(1) is); VL(d,v) is the face average of
// SPACEINTERP_GetSurfCenterVars where that routine writes it and 0 elsewhere.  RCCorrection
// runs after BC_Boundarys(0) (main.F90:89); its inputs do not change until the update, so the
// LU-SGS preparation evaluates it.
template <typename R>
__device__ inline R rc_fr1(const ParamsT<R>& p, const DevBlock& b, int I, int J, int K, int c) {
    const int st[3] = {1, b.PI, b.PI * b.PJ};
    auto DQ = [&](int L, int cc) { return rs<R>(b, S_DQ + L - 1)[cc]; };         // DqDxyz(L), L 1-based
    R St2[4][4], Wij[4][4];
    for (int a = 0; a < 4; ++a)
        for (int e = 0; e < 4; ++e) { St2[a][e] = R(0.0); Wij[a][e] = R(0.0); }
    const R DuDx = DQ(1, c), DuDy = DQ(2, c), DuDz = DQ(3, c), DvDx = DQ(4, c), DvDy = DQ(5, c), DvDz = DQ(6, c);
    const R DwDx = DQ(7, c), DwDy = DQ(8, c);
    const R h = R(0.5), om = R(p.omega0);
    St2[1][1] = DuDx; St2[1][2] = h * (DuDy + DvDx); St2[1][3] = h * (DuDz + DwDx);
    St2[2][1] = St2[1][2]; St2[2][2] = DvDy; St2[2][3] = h * (DvDz + DwDy);
    St2[3][1] = St2[1][3]; St2[3][2] = St2[2][3];
    Wij[1][2] = h * (DuDy - DvDx); Wij[1][3] = h * (DuDz - DwDx); Wij[2][3] = h * (DvDz - DwDy) - om;
    Wij[2][1] = -Wij[1][2]; Wij[3][1] = -Wij[1][3]; Wij[3][2] = -Wij[2][3];
    R SSum = R(0.0), WSum = R(0.0);
    for (int JJ = 1; JJ <= 3; ++JJ)
        for (int II = 1; II <= 3; ++II) {
            SSum = SSum + St2[II][JJ] * St2[II][JJ];
            WSum = WSum + Wij[II][JJ] * Wij[II][JJ];
        }
    SSum = SSum * R(2.0);
    WSum = WSum * R(2.0);
    // VL(d,v) at face index (i,j,k) where SPACEINTERP writes it (d = 1: j, k interior; d = 2:
    // i, k interior; d = 3: i, j interior), 0 elsewhere
    auto VLf = [&](int d, int v, int i, int j, int k) -> R {
        const bool in = d == 1 ? (j >= 1 && j <= b.NJ1 && k >= 1 && k <= b.NK1)
                      : d == 2 ? (i >= 1 && i <= b.NI1 && k >= 1 && k <= b.NK1)
                               : (i >= 1 && i <= b.NI1 && j >= 1 && j <= b.NJ1);
        if (!in) return R(0.0);
        return favg<R>(rs<R>(b, S_PRIM + v - 1), rs<R>(b, S_ALAGM + d - 1), rs<R>(b, S_AINV + d - 1), cidx(b, i, j, k), st[d - 1]);
    };
    auto U = [&](int v, int i, int j, int k) {      // the VL*SD sum of RC_Correction.F90:95-100
        const int cf = cidx(b, i, j, k);
        return VLf(1, v, i, j, k) * rs<R>(b, S_SD + v - 1)[cf] + VLf(2, v, i, j, k) * rs<R>(b, S_SD + 3 + v - 1)[cf] +
               VLf(3, v, i, j, k) * rs<R>(b, S_SD + 6 + v - 1)[cf];
    };
    const R Ui1 = U(1, I + 1, J, K), Ui0 = U(1, I, J, K), Uj1 = U(2, I, J + 1, K), Uj0 = U(2, I, J, K);
    const R Uk1 = U(3, I, J, K + 1), Uk0 = U(3, I, J, K);
    const R* Vol = rs<R>(b, S_VOL);
    R r_bar = R(0.0);
    for (int JJ = 1; JJ <= 3; ++JJ)
        for (int II = 1; II <= 3; ++II) {
            const int LL1 = (II - 1) * 3 + JJ, LL2 = (JJ - 1) * 3 + II;
            const R Sij = DQ(LL1, c) + DQ(LL2, c);
            auto face = [&](int cn) {
                R vol1 = Vol[cn] / (Vol[cn] + Vol[c]);
                return vol1 * (DQ(LL1, cn) + DQ(LL2, cn)) + (R(1.0) - vol1) * Sij;
            };
            const R Sijf1 = face(c - st[0]), Sijf2 = face(c + st[0]), Sijf3 = face(c - st[1]), Sijf4 = face(c + st[1]);
            const R Sijf5 = face(c - st[2]), Sijf6 = face(c + st[2]);
            const R volinv = R(1.0) / Vol[c];
            R DsijDt = Ui1 * Sijf2 - Ui0 * Sijf1 + Uj1 * Sijf4 - Uj0 * Sijf3 + Uk1 * Sijf6 - Uk0 * Sijf5;
            R DsDt = DsijDt * R(0.5) * volinv;
            R DsDt2 = R(0.0);
            for (int MM = 1; MM <= 1; ++MM)
                for (int NN = 1; NN <= 3; ++NN) {
                    const R epsIMN = R(0.5 * (II - MM) * (MM - NN) * (NN - II));
                    const R epsJMN = R(0.5 * (JJ - MM) * (MM - NN) * (NN - JJ));
                    DsDt2 = DsDt2 + (epsIMN * St2[JJ][NN] + epsJMN * St2[II][NN]) * om;
                }
            DsDt = DsDt + DsDt2;
            for (int KK = 1; KK <= 3; ++KK) r_bar = r_bar + Wij[II][KK] * St2[JJ][KK] * DsDt;
        }
    const R Dsum = dmax(SSum, R(0.09) * sq(rs<R>(b, S_V + 6)[c] / rs<R>(b, S_V)[c]));
    const R r_star = sqrt(SSum / WSum);
    r_bar = R(2.0) * r_bar / (sqrt(WSum) * p15(Dsum));
    const R cr1 = R(1.0), cr2 = R(2.0), cr3 = R(1.0);
    const R f_rot = (R(1) + cr1) * R(2.0) * r_star / (R(1.0) + r_star) * (R(1) - cr3 * tatan(cr2 * r_bar)) - cr1;
    return dmax(dmin(f_rot, R(1.25)), R(0.0));
}

// (FP32: two resident CTAs of 256 threads per SM, i.e. at most 128 registers)
#ifndef TG_PREP_MINB
#define TG_PREP_MINB 3      // resident CTAs per SM of the FP32 preparation (84 registers, 80-byte spill)
#endif
#ifndef TG_PREP_MINB_F64
#define TG_PREP_MINB_F64 2  // ... and of the FP64 one (128 registers, 84-byte spill; 254 at one CTA per SM)
#endif
template <typename R>
__global__ void __launch_bounds__(CELL_TILE, sizeof(R) == 4 ? TG_PREP_MINB : TG_PREP_MINB_F64) k_lusgs_prep(const DevBlock* __restrict__ blks, const Tile* __restrict__ tiles, const int* __restrict__ qpos,
                             R* __restrict__ rec, R* __restrict__ dq, const CaseDev* __restrict__ cdev) {
    const Tile t = tiles[blockIdx.x];
    if ((int)threadIdx.x >= t.count) return;
    const DevBlock b = blks[t.blk];
    const Params pd = cdev[b.cs].p;
    const ParamsT<R> p = cparams<R>(cdev[b.cs]);
    const int turb = cdev[b.cs].turb;
    const int nlex = t.start + threadIdx.x;                              // lexicographic interior index
    const int I = nlex % b.NI1 + 1, J = (nlex / b.NI1) % b.NJ1 + 1, K = nlex / (b.NI1 * b.NJ1) + 1;
    const long long q = qpos[(size_t)blockIdx.x * CELL_TILE + threadIdx.x];
    const int c = cidx(b, I, J, K);
    auto REC = [&](int m) -> R& { return rec[sw_at(q, m, NREC)]; };
    auto DQ = [&](int L) -> R& { return dq[sw_at(q, L, DQ_STRIDE)]; };
    // BDF2 right-hand side and the mean-flow diagonal (TIME_LUSGS.F90:73-108).  FP64 path: the
    // reference's operations.  Mixed path: the time-level difference 3V - 4Wt0 + Wt1 in FP64
    // (it cancels), everything else in FP32 with one reciprocal of the volume.  (This kernel is
    // bound by load latency at its register limit, so the hardware conversion stays: the
    // integer-pipe one of cvt.cuh measured 50% slower here.)
    const double DT = pd.DT_LUSGS_Main;
    constexpr bool MIXED = sizeof(R) == 4;
    R stept, cvs, fm;
    auto rhs = [&](int L) {
        const double bdf = 3.0 * slot(b, S_V + L)[c] - 4.0 * slot(b, S_WT0 + L)[c] + slot(b, S_WT1 + L)[c];
        if constexpr (MIXED) {
            const R rvol = R(1.0) / rs<R>(b, S_VOL)[c];
            return rs<R>(b, S_D + L)[c] * rvol - R(bdf) * (R(0.5) / R(DT));
        } else {
            return R((double)rs<R>(b, S_D + L)[c] / slot(b, S_VOL)[c] - bdf * 0.5 / DT);
        }
    };
    if constexpr (MIXED) {
        const R Dtm = rs<R>(b, S_DTM)[c], vol = rs<R>(b, S_VOL)[c];
        stept = R(2.0) * Dtm / (R(3.0) * Dtm / R(DT) + R(2.0));
        cvs = stept / vol;
        fm = R(1.0) + (rs<R>(b, S_RDS)[c] + rs<R>(b, S_RDS + 1)[c] + rs<R>(b, S_RDS + 2)[c]) * cvs;
    } else {
        const double Dtm = slot(b, S_DTM)[c], vol = slot(b, S_VOL)[c];
        const double st = 2.0 * Dtm / (3.0 * Dtm / DT + 2.0);
        const double cv = st / vol;
        const double rsum = slot(b, S_RDS)[c] + slot(b, S_RDS + 1)[c] + slot(b, S_RDS + 2)[c];
        stept = R(st); cvs = R(cv); fm = R(1.0 + rsum * cv);
    }
    // the diagonal terms into the record: FP64 path its four entries; mixed path the compact
    // record of this position (CompactRec: metric and radius per direction, velocity and total
    // enthalpy, stept, cvs and the reciprocals of the two diagonals)
    auto finish = [&](R ft) {
        if constexpr (MIXED) {
            float4* R4 = reinterpret_cast<float4*>(rec) + (size_t)q * (NCREC / 4);
#pragma unroll
            for (int d = 0; d < 3; ++d)
                R4[d] = make_float4(rs<R>(b, S_ASD + 3 * d)[c], rs<R>(b, S_ASD + 3 * d + 1)[c], rs<R>(b, S_ASD + 3 * d + 2)[c],
                                    rs<R>(b, S_RDS + d)[c]);
            const float u = rs<R>(b, S_SVEL)[c], v = rs<R>(b, S_SVEL + 1)[c], w = rs<R>(b, S_SVEL + 2)[c];
            const float H = 0.5f * (u * u + v * v + w * w) + 1.4f * rs<R>(b, S_PP)[c] * rs<R>(b, S_RINV)[c] / 0.4f;
            R4[CR_VEL / 4] = make_float4(u, v, w, H);
            R4[CR_DIAG / 4] = make_float4(stept, cvs, 1.0f / fm, 1.0f / ft);
        } else {
            REC(REC_STEPT) = stept;
            REC(REC_CVS) = cvs;
            REC(REC_FM) = fm;
            REC(REC_FT) = ft;
        }
    };
    for (int L = 0; L < 5; ++L) DQ(L) = rhs(L);
    if constexpr (!MIXED) {
        if (pd.IF_Precondition) {     // the right-hand side preconditioned (TIME_LUSGS.F90:113-160)
            double A[5] = {DQ(0), DQ(1), DQ(2), DQ(3), DQ(4)}, tpc[NPC];
            precond_terms_at(pd, b, c, tpc);
            precond_apply<double>(A, tpc);
            for (int L = 0; L < 5; ++L) DQ(L) = A[L];
        }
    }
    if (!turb) {            // the k-omega lanes of the sweeps then produce zeros
        DQ(5) = rs<R>(b, S_D + 5)[c];
        DQ(6) = rs<R>(b, S_D + 6)[c];
        finish(R(1.0));
        return;
    }
    for (int L = 5; L < 7; ++L) DQ(L) = rhs(L);
    auto G = [&](int q) { return rs<R>(b, S_DQ + q)[c]; };
    R dudx = G(0), dudy = G(1), dudz = G(2), dvdx = G(3), dvdy = G(4), dvdz = G(5), dwdx = G(6), dwdy = G(7), dwdz = G(8);
    R dtkdx = G(12), dtkdy = G(13), dtkdz = G(14), dtodx = G(15), dtody = G(16), dtodz = G(17);
    R Div = dudx + dvdy + dwdz;
    R Votg = sq(dudy - dvdx) + sq(dvdz - dwdy) + sq(dwdx - dudz);
    R prod = (R(2.0) * (dudx * dudx + dvdy * dvdy + dwdz * dwdz) + sq(dudy + dvdx) + sq(dvdz + dwdy) + sq(dwdx + dudz)
              - R(2.0 / 3.0) * Div * Div);
    R cdif = dtkdx * dtodx + dtkdy * dtody + dtkdz * dtodz;
    const R Ref = R(p.Ref), Bs = R(p.Beta_star), Sigo2 = R(p.Sigo2);
    R tprod = dmin(prod, Votg) * (rs<R>(b, S_RMIU)[c]) / Ref;
    R ARo = (rs<R>(b, S_V)[c]), ARTk = (rs<R>(b, S_V + 5)[c]), ARTO = (rs<R>(b, S_V + 6)[c]);
    R tprodl1 = R(p.Prod_Lmt) * Bs * ARTk * ARTO / ARo * Ref;
    tprod = dmin(tprod, tprodl1);
    if (p.Kind_Model == 2) {    // Wilcox 2006 k-omega (TURBTWO_TIME_LUSGS_SST.F90:418-547)
        const R c23 = R(2.0 / 3.0);
        R SourceN1 = -(c23 * dmax(Div, R(0.0))) - Bs * ARTO / ARo * Ref;
        DQ(5) = DQ(5) + ((tprod - c23 * dmin(Div, R(0.0)) * ARTk) + SourceN1 * ARTk);
        const R CnegTk = fabs(SourceN1);
        tprod = dmin(prod, Votg) / Ref;
        const R h = R(0.5);
        const R W[3][3] = {{R(0.), h * (dudy - dvdx), h * (dudz - dwdx)},
                           {-(h * (dudy - dvdx)), R(0.), h * (dvdz - dwdy)},
                           {-(h * (dudz - dwdx)), -(h * (dvdz - dwdy)), R(0.)}};
        const R Sxy = h * (dudy + dvdx), Sxz = h * (dudz + dwdx), Syz = h * (dvdz + dwdy);
        const R S[3][3] = {{h * (dudx + dudx), Sxy, Sxz}, {Sxy, h * (dvdy + dvdy), Syz}, {Sxz, Syz, h * (dwdz + dwdz)}};
        R WWSg = R(0.);
#pragma unroll
        for (int ii = 0; ii < 3; ++ii)
#pragma unroll
            for (int jj = 0; jj < 3; ++jj)
#pragma unroll
                for (int kk = 0; kk < 3; ++kk) WWSg = WWSg + W[ii][jj] * W[jj][kk] * S[kk][ii];
        R aK_omg = fabs(WWSg / cube_pow(R(0.09) * ARTO / ARo * Ref));
        R Beta_06 = R(p.Beta1) * ((R(1.) + R(85.) * aK_omg) / (R(1.) + R(100.) * aK_omg));
        const R G1 = R(p.Gama1);
        R SourceP = G1 * ARo * tprod - c23 * G1 * dmin(Div, R(0.0)) * ARTO;
        SourceN1 = -(c23 * G1 * dmax(Div, R(0.0))) - Beta_06 * ARTO / ARo * Ref;
        R Source = SourceP + SourceN1 * ARTO;
        R dltCD = cdif <= R(0.) ? R(0.) : R(0.125);
        Source = Source + dltCD * ARo * ARo / ARTO / Ref * cdif;
        DQ(6) = DQ(6) + Source;
        finish(R(fm) + (CnegTk + R(2.0) * fabs(SourceN1)) * R(stept));
        return;
    }
    R TT = (rs<R>(b, S_T)[c]);
    R RmiuL = mu_suth<R>(p, TT);
    R Fdes = R(1.0);
    R alIDDES = R(1.0);
    const bool iddes = p.Kind_Hybrid == 3 && p.Kind_SubHY == 5;
    if (p.Kind_Hybrid == 3) {
        // DES length scale with the loop-carried F1 and omega of the previous interior cell
        // (TURBTWO_TIME_LUSGS_SST.F90:192-213); the first cell uses F1 = 0 and its own omega
        int np = nlex - 1;
        R arg1p = R(0.0), Vomp = ARTO / ARo;
        if (np >= 0) {
            int Ip = np % b.NI1 + 1, Jp = (np / b.NI1) % b.NJ1 + 1, Kp = np / (b.NI1 * b.NJ1) + 1;
            int cq = cidx(b, Ip, Jp, Kp);
            arg1p = (rs<R>(b, S_FC1)[cq]);
            Vomp = (rs<R>(b, S_V + 6)[cq]) / (rs<R>(b, S_V)[cq]);
        }
        R aLt = sqrt(ARTk / ARo) / (Bs * ARTO / ARo * Ref);
        R Cdiff = (R(2. * 0.856) / Vomp) / Ref * cdif;
        R vOmega = ARTO / ARo;
        R Fsst = fsst<R>(p, ARo, ARTk / ARo, vOmega, (rs<R>(b, S_DST)[c]), RmiuL, Cdiff);
        R aLgrd = ((R(1.) - arg1p) * R(0.61) + arg1p * R(0.78)) * (rs<R>(b, S_ALENG)[c]);
        Fdes = dmax(aLt * (R(1.) - Fsst) / aLgrd, R(1.0));
        if (iddes) {        // IDDES length scale (TURBTWO_TIME_LUSGS_SST.F90:218-252)
            const R aLmax = rs<R>(b, S_ALENG)[c], aDst = rs<R>(b, S_DST)[c], aLmin = rs<R>(b, S_ASENG)[c];
            const R Cw = R(0.15);
            R Cdes = (R(1.) - arg1p) * R(0.61) + arg1p * R(0.78);
            R dlt = dmin(dmax(dmax(Cw * aLmax, Cw * aDst), aLmin), aLmax);
            aLgrd = Cdes * dlt;
            const R g[9] = {dudx, dudy, dudz, dvdx, dvdy, dvdz, dwdx, dwdy, dwdz};
            const R RmiuT = rs<R>(b, S_RMIU)[c];
            R fd = fd_function<R>(p, ARo, RmiuT, aDst, aLmax, g);
            R fe = fe_function<R>(p, ARo, RmiuT, RmiuL, aDst, aLmax, g);
            alIDDES = (R(1.) + fe) * fd * aLt + (R(1.) - fd) * aLgrd;
        }
    }
    R DistN = (rs<R>(b, S_DST)[c]);
    R CDKO = dmax(R(2.0) * ARo * Sigo2 / (ARTO / ARo) * cdif, R(1.0e-10));
    R arg1 = dmax(sqrt(ARTk / ARo) / Bs / (ARTO / ARo) / DistN / Ref, R(500.0) * RmiuL / DistN / DistN / ARTO / Ref / Ref);
    arg1 = dmin(arg1, R(4.0) * Sigo2 * ARTk / CDKO / DistN / DistN);
    R a2 = arg1 * arg1;
    arg1 = ttanh(a2 * a2);
    R AA = sqrt(R(1.4) * (rs<R>(b, S_PP)[c]) / ARo);
    R Mt = sqrt(ARTk / ARo) / AA;
    const R Alf1 = R(1.0), Alf2 = R(0.4), Alf3 = R(0.2);
    const R c23 = R(2.0 / 3.0);
    R SourceP, SourceN1, Source, CnegTk, CnegTO;
    // the rotation/curvature factor of the production (TURBTWO_TIME_LUSGS_SST.F90:286,325,343,384;
    // 1 unless Kind_RotMod = 1)
    const bool rc = p.Kind_RotMod == 1;
    const R f_r1 = rc ? rc_fr1<R>(p, b, I, J, K, c) : R(1.0);
    if (p.IF_Comppress == 0) {
        SourceP = tprod - c23 * dmin(Div, R(0.0)) * ARTk;
        if (rc) SourceP = SourceP * f_r1;
        SourceN1 = -(c23 * dmax(Div, R(0.0))) - Bs * ARTO / ARo * Ref * Fdes;
    } else {
        SourceP = (R(1.) - (R(1.) - arg1) * Alf2 * Mt * Mt) * tprod - c23 * dmin(Div, R(0.0)) * ARTk;
        if (rc) SourceP = SourceP * f_r1;
        SourceN1 = -(c23 * dmax(Div, R(0.0))) - (R(1.) + (R(1.) - arg1) * (Alf1 - Alf3) * Mt * Mt) * Bs * ARTO / ARo * Ref * Fdes;
    }
    Source = SourceP + SourceN1 * ARTk;
    CnegTk = fabs(SourceN1);
    if (p.If_fix_Transition && rs<R>(b, S_XC)[c] < p.Trans_location) Source = R(0.0);
    if (iddes) {            // the IDDES destruction (TURBTWO_TIME_LUSGS_SST.F90:299-310, 354-366)
        if (p.IF_Comppress == 0) SourceN1 = -(c23 * dmax(Div, R(0.0))) - sqrt(ARTk / ARo) / alIDDES;
        else SourceN1 = -(c23 * dmax(Div, R(0.0))) - (R(1.) + (R(1.) - arg1) * (Alf1 - Alf3) * Mt * Mt) * sqrt(ARTk / ARo) / alIDDES;
        Source = SourceP + SourceN1 * ARTk;
        CnegTk = fabs(-(c23 * dmax(Div, R(0.0))) - R(1.5) * sqrt(ARTk / ARo) / alIDDES);
        if (p.If_fix_Transition && rs<R>(b, S_XC)[c] < p.Trans_location) Source = R(0.0);
    }
    DQ(5) = DQ(5) + Source;
    tprod = dmin(prod, Votg) / Ref;
    R GamaAB = R(p.Gama1) * arg1 + R(p.Gama2) * (R(1.0) - arg1);
    R BetaAB = R(p.Beta1) * arg1 + R(p.Beta2) * (R(1.0) - arg1);
    if (p.IF_Comppress == 0) {
        SourceP = GamaAB * ARo * tprod - c23 * GamaAB * dmin(Div, R(0.0)) * ARTO;
        if (rc) SourceP = SourceP * f_r1;
        SourceN1 = -(c23 * GamaAB * dmax(Div, R(0.0))) - BetaAB * ARTO / ARo * Ref;
    } else {
        SourceP = (GamaAB + (R(1.) - arg1) * Alf2 * Mt * Mt) * ARo * tprod - c23 * GamaAB * dmin(Div, R(0.0)) * ARTO;
        if (rc) SourceP = SourceP * f_r1;
        SourceN1 = -(c23 * GamaAB * dmax(Div, R(0.0))) - (R(1.) - (R(1.) - arg1) * (Alf1 - Alf3) * Mt * Mt) * BetaAB * ARTO / ARo * Ref;
    }
    Source = SourceP + SourceN1 * ARTO;
    R SourceCross = R(2.0) * (R(1) - arg1) * ARo * Sigo2 / (ARTO / ARo) * cdif / Ref;
    SourceCross = sgn1(SourceCross) * dmin(fabs(SourceCross), fabs(SourceP) * R(0.5));
    Source = Source + SourceCross;
    DQ(6) = DQ(6) + Source;
    CnegTO = R(2.0) * fabs(SourceN1);
    finish(R(fm) + (CnegTk + CnegTO) * R(stept));
}

// The neighbours' Jacobian terms and spectral radii of the sweep records: 6 threads per
// position (one per neighbour) compute into shared memory, then the block writes its 32
// consecutive records as one contiguous, coalesced range (the diagonal entries excepted,
// which k_lusgs_prep writes).  A missing neighbour (nbp < 0) leaves its entries unused.
template <typename R>
__global__ void __launch_bounds__(6 * 32) k_lusgs_jac(const DevBlock* __restrict__ blks, const SweepCell* __restrict__ cells,
                                                      const int* __restrict__ nbp, R* __restrict__ rec, long long N) {
    __shared__ R stage[32][6 * NBREC];
    const long long q0 = (long long)blockIdx.x * 32;
    const int t = threadIdx.x, r = t / 6, k = t % 6;
    const long long q = q0 + r;
    if (q < N && nbp[sw_at(q, k, 6)] >= 0) {
        const SweepCell sc = cells[q];
        const DevBlock b = blks[sc.blk];
        const int c = cidx(b, sc.i, sc.j, sc.k);
        const size_t nc = (size_t)b.ncell;
        const int d = k % 3;
        const int st = d == 0 ? 1 : (d == 1 ? b.PI : b.PI * b.PJ);
        const int nb = k < 3 ? c - st : c + st;
        const R* sv = rs<R>(b, S_SVEL);
        const R* asd = rs<R>(b, S_ASD + 3 * d);
        R Jt[NJAC];
        jac_terms<R>(sv[nb], sv[nb + nc], sv[nb + 2 * nc], asd[nb], asd[nb + nc], asd[nb + 2 * nc], rs<R>(b, S_PP)[nb],
                     rs<R>(b, S_RINV)[nb], Jt);
        for (int m = 0; m < NJAC; ++m) stage[r][NBREC * k + m] = Jt[m];
        stage[r][NBREC * k + NJAC] = rs<R>(b, S_RDS + d)[nb];
    }
    __syncthreads();
    const long long nq = N - q0 < 32 ? N - q0 : 32;
    for (int e = t; e < nq * NREC; e += blockDim.x) {
        const int rr = e / NREC, m = e % NREC;
        if (m < 6 * NBREC) rec[sw_at(q0 + rr, m, NREC)] = stage[rr][m];
    }
}


// The PrecondDW coefficients of the six neighbours of every sweep position (FP64 path, low-Mach
// preconditioning): one thread per (position, neighbour); a missing neighbour is left unused
static __global__ void k_lusgs_jac_pc(const DevBlock* __restrict__ blks, const SweepCell* __restrict__ cells, const int* __restrict__ nbp,
                               const CaseDev* __restrict__ cdev, double* __restrict__ pc, long long N) {
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= 6 * N) return;
    const long long q = g / 6;
    const int k = (int)(g % 6);
    if (nbp[sw_at(q, k, 6)] < 0) return;
    const SweepCell sc = cells[q];
    const DevBlock b = blks[sc.blk];
    const Params p = cdev[b.cs].p;
    const int c = cidx(b, sc.i, sc.j, sc.k);
    const int d = k % 3;
    const int st = d == 0 ? 1 : (d == 1 ? b.PI : b.PI * b.PJ);
    double t[NPC];
    precond_terms_at(p, b, k < 3 ? c - st : c + st, t);
    for (int m = 0; m < NPC; ++m) pc[sw_at(q, k * NPC + m, 6 * NPC)] = t[m];
}

// ---------------------------------------------------------------------------------------
// LU-SGS sweeps (Time/TIME_LUSGS.F90:172-675, Time/TURBTWO_TIME_LUSGS_SST.F90:562-766) on the
// i+j+k hyperplanes of every block.  Any order of the (i-1,j-1,k-1) dependency graph
// reproduces the lexicographic sweep exactly; hyperplanes are such an order.  A hyperplane is
// a contiguous range of sweep positions.
//
// SWEEP_LANES lanes per cell, lane L = component L of DeltaQ (0..4 mean flow, 5..6 k and
// omega, the rest idle), so that the few FP64 operations left on the critical path (the
// products with the neighbours' DeltaQ and one division) spread over many SM sub-partitions.
// turb selects the components swept: 0 mean flow, 1 all, 2 k and omega only (the Runge-Kutta
// path, whose mean flow is explicit).
// ---------------------------------------------------------------------------------------
// The sweep kernels' `lanes` argument: bits 0-1 select the components swept (0 mean flow,
// 1 all, 2 k and omega only), bit SWEEP_WPC the thread mapping.  Lane-major (bit clear): the
// 8 threads of a position are adjacent lanes of one warp (component = lane % 8).  Warp per
// component (bit set): a warp holds one component of 32 consecutive positions, so its lanes
// take one code path -- on GB300 a warp's FP64 instruction occupies the FP64 unit of its
// sub-partition for ~64 cycles whatever its active lanes, and the lane-major warp's four
// divergent component paths issue ~5x the FP64 instructions per position.
__device__ inline void sweep_map(int g, int lanes, int& e, int& L) {
    if (lanes & SWEEP_WPC) { e = (g / (32 * SWEEP_LANES)) * 32 + (g & 31); L = (g >> 5) % SWEEP_LANES; }
    else { e = g / SWEEP_LANES; L = g % SWEEP_LANES; }
}

// Mixed-path (FP32) sweep step of one position, all seven components, from the compact records
// (CompactRec).  Each neighbour's Jacobian row is rebuilt from its metric s, velocity v and total
// enthalpy H: with VP = v.s, th = s.dm - VP dr and ph = (gamma-1)(|v|^2/2 dr - v.dm + dE),
//   row 0 = s.dm,   rows 1-3 = v_a th + s_a ph + VP dm_a,   row 4 = H th + VP (ph + dE),
// the rows of A(Q) DeltaQ of TIME_LUSGS.F90:696-768 re-associated (the FP32 path does not keep
// the reference's operation order); the k and omega rows are VP dq (TURBTWO_TIME_LUSGS_SST.F90:
// 562-766).  The neighbour terms are 0.5 (row + sgn Rds dq), summed over the three neighbours;
// then D = (own stept + sum cvs) / diag in the lower sweep, own - sum cvs / diag in the upper.
// turb: 0 mean flow, 1 all, 2 k and omega only (the others are stored back unchanged).
// chained: griddepcontrol.wait before the first DeltaQ access.
// the static inputs of one position (records and neighbour positions never change during a
// sweep, so they load before the wait for the previous hyperplane): the neighbours on the
// side the sweep comes from, their metric and radius (g) and velocity and enthalpy (h) of the
// direction, VP = v.s and |v|^2/2, and the position's diagonal record
struct SweepStatic {
    int np[3];
    float4 g[3], h[3], dg;
    float VP[3], q2[3];
};
template <bool LOWER>
__device__ __forceinline__ void sweep_static(const int* __restrict__ nbp, const float4* __restrict__ R4, long long q, SweepStatic& s) {
    const int side = LOWER ? 0 : 3;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        s.np[d] = nbp[sw_at(q, side + d, 6)];
        const long long r = s.np[d] >= 0 ? s.np[d] : q;
        s.g[d] = __ldg(R4 + (size_t)r * (NCREC / 4) + d);               // s of direction d, Rds(d)
        s.h[d] = __ldg(R4 + (size_t)r * (NCREC / 4) + CR_VEL / 4);      // u, v, w, H
    }
    s.dg = __ldg(R4 + (size_t)q * (NCREC / 4) + CR_DIAG / 4);          // stept, cvs, 1/fm, 1/ft
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        s.VP[d] = s.h[d].x * s.g[d].x + s.h[d].y * s.g[d].y + s.h[d].z * s.g[d].z;
        s.q2[d] = 0.5f * (s.h[d].x * s.h[d].x + s.h[d].y * s.h[d].y + s.h[d].z * s.h[d].z);
    }
}
// the neighbours' DeltaQ (written during the sweep by other SMs: read through L2); a missing
// neighbour reads the position's own entry, unused
__device__ __forceinline__ void sweep_nbvals(const float* dq, const SweepStatic& s, long long q, float4 a[3], float4 t[3]) {
    const float4* D4 = reinterpret_cast<const float4*>(dq);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const long long r = s.np[d] >= 0 ? s.np[d] : q;
        a[d] = __ldcg(D4 + (size_t)r * 2);
        t[d] = __ldcg(D4 + (size_t)r * 2 + 1);
    }
}
// the arithmetic of one position: own DeltaQ (o0, o1) and the neighbours' (a: components 0-3,
// t: 4-6) -> out[0..6], out[7] = the pad word kept
template <bool LOWER>
__device__ __forceinline__ void sweep_core(const SweepStatic& s, float4 o0, float4 o1, const float4 a[3], const float4 t[3],
                                           int turb, float out[8]) {
    const float sgn = LOWER ? 1.0f : -1.0f;
    float acc[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    const float Gm1 = 0.4f;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if (s.np[d] < 0) continue;
        const float a0 = a[d].x, a1 = a[d].y, a2 = a[d].z, a3 = a[d].w, a4 = t[d].x, a5 = t[d].y, a6 = t[d].z;
        const float sx = s.g[d].x, sy = s.g[d].y, sz = s.g[d].z, sr = sgn * s.g[d].w;
        const float u = s.h[d].x, v = s.h[d].y, w = s.h[d].z, H = s.h[d].w, vp = s.VP[d];
        const float sm = sx * a1 + sy * a2 + sz * a3;
        const float th = sm - vp * a0;
        const float ph = Gm1 * (s.q2[d] * a0 - (u * a1 + v * a2 + w * a3) + a4);
        acc[0] += sm + sr * a0;
        acc[1] += u * th + sx * ph + (vp + sr) * a1;
        acc[2] += v * th + sy * ph + (vp + sr) * a2;
        acc[3] += w * th + sz * ph + (vp + sr) * a3;
        acc[4] += H * th + vp * (ph + a4) + sr * a4;
        acc[5] += (vp + sr) * a5;
        acc[6] += (vp + sr) * a6;
    }
    const float own[7] = {o0.x, o0.y, o0.z, o0.w, o1.x, o1.y, o1.z};
    const float stept = s.dg.x, hc = 0.5f * s.dg.y;
#pragma unroll
    for (int L = 0; L < 7; ++L) {
        const float iden = L < 5 ? s.dg.z : s.dg.w;
        const bool act = turb == 1 || (turb == 0 ? L < 5 : L >= 5);
        const float nv = LOWER ? (own[L] * stept + acc[L] * hc) * iden : own[L] - acc[L] * hc * iden;
        out[L] = act ? nv : own[L];
    }
    out[7] = o1.w;
}
__device__ __forceinline__ void sweep_store(float* dq, long long q, const float out[8]) {
    float4* W4 = reinterpret_cast<float4*>(dq) + (size_t)q * 2;
    __stcg(W4, make_float4(out[0], out[1], out[2], out[3]));
    __stcg(W4 + 1, make_float4(out[4], out[5], out[6], out[7]));
}

template <bool LOWER>
__device__ inline void sweep_pos_compact(const int* __restrict__ nbp, const float* __restrict__ rec, float* dq, long long q,
                                         int turb, bool chained) {
    SweepStatic s;
    sweep_static<LOWER>(nbp, reinterpret_cast<const float4*>(rec), q, s);
    if (chained) asm volatile("griddepcontrol.wait;" ::: "memory");
    float4 a[3], t[3];
    sweep_nbvals(dq, s, q, a, t);
    const float4* D4 = reinterpret_cast<const float4*>(dq);
    const float4 o0 = __ldcg(D4 + (size_t)q * 2), o1 = __ldcg(D4 + (size_t)q * 2 + 1);
    float out[8];
    sweep_core<LOWER>(s, o0, o1, a, t, turb, out);
    sweep_store(dq, q, out);
}

template <typename R, bool LOWER>
__device__ inline void sweep_item(const int* __restrict__ nbp, const R* __restrict__ rec, R* dq, long long N, long long q,
                                  int L, int turb, bool chained = false, bool hoist = true, bool release = true,
                                  const R* __restrict__ pc = nullptr) {
    if constexpr (sizeof(R) == 4) {     // mixed path: lane 0 of a position computes all its components
        if (L != 0) {
            if (chained) { asm volatile("griddepcontrol.wait;" ::: "memory"); asm volatile("griddepcontrol.launch_dependents;"); }
            return;
        }
        sweep_pos_compact<LOWER>(nbp, (const float*)rec, (float*)dq, q, turb, chained);
        if (chained) asm volatile("griddepcontrol.launch_dependents;");
        return;
    }
    if (L >= 7 || (L >= 5 && turb == 0) || (L < 5 && turb == 2)) {
        if (chained) {
            asm volatile("griddepcontrol.wait;" ::: "memory");
            if (release) asm volatile("griddepcontrol.launch_dependents;");
        }
        return;
    }
    const int side = LOWER ? 0 : 3;
    const R sgn = LOWER ? R(1.0) : R(-1.0);
    auto REC = [&](int m) { return rec[sw_at(q, m, NREC)]; };
    // Everything that does not depend on the previous hyperplane first: neighbour positions,
    // this lane's Jacobian terms and radii, the diagonal.  A missing neighbour (nbp < 0) reads
    // this cell's own entries instead and its term is replaced by 0 afterwards.
    long long npv[3];
    R k[3][7];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        npv[d] = nbp[sw_at(q, side + d, 6)];
        const int jd = NBREC * (side + d);
        k[d][6] = REC(jd + NJAC);                                   // spectral radius
        if (L == 0) {
            for (int m = 0; m < 3; ++m) k[d][m] = REC(jd + JC_R0 + m);
        } else if (L < 4) {
            for (int m = 0; m < 5; ++m) k[d][m] = REC(jd + JC_R1 + 5 * (L - 1) + m);
        } else if (L == 4) {
            for (int m = 0; m < 4; ++m) k[d][m] = REC(jd + JC_R4 + m);
            k[d][4] = REC(jd + JC_VP);
            k[d][5] = REC(jd + JC_GET1);
        } else {
            k[d][0] = REC(jd + JC_VPT);
        }
    }
    const R stept = REC(REC_STEPT), cvs = REC(REC_CVS);
    const R den = L < 5 ? REC(REC_FM) : REC(REC_FT);
    // one launch per hyperplane chained with programmatic dependent launch: wait for the
    // previous hyperplane to complete, then let the next one start its loads (unless the
    // kernel released it at entry)
    if (chained) {
        asm volatile("griddepcontrol.wait;" ::: "memory");
        if (release) asm volatile("griddepcontrol.launch_dependents;");
    }
    // DeltaQ is written during the sweep by other SMs: read it through L2 (never a stale L1
    // line).  Every lane loads in converged code, before the per-component branches, so that a
    // warp waits for one dependent L2 round trip instead of one per divergent branch.
    // (A warp of the warp-per-component mapping takes one branch: it loads inside it.)
    R nq[3][5], nt[3];
    if (hoist) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const long long np = npv[d] >= 0 ? npv[d] : q;
#pragma unroll
            for (int m = 0; m < 5; ++m) nq[d][m] = __ldcg(dq + sw_at(np, m, DQ_STRIDE));
            nt[d] = __ldcg(dq + sw_at(np, L < 5 ? 0 : L, DQ_STRIDE));
        }
    }
    R* D = dq + sw_at(q, L, DQ_STRIDE);
    const R own = __ldcg(D);
    R acc[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const bool has = npv[d] >= 0;
        const long long np = has ? npv[d] : q;
        const R RDSt = k[d][6];
        R val;
        if (L < 5) {
            if (!hoist)
#pragma unroll
                for (int m = 0; m < 5; ++m) nq[d][m] = __ldcg(dq + sw_at(np, m, DQ_STRIDE));
            const R AinRo = nq[d][0], AinRx = nq[d][1], AinRy = nq[d][2], AinRz = nq[d][3], AinRe = nq[d][4];
            R Dif;
            if (L == 0) {
                const R aSDt = R(0.0);
                Dif = AinRo * aSDt + AinRx * k[d][0] + AinRy * k[d][1] + AinRz * k[d][2] + AinRe * R(0.0);
            } else if (L < 4) {
                Dif = AinRo * k[d][0] + AinRx * k[d][1] + AinRy * k[d][2] + AinRz * k[d][3] + AinRe * k[d][4];
            } else {
                Dif = AinRo * k[d][4] * k[d][5] + AinRx * k[d][0] + AinRy * k[d][1] + AinRz * k[d][2] + AinRe * k[d][3];
            }
            if constexpr (sizeof(R) == 8) {
                if (pc && (L == 0 || L == 4)) {
                    // low-Mach preconditioning: PrecondDW of the neighbour's whole A(Q) DeltaQ
                    // (TIME_LUSGS.F90:235-248); its rows as the lanes form them, then the map
                    const int jd = NBREC * (side + d);
                    R A[5];
                    A[0] = AinRo * R(0.0) + AinRx * REC(jd + JC_R0) + AinRy * REC(jd + JC_R0 + 1) + AinRz * REC(jd + JC_R0 + 2) +
                           AinRe * R(0.0);
                    for (int l = 1; l < 4; ++l) {
                        const int o = jd + JC_R1 + 5 * (l - 1);
                        A[l] = AinRo * REC(o) + AinRx * REC(o + 1) + AinRy * REC(o + 2) + AinRz * REC(o + 3) + AinRe * REC(o + 4);
                    }
                    A[4] = AinRo * REC(jd + JC_VP) * REC(jd + JC_GET1) + AinRx * REC(jd + JC_R4) + AinRy * REC(jd + JC_R4 + 1) +
                           AinRz * REC(jd + JC_R4 + 2) + AinRe * REC(jd + JC_R4 + 3);
                    R tpc[NPC];
                    for (int m = 0; m < NPC; ++m) tpc[m] = pc[sw_at(q, (side + d) * NPC + m, 6 * NPC)];
                    precond_apply<R>(A, tpc);
                    Dif = A[L];
                }
            }
            const R Din = L == 0 ? AinRo : L == 1 ? AinRx : L == 2 ? AinRy : L == 3 ? AinRz : AinRe;
            val = R(0.5) * (Dif + sgn * (RDSt * Din));
        } else {
            const R VP = k[d][0];
            const R Dq = hoist ? nt[d] : __ldcg(dq + sw_at(np, L, DQ_STRIDE));
            val = R(0.5) * (Dq * VP + sgn * (RDSt * Dq));
        }
        acc[d] = has ? val : R(0.0);
    }
    const R sum = acc[0] + acc[1] + acc[2];
    if (LOWER) *D = (own * stept + sum * cvs) / den;
    else *D = own - sum * cvs / den;
}

// one hyperplane [first, first+count) per launch (chained: launched with programmatic
// stream serialisation, see sweep_item)
__device__ inline void prefetch_l2_range(const void* p, size_t bytes, size_t t, size_t stride) {
    const char* a = (const char*)p;
    const char* a0 = (const char*)((uintptr_t)a & ~(uintptr_t)127);     // allocations are 256-byte aligned
    const size_t lines = (size_t)(a + bytes - a0 + 127) / 128;
    for (size_t l = t; l < lines; l += stride) asm volatile("prefetch.global.L2 [%0];" ::"l"(a0 + l * 128));
}

// pf_first/pf_count: a later hyperplane whose records and neighbour positions this launch
// pulls into L2 (otherwise they come from DRAM on the path between two dependent steps)
// chained: 1 = the next hyperplane's launch is released after this one's wait, 2 = at entry
template <typename R, bool LOWER>
__global__ void k_sweep(const int* __restrict__ nbp, const R* __restrict__ rec, R* dq, long long N, int first, int count, int lanes,
                        int chained, int pf_first, int pf_count, const R* __restrict__ pc) {
    if (chained == 2) asm volatile("griddepcontrol.launch_dependents;");
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (pf_count > 0) {
        const size_t T = (size_t)gridDim.x * blockDim.x;
        prefetch_l2_range(rec + sw_at(pf_first, 0, NREC), (size_t)pf_count * NREC * sizeof(R), g, T);
        prefetch_l2_range(nbp + sw_at(pf_first, 0, 6), (size_t)pf_count * 6 * sizeof(int), g, T);
    }
    int e, L;
    sweep_map(g, lanes, e, L);
    if (e >= count) {
        if (chained) {
            asm volatile("griddepcontrol.wait;" ::: "memory");
            if (chained == 1) asm volatile("griddepcontrol.launch_dependents;");
        }
        return;
    }
    sweep_item<R, LOWER>(nbp, rec, dq, N, (long long)first + e, L, lanes & 3, chained != 0, !(lanes & SWEEP_WPC), chained == 1, pc);
}

// Mixed path: one hyperplane per launch, one thread per position (sweep_pos_compact).
// chained: 1 = the next hyperplane's launch is released after this one's wait, 2 = at entry,
// so that its DeltaQ-independent loads (records, neighbour positions) run while this hyperplane
// still waits for the previous one (every DeltaQ access stays after griddepcontrol.wait).
template <bool LOWER>
__global__ void k_sweep_c(const int* __restrict__ nbp, const float* __restrict__ rec, float* dq, int first, int count, int turb,
                          int chained, int pf_first, int pf_count) {
    if (chained == 2) asm volatile("griddepcontrol.launch_dependents;");
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (pf_count > 0) {
        const size_t T = (size_t)gridDim.x * blockDim.x;
        prefetch_l2_range(rec + sw_at(pf_first, 0, NCREC), (size_t)pf_count * NCREC * sizeof(float), g, T);
        prefetch_l2_range(nbp + sw_at(pf_first, 0, 6), (size_t)pf_count * 6 * sizeof(int), g, T);
    }
    if (g >= count) {
        if (chained) asm volatile("griddepcontrol.wait;" ::: "memory");
        if (chained == 1) asm volatile("griddepcontrol.launch_dependents;");
        return;
    }
    sweep_pos_compact<LOWER>(nbp, rec, dq, (long long)first + g, turb, chained != 0);
    if (chained == 1) asm volatile("griddepcontrol.launch_dependents;");
}

// Two hyperplanes per launch (mixed path): four lanes per position p of the second plane.
// Lanes 0-2 compute p's neighbour on the first plane in direction 0-2 -- each from its own
// neighbours on the plane before, which the previous launch finished -- and pass it to lane 3
// by warp shuffle, which then computes p.  A position of the first plane is so computed by
// each of its neighbours on the second plane, with the same inputs and arithmetic (sweep_core,
// shared with k_sweep_c), and each stores the same value; positions of the first plane with no
// neighbour on the second (block corners) come as a list of their own (orph) and are computed
// by lane 0 of an item alone.  One dependent launch and one L2 round trip per two planes
// instead of per plane.  Reads and writes go to different arrays, so that no thread can see a
// value another one is replacing: the lower sweep reads the right-hand sides from X and
// writes Y, the upper sweep reads the lower results from Y and writes the final DeltaQ back to
// X.  p_first, p_count: the second plane's positions; chained, pf_first, pf_count as in
// k_sweep_c.  (One thread computing all four positions held 255 registers and took 1.40 ms of
// sweeps per cascade iteration; a host-built table of the neighbours' neighbours, one load
// round before the wait instead of two dependent ones, measured slower still.)
template <bool LOWER>
__global__ void __launch_bounds__(128) k_sweep_pair(const int* __restrict__ nbp, const float* __restrict__ rec, float* X, float* Y,
                                                    int p_first, int p_count, const int* __restrict__ orph, int o_count, int turb,
                                                    int chained, int pf_first, int pf_count) {
    if (chained == 2) asm volatile("griddepcontrol.launch_dependents;");
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (pf_count > 0) {
        const size_t T = (size_t)gridDim.x * blockDim.x;
        prefetch_l2_range(rec + sw_at(pf_first, 0, NCREC), (size_t)pf_count * NCREC * sizeof(float), g, T);
        prefetch_l2_range(nbp + sw_at(pf_first, 0, 6), (size_t)pf_count * 6 * sizeof(int), g, T);
    }
    const int item = g >> 2, l = g & 3;
    const bool valid = item < p_count + o_count;
    const bool pair = item < p_count;
    const float* own_src = LOWER ? X : Y;          // the DeltaQ this sweep starts from
    float* dst = LOWER ? Y : X;                    // this sweep's results (neighbours read here)
    const float4* R4 = reinterpret_cast<const float4*>(rec);
    const float4* O4 = reinterpret_cast<const float4*>(own_src);
    // the position this lane computes: p (lane 3 of a pair item, lane 0 of an orphan) or p's
    // neighbour on the first plane in direction l (lanes 0-2 of a pair item), -1 = none
    long long p = -1, q = -1;
    if (valid) {
        p = pair ? (long long)p_first + item : (long long)orph[item - p_count];
        if (!pair) q = l == 0 ? p : -1;
        else if (l == 3) q = p;
        else q = nbp[sw_at(p, (LOWER ? 0 : 3) + l, 6)];
    }
    SweepStatic st;
    if (q >= 0) sweep_static<LOWER>(nbp, R4, q, st);
    if (chained) asm volatile("griddepcontrol.wait;" ::: "memory");
    float out[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    const bool first = q >= 0 && (!pair || l < 3);     // computes from the plane before
    float4 o0 = make_float4(0.f, 0.f, 0.f, 0.f), o1 = o0;
    if (q >= 0) {
        o0 = __ldcg(O4 + (size_t)q * 2);
        o1 = __ldcg(O4 + (size_t)q * 2 + 1);
    }
    if (first) {
        float4 a[3], t[3];
        sweep_nbvals(dst, st, q, a, t);
        sweep_core<LOWER>(st, o0, o1, a, t, turb, out);
        sweep_store(dst, q, out);
    }
    // lane 3 takes the first-plane values of lanes 0-2 (every lane shuffles)
    float nb[3][8];
    const int base = threadIdx.x & ~3 & 31;
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int m = 0; m < 8; ++m) nb[d][m] = __shfl_sync(0xffffffffu, out[m], base + d);
    if (pair && l == 3) {
        float4 a[3], t[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            a[d] = make_float4(nb[d][0], nb[d][1], nb[d][2], nb[d][3]);
            t[d] = make_float4(nb[d][4], nb[d][5], nb[d][6], nb[d][7]);
        }
        sweep_core<LOWER>(st, o0, o1, a, t, turb, out);
        sweep_store(dst, q, out);
    }
    if (chained == 1) asm volatile("griddepcontrol.launch_dependents;");
}

// Grid-wide barrier of a co-resident (cooperative) grid.  The wait is bounded: after `limit`
// polls the barrier records an error and every block leaves the kernel at its next check.
__device__ inline bool grid_barrier(SweepSync* sy, unsigned nblocks, unsigned limit) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* vgen = &sy->gen;
        const unsigned g0 = *vgen;
        __threadfence();
        if (atomicAdd(&sy->count, 1u) == nblocks - 1) {
            atomicExch(&sy->count, 0u);
            __threadfence();
            atomicAdd(&sy->gen, 1u);
        } else {
            unsigned it = 0;
            while (*vgen == g0) {
                if (++it > limit) { atomicExch(&sy->err, 1); break; }
            }
        }
        __threadfence();
        ok = *((volatile int*)&sy->err) == 0;      // one answer for the whole block
    }
    __syncthreads();
    return ok != 0;
}

// Both sweeps over all hyperplanes in one cooperative launch: the items of hyperplane h are
// spread over the whole grid, then a grid barrier; U runs the hyperplanes in reverse.
template <typename R>
__global__ void k_sweep_all(const int* __restrict__ nbp, const R* __restrict__ rec, R* dq, long long N,
                            const int* __restrict__ plane_off, int nplanes, int lanes, SweepSync* sy, unsigned limit,
                            const R* __restrict__ pc) {
    const int stride = gridDim.x * blockDim.x;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    for (int h = 0; h < nplanes; ++h) {
        const int first = plane_off[h], n = plane_off[h + 1] - first, items = sweep_items(n, lanes);
        for (int g = tid; g < items; g += stride) {
            int e, L;
            sweep_map(g, lanes, e, L);
            if (e < n) sweep_item<R, true>(nbp, rec, dq, N, (long long)first + e, L, lanes & 3, false, !(lanes & SWEEP_WPC), true, pc);
        }
        if (!grid_barrier(sy, gridDim.x, limit)) return;
    }
    for (int h = nplanes - 1; h >= 0; --h) {
        const int first = plane_off[h], n = plane_off[h + 1] - first, items = sweep_items(n, lanes);
        for (int g = tid; g < items; g += stride) {
            int e, L;
            sweep_map(g, lanes, e, L);
            if (e < n) sweep_item<R, false>(nbp, rec, dq, N, (long long)first + e, L, lanes & 3, false, !(lanes & SWEEP_WPC), true, pc);
        }
        if (h > 0 && !grid_barrier(sy, gridDim.x, limit)) return;
    }
}

// Both sweeps as one dataflow over all positions (one cooperative launch): item (q, L) starts
// as soon as its three neighbours of the previous hyperplane have published their DeltaQ
// (flag[q'] counts the 7 lanes of q' that have written), instead of waiting for the whole
// hyperplane.  Items go to threads round-robin in sweep order (L sweep ascending, then U
// descending), so a thread only ever waits on items that come earlier in that order: with the
// whole grid resident nothing can wait forever.  Every wait is bounded; on expiry the kernel
// records an error and all threads leave.
template <typename R>
__device__ inline bool flow_wait(const int* flag, long long q, int want, SweepSync* sy, unsigned limit) {
    const volatile int* f = flag + q;
    unsigned it = 0;
    while (*f < want) {
        if ((++it & 255) == 0 && *((volatile int*)&sy->err)) return false;
        if (it > limit) { atomicExch(&sy->err, 2); return false; }
        __nanosleep(32);
    }
    __threadfence();
    return true;
}

template <typename R>
__global__ void k_sweep_flow(const int* __restrict__ nbp, const R* __restrict__ rec, R* dq, long long N, int* flagL, int* flagU,
                             int turb, SweepSync* sy, unsigned limit, const R* __restrict__ pc) {
    const long long T = (long long)gridDim.x * blockDim.x;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long items = N * SWEEP_LANES;
    for (long long it = t; it < items; it += T) {                  // L sweep, ascending
        const long long q = it / SWEEP_LANES;
        const int L = (int)(it % SWEEP_LANES);
        if (L >= 7) continue;
        bool ok = true;
        for (int d = 0; d < 3 && ok; ++d) {
            const long long np = nbp[sw_at(q, d, 6)];
            if (np >= 0) ok = flow_wait<R>(flagL, np, 7, sy, limit);
        }
        if (!ok) return;
        sweep_item<R, true>(nbp, rec, dq, N, q, L, turb & 3, false, true, true, pc);
        __threadfence();
        atomicAdd(flagL + q, 1);
    }
    for (long long it = t; it < items; it += T) {                  // U sweep, descending
        const long long q = N - 1 - it / SWEEP_LANES;
        const int L = (int)(it % SWEEP_LANES);
        if (L >= 7) continue;
        bool ok = flow_wait<R>(flagL, q, 7, sy, limit);             // own L result
        for (int d = 0; d < 3 && ok; ++d) {
            const long long np = nbp[sw_at(q, 3 + d, 6)];
            if (np >= 0) ok = flow_wait<R>(flagU, np, 7, sy, limit);
        }
        if (!ok) return;
        sweep_item<R, false>(nbp, rec, dq, N, q, L, turb & 3, false, true, true, pc);
        __threadfence();
        atomicAdd(flagU + q, 1);
    }
}

// Both sweeps as a tiled wavefront (one cooperative launch): every CTA takes the next tile of
// the topological order from a counter (L sweep tiles first, then the U sweep tiles in
// reverse), waits until the tiles holding its lower (upper) neighbours have published, sweeps
// the tile's own planes with a CTA barrier between them, and publishes the tile.  A CTA only
// waits on tiles taken before its own by CTAs that are running, so the smallest unfinished
// tile can always proceed.  Waits are bounded: on expiry the kernel records an error and
// every CTA leaves at its next check.
__device__ inline bool tile_wait(const int* flag, SweepSync* sy, unsigned limit) {
    const volatile int* f = flag;
    unsigned it = 0;
    while (*f == 0) {
        if ((++it & 255) == 0 && *((volatile int*)&sy->err)) return false;
        if (it > limit) { atomicExch(&sy->err, 3); return false; }
        __nanosleep(64);
    }
    __threadfence();
    return true;
}

template <typename R>
__global__ void k_sweep_tiles(const int* __restrict__ nbp, const R* __restrict__ rec, R* dq, long long N, TileView tv,
                              int lanes, int* flags, int* counter, SweepSync* sy, unsigned limit, const R* __restrict__ pc) {
    __shared__ int s_t, s_ok;
    const int nt = tv.ntiles;
    for (;;) {
        if (threadIdx.x == 0) s_t = *((volatile int*)&sy->err) ? 2 * nt : atomicAdd(counter, 1);
        __syncthreads();
        const int t = s_t;
        if (t >= 2 * nt) return;
        const bool lower = t < nt;
        const int T = lower ? t : 2 * nt - 1 - t;
        if (threadIdx.x == 0) {
            bool ok = true;
            for (int d = 0; d < 3 && ok; ++d) {
                const int dep = tv.dep[6 * T + (lower ? 0 : 3) + d];
                if (dep >= 0) ok = tile_wait(flags + (lower ? 0 : nt) + dep, sy, limit);
            }
            if (ok && !lower) ok = tile_wait(flags + T, sy, limit);      // the tile's own L result
            s_ok = ok ? 1 : 0;
        }
        __syncthreads();
        if (!s_ok) return;
        const int p0 = tv.plane0[T], np = tv.plane0[T + 1] - p0;
        for (int pp = 0; pp < np; ++pp) {
            const int p = lower ? p0 + pp : p0 + np - 1 - pp;
            const int a = tv.pitem[p], n = tv.pitem[p + 1] - a, items = sweep_items(n, lanes);
            for (int g = threadIdx.x; g < items; g += blockDim.x) {
                int e, L;
                sweep_map(g, lanes, e, L);
                if (e >= n) continue;
                const long long q = tv.item[a + e];
                if (lower) sweep_item<R, true>(nbp, rec, dq, N, q, L, lanes & 3, false, !(lanes & SWEEP_WPC), true, pc);
                else sweep_item<R, false>(nbp, rec, dq, N, q, L, lanes & 3, false, !(lanes & SWEEP_WPC), true, pc);
            }
            __syncthreads();
        }
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) atomicExch(flags + (lower ? 0 : nt) + T, 1);
    }
}

// DeltaQ back to the cells (the update and trans_get_field read it there), one thread per
// interior cell of the cell tiles: a sweep position's components share one sector of dq, so
// each cell reads one sector and the stores to the D slots are coalesced (components l0..6:
// the Runge-Kutta path sweeps and returns only k and omega, l0 = 5)
template <typename R>
__global__ void k_sweep_scatter(const DevBlock* __restrict__ blks, const Tile* __restrict__ tiles, const int* __restrict__ qpos,
                                const R* __restrict__ dq, int l0) {
    const Tile t = tiles[blockIdx.x];
    if ((int)threadIdx.x >= t.count) return;
    const DevBlock b = blks[t.blk];
    const int n = t.start + threadIdx.x;
    const int I = n % b.NI1 + 1, J = (n / b.NI1) % b.NJ1 + 1, K = n / (b.NI1 * b.NJ1) + 1;
    const int c = cidx(b, I, J, K);
    const long long q = qpos[(size_t)blockIdx.x * CELL_TILE + threadIdx.x];
    R d[7];
#pragma unroll
    for (int L = 0; L < 7; ++L) d[L] = L >= l0 ? dq[sw_at(q, L, DQ_STRIDE)] : R(0);
#pragma unroll
    for (int L = 0; L < 7; ++L)
        if (L >= l0) rs<R>(b, S_D + L)[c] = d[L];
}

#ifdef TG_COMMON_KERNELS
// ---------------------------------------------------------------------------------------
// SST update of k and omega at the end of an iteration (Time/TIME_Update_V.F90:709-816,
// Time/TIME_RK_V_Update_New.F90:97-187, Kind_Model = 1): exp-positivity increments, the
// F2-limited Cmu, the omega and k realizability limits and the eddy viscosity.  RmiuL is the
// caller's laminar viscosity (the two routines evaluate Sutherland differently).
// ---------------------------------------------------------------------------------------
__device__ inline void sst_update(const Params& p, const DevBlock& b, int c, int d_fp32, double d6, double d7, double pRo,
                                  double RmiuL) {
    double* V5 = slot(b, S_V + 5);
    double* V6 = slot(b, S_V + 6);
    double ARTk = V5[c], ARTO = V6[c];
    if (d6 >= 0.0) ARTk = ARTk + d6;
    else ARTk = ARTk * tmx::exp_(d6 / (ARTk + 1.e-10));
    ARTk = dmax(ARTk, 1.0e-10);
    if (d7 >= 0.0) ARTO = ARTO + d7;
    else ARTO = ARTO * tmx::exp_(d7 / (ARTO + 1.e-10));
    ARTO = dmax(ARTO, 1.0e-10);
    double DistN = slot(b, S_DST)[c];
    auto G = [&](int q) { return d_fp32 ? (double)fslot(b, S_DQ + q)[c] : slot(b, S_DQ + q)[c]; };
    double Dudx = G(0), Dudy = G(1), Dudz = G(2), Dvdx = G(3), Dvdy = G(4), Dvdz = G(5), Dwdx = G(6), Dwdy = G(7), Dwdz = G(8);
    double Div = Dudx + Dvdy + Dwdz;
    double prod = (2.0 * (Dudx * Dudx + Dvdy * Dvdy + Dwdz * Dwdz) + sq(Dudy + Dvdx) + sq(Dvdz + Dwdy) + sq(Dwdx + Dudz)
                   - 2.0 / 3.0 * Div * Div);
    if (p.Kind_Model == 2) {    // Wilcox 2006 (TIME_Update_V.F90:821-858, TIME_RK_V_Update_New.F90:195-232)
        double Sii = Dudx - (Dudx + Dvdy + Dwdz) / 3.;
        double Sjj = Dvdy - (Dudx + Dvdy + Dwdz) / 3.;
        double Skk = Dwdz - (Dudx + Dvdy + Dwdz) / 3.;
        double Sij = (Dudy + Dvdx) / 2.0, Sik = (Dudz + Dwdx) / 2.0, Sjk = (Dvdz + Dwdy) / 2.0;
        double Skl = sqrt(1.0 * Sii * Sii + 1.0 * Sjj * Sjj + 1.0 * Skk * Skk + 2.0 * Sij * Sij + 2.0 * Sik * Sik + 2.0 * Sjk * Sjk);
        ARTO = dmax(ARTO, sqrt(pRo * fabs(prod) / (p.Prod_Lmt * p.Beta_star)) / p.Ref);
        ARTk = dmin(ARTk, 100000.0 * RmiuL * ARTO / pRo);
        V5[c] = ARTk;
        V6[c] = ARTO;
        ARTO = dmax(ARTO, 7. / 8. * pRo * sqrt(Skl * Skl * 2. / 0.09) / p.Ref);
        slot(b, S_RMIU)[c] = ARTk / ARTO * pRo;
        return;
    }
    double arg2 = 2.0 * sqrt(ARTk / pRo) / p.Beta_star / (ARTO / pRo) / DistN / p.Ref;
    arg2 = dmax(arg2, 500.0 * RmiuL / DistN / DistN / ARTO / p.Ref / p.Ref);
    arg2 = tmx::tanh_(arg2 * arg2);
    double Sii = Dudx, Sjj = Dvdy, Skk = Dwdz;
    double Sij = (Dudy + Dvdx) / 2.0, Sik = (Dudz + Dwdx) / 2.0, Sjk = (Dvdz + Dwdy) / 2.0;
    double Skl = sqrt(2.0 * (1.0 * Sii * Sii + 1.0 * Sjj * Sjj + 1.0 * Skk * Skk + 2.0 * Sij * Sij + 2.0 * Sik * Sik + 2.0 * Sjk * Sjk));
    double Cmua = dmin(1.0, p.A1 * ARTO / pRo / ((Skl) * arg2 + 1.e-10) * p.Ref);
    ARTO = dmax(ARTO, sqrt(pRo * Cmua * fabs(prod) / (p.Prod_Lmt * p.Beta_star)) / p.Ref);
    ARTk = dmin(ARTk, 100000.0 * RmiuL * ARTO / pRo / Cmua);
    V5[c] = ARTk;
    V6[c] = ARTO;
    slot(b, S_RMIU)[c] = Cmua * ARTk / ARTO * pRo;
}

// ---------------------------------------------------------------------------------------
// Time/TIME_Update_V.F90:106-294 (norms) and :502-859 (update), FP64 in both paths
// ---------------------------------------------------------------------------------------
__global__ void k_update(const DevBlock* __restrict__ blks, const Tile* __restrict__ tiles, const CaseDev* __restrict__ cdev,
                         NormPart* __restrict__ parts, int d_fp32) {
    const Tile t = tiles[blockIdx.x];
    const DevBlock b = blks[t.blk];
    const Params p = cdev[b.cs].p;
    const int turb_upd = cdev[b.cs].turb_upd;
    int tid = threadIdx.x;
    double sa = 0, ma = -1, sk = 0, mk = 0, so = 0, mo = 0;
    long long ia = -1;
    int nanf = 0;
    if (tid < t.count) {
        int n = t.start + tid;
        int I = n % b.NI1 + 1, J = (n / b.NI1) % b.NJ1 + 1, K = n / (b.NI1 * b.NJ1) + 1;
        int c = cidx(b, I, J, K);
        double* V[7];
        for (int m = 0; m < 7; ++m) V[m] = slot(b, S_V + m);
        double* PP = slot(b, S_PP);
        double* T = slot(b, S_T);
        double v1 = V[0][c];
        // DeltaQ from the sweeps: FP64, or FP32 in the mixed path
        auto Dq = [&](int L) { return d_fp32 ? (double)fslot(b, S_D + L)[c] : slot(b, S_D + L)[c]; };
        double d1 = Dq(0), d6 = Dq(5), d7 = Dq(6);
        double DR = fabs(d1 / v1);
        nanf = isnan(d1) ? 1 : 0;
        sa = DR * DR; ma = DR; ia = n;
        double DRk = fabs(d6 / v1), DRo = fabs(d7 / v1);
        sk = DRk * DRk; mk = DRk; so = DRo * DRo; mo = DRo;
        // mean flow (non-preconditioned, TIME_Update_V.F90:621-689)
        double AinRo = d1, AinRx = Dq(1), AinRy = Dq(2), AinRz = Dq(3);
        double AinRe = Dq(4);
        double pRo = v1;
        double roinv = 1.0 / pRo;
        double rr = p.omega0 * slot(b, S_RAD)[c];
        if (p.IF_Precondition) {
            // preconditioned (TIME_Update_V.F90:580-607): conservative increments; the kinetic
            // energy takes the new momenta with the old 1/rho, and T the old pressure with the
            // new density
            double pRx = V[1][c], pRy = V[2][c], pRz = V[3][c], pRe = V[4][c];
            pRo = pRo + AinRo;
            pRo = fabs(pRo);
            pRx = pRx + AinRx; pRy = pRy + AinRy; pRz = pRz + AinRz;
            pRe = pRe + AinRe;
            pRe = fabs(pRe);
            double DV = 0.5 * (pRx * pRx + pRy * pRy + pRz * pRz) * roinv;
            double pPP = (pRe - DV) * (1.4 - 1.0);
            if (pPP <= 0.0) {
                pPP = fabs(pPP);
                pRe = pPP / (1.4 - 1.0) + DV;
            }
            double pTT = p.RXM2 * PP[c] / pRo;
            V[0][c] = pRo; V[1][c] = pRx; V[2][c] = pRy; V[3][c] = pRz; V[4][c] = pRe;
            PP[c] = pPP;
            T[c] = pTT;
        } else {
        double pVx = V[1][c] * roinv, pVy = V[2][c] * roinv, pVz = V[3][c] * roinv;
        double AinX = (AinRx - pVx * AinRo) * roinv;
        double AinY = (AinRy - pVy * AinRo) * roinv;
        double AinZ = (AinRz - pVz * AinRo) * roinv;
        double AinP = (1.4 - 1.0) * (AinRe - 0.5 * AinRo * (pVx * pVx + pVy * pVy + pVz * pVz) - pRo * (AinX * pVx + AinY * pVy + AinZ * pVz));
        if (AinRo >= 0.) pRo = pRo + AinRo;
        else pRo = pRo * tmx::exp_(AinRo / (pRo + 1.e-10));
        pRo = fabs(pRo);
        double pp = PP[c];
        if (AinP >= 0.) pp = pp + AinP;
        else pp = pp * tmx::exp_(AinP / (pp + 1.e-10));
        pp = fabs(pp);
        PP[c] = pp;
        T[c] = p.RXM2 * pp / pRo;
        pVx = pVx + AinX; pVy = pVy + AinY; pVz = pVz + AinZ;
        V[0][c] = pRo;
        V[1][c] = pRo * pVx;
        V[2][c] = pRo * pVy;
        V[3][c] = pRo * pVz;
        double DV = 0.5 * (pVx * pVx + pVy * pVy + pVz * pVz);
        V[4][c] = pp / (1.4 - 1.0) + DV * pRo - 0.5 * sq(rr) * pRo;
        }
        if (turb_upd) {   // TIME_Update_V.F90:709-816
            double VV = sq(V[1][c]) + sq(V[2][c]) + sq(V[3][c]);
            double PPP = (1.4 - 1.0) * V[4][c] - 0.5 * (1.4 - 1.0) * (VV / pRo - sq(rr) * pRo);
            double TT = p.RXM2 * PPP / pRo;
            sst_update(p, b, c, d_fp32, d6, d7, pRo, mu_suth<double>(p, TT));
        }
    }
    NormPart P;
    P.sa = sa; P.ma = ma; P.sk = sk; P.mk = mk; P.so = so; P.mo = mo; P.ia = ia; P.nan = nanf; P.pad_ = 0;
    P = norm_reduce_cta(P);
    if (tid == 0) parts[blockIdx.x] = P;
}

// ---------------------------------------------------------------------------------------
// Runge-Kutta marching (IF_RK = 1), FP64 in both paths.
// Time/TIME_RK_Save.F90:16-28 (Wt2 <- V at stage 1) and Time/TIME_RK.F90:27-86: the norms of
// |D1/V1| on the residual before the update, then the SSP-RK3 stage on V(1:5).  Also leaves
// 1/rho and the velocities of the new state for the k-omega sweep Jacobians (FP32 copies of
// them and of V(1:5) in the mixed path), which TURBTWO_TIME_LUSGS_SST evaluates on it.
// ---------------------------------------------------------------------------------------
__global__ void k_rk_update(const DevBlock* __restrict__ blks, const Tile* __restrict__ tiles, NormPart* __restrict__ parts,
                            int d_fp32, int itr) {
    const Tile t = tiles[blockIdx.x];
    const DevBlock b = blks[t.blk];
    const int tid = threadIdx.x;
    double sa = 0, ma = -1;
    long long ia = -1;
    int nanf = 0;
    if (tid < t.count) {
        const int n = t.start + tid;
        const int I = n % b.NI1 + 1, J = (n / b.NI1) % b.NJ1 + 1, K = n / (b.NI1 * b.NJ1) + 1;
        const int c = cidx(b, I, J, K);
        if (itr == 1)
            for (int L = 0; L < 7; ++L) slot(b, S_WT2 + L)[c] = slot(b, S_V + L)[c];
        auto Dq = [&](int L) { return d_fp32 ? (double)fslot(b, S_D + L)[c] : slot(b, S_D + L)[c]; };
        const double d1 = Dq(0);
        const double DR = fabs(d1 / slot(b, S_V)[c]);
        nanf = isnan(d1) ? 1 : 0;
        sa = DR * DR; ma = DR; ia = n;
        const double dtm = slot(b, S_DTM)[c], vol = slot(b, S_VOL)[c];
        double v[5];
        for (int L = 0; L < 5; ++L) {
            const double d = Dq(L), w = slot(b, S_WT2 + L)[c];
            double x = slot(b, S_V + L)[c];
            if (itr == 1) x = x + dtm * d / vol;
            else if (itr == 2) x = 0.75 * w + 0.25 * x + 0.25 * dtm * d / vol;
            else x = 1.0 / 3.0 * w + 2.0 / 3.0 * x + 2.0 / 3.0 * dtm * d / vol;
            slot(b, S_V + L)[c] = x;
            v[L] = x;
        }
        const double ri = 1.0 / v[0];
        const double u = v[1] * ri, vv = v[2] * ri, w = v[3] * ri;
        slot(b, S_RINV)[c] = ri;
        slot(b, S_SVEL)[c] = u;
        slot(b, S_SVEL + 1)[c] = vv;
        slot(b, S_SVEL + 2)[c] = w;
        if (d_fp32) {
            for (int L = 0; L < 5; ++L) fslot(b, S_V + L)[c] = (float)v[L];
            fslot(b, S_RINV)[c] = (float)ri;
            fslot(b, S_SVEL)[c] = (float)u;
            fslot(b, S_SVEL + 1)[c] = (float)vv;
            fslot(b, S_SVEL + 2)[c] = (float)w;
        }
    }
    NormPart P = norm_identity();
    P.sa = sa; P.ma = ma; P.ia = ia; P.nan = nanf;
    P = norm_reduce_cta(P);
    if (tid == 0) {      // the k and omega parts are written by k_rk_vupdate
        NormPart& Q = parts[blockIdx.x];
        Q.sa = P.sa; Q.ma = P.ma; Q.ia = P.ia; Q.nan = P.nan; Q.pad_ = 0;
    }
}

// Time/TIME_RK_V_Update_New.F90:66-320: p and T from the new V (no rotation term), the SST
// update from the k-omega increments (Sutherland without Csth1), then the k and omega norms
// on the updated density.
__global__ void k_rk_vupdate(const DevBlock* __restrict__ blks, const Tile* __restrict__ tiles, const CaseDev* __restrict__ cdev,
                             NormPart* __restrict__ parts, int d_fp32) {
    const Tile t = tiles[blockIdx.x];
    const DevBlock b = blks[t.blk];
    const Params p = cdev[b.cs].p;
    const int turb_upd = cdev[b.cs].turb_upd;
    const int tid = threadIdx.x;
    double sk = 0, mk = 0, so = 0, mo = 0;
    if (tid < t.count) {
        const int n = t.start + tid;
        const int I = n % b.NI1 + 1, J = (n / b.NI1) % b.NJ1 + 1, K = n / (b.NI1 * b.NJ1) + 1;
        const int c = cidx(b, I, J, K);
        const double v1 = slot(b, S_V)[c], v2 = slot(b, S_V + 1)[c], v3 = slot(b, S_V + 2)[c];
        const double v4 = slot(b, S_V + 3)[c], v5 = slot(b, S_V + 4)[c];
        double VV = v2 * v2 + v3 * v3 + v4 * v4;
        const double pp = (1.4 - 1.0) * v5 - 0.5 * (1.4 - 1.0) * VV / v1;
        slot(b, S_PP)[c] = pp;
        slot(b, S_T)[c] = p.RXM2 * pp / v1;
        auto Dq = [&](int L) { return d_fp32 ? (double)fslot(b, S_D + L)[c] : slot(b, S_D + L)[c]; };
        const double d6 = Dq(5), d7 = Dq(6);
        if (turb_upd) {
            VV = sq(v2) + sq(v3) + sq(v4);
            const double PPP = 0.4 * v5 - 0.2 * VV / v1;
            const double TT = p.RXM2 * PPP / v1;
            sst_update(p, b, c, d_fp32, d6, d7, v1, mu_suth_nocs<double>(p, TT));
        }
        const double DRk = fabs(d6 / v1), DRo = fabs(d7 / v1);
        sk = DRk * DRk; mk = DRk; so = DRo * DRo; mo = DRo;
    }
    NormPart P = norm_identity();
    P.sk = sk; P.so = so; P.mk = mk; P.mo = mo;
    P = norm_reduce_cta(P);
    if (tid == 0) {
        NormPart& Q = parts[blockIdx.x];
        Q.sk = P.sk; Q.so = P.so; Q.mk = P.mk; Q.mo = P.mo;
    }
}

// Per-block norms from the per-tile partials (Time/TIME_Update_V.F90:116-146, 892-908): one
// block of threads per solver block, fixed summation order (strided partial sums, then the
// warp-shuffle reduction), the maximum of |D1/V1| with the later cell winning ties.
__global__ void k_block_norms(const DevBlock* __restrict__ blks, const NormPart* __restrict__ parts,
                              const int* __restrict__ tile_first, BlockNorms* __restrict__ out) {
    const int bi = blockIdx.x, tid = threadIdx.x;
    double sa = 0, sk = 0, so = 0, ma = -1, mk = 0, mo = 0;
    long long ia = 0;
    int nan = 0;
    for (int t = tile_first[bi] + tid; t < tile_first[bi + 1]; t += blockDim.x) {
        const NormPart P = parts[t];
        sa += P.sa; sk += P.sk; so += P.so;
        if (P.ma > ma || (P.ma == ma && P.ia > ia)) { ma = P.ma; ia = P.ia; }
        mk = dmax(mk, P.mk); mo = dmax(mo, P.mo);
        nan |= P.nan;
    }
    NormPart P;
    P.sa = sa; P.ma = ma; P.sk = sk; P.mk = mk; P.so = so; P.mo = mo; P.ia = ia; P.nan = nan; P.pad_ = 0;
    P = norm_reduce_cta(P);
    if (tid == 0) {
        const DevBlock B = blks[bi];
        BlockNorms N;
        N.DRSa = sqrt(P.sa / B.NI1 / B.NJ1 / B.NK1);
        N.DRSk = sqrt(P.sk / B.NI1 / B.NJ1 / B.NK1);
        N.DRSo = sqrt(P.so / B.NI1 / B.NJ1 / B.NK1);
        N.DUa = P.ma; N.DUk = P.mk; N.DUo = P.mo;
        const long long i0 = P.ia;
        N.Ima = (int)(i0 % B.NI1) + 1; N.Jma = (int)((i0 / B.NI1) % B.NJ1) + 1; N.Kma = (int)(i0 / ((long long)B.NI1 * B.NJ1)) + 1;
        N.nan_flag = P.nan;
        out[bi] = N;
    }
}

// Time/TIME_Update_U.F90:16-44
__global__ void k_update_u(const DevBlock* __restrict__ blks, const Tile* __restrict__ tiles, const CaseDev* __restrict__ cdev) {
    const Tile t = tiles[blockIdx.x];
    if ((int)threadIdx.x >= t.count) return;
    const DevBlock b = blks[t.blk];
    const int kind_dual = cdev[b.cs].p.Kind_Dual;
    if (kind_dual == 0) return;
    int n = t.start + threadIdx.x;
    int I = n % b.NI1 + 1, J = (n / b.NI1) % b.NJ1 + 1, K = n / (b.NI1 * b.NJ1) + 1;
    int c = cidx(b, I, J, K);
    // every load before the first store: the slots share one arena, so loads placed after a
    // store would each wait for the previous component's round trip
    double w0[7], v[7];
#pragma unroll
    for (int L = 0; L < 7; ++L) {
        w0[L] = slot(b, S_WT0 + L)[c];
        v[L] = slot(b, S_V + L)[c];
    }
#pragma unroll
    for (int L = 0; L < 7; ++L) {
        if (kind_dual == 2) slot(b, S_WT1 + L)[c] = w0[L];
        slot(b, S_WT0 + L)[c] = v[L];
    }
}

// static metric products (computed once per geometry upload)
__global__ void k_geom_static(const DevBlock* __restrict__ blks, int nblk, long long total, const long long* __restrict__ off) {
    long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total) return;
    int lo = 0, hi = nblk - 1;
    while (lo < hi) { int mid = (lo + hi + 1) >> 1; if (off[mid] <= g) lo = mid; else hi = mid - 1; }
    const DevBlock b = blks[lo];
    int c = (int)(g - off[lo]);
    int i = c % b.PI, j = (c / b.PI) % b.PJ, k = c / (b.PI * b.PJ);
    const int st[3] = {1, b.PI, b.PI * b.PJ};
    const int pos[3] = {i, j, k};
    const int ext[3] = {b.NI + 5, b.PJ, b.PK};       // the ghost extent (row padding excluded)
    for (int d = 0; d < 3; ++d) {
        if (pos[d] >= 1) {
            const double* al = slot(b, S_ALAGM + d);
            slot(b, S_AINV + d)[c] = 1.0 / (al[c] + al[c - st[d]]);
            const double* vo = slot(b, S_VOL);
            slot(b, S_VINV + d)[c] = 1.0 / (vo[c] + vo[c - st[d]]);
        }
        if (pos[d] + 1 < ext[d])
            for (int m = 0; m < 3; ++m) {
                const double* S = slot(b, S_SD + 3 * d + m);
                slot(b, S_ASD + 3 * d + m)[c] = 0.5 * (S[c] + S[c + st[d]]);
            }
    }
}

#endif  // TG_COMMON_KERNELS

}  // namespace tg

namespace tg {
#ifdef TG_COMMON_KERNELS
// Fortran-layout (component fastest, lower bound lb) <-> slots, one thread per Fortran cell
// one thread per element of the Fortran array (component fastest), so that the array side --
// a staging buffer, or the caller's page-locked array over the host link -- is read and written
// in whole consecutive lines
__global__ void k_field_xfer(DevBlock b, int slot0, int ncomp, int lb, int is_sd, double* __restrict__ stage, int to_slots) {
    int ei = b.NI + 2 - lb + 1, ej = b.NJ + 2 - lb + 1, ek = b.NK + 2 - lb + 1;
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)ei * ej * ek * ncomp) return;
    long long n = e / ncomp;
    int m = (int)(e - n * ncomp);
    int i = (int)(n % ei), j = (int)((n / ei) % ej), k = (int)(n / ((long long)ei * ej));
    int c = cidx(b, i + lb, j + lb, k + lb);
    int so = is_sd ? 3 * (m % 3) + m / 3 : m;
    double* sl = slot(b, slot0 + so);
    if (to_slots) sl[c] = stage[e];
    else stage[e] = sl[c];
}

// Cross-rank 1-to-1 interfaces (BC/PARALLEL_BC_P2P.F90:1-257): the words of a segment's face
// cells in the reference's buffer layout.  Pack: cells[3q+L] is the source cell of layer L of
// face cell q; sweep -1 sends per face cell layer 0: V(1:7), PP, T, Rmiu, Rds(1:3), shock and
// layers 1, 2: V(1:7), PP, T, Rmiu, shock (36 words); sweep 0 the 18 gradients of layer 0
// (from the FP32 copies when dq_fp32).  Unpack (k_halo_unpack): tab[4q] is the partner's face
// cell whose words fill face cell q, tab[4q+1+L] the ghost cell of layer L; the state and
// gradients are rotated by the interface's angle exactly as the same-rank copy (k_bc_state,
// k_bc_grad) rotates them; Rds and shock travel but are not written (the ghost shock is
// overwritten by the extrapolation, the ghost Rds is read by nothing).
__global__ void k_halo_pack(DevBlock b, const int* __restrict__ cells, int n, int sweep, int dq_fp32, double* __restrict__ out) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    if (sweep == -1) {
        double* w = out + (size_t)36 * q;
        int k = 0;
        for (int L = 0; L < 3; ++L) {
            const int c = cells[3 * q + L];
            for (int m = 0; m < 7; ++m) w[k++] = slot(b, S_V + m)[c];
            w[k++] = slot(b, S_PP)[c];
            w[k++] = slot(b, S_T)[c];
            w[k++] = slot(b, S_RMIU)[c];
            if (L == 0)
                for (int d = 0; d < 3; ++d) w[k++] = slot(b, S_RDS + d)[c];
            w[k++] = dq_fp32 ? (double)fslot(b, S_SHOCK)[c] : slot(b, S_SHOCK)[c];
        }
    } else {
        const int c = cells[3 * q];
        for (int m = 0; m < 18; ++m) out[(size_t)18 * q + m] = dq_fp32 ? (double)fslot(b, S_DQ + m)[c] : slot(b, S_DQ + m)[c];
    }
}

// Several Fortran-layout arrays in page-locked host memory <-> slots in one launch: each thread
// moves a chunk of ch consecutive elements of one array (component fastest); uploads take chunks
// of XFER_CHUNK with 16-byte reads of the host side (a warp keeps 1 KB of the host link in
// flight per access), downloads one element per thread (measured faster: the writes to the host
// side stream from many more threads).  Entry q owns chunks [off[q], off[q+1]); the arrays start
// on 16-byte boundaries (page-locked allocations), and every chunk starts at a multiple of ch
// within its array.
__global__ void k_fields_xfer(XferBatch x, long long total, int to_slots, int ch) {
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total) return;
    int lo = 0, hi = x.n - 1;
    while (lo < hi) { int mid = (lo + hi + 1) >> 1; if (x.e[mid].off <= g) lo = mid; else hi = mid - 1; }
    const XferEntry& E = x.e[lo];
    const long long r0 = (g - E.off) * ch;
    const int m = (int)(E.count - r0 < ch ? E.count - r0 : ch);
    double v[XFER_CHUNK];
    long long cs[XFER_CHUNK];
#pragma unroll
    for (int u = 0; u < XFER_CHUNK; ++u) {
        if (u >= m) break;
        const long long r = r0 + u;
        const long long n = r / E.ncomp;
        const int mc = (int)(r - n * E.ncomp);
        const int i = (int)(n % E.ei), j = (int)((n / E.ei) % E.ej), k = (int)(n / ((long long)E.ei * E.ej));
        const long long c = (long long)(i + E.lb + 2) + (long long)E.PI * ((j + E.lb + 2) + (long long)E.PJ * (k + E.lb + 2));
        const int so = E.is_sd ? 3 * (mc % 3) + mc / 3 : mc;
        cs[u] = (long long)(E.slot0 + so) * (long long)E.ncell + c;
    }
    if (to_slots) {
        if (m == XFER_CHUNK && ch == XFER_CHUNK) {
            const double2* h = reinterpret_cast<const double2*>(E.host + r0);
#pragma unroll
            for (int u = 0; u < XFER_CHUNK / 2; ++u) {
                const double2 w = h[u];
                v[2 * u] = w.x;
                v[2 * u + 1] = w.y;
            }
        } else {
            for (int u = 0; u < m; ++u) v[u] = E.host[r0 + u];
        }
        for (int u = 0; u < m; ++u) E.base[cs[u]] = v[u];
    } else {
        for (int u = 0; u < m; ++u) v[u] = E.base[cs[u]];
        if (m == XFER_CHUNK && ch == XFER_CHUNK) {
            double2* h = reinterpret_cast<double2*>(E.host + r0);
#pragma unroll
            for (int u = 0; u < XFER_CHUNK / 2; ++u) h[u] = make_double2(v[2 * u], v[2 * u + 1]);
        } else {
            for (int u = 0; u < m; ++u) E.host[r0 + u] = v[u];
        }
    }
}
#endif  // TG_COMMON_KERNELS
}  // namespace tg
