// kernels_mixed.cuh -- the FP64-state kernels of the mixed-precision path in a reduced-operation
// form (included by k_mixed.cu only).
//
// On GB300 every FP64 instruction -- and every double <-> float conversion -- issues at 1/64 of
// the FP32 rate, and a double division or square root is ~10 of them.  The FP64 path evaluates
// Time/SpectralRadius.F90 and Time/TIME_Update_V.F90 operation by operation (bit-identical to
// the reference's arithmetic); these mixed-path versions keep the state in FP64 -- the
// conserved variables and pressure are FP64 values that FP32 increments are added to -- and
//   - convert between double and float on the integer pipe (cvt.cuh),
//   - evaluate the increments of the update (velocity, pressure, the norms' |D/V| terms) in
//     FP32, from the FP32 DeltaQ the sweeps produce: the momentum update
//     rho'(m/rho + a) = m + (m r + rho' a), with r = rho'/rho - 1, becomes one FP32 increment
//     added to the FP64 momentum, so no FP64 division is left per cell,
//   - evaluate the positivity-preserving update p*exp(dp/p) = p + p*expm1(dp/p) with an FP32
//     expm1 scaled by the FP64 value (the FP32 error scales with the increment, so it vanishes
//     as the iteration converges),
//   - evaluate the spectral radii and the local time step in FP32 (they set the pseudo-time
//     step, not the converged solution), and the SST model algebra of the update (the
//     F2-limited C_mu, the realizability limits of omega and k) in FP32, like the other SST and
//     sweep arithmetic of the mixed path,
//   - reduce the residual norms in FP32 within a warp and in FP64 across the CTA's warps.
#pragma once
#include "cvt.cuh"

namespace tg {

// ---------------------------------------------------------------------------------------
// Time/SpectralRadius.F90:47-180, mixed path: spectral radii and local time step in FP32 from
// the FP64 state (converted on the integer pipe) and the FP32 copies of the metrics; written to
// the FP64 slots (exact values of the FP32 results), which k_prims_mixed copies for the sweeps.
// ---------------------------------------------------------------------------------------
__global__ void k_specrad_mixed(const DevBlock* __restrict__ blks, const Tile* __restrict__ tiles,
                                const CaseDev* __restrict__ cdev) {
    const Tile t = tiles[blockIdx.x];
    if ((int)threadIdx.x >= t.count) return;
    const DevBlock b = blks[t.blk];
    const CaseDev& cd = cdev[b.cs];
    const ParamsT<float>& pf = cd.pf;
    const int n = t.start + threadIdx.x;
    const int I = n % b.NI1 + 1, J = (n / b.NI1) % b.NJ1 + 1, K = n / (b.NI1 * b.NJ1) + 1;
    const int c = cidx(b, I, J, K);
    const float rden = 1.0f / f32_rn(slot(b, S_V)[c]);
    const float Vxi = f32_rn(slot(b, S_V + 1)[c]) * rden, Vyi = f32_rn(slot(b, S_V + 2)[c]) * rden;
    const float Vzi = f32_rn(slot(b, S_V + 3)[c]) * rden;
    const float AAc = sqrtf(1.4f * f32_rn(slot(b, S_PP)[c]) * rden);
    const float RmiuL = mu_suth<float>(pf, f32_rn(slot(b, S_T)[c]));
    const float RmiuTL = f32_rn(slot(b, S_RMIU)[c]);
    const float uvmu = (RmiuL + RmiuTL + 1.0e-20f) * (4.0f / 3.0f);
    const float uvmupr = (RmiuL * (1.0f / 0.72f) + RmiuTL * (1.0f / 0.9f) + 1.0e-20f) * 1.4f;
    const float vol = fslot(b, S_VOL)[c];
    float A[9];                                      // all loads before the first store
#pragma unroll
    for (int q = 0; q < 9; ++q) A[q] = fslot(b, S_ASD + q)[c];
    const float visc = 2.0f * fmaxf(uvmu, uvmupr) * rden / (vol * pf.Ref);
    float rs = 0.0f;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const float ARX = A[3 * d], ARY = A[3 * d + 1], ARZ = A[3 * d + 2];
        const float STsq = ARX * ARX + ARY * ARY + ARZ * ARZ;
        const float UU = Vxi * ARX + Vyi * ARY + Vzi * ARZ;
        const float Rd = fabsf(UU) + sqrtf(STsq) * AAc + STsq * visc;
        slot(b, S_RDS + d)[c] = f64_of(Rd);
        rs += Rd;
    }
    const float Dtm_local = vol / rs;
    const Params& p = cd.p;
    double dtm = p.IF_Local_Main == 1 ? f64_of(pf.CFL_Main * Dtm_local) : p.DT_LUSGS_Main;
    if (p.Kind_Dual != 0) dtm = p.IF_Local_Sub == 1 ? f64_of(f32_rn(cd.CFL_sub) * Dtm_local) : p.DT_LUSGS_Sub;
    slot(b, S_DTM)[c] = dtm;
}

// ---------------------------------------------------------------------------------------
// Mixed path: the FP32 copies the FP32 kernels read, in one pass over every padded cell: the
// state V(7), p, T, mu_t, the spectral radii and time step, and the primitives u, v, w,
// k/rho, omega/rho, 1/rho and the LU-SGS velocities from one FP32 reciprocal of rho (the FP64
// path's k_prims divides per component and keeps FP64 primitives, which nothing in the mixed
// path reads).  The conversions run on the integer pipe (cvt.cuh).
// ---------------------------------------------------------------------------------------
__global__ void k_prims_mixed(const DevBlock* __restrict__ blks, int nblk, long long total, const long long* __restrict__ off) {
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total) return;
    int lo = 0, hi = nblk - 1;
    while (lo < hi) { int mid = (lo + hi + 1) >> 1; if (off[mid] <= g) lo = mid; else hi = mid - 1; }
    const DevBlock b = blks[lo];
    const int c = (int)(g - off[lo]);
    // every load before the first store (the FP32 copies could alias the FP64 slots as far as
    // the compiler knows, and a load after a store would wait for the previous round trip)
    double x[14];
#pragma unroll
    for (int L = 0; L < 7; ++L) x[L] = slot(b, S_V + L)[c];
#pragma unroll
    for (int q = 0; q < 3; ++q) x[7 + q] = slot(b, S_PP + q)[c];
#pragma unroll
    for (int q = 0; q < 4; ++q) x[10 + q] = slot(b, S_RDS + q)[c];
    float v[7];
#pragma unroll
    for (int L = 0; L < 7; ++L) {
        v[L] = f32_rn(x[L]);
        fslot(b, S_V + L)[c] = v[L];
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) fslot(b, S_PP + q)[c] = f32_rn(x[7 + q]);
#pragma unroll
    for (int q = 0; q < 4; ++q) fslot(b, S_RDS + q)[c] = f32_rn(x[10 + q]);
    const float ri = 1.0f / v[0];
    const float u = v[1] * ri, vv = v[2] * ri, w = v[3] * ri;
    fslot(b, S_PRIM)[c] = u;
    fslot(b, S_PRIM + 1)[c] = vv;
    fslot(b, S_PRIM + 2)[c] = w;
    fslot(b, S_PRIM + 3)[c] = v[5] * ri;
    fslot(b, S_PRIM + 4)[c] = v[6] * ri;
    fslot(b, S_RINV)[c] = ri;
    fslot(b, S_SVEL)[c] = u;
    fslot(b, S_SVEL + 1)[c] = vv;
    fslot(b, S_SVEL + 2)[c] = w;
}

// ---------------------------------------------------------------------------------------
// BC/BC_Outlet.F90:37-107, mixed path: one warp per outlet line.  The radial-equilibrium
// recurrence along j,
//     p_j = p_{j-1} + |dr_j * rho_{j-1} * (w_{j-1} cos - sin v_{j-1} + omega r)^2| / (r_j + tiny),
//     rho_j = p_j * RXM2 / T_j,
// has coefficients that depend only on interior values (the previous j's velocities enter as
// V(3:4)/V(1) of its interior cell, equal to the ghost's rho*v / rho), so the lanes load and
// prepare 32 entries at a time in parallel and only the multiply-add chain runs lane by lane
// (through shuffles); the ghost writes are again parallel.
// ---------------------------------------------------------------------------------------
__global__ void k_bc_outlet_mixed(const DevBlock* __restrict__ blks, const BCEntry* __restrict__ ent,
                                  const OutletLine* __restrict__ lines, int nl, const CaseDev* __restrict__ cdev) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= nl) return;                                   // whole warps leave together
    const OutletLine Ln = lines[w];
    const DevBlock b = blks[Ln.blk];
    const Params& p = cdev[b.cs].p;
    const int turb = cdev[b.cs].turb;
    double* V0 = slot(b, S_V);
    double* PP = slot(b, S_PP);
    double* T = slot(b, S_T);
    double* Rm = slot(b, S_RMIU);
    const double* rad = slot(b, S_RAD);
    const double* sint = slot(b, S_SINT);
    const double* cost = slot(b, S_COST);
    double pp_carry = 0.0, den_carry = 1.0, vy_carry = 0.0, vz_carry = 0.0;
    for (int j0 = 0; j0 < Ln.n; j0 += 32) {
        const int e = Ln.first + j0 + lane;
        const bool act = j0 + lane < Ln.n;
        BCEntry E;
        double Tl = 1.0, rv1 = 0.0, vy = 0.0, vz = 0.0, a = 0.0, k1 = 0.0;
        bool first = false;
        if (act) {
            E = ent[e];
            Tl = T[E.s[0]];
            rv1 = 1.0 / V0[E.s[0]];
            vy = slot(b, S_V + 2)[E.s[0]] * rv1;
            vz = slot(b, S_V + 3)[E.s[0]] * rv1;
            k1 = p.RXM2 / Tl;
            first = E.sub == 1;
        }
        // velocities of the previous entry (lane - 1, or the previous chunk's last)
        double vy_p = __shfl_up_sync(0xffffffffu, vy, 1), vz_p = __shfl_up_sync(0xffffffffu, vz, 1);
        if (lane == 0) { vy_p = vy_carry; vz_p = vz_carry; }
        if (act && !first) {
            const int lm = E.l[0] - b.PI;              // (il, jl-1, kl)
            const double rcs1 = rad[E.l[0]], rcs2 = rad[lm];
            const double RoVr2 = sq(vz_p * cost[lm] - sint[lm] * vy_p + p.omega0 * rcs2);
            a = fabs((rcs1 - rcs2) * RoVr2) * (1.0 / (rcs2 + p.Tiny));
        }
        // the chain, lane by lane
        double pp = 0.0, den = 0.0, pp_c = pp_carry, den_c = den_carry;
        for (int i = 0; i < 32; ++i) {
            const double ai = __shfl_sync(0xffffffffu, a, i), ki = __shfl_sync(0xffffffffu, k1, i);
            const int fi = __shfl_sync(0xffffffffu, first ? 1 : 0, i);
            const double ppi = fi ? p.Pouthub : pp_c + ai * den_c;
            const double deni = ppi * ki;
            if (lane == i) { pp = ppi; den = deni; }
            if (j0 + i < Ln.n) { pp_c = ppi; den_c = deni; }
        }
        pp_carry = pp_c; den_carry = den_c;
        vy_carry = __shfl_sync(0xffffffffu, vy, 31);
        vz_carry = __shfl_sync(0xffffffffu, vz, 31);
        if (Ln.n - j0 < 32) {                          // a partial chunk: its last entry's values
            const int last = Ln.n - j0 - 1;
            vy_carry = __shfl_sync(0xffffffffu, vy, last);
            vz_carry = __shfl_sync(0xffffffffu, vz, last);
        }
        if (!act) continue;
        const int s0 = E.s[0];
        const double den_ratio = den * rv1;
        const double v2 = slot(b, S_V + 1)[s0] * den_ratio, v3 = slot(b, S_V + 2)[s0] * den_ratio;
        const double v4 = slot(b, S_V + 3)[s0] * den_ratio;
        for (int L = 0; L < 3; ++L) {
            const int ig = E.l[L];
            V0[ig] = den; slot(b, S_V + 1)[ig] = v2; slot(b, S_V + 2)[ig] = v3; slot(b, S_V + 3)[ig] = v4;
            PP[ig] = pp;
            T[ig] = Tl;
        }
        if (turb) {
            const double k6 = slot(b, S_V + 5)[s0], k7 = slot(b, S_V + 6)[s0], rm = Rm[s0];
            for (int L = 0; L < 3; ++L) {
                const int ig = E.l[L];
                slot(b, S_V + 5)[ig] = k6; slot(b, S_V + 6)[ig] = k7; Rm[ig] = rm;
            }
        }
    }
}

// p + p*expm1(dp/(p+1e-10)) for dp < 0, p + dp otherwise (Time/TIME_Update_V.F90:660-675)
__device__ inline double positive_add(double p, float dp) {
    if (dp >= 0.0f) return p + f64_of(dp);
    const float x = dp / (f32_rn(p) + 1.0e-10f);
    return p + p * f64_of(expm1f(x));
}

// Residual-norm partials of one thread in FP32 (the terms |D/V| come from FP32 increments),
// joined as NormPart's (the later cell kept on ties of the maximum); a warp reduces them by
// shuffles in FP32, warp 0 then the CTA's warps the same way, and the CTA's result goes out as
// a NormPart (FP64), which k_block_norms sums over the tiles of a block in FP64.
struct NormPartF {
    float sa, ma, sk, mk, so, mo;
    int ia, nan;
};
__device__ inline void normf_join(NormPartF& a, const NormPartF& b) {
    a.sa += b.sa; a.sk += b.sk; a.so += b.so;
    if (b.ma > a.ma || (b.ma == a.ma && b.ia > a.ia)) { a.ma = b.ma; a.ia = b.ia; }
    a.mk = fmaxf(a.mk, b.mk); a.mo = fmaxf(a.mo, b.mo);
    a.nan |= b.nan;
}
__device__ inline NormPartF normf_reduce_warp(NormPartF a) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    for (int w = 16; w > 0; w >>= 1) {
        NormPartF o;
        o.sa = __shfl_down_sync(full, a.sa, w); o.ma = __shfl_down_sync(full, a.ma, w);
        o.sk = __shfl_down_sync(full, a.sk, w); o.mk = __shfl_down_sync(full, a.mk, w);
        o.so = __shfl_down_sync(full, a.so, w); o.mo = __shfl_down_sync(full, a.mo, w);
        o.ia = __shfl_down_sync(full, a.ia, w); o.nan = __shfl_down_sync(full, a.nan, w);
        if (lane + w < 32) normf_join(a, o);
    }
    return a;
}
// the CTA's reduction, valid in thread 0 (blockDim a multiple of 32); every thread calls it
__device__ inline NormPart norm_reduce_cta_f(NormPartF a) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    a = normf_reduce_warp(a);
    __shared__ NormPartF s_warp[32];
    if (lane == 0) s_warp[wid] = a;
    __syncthreads();
    NormPart r = norm_identity();
    if (wid == 0) {
        NormPartF e;
        e.sa = 0.0f; e.ma = -1.0f; e.sk = 0.0f; e.mk = 0.0f; e.so = 0.0f; e.mo = 0.0f; e.ia = -1; e.nan = 0;
        const NormPartF b = normf_reduce_warp(lane < (int)(blockDim.x >> 5) ? s_warp[lane] : e);
        r.sa = f64_of(b.sa); r.ma = f64_of(b.ma); r.sk = f64_of(b.sk); r.mk = f64_of(b.mk);
        r.so = f64_of(b.so); r.mo = f64_of(b.mo); r.ia = b.ia; r.nan = b.nan; r.pad_ = 0;
    }
    return r;
}

// ---------------------------------------------------------------------------------------
// Time/TIME_Update_V.F90:106-294 (norms) and :621-816 (update), mixed path.  DeltaQ and the
// gradients come from the FP32 copies; the increments are FP32, the state they are added to
// FP64.
// ---------------------------------------------------------------------------------------
__global__ void k_update_mixed(const DevBlock* __restrict__ blks, const Tile* __restrict__ tiles,
                               const CaseDev* __restrict__ cdev, NormPart* __restrict__ parts) {
    const Tile t = tiles[blockIdx.x];
    const DevBlock b = blks[t.blk];
    const CaseDev& cd = cdev[b.cs];
    const int turb_upd = cd.turb_upd;
    const int tid = threadIdx.x;
    NormPartF P;
    P.sa = 0.0f; P.ma = -1.0f; P.sk = 0.0f; P.mk = 0.0f; P.so = 0.0f; P.mo = 0.0f; P.ia = -1; P.nan = 0;
    if (tid < t.count) {
        const int n = t.start + tid;
        const int I = n % b.NI1 + 1, J = (n / b.NI1) % b.NJ1 + 1, K = n / (b.NI1 * b.NJ1) + 1;
        const int c = cidx(b, I, J, K);
        double* V0 = slot(b, S_V);
        double* V1 = slot(b, S_V + 1);
        double* V2 = slot(b, S_V + 2);
        double* V3 = slot(b, S_V + 3);
        double* V4 = slot(b, S_V + 4);
        auto Dq = [&](int L) { return fslot(b, S_D + L)[c]; };
        const float AinRo = Dq(0), AinRx = Dq(1), AinRy = Dq(2), AinRz = Dq(3), AinRe = Dq(4);
        const float d6 = Dq(5), d7 = Dq(6);
        double* PP = slot(b, S_PP);
        const double rho0 = V0[c], m1 = V1[c], m2 = V2[c], m3 = V3[c], p0 = PP[c];
        const float radc = fslot(b, S_RAD)[c];
        const float rof = f32_rn(rho0), roinv = 1.0f / rof;
        const float m1f = f32_rn(m1), m2f = f32_rn(m2), m3f = f32_rn(m3);
        P.nan = isnan(AinRo) ? 1 : 0;
        const float DR = fabsf(AinRo) * roinv, DRk = fabsf(d6) * roinv, DRo = fabsf(d7) * roinv;
        P.sa = DR * DR; P.ma = DR; P.ia = n;
        P.sk = DRk * DRk; P.mk = DRk; P.so = DRo * DRo; P.mo = DRo;
        const float pVx = m1f * roinv, pVy = m2f * roinv, pVz = m3f * roinv;
        const float AinX = (AinRx - pVx * AinRo) * roinv;
        const float AinY = (AinRy - pVy * AinRo) * roinv;
        const float AinZ = (AinRz - pVz * AinRo) * roinv;
        const float AinP = (1.4f - 1.0f) * (AinRe - 0.5f * AinRo * (pVx * pVx + pVy * pVy + pVz * pVz)
                                            - rof * (AinX * pVx + AinY * pVy + AinZ * pVz));
        // density rho' = |rho exp(dRo/rho)| (rho + dRo for dRo >= 0); r = rho'/rho - 1
        float r;
        double rho;
        if (AinRo >= 0.0f) {
            r = AinRo * roinv;
            rho = rho0 + f64_of(AinRo);
        } else {
            r = expm1f(AinRo / (rof + 1.0e-10f));
            rho = rho0 + rho0 * f64_of(r);
        }
        rho = fabs(rho);
        const float rhof = f32_rn(rho);
        // momentum rho'(m/rho + a) = m + (m r + rho' a)
        V1[c] = m1 + f64_of(m1f * r + rhof * AinX);
        V2[c] = m2 + f64_of(m2f * r + rhof * AinY);
        V3[c] = m3 + f64_of(m3f * r + rhof * AinZ);
        V0[c] = rho;
        const double pp = fabs(positive_add(p0, AinP));
        PP[c] = pp;
        const float Tf = cd.pf.RXM2 * f32_rn(pp) / rhof;
        slot(b, S_T)[c] = f64_of(Tf);
        const float ux = pVx + AinX, uy = pVy + AinY, uz = pVz + AinZ;
        const float rr = cd.pf.omega0 * radc;
        V4[c] = pp * (1.0 / (1.4 - 1.0)) + f64_of((0.5f * (ux * ux + uy * uy + uz * uz) - 0.5f * rr * rr) * rhof);
        if (turb_upd) {   // TIME_Update_V.F90:709-816
            // the SST inputs as one batch of loads after the mean-flow stores (hoisting them
            // above those too raised the kernel from 56 to 70 registers and measured slower)
            double* V5 = slot(b, S_V + 5);
            double* V6 = slot(b, S_V + 6);
            double ARTk = dmax(positive_add(V5[c], d6), 1.0e-10);
            double ARTO = dmax(positive_add(V6[c], d7), 1.0e-10);
            const ParamsT<float>& p = cd.pf;
            const float ro = rhof, kf = f32_rn(ARTk);
            float of = f32_rn(ARTO);
            const float RmiuL = mu_suth<float>(p, Tf);
            const float DistN = fslot(b, S_DST)[c];
            float Gq[9];
#pragma unroll
            for (int q = 0; q < 9; ++q) Gq[q] = fslot(b, S_DQ + q)[c];
            const float Dudx = Gq[0], Dudy = Gq[1], Dudz = Gq[2], Dvdx = Gq[3], Dvdy = Gq[4], Dvdz = Gq[5];
            const float Dwdx = Gq[6], Dwdy = Gq[7], Dwdz = Gq[8];
            const float Div = Dudx + Dvdy + Dwdz;
            const float prod = 2.0f * (Dudx * Dudx + Dvdy * Dvdy + Dwdz * Dwdz) + sq(Dudy + Dvdx) + sq(Dvdz + Dwdy)
                               + sq(Dwdx + Dudz) - (2.0f / 3.0f) * Div * Div;
            const float Ref = p.Ref, Bs = p.Beta_star;
            if (p.Kind_Model == 2) {    // Wilcox 2006 (TIME_Update_V.F90:821-858), in FP32
                const float t3 = Div / 3.0f;
                const float Sii = Dudx - t3, Sjj = Dvdy - t3, Skk = Dwdz - t3;
                const float Sij = 0.5f * (Dudy + Dvdx), Sik = 0.5f * (Dudz + Dwdx), Sjk = 0.5f * (Dvdz + Dwdy);
                const float Skl = sqrtf(Sii * Sii + Sjj * Sjj + Skk * Skk + 2.0f * (Sij * Sij + Sik * Sik + Sjk * Sjk));
                of = fmaxf(of, sqrtf(ro * fabsf(prod) / (p.Prod_Lmt * Bs)) / Ref);
                const float kl = fminf(kf, 100000.0f * RmiuL * of / ro);
                ARTO = of == f32_rn(ARTO) ? ARTO : f64_of(of);
                ARTk = kl == kf ? ARTk : f64_of(kl);
                V5[c] = ARTk;
                V6[c] = ARTO;
                const float om = fmaxf(of, 0.875f * ro * sqrtf(Skl * Skl * (2.0f / 0.09f)) / Ref);
                slot(b, S_RMIU)[c] = f64_of(kl / om * ro);
            } else {
            float arg2 = 2.0f * sqrtf(kf / ro) / Bs / (of / ro) / DistN / Ref;
            arg2 = fmaxf(arg2, 500.0f * RmiuL / DistN / DistN / of / Ref / Ref);
            arg2 = tanhf(arg2 * arg2);
            const float Sij = 0.5f * (Dudy + Dvdx), Sik = 0.5f * (Dudz + Dwdx), Sjk = 0.5f * (Dvdz + Dwdy);
            const float Skl = sqrtf(2.0f * (Dudx * Dudx + Dvdy * Dvdy + Dwdz * Dwdz + 2.0f * (Sij * Sij + Sik * Sik + Sjk * Sjk)));
            const float Cmua = fminf(1.0f, p.A1 * of / ro / (Skl * arg2 + 1.e-10f) * Ref);
            of = fmaxf(of, sqrtf(ro * Cmua * fabsf(prod) / (p.Prod_Lmt * Bs)) / Ref);
            const float kl = fminf(kf, 100000.0f * RmiuL * of / ro / Cmua);
            ARTO = of == f32_rn(ARTO) ? ARTO : f64_of(of);
            ARTk = kl == kf ? ARTk : f64_of(kl);
            V5[c] = ARTk;
            V6[c] = ARTO;
            slot(b, S_RMIU)[c] = f64_of(Cmua * kl / of * ro);
            }
        }
    }
    const NormPart R = norm_reduce_cta_f(P);
    if (tid == 0) parts[blockIdx.x] = R;
}

// ---------------------------------------------------------------------------------------
// Both LU-SGS sweeps of the mixed path with one thread-block cluster per solver block
// (Time/TIME_LUSGS.F90:73-215 order): the cluster's CTAs take the block's positions of
// hyperplane h, then meet at a cluster barrier (arrive.release / wait.acquire) before h+1; the
// lower sweep ascends, the upper descends.  The sweeps stop at block faces, so clusters never
// wait on one another and need no co-residency beyond their own CTAs, which the hardware
// schedules together; a cluster barrier is a hardware barrier every thread reaches, not a spin.
// Every position runs sweep_pos_compact, as in the other schedules (bit-identical results);
// DeltaQ written by other SMs of the cluster is read through L2.  pb_off[h*(nblk+1) + b] is the
// first sweep position of block b in hyperplane h; pf > 0 prefetches the block's records of
// hyperplane h +- pf into L2 while h is swept.
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ void cluster_barrier() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ unsigned cluster_reg(int which) {
    unsigned r;
    if (which == 0) asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    else if (which == 1) asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    else asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
    return r;
}

__global__ void k_sweep_cluster(const int* __restrict__ nbp, const float* __restrict__ rec, float* dq,
                                const int* __restrict__ pb_off, int nh, int nblk, int turb, int pf) {
    const int rank = (int)cluster_reg(0), ncta = (int)cluster_reg(1), b = (int)cluster_reg(2);
    const int nt = ncta * blockDim.x, t = rank * blockDim.x + threadIdx.x;
    auto first = [&](int h) { return pb_off[(size_t)h * (nblk + 1) + b]; };
    auto last = [&](int h) { return pb_off[(size_t)h * (nblk + 1) + b + 1]; };
    auto prefetch = [&](int h) {
        if (pf > 0 && h >= 0 && h < nh && last(h) > first(h))
            prefetch_l2_range(rec + sw_at(first(h), 0, NCREC), (size_t)(last(h) - first(h)) * NCREC * sizeof(float), t, nt);
    };
    for (int h = 0; h < nh; ++h) {
        const int p0 = first(h), p1 = last(h);
        if (p0 == p1) continue;             // the same for every thread of the cluster
        prefetch(h + pf);
        for (int q = p0 + t; q < p1; q += nt) sweep_pos_compact<true>(nbp, rec, dq, q, turb, false);
        cluster_barrier();
    }
    for (int h = nh - 1; h >= 0; --h) {
        const int p0 = first(h), p1 = last(h);
        if (p0 == p1) continue;
        prefetch(h - pf);
        for (int q = p0 + t; q < p1; q += nt) sweep_pos_compact<false>(nbp, rec, dq, q, turb, false);
        cluster_barrier();
    }
}

}  // namespace tg
