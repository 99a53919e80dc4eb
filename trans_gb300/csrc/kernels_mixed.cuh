// kernels_mixed.cuh -- the FP64-state kernels of the mixed-precision path in a reduced-operation
// form (included by k_mixed.cu only).
//
// On GB300 every FP64 instruction issues at 1/64 of the FP32 rate, and a double division or
// square root is ~10 of them.  The FP64 path evaluates Time/SpectralRadius.F90 and
// Time/TIME_Update_V.F90 operation by operation (bit-identical to the reference's arithmetic);
// these mixed-path versions keep the same quantities in FP64 -- the conserved-variable update,
// the local time step and the residual norms -- but
//   - divide once per cell (a reciprocal) where the reference divides by the same value
//     several times,
//   - evaluate the increments of the positivity-preserving update, p*exp(dp/p) = p + p*expm1(dp/p),
//     as an FP32 expm1 added to the FP64 value (the FP32 error scales with the increment, so it
//     vanishes as the iteration converges),
//   - evaluate the SST model algebra of the update (the F2-limited C_mu and the realizability
//     limits of omega and k) and the spectral radii's square roots and Sutherland law in FP32,
//     like the other SST and sweep arithmetic of the mixed path.
#pragma once

namespace tg {

// ---------------------------------------------------------------------------------------
// Time/SpectralRadius.F90:47-180, mixed path: spectral radii with FP32 square roots and
// Sutherland law, accumulated in FP64; the local time step divides in FP64.
// ---------------------------------------------------------------------------------------
__global__ void k_specrad_mixed(const DevBlock* __restrict__ blks, const Tile* __restrict__ tiles,
                                const CaseDev* __restrict__ cdev) {
    const Tile t = tiles[blockIdx.x];
    if ((int)threadIdx.x >= t.count) return;
    const DevBlock b = blks[t.blk];
    const CaseDev& cd = cdev[b.cs];
    const Params& p = cd.p;
    const double CFL_sub = cd.CFL_sub;
    const int n = t.start + threadIdx.x;
    const int I = n % b.NI1 + 1, J = (n / b.NI1) % b.NJ1 + 1, K = n / (b.NI1 * b.NJ1) + 1;
    const int c = cidx(b, I, J, K);
    const double Den = slot(b, S_V)[c];
    const double rden = 1.0 / Den;
    const double Vxi = slot(b, S_V + 1)[c] * rden, Vyi = slot(b, S_V + 2)[c] * rden, Vzi = slot(b, S_V + 3)[c] * rden;
    const double AAc = (double)sqrtf((float)(1.4 * slot(b, S_PP)[c] * rden));
    const double RmiuL = (double)mu_suth<float>(cd.pf, (float)slot(b, S_T)[c]);
    const double RmiuTL = slot(b, S_RMIU)[c];
    const double uvmu = (RmiuL + RmiuTL + 1.0e-20) * (4.0 / 3.0);
    const double uvmupr = (RmiuL * (1.0 / 0.72) + RmiuTL * (1.0 / 0.9) + 1.0e-20) * 1.4;
    const double vol = slot(b, S_VOL)[c];
    const double visc = 2.0 * dmax(uvmu, uvmupr) * rden / (vol * p.Ref);
    double rs = 0.0;
    for (int d = 0; d < 3; ++d) {
        const double ARX = slot(b, S_ASD + 3 * d)[c], ARY = slot(b, S_ASD + 3 * d + 1)[c], ARZ = slot(b, S_ASD + 3 * d + 2)[c];
        const double STsq = ARX * ARX + ARY * ARY + ARZ * ARZ;
        const double UU = Vxi * ARX + Vyi * ARY + Vzi * ARZ;
        const double Rd = fabs(UU) + (double)sqrtf((float)STsq) * AAc + STsq * visc;
        slot(b, S_RDS + d)[c] = Rd;
        rs += Rd;
    }
    const double Dtm_local = vol / rs;
    double dtm = p.IF_Local_Main == 1 ? p.CFL_Main * Dtm_local : p.DT_LUSGS_Main;
    if (p.Kind_Dual != 0) dtm = p.IF_Local_Sub == 1 ? CFL_sub * Dtm_local : p.DT_LUSGS_Sub;
    slot(b, S_DTM)[c] = dtm;
}

// ---------------------------------------------------------------------------------------
// Mixed path: the FP32 copies the FP32 kernels read, in one pass over every padded cell: the
// state V(7), p, T, mu_t, the spectral radii and time step, and the primitives u, v, w,
// k/rho, omega/rho, 1/rho and the LU-SGS velocities from one FP64 reciprocal of rho (the FP64
// path's k_prims divides per component and keeps FP64 primitives, which nothing in the mixed
// path reads).
// ---------------------------------------------------------------------------------------
__global__ void k_prims_mixed(const DevBlock* __restrict__ blks, int nblk, long long total, const long long* __restrict__ off) {
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total) return;
    int lo = 0, hi = nblk - 1;
    while (lo < hi) { int mid = (lo + hi + 1) >> 1; if (off[mid] <= g) lo = mid; else hi = mid - 1; }
    const DevBlock b = blks[lo];
    const int c = (int)(g - off[lo]);
    double v[7];
    for (int L = 0; L < 7; ++L) {
        v[L] = slot(b, S_V + L)[c];
        fslot(b, S_V + L)[c] = (float)v[L];
    }
    for (int q = S_PP; q <= S_RMIU; ++q) fslot(b, q)[c] = (float)slot(b, q)[c];
    for (int q = S_RDS; q <= S_DTM; ++q) fslot(b, q)[c] = (float)slot(b, q)[c];
    const double ri = 1.0 / v[0];
    const float u = (float)(v[1] * ri), vv = (float)(v[2] * ri), w = (float)(v[3] * ri);
    fslot(b, S_PRIM)[c] = u;
    fslot(b, S_PRIM + 1)[c] = vv;
    fslot(b, S_PRIM + 2)[c] = w;
    fslot(b, S_PRIM + 3)[c] = (float)(v[5] * ri);
    fslot(b, S_PRIM + 4)[c] = (float)(v[6] * ri);
    fslot(b, S_RINV)[c] = (float)ri;
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
__device__ inline double positive_add(double p, double dp) {
    if (dp >= 0.0) return p + dp;
    const float x = (float)dp / ((float)p + 1.0e-10f);
    return p + p * (double)expm1f(x);
}

// ---------------------------------------------------------------------------------------
// Time/TIME_Update_V.F90:106-294 (norms) and :621-816 (update), mixed path.  DeltaQ and the
// gradients come from the FP32 copies.
// ---------------------------------------------------------------------------------------
__global__ void k_update_mixed(const DevBlock* __restrict__ blks, const Tile* __restrict__ tiles,
                               const CaseDev* __restrict__ cdev, NormPart* __restrict__ parts) {
    const Tile t = tiles[blockIdx.x];
    const DevBlock b = blks[t.blk];
    const CaseDev& cd = cdev[b.cs];
    const int turb_upd = cd.turb_upd;
    const int tid = threadIdx.x;
    double sa = 0, ma = -1, sk = 0, mk = 0, so = 0, mo = 0;
    long long ia = -1;
    int nanf = 0;
    if (tid < t.count) {
        const int n = t.start + tid;
        const int I = n % b.NI1 + 1, J = (n / b.NI1) % b.NJ1 + 1, K = n / (b.NI1 * b.NJ1) + 1;
        const int c = cidx(b, I, J, K);
        double* V0 = slot(b, S_V);
        double* V1 = slot(b, S_V + 1);
        double* V2 = slot(b, S_V + 2);
        double* V3 = slot(b, S_V + 3);
        double* V4 = slot(b, S_V + 4);
        auto Dq = [&](int L) { return (double)fslot(b, S_D + L)[c]; };
        const double AinRo = Dq(0), AinRx = Dq(1), AinRy = Dq(2), AinRz = Dq(3), AinRe = Dq(4);
        const double d6 = Dq(5), d7 = Dq(6);
        double pRo = V0[c];
        const double roinv = 1.0 / pRo;
        nanf = isnan(AinRo) ? 1 : 0;
        const double DR = fabs(AinRo) * roinv, DRk = fabs(d6) * roinv, DRo = fabs(d7) * roinv;
        sa = DR * DR; ma = DR; ia = n;
        sk = DRk * DRk; mk = DRk; so = DRo * DRo; mo = DRo;
        double pVx = V1[c] * roinv, pVy = V2[c] * roinv, pVz = V3[c] * roinv;
        const double AinX = (AinRx - pVx * AinRo) * roinv;
        const double AinY = (AinRy - pVy * AinRo) * roinv;
        const double AinZ = (AinRz - pVz * AinRo) * roinv;
        const double AinP = (1.4 - 1.0) * (AinRe - 0.5 * AinRo * (pVx * pVx + pVy * pVy + pVz * pVz)
                                           - pRo * (AinX * pVx + AinY * pVy + AinZ * pVz));
        pRo = fabs(positive_add(pRo, AinRo));
        double* PP = slot(b, S_PP);
        const double pp = fabs(positive_add(PP[c], AinP));
        PP[c] = pp;
        const double T = cd.p.RXM2 * pp / pRo;
        slot(b, S_T)[c] = T;
        pVx += AinX; pVy += AinY; pVz += AinZ;
        V0[c] = pRo;
        V1[c] = pRo * pVx;
        V2[c] = pRo * pVy;
        V3[c] = pRo * pVz;
        const double rr = cd.p.omega0 * slot(b, S_RAD)[c];
        V4[c] = pp * (1.0 / (1.4 - 1.0)) + (0.5 * (pVx * pVx + pVy * pVy + pVz * pVz) - 0.5 * rr * rr) * pRo;
        if (turb_upd) {   // TIME_Update_V.F90:709-816
            double* V5 = slot(b, S_V + 5);
            double* V6 = slot(b, S_V + 6);
            double ARTk = dmax(positive_add(V5[c], d6), 1.0e-10);
            double ARTO = dmax(positive_add(V6[c], d7), 1.0e-10);
            const ParamsT<float>& p = cd.pf;
            const float ro = (float)pRo, kf = (float)ARTk;
            float of = (float)ARTO;
            const float RmiuL = mu_suth<float>(p, (float)T);
            const float DistN = fslot(b, S_DST)[c];
            auto G = [&](int q) { return fslot(b, S_DQ + q)[c]; };
            const float Dudx = G(0), Dudy = G(1), Dudz = G(2), Dvdx = G(3), Dvdy = G(4), Dvdz = G(5);
            const float Dwdx = G(6), Dwdy = G(7), Dwdz = G(8);
            const float Div = Dudx + Dvdy + Dwdz;
            const float prod = 2.0f * (Dudx * Dudx + Dvdy * Dvdy + Dwdz * Dwdz) + sq(Dudy + Dvdx) + sq(Dvdz + Dwdy)
                               + sq(Dwdx + Dudz) - (2.0f / 3.0f) * Div * Div;
            const float Ref = p.Ref, Bs = p.Beta_star;
            if (p.Kind_Model == 2) {    // Wilcox 2006 (TIME_Update_V.F90:821-858), in FP32
                const float t3 = Div / 3.0f;
                const float Sii = Dudx - t3, Sjj = Dvdy - t3, Skk = Dwdz - t3;
                const float Sij = 0.5f * (Dudy + Dvdx), Sik = 0.5f * (Dudz + Dwdx), Sjk = 0.5f * (Dvdz + Dwdy);
                const float Skl = sqrtf(Sii * Sii + Sjj * Sjj + Skk * Skk + 2.0f * (Sij * Sij + Sik * Sik + Sjk * Sjk));
                ARTO = dmax(ARTO, (double)(sqrtf(ro * fabsf(prod) / (p.Prod_Lmt * Bs)) / Ref));
                of = (float)ARTO;
                ARTk = dmin(ARTk, (double)(100000.0f * RmiuL * of / ro));
                V5[c] = ARTk;
                V6[c] = ARTO;
                const float om = fmaxf(of, 0.875f * ro * sqrtf(Skl * Skl * (2.0f / 0.09f)) / Ref);
                slot(b, S_RMIU)[c] = (double)((float)ARTk / om * ro);
            } else {
            float arg2 = 2.0f * sqrtf(kf / ro) / Bs / (of / ro) / DistN / Ref;
            arg2 = fmaxf(arg2, 500.0f * RmiuL / DistN / DistN / of / Ref / Ref);
            arg2 = tanhf(arg2 * arg2);
            const float Sij = 0.5f * (Dudy + Dvdx), Sik = 0.5f * (Dudz + Dwdx), Sjk = 0.5f * (Dvdz + Dwdy);
            const float Skl = sqrtf(2.0f * (Dudx * Dudx + Dvdy * Dvdy + Dwdz * Dwdz + 2.0f * (Sij * Sij + Sik * Sik + Sjk * Sjk)));
            const float Cmua = fminf(1.0f, p.A1 * of / ro / (Skl * arg2 + 1.e-10f) * Ref);
            ARTO = dmax(ARTO, (double)(sqrtf(ro * Cmua * fabsf(prod) / (p.Prod_Lmt * Bs)) / Ref));
            of = (float)ARTO;
            ARTk = dmin(ARTk, (double)(100000.0f * RmiuL * of / ro / Cmua));
            V5[c] = ARTk;
            V6[c] = ARTO;
            slot(b, S_RMIU)[c] = (double)(Cmua * (float)ARTk / of * ro);
            }
        }
    }
    NormPart P;
    P.sa = sa; P.ma = ma; P.sk = sk; P.mk = mk; P.so = so; P.mo = mo; P.ia = ia; P.nan = nanf; P.pad_ = 0;
    P = norm_reduce_cta(P);
    if (tid == 0) parts[blockIdx.x] = P;
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
