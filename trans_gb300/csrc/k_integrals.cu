// k_integrals.cu -- integrated quantities of a solution on the device: mass flow and mass-averaged
// total and static pressure through every inlet (kind 5) and outlet (kind 7) face, pressure and
// viscous force on every wall (kind 1) face, and the wall pressure coefficient of one segment.
//
// The per-face expressions restate the reference's output routines:
//   mass flux   Output/OUTPUT_Residual_NS.F90:37-75: face momentum = volume-weighted average of
//               the two cells with the weights crossed, dotted with SD of the face (the reference
//               evaluates one i-plane of one block; here every face of every kind-5/7 segment)
//   p0          Output/Average_Field.F90:66,157: p (1 + 0.2 M^2)^3.5 (not divided by PPF here),
//               from the face-averaged state, mass averaged over the faces
//   force       Output/OUTPUT_ClCdCm.F90:114-264: pressure part (PP - PPF) S Sgn with Sgn = -1 on
//               a min face, +1 on a max face; viscous part tau (u S - (u.S) S/|S|), tau =
//               mu_w/(Dst Ref) with Sutherland mu_w, no Sgn (the reference comments it out);
//               summed before the 2/Area_Ref scaling
//   Cp          Output/OUTPUT_Surfaces.F90:303-305: 2 (PP - PPF) at the wall cell
// Sums are taken in a fixed order (each thread a fixed stride of the case's faces, then a fixed
// tree), so the result does not depend on scheduling: the same state gives the same bits.
#include "launch.h"
#include "types.cuh"

namespace tg {

namespace {

constexpr int INTG_THREADS = 256;

__device__ void face_terms(const DevBlock* __restrict__ blks, const BCEntry& E, const CaseDev& cd, double* q) {
    const DevBlock& b = blks[E.blk];
    const int d = E.dir - 1;
    const int pt = d == 0 ? E.i : (d == 1 ? E.j : E.k);
    const bool is_min = pt == 1;
    const int ci = E.s[0];                       // interior cell on the face
    const int cg = E.l[0];                       // first ghost cell
    const int cf = cidx(b, E.i, E.j, E.k);       // face index of SD and Grad
    const double* V = slot(b, S_V);
    const size_t nc = (size_t)b.ncell;
    const double* PP = slot(b, S_PP);
    const double S0 = slot(b, S_SD + 3 * d)[cf], S1 = slot(b, S_SD + 3 * d + 1)[cf], S2 = slot(b, S_SD + 3 * d + 2)[cf];
    if (E.kind == 5 || E.kind == 7) {
        const double* vol = slot(b, S_VOL);
        const double w1 = vol[cg], w2 = vol[ci];
        const double ws = w1 + w2;
        const double rho = (w1 * V[ci] + w2 * V[cg]) / ws;
        const double ru = (w1 * V[nc + ci] + w2 * V[nc + cg]) / ws;
        const double rv = (w1 * V[2 * nc + ci] + w2 * V[2 * nc + cg]) / ws;
        const double rw = (w1 * V[3 * nc + ci] + w2 * V[3 * nc + cg]) / ws;
        const double p = (w1 * PP[ci] + w2 * PP[cg]) / ws;
        const double flux = ru * S0 + rv * S1 + rw * S2;          // along +IJKDirect
        const bool into = (E.kind == 5) == is_min;               // inflow at a min face, outflow at a max face
        const double mf = into ? flux : -flux;
        const double u2 = (ru * ru + rv * rv + rw * rw) / (rho * rho);
        const double M2 = u2 / (1.4 * p / rho);
        const double p0 = p * pow(1.0 + 0.5 * (1.4 - 1.0) * M2, 1.4 / (1.4 - 1.0));
        const int o = E.kind == 5 ? 0 : 3;
        q[o] = mf;
        q[o + 1] = mf * p0;
        q[o + 2] = mf * p;
    } else if (E.kind == 1) {
        const Params& P = cd.p;
        const double Sl = slot(b, S_GRAD + d)[cf];
        const double Sx = S0 / Sl, Sy = S1 / Sl, Sz = S2 / Sl;
        const double Sgn = is_min ? -1.0 : 1.0;
        const double P2 = PP[ci] - P.PPF;
        q[6] = P2 * Sx * Sl * Sgn;
        q[7] = P2 * Sy * Sl * Sgn;
        q[8] = P2 * Sz * Sl * Sgn;
        const double TT = slot(b, S_T)[ci];
        const double RmiuW = (1.0 + P.Csthlnd) / (TT * P.Csth1 + P.Csthlnd) * pow(P.Csth1 * TT, 1.5);
        const double Dn = slot(b, S_DST)[ci];
        const double Denw = V[ci];
        const double u = V[nc + ci] / Denw, v = V[2 * nc + ci] / Denw, w = V[3 * nc + ci] / Denw;
        const double Vcon = u * Sx * Sl + v * Sy * Sl + w * Sz * Sl;
        const double tau = 1.0 * RmiuW / Dn / P.Ref;
        q[9] = tau * (u * Sl - Vcon * Sx);
        q[10] = tau * (v * Sl - Vcon * Sy);
        q[11] = tau * (w * Sl - Vcon * Sz);
    }
}

// one CTA per case over the case's boundary faces [first[cs], first[cs+1])
__global__ void __launch_bounds__(INTG_THREADS)
k_integrals(const DevBlock* __restrict__ blks, const BCEntry* __restrict__ ent, const int* __restrict__ first,
            const CaseDev* __restrict__ cdev, double* __restrict__ out) {
    __shared__ double red[NINTG][INTG_THREADS];
    const int cs = blockIdx.x, t = threadIdx.x;
    double acc[NINTG];
    for (int m = 0; m < NINTG; ++m) acc[m] = 0.0;
    const CaseDev& cd = cdev[cs];
    for (int e = first[cs] + t; e < first[cs + 1]; e += INTG_THREADS) {
        const BCEntry E = ent[e];
        if (E.kind != 1 && E.kind != 5 && E.kind != 7) continue;
        double q[NINTG];
        for (int m = 0; m < NINTG; ++m) q[m] = 0.0;
        face_terms(blks, E, cd, q);
        for (int m = 0; m < NINTG; ++m) acc[m] += q[m];
    }
    for (int m = 0; m < NINTG; ++m) red[m][t] = acc[m];
    __syncthreads();
    for (int h = INTG_THREADS / 2; h > 0; h >>= 1) {
        if (t < h)
            for (int m = 0; m < NINTG; ++m) red[m][t] += red[m][t + h];
        __syncthreads();
    }
    if (t < NINTG) out[(size_t)cs * NINTG + t] = red[t][0];
}

// Cp = 2 (PP - PPF) at the wall cell of each face of one segment (entries [e0, e0+n) of the table)
__global__ void k_wall_cp(const DevBlock* __restrict__ blks, const BCEntry* __restrict__ ent, int e0, int n,
                          const CaseDev* __restrict__ cdev, double* __restrict__ cp) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const BCEntry& E = ent[e0 + r];
    const DevBlock& b = blks[E.blk];
    cp[r] = 2.0 * (slot(b, S_PP)[E.s[0]] - cdev[b.cs].p.PPF);
}

// pressure and viscous force of each face of one segment: f[6r .. 6r+5] = (pressure x, y, z,
// viscous x, y, z) of face r, the terms k_integrals sums
__global__ void k_wall_forces(const DevBlock* __restrict__ blks, const BCEntry* __restrict__ ent, int e0, int n,
                              const CaseDev* __restrict__ cdev, double* __restrict__ f) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const BCEntry E = ent[e0 + r];
    double q[NINTG];
    for (int m = 0; m < NINTG; ++m) q[m] = 0.0;
    face_terms(blks, E, cdev[blks[E.blk].cs], q);
    for (int m = 0; m < 6; ++m) f[(size_t)6 * r + m] = q[6 + m];
}

}  // namespace

void launch_wall_forces(cudaStream_t s, const DevBlock* blks, const BCEntry* ent, int e0, int n, const CaseDev* cdev,
                        double* f) {
    if (n > 0) k_wall_forces<<<(n + 127) / 128, 128, 0, s>>>(blks, ent, e0, n, cdev, f);
}

void launch_integrals(cudaStream_t s, const DevBlock* blks, const BCEntry* ent, const int* first, int ncase,
                      const CaseDev* cdev, double* out) {
    if (ncase > 0) k_integrals<<<ncase, INTG_THREADS, 0, s>>>(blks, ent, first, cdev, out);
}

void launch_wall_cp(cudaStream_t s, const DevBlock* blks, const BCEntry* ent, int e0, int n, const CaseDev* cdev,
                    double* cp) {
    if (n > 0) k_wall_cp<<<(n + 127) / 128, 128, 0, s>>>(blks, ent, e0, n, cdev, cp);
}

}  // namespace tg
