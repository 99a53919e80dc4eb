// resid_tma.cuh -- the mixed path's residual from shared-memory tiles staged by the tensor
// memory access (TMA) unit: Space/ residual of main.F90:92-133 in FP32, one launch per face
// direction, each CTA a brick of cells with its halo along that direction.
//
// A CTA stages every slot its faces read -- the reconstruction stencil (cells -3..+2 along the
// direction) and the two-point fields (cells -1, 0) -- with one cp.async.bulk.tensor per slot
// into shared memory, waits on one mbarrier, computes each face's NFX fluxes with the shared
// physics (face_flux_body) reading shared memory, and adds the flux differences of its cells to
// D.  The FX slots and the gather pass of the FP64 path are not used: the per-direction sums go
// straight to D (direction 1 writes, 2 and 3 add), so the FP32 sum order is
//   D = (-Fv1 + Fv1' [+ rotating source] - Fc1 + Fc1') + (-Fv2 + ...) + (-Fv3 + ...).
//
// Tiles (array indices, i.e. Fortran index + 2; interior cells 3..N+1):
//   direction 1: 28 cells along i x 8 rows along j x 1 k; staged box 36 x 8 from x0-4 (29
//                faces per row, one warp per row; the neighbour face's flux comes from the
//                next lane by a warp shuffle);
//   directions 2, 3: 32 cells along i x 8 cells along the direction; staged boxes 32 x 14
//                (stencil, from y0-3) and 32 x 10 (two-point fields, from y0-1); 9 faces per
//                column, one thread per face, the fluxes exchanged through shared memory.
// Two CTAs are resident per SM (registers and shared memory); 4-cell bricks with four CTAs
// measured slower (more halo faces, more instructions per cell).
// The x origin of every box is a multiple of 4 cells (16 bytes) and the row pitch PI a
// multiple of 4, as the TMA unit requires; boxes reaching outside the block read zeros, which
// no valid face uses.
#pragma once
#include <cuda.h>
#include <stdint.h>
#include "kernels.cuh"
#include "launch.h"

namespace tg {

// tile geometry (RT_X, RT_X1, RT_D, RT_W1, RT_WIDE, RT_NARROW, NRMAP) is in launch.h
constexpr int RT_NWIDE = 14, RT_NNARROW = 25, RT_NFIELD = RT_NWIDE + RT_NNARROW;
constexpr int RT_FACES = RT_X * (RT_D + 1);                       // faces of a direction-2/3 tile
constexpr int RT_B1 = RT_W1 * RT_R1;                              // floats of a direction-1 box
constexpr int RT_F1 = (RT_B1 + 31) / 32 * 32;                     // floats per field, direction 1 (128-byte multiple)
constexpr int RT_FW = RT_X * RT_WIDE, RT_FN = RT_X * RT_NARROW;   // floats per field, directions 2, 3
constexpr int RT_FIELDS1 = RT_NFIELD * RT_F1;
constexpr int RT_FIELDS23 = RT_NWIDE * RT_FW + RT_NNARROW * RT_FN;
// every field starts on a 128-byte boundary: a TMA tensor copy's shared-memory destination must
static_assert(RT_F1 * 4 % 128 == 0 && RT_FW * 4 % 128 == 0 && RT_FN * 4 % 128 == 0 && RT_NWIDE * RT_FW * 4 % 128 == 0,
              "TMA destinations must be 128-byte aligned");
// dynamic shared memory of a CTA: fields, face fluxes (directions 2, 3), mbarrier, alignment slack
constexpr size_t rt_smem_bytes(int dir) {
    return (size_t)(dir == 1 ? RT_FIELDS1 : RT_FIELDS23 + NFX * RT_FACES) * 4 + 16 + 128;
}

// staged field of a slot for direction DIR: 0..13 the stencil fields, 14..38 the two-point
// fields, -1 a slot read from global memory
template <int DIR>
__host__ __device__ constexpr int rt_field(int slot) {
    return (slot >= S_PRIM && slot < S_PRIM + 5) ? slot - S_PRIM
         : slot == S_PP ? 5 : slot == S_T ? 6 : slot == S_SHOCK ? 7 : slot == S_RAD ? 8
         : slot == S_ALAGM + DIR - 1 ? 9 : slot == S_AINV + DIR - 1 ? 10
         : (slot >= S_SD + 3 * (DIR - 1) && slot < S_SD + 3 * DIR) ? 11 + slot - (S_SD + 3 * (DIR - 1))
         : (slot >= S_DQ && slot < S_DQ + 18) ? 14 + slot - S_DQ
         : slot == S_RMIU ? 32 : slot == S_VOL ? 33 : slot == S_V ? 34 : slot == S_DST ? 35
         : slot == S_VINV + DIR - 1 ? 36 : slot == S_WALL + DIR - 1 ? 37 : slot == S_GRAD + DIR - 1 ? 38 : -1;
}

template <int DIR>
__host__ __device__ constexpr int rt_offset(int field) {       // first float of a field
    return DIR == 1 ? field * RT_F1 : (field < RT_NWIDE ? field * RT_FW : RT_NWIDE * RT_FW + (field - RT_NWIDE) * RT_FN);
}

// face inputs from the staged tile: pos is the face's offset-0 element within a field (direction
// 1: row * RT_W1 + lane + 4; directions 2, 3: face * 32 + column); anything not staged, or at an
// offset outside the staged range, is read from the slot arrays
template <int DIR>
struct FaceTile {
    const float* sm;
    const DevBlock& b;
    int c, s, pos;
    __device__ float v(int slot, int o) const {
        const int f = rt_field<DIR>(slot);
        if (DIR == 1) {
            if (f >= 0 && o >= -4 && o <= 3) return sm[rt_offset<DIR>(f) + pos + o];
        } else {
            if (f >= 0 && f < RT_NWIDE && o >= -3 && o <= 2) return sm[rt_offset<DIR>(f) + pos + (o + 3) * RT_X];
            if (f >= RT_NWIDE && o >= -1 && o <= 0) return sm[rt_offset<DIR>(f) + pos + (o + 1) * RT_X];
        }
        return fslot(b, slot)[c + o * s];
    }
};

// ---- mbarrier and TMA (PTX) ----
__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait for the phase of the given parity: false after `limit` polls
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, unsigned limit) {
    for (unsigned n = 0; n < limit; ++n)
        if (mbar_test(bar, parity)) return true;
    return false;
}
// the tensor maps live in global memory, written by the host before the launch
__device__ __forceinline__ void tensormap_acquire(const void* map) {
    asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(map) : "memory");
}
__device__ __forceinline__ void tma_load_4d(float* dst, const void* map, int x, int y, int z, int w, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];"
        ::"r"(smem_addr(dst)), "l"(map), "r"(x), "r"(y), "r"(z), "r"(w), "r"(smem_addr(bar))
        : "memory");
}

// flux differences of one cell in the mixed path's order (see the file comment); Fm = the
// fluxes of the face on the cell's minus side, Fp of the face on its plus side
// (first: direction 1, which writes D; directions 2, 3 add to it)
__device__ __forceinline__ void rt_cell(const DevBlock& b, int c, int turb, const float* Fm, const float* Fp, bool first,
                                        float om) {
    const size_t nc = (size_t)b.ncell;
    float* D = fslot(b, S_D);
    float a = 0.f - Fm[FX_C0] + Fp[FX_C0];
    D[c] = first ? a : D[c] + a;
#pragma unroll
    for (int L = 1; L < 5; ++L) {
        a = 0.f - Fm[FX_VX + L - 1] + Fp[FX_VX + L - 1];
        if (first && (L == 2 || L == 3) && om != 0.f) {
            // rotating-frame source of DIFFUSION_Centered (:812-822), after the viscous terms
            const float* V = fslot(b, S_V);
            const float V1 = V[c];
            const float ss = L == 2 ? 2.f * om * V[3 * nc + c] + om * fslot(b, S_YC)[c] * om * V1
                                    : -2.f * om * V[2 * nc + c] + om * fslot(b, S_ZC)[c] * om * V1;
            a = a + ss * fslot(b, S_VOL)[c];
        }
        a = a - Fm[FX_C0 + L] + Fp[FX_C0 + L];
        D[L * nc + c] = first ? a : D[L * nc + c] + a;
    }
    if (turb) {
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            a = 0.f - Fm[FX_TK + q] + Fp[FX_TK + q] - Fm[FX_CK + q] + Fp[FX_CK + q];
            D[(5 + q) * nc + c] = first ? a : D[(5 + q) * nc + c] + a;
        }
    } else if (first) {
        D[5 * nc + c] = 0.f;
        D[6 * nc + c] = 0.f;
    }
}

template <int DIR>
__global__ void __launch_bounds__(DIR == 1 ? 32 * RT_R1 : RT_FACES, 2)
    k_resid_tma(const DevBlock* __restrict__ blks, const ResidTile* __restrict__ tiles, const CaseDev* __restrict__ cdev,
                const CUtensorMap* __restrict__ maps, int* __restrict__ err, unsigned limit) {
    extern __shared__ unsigned char rt_raw[];
    float* sm = (float*)(((uintptr_t)rt_raw + 127) & ~(uintptr_t)127);
    float* Fb = sm + (DIR == 1 ? RT_FIELDS1 : RT_FIELDS23);
    uint64_t* bar = (uint64_t*)(Fb + (DIR == 1 ? 0 : NFX * RT_FACES));
    const ResidTile t = tiles[blockIdx.x];
    const DevBlock b = blks[t.blk];
    const CaseDev& cd = cdev[b.cs];
    const int turb = cd.turb;
    const int tid = threadIdx.x;
    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (tid == 0) {
        const CUtensorMap* mw = maps + (size_t)t.blk * NRMAP + (DIR == 1 ? 0 : (DIR == 2 ? 1 : 3));
        const CUtensorMap* mn = DIR == 1 ? mw : mw + 1;
        tensormap_acquire(mw);
        if (DIR != 1) tensormap_acquire(mn);
        // box origins (x, y, z): the stencil from 3 cells before the first face, the two-point
        // fields from 1 cell before (direction 1: both from 4 cells before, one box shape)
        const int wx = DIR == 1 ? t.x0 - 4 : t.x0, wy = DIR == 2 ? t.y0 - 3 : t.y0, wz = DIR == 3 ? t.z0 - 3 : t.z0;
        const int ny = DIR == 2 ? t.y0 - 1 : t.y0, nz = DIR == 3 ? t.z0 - 1 : t.z0;
        int wl[RT_NWIDE], nl[RT_NNARROW], nw = 0, nn = 0;
        wl[nw++] = S_PRIM; wl[nw++] = S_PRIM + 1; wl[nw++] = S_PRIM + 2;
        if (turb) { wl[nw++] = S_PRIM + 3; wl[nw++] = S_PRIM + 4; }
        wl[nw++] = S_PP; wl[nw++] = S_T; wl[nw++] = S_SHOCK;
        if (cd.p.omega0 != 0.0) wl[nw++] = S_RAD;
        wl[nw++] = S_ALAGM + DIR - 1; wl[nw++] = S_AINV + DIR - 1;
        for (int m = 0; m < 3; ++m) wl[nw++] = S_SD + 3 * (DIR - 1) + m;
        for (int m = 0; m < (turb ? 18 : 12); ++m) nl[nn++] = S_DQ + m;
        nl[nn++] = S_RMIU; nl[nn++] = S_VOL;
        if (turb) { nl[nn++] = S_V; nl[nn++] = S_DST; }
        nl[nn++] = S_VINV + DIR - 1; nl[nn++] = S_WALL + DIR - 1; nl[nn++] = S_GRAD + DIR - 1;
        // bytes the copies deliver: the boxes' sizes (a direction-1 field is padded beyond its box)
        const unsigned wb = (DIR == 1 ? RT_B1 : RT_FW) * 4, nb = (DIR == 1 ? RT_B1 : RT_FN) * 4;
        mbar_arrive_expect_tx(bar, nw * wb + nn * nb);
        for (int q = 0; q < nw; ++q) tma_load_4d(sm + rt_offset<DIR>(rt_field<DIR>(wl[q])), mw, wx, wy, wz, wl[q], bar);
        for (int q = 0; q < nn; ++q) tma_load_4d(sm + rt_offset<DIR>(rt_field<DIR>(nl[q])), mn, wx, ny, nz, nl[q], bar);
    }
    // one verdict for the whole CTA, so that no thread is left at a barrier
    if (__syncthreads_or(!mbar_wait(bar, 0, limit))) {
        // the copies did not land in time: record it, give the ones in flight the default
        // bounded wait (their shared memory must outlive them), return
        if (tid == 0) {
            atomicExch(err, 1);
            mbar_wait(bar, 0, RT_WAIT_LIMIT);
        }
        __syncthreads();
        return;
    }
    const ParamsT<float> p = cd.pf;
    if (DIR == 1) {
        const int r = tid >> 5, l = tid & 31;
        const int ia = t.x0 + l, ja = t.y0 + r, ka = t.z0;
        const int c = ia + b.PI * (ja + b.PJ * ka);
        float F[NFX];
#pragma unroll
        for (int m = 0; m < NFX; ++m) F[m] = 0.f;
        if (l <= RT_X1 && ia >= 3 && ia <= b.NI + 2 && ja <= b.NJ + 1 && ka <= b.NK + 1) {
            const FaceTile<DIR> q{sm, b, c, 1, r * RT_W1 + l + 4};
            face_flux_body<float, DIR>(p, turb, q, F);
        }
        float Fp[NFX];          // the plus-side face of this lane's cell: the next lane's face
#pragma unroll
        for (int m = 0; m < NFX; ++m) Fp[m] = __shfl_down_sync(0xffffffffu, F[m], 1);
        if (l < RT_X1 && ia >= 3 && ia <= b.NI + 1 && ja <= b.NJ + 1 && ka <= b.NK + 1)
            rt_cell(b, c, turb, F, Fp, true, p.omega0);
    } else {
        const int x = tid & 31, f = tid >> 5;
        const int ia = t.x0 + x;
        const int ja = DIR == 2 ? t.y0 + f : t.y0, ka = DIR == 3 ? t.z0 + f : t.z0;
        const int s = DIR == 2 ? b.PI : b.PI * b.PJ;
        const int c = ia + b.PI * (ja + b.PJ * ka);
        const bool along_ok = DIR == 2 ? (ja <= b.NJ + 2 && ka <= b.NK + 1) : (ka <= b.NK + 2 && ja <= b.NJ + 1);
        if (ia >= 3 && ia <= b.NI + 1 && along_ok) {
            float F[NFX];
#pragma unroll
            for (int m = 0; m < NFX; ++m) F[m] = 0.f;
            const FaceTile<DIR> q{sm, b, c, s, x + RT_X * f};
            face_flux_body<float, DIR>(p, turb, q, F);
#pragma unroll
            for (int m = 0; m < NFX; ++m) Fb[m * RT_FACES + tid] = F[m];
        }
        __syncthreads();
        const bool cell_ok = DIR == 2 ? (ja <= b.NJ + 1 && ka <= b.NK + 1) : (ka <= b.NK + 1 && ja <= b.NJ + 1);
        if (f < RT_D && ia >= 3 && ia <= b.NI + 1 && cell_ok) {
            float Fm[NFX], Fp[NFX];
#pragma unroll
            for (int m = 0; m < NFX; ++m) {
                Fm[m] = Fb[m * RT_FACES + tid];
                Fp[m] = Fb[m * RT_FACES + tid + RT_X];
            }
            rt_cell(b, c, turb, Fm, Fp, false, 0.f);
        }
    }
}

}  // namespace tg
