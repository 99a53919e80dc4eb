// k_geometry.cu -- GEOM_CalcDST (Geom/CalcDst.F90:28-719) on the device: the wall distance
// (:127-164) and the per-cell and per-face metrics of one block.
//
// Wall distance.
//
// The reference computes, for every interior cell centre, the squared distance
// DDD = Dx*Dx + Dy*Dy + Dz*Dz to the centre of every panel of every wall surface (panel centre =
// the average of its 4 nodes), keeps the minimum per surface (Dst_minN), combines the surfaces
// in order as  d = max(d, tiny); if (Dst_minN < d) d = Dst_minN  (starting from d = 1e20), and
// stores sqrt(d).  That is O(cells x panels): 8.8e11 pairs for a 5.7 M-cell cascade.
//
// Here each surface is scanned twice per cell in FP32 (the FP32 pipe is 58x the FP64 pipe on
// GB300): pass A finds the FP32 minimum m of the squared distances; pass B evaluates the
// reference's FP64 expression only for the panels whose FP32 squared distance is within
// (sqrt(m)(1 + 1e-5) + 2 Eabs)^2 (1 + 1e-5) of it, where Eabs = 1e-6 R bounds the error of an
// FP32 distance (coordinates rounded to FP32: 2^-24 |x| each, |x| <= R <= 1e18, three
// components; 1e-37 floor for subnormal FP32) and the relative slack covers the FP32 arithmetic.  The panel that minimises the FP64 DDD has an
// FP32 distance within 2 Eabs (+ the relative slack) of the FP32 minimum, so it is always
// evaluated, and the minimum of the evaluated FP64 values is the reference's Dst_minN exactly.
// The FP64 arithmetic is compiled without contraction (-fmad=false), so the result is
// bit-identical to a sequential CPU evaluation of the reference's loop.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/trans_gpu.h"

namespace tg {

thread_local std::string g_stateless_err;
namespace eng {
const char* stateless_error() { return g_stateless_err.c_str(); }
}  // namespace eng

namespace {

constexpr int WD_THREADS = 256;
constexpr int WD_TILE = 2048;             // panels per shared-memory tile (float4: 32 KB)

constexpr int WD_CAND = 8;                // candidates per surface held for the converged FP64 pass

// the reference's DDD (Geom/CalcDst.F90:150-155), in its order
__device__ __forceinline__ double ddd64(double px, double py, double pz, const double* __restrict__ q) {
    const double Dx = px - q[0], Dy = py - q[1], Dz = pz - q[2];
    return Dx * Dx + Dy * Dy + Dz * Dz;
}

__device__ __forceinline__ float d2f(float fx, float fy, float fz, float4 q) {
    const float dx = fx - q.x, dy = fy - q.y, dz = fz - q.z;
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, dx * dx));
}

__global__ void __launch_bounds__(WD_THREADS)
k_wall_distance(long long n, const double* __restrict__ pts, const float4* __restrict__ pan32,
                const double* __restrict__ pan64, const long long* __restrict__ soff, int nsurf, float eabs,
                double tiny, double* __restrict__ dst) {
    __shared__ float4 tile[WD_TILE];
    const long long c = (long long)blockIdx.x * WD_THREADS + threadIdx.x;
    const bool live = c < n;
    const double px = live ? pts[3 * c] : 0.0, py = live ? pts[3 * c + 1] : 0.0, pz = live ? pts[3 * c + 2] : 0.0;
    const float fx = (float)px, fy = (float)py, fz = (float)pz;
    double d = 1.0e20;
    for (int s = 0; s < nsurf; ++s) {
        const long long p0 = soff[s], p1 = soff[s + 1];
        // pass A: FP32 minimum over the surface
        float m = INFINITY, m1 = INFINITY;     // two chains of minima
        for (long long t0 = p0; t0 < p1; t0 += WD_TILE) {
            const int cnt = (int)min((long long)WD_TILE, p1 - t0);
            __syncthreads();
            for (int r = threadIdx.x; r < cnt; r += WD_THREADS) tile[r] = pan32[t0 + r];
            __syncthreads();
            int r = 0;
#pragma unroll 4
            for (; r + 1 < cnt; r += 2) {
                m = fminf(m, d2f(fx, fy, fz, tile[r]));
                m1 = fminf(m1, d2f(fx, fy, fz, tile[r + 1]));
            }
            if (r < cnt) m = fminf(m, d2f(fx, fy, fz, tile[r]));
        }
        m = fminf(m, m1);
        const float sm = sqrtf(m);
        const float bd = __fmaf_rn(sm, 1.0e-5f, sm) + 2.0f * eabs;
        const float thr = bd * bd * (1.0f + 1.0e-5f);
        // pass B: collect the candidates, then evaluate the reference's FP64 expression for them
        // with the warp's lanes together (a candidate found by one lane alone would otherwise
        // cost the whole warp's FP64 issue slots); a lane with more than WD_CAND candidates
        // evaluates the extra ones at once
        double a = 1.0e20;
        long long cand[WD_CAND];
        int nc = 0;
        for (long long t0 = p0; t0 < p1; t0 += WD_TILE) {
            const int cnt = (int)min((long long)WD_TILE, p1 - t0);
            __syncthreads();
            for (int r = threadIdx.x; r < cnt; r += WD_THREADS) tile[r] = pan32[t0 + r];
            __syncthreads();
            for (int r = 0; r < cnt; ++r) {
                if (d2f(fx, fy, fz, tile[r]) <= thr) {
                    if (nc < WD_CAND) {
                        cand[nc++] = t0 + r;
                    } else {
                        const double DDD = ddd64(px, py, pz, pan64 + 3 * (t0 + r));
                        if (DDD < a) a = DDD;
                    }
                }
            }
        }
#pragma unroll
        for (int j = 0; j < WD_CAND; ++j) {
            if (j < nc) {
                const double DDD = ddd64(px, py, pz, pan64 + 3 * cand[j]);
                if (DDD < a) a = DDD;
            }
        }
        if (d < tiny) d = tiny;          // amax1(dst_minimum, tiny)
        if (a < d) d = a;
    }
    if (live) dst[c] = sqrt(d);
}

// ---------------------------------------------------------------------------------------
// Block metrics (Geom/CalcDst.F90:95-521).  Arrays are ghost-padded (NI+5)(NJ+5)(NK+5), index
// -2..N+2 per direction; nodes are X, Y, Z of NI x NJ x NK, I fastest.  Every expression keeps
// the reference's operation order (no contraction), so the results equal a CPU evaluation.
// ---------------------------------------------------------------------------------------
struct Geo {
    int NI, NJ, NK, PI, PJ;
    const double* X;            // nodes: X, Y, Z planes
    double* out;                // GEO_NF padded fields
    size_t P;                   // padded cells per field
};
enum GeoField { G_XC = 0, G_YC, G_ZC, G_DST, G_ALENG, G_ASENG, G_VOL, G_RAD, G_THTC, G_SD = 9, G_GRAD = 18, G_ALAGM = 21,
                GEO_NF = 24 };

__device__ __forceinline__ size_t gp(const Geo& g, int i, int j, int k) {
    return (size_t)(i + 2) + (size_t)g.PI * ((size_t)(j + 2) + (size_t)g.PJ * (size_t)(k + 2));
}
__device__ __forceinline__ double nd(const Geo& g, int q, int I, int J, int K) {   // node (I,J,K), 1-based
    return g.X[(size_t)q * g.NI * g.NJ * g.NK + (size_t)(I - 1) + (size_t)g.NI * ((size_t)(J - 1) + (size_t)g.NJ * (K - 1))];
}
__device__ __forceinline__ double* gf(const Geo& g, int f) { return g.out + (size_t)f * g.P; }

// cell centre of cell (I,J,K) from its 8 nodes (:97-112)
__device__ __forceinline__ double cell_centre(const Geo& g, int q, int I, int J, int K) {
    const int I1 = I + 1, J1 = J + 1, K1 = K + 1;
    return (nd(g, q, I1, J1, K1) + nd(g, q, I1, J1, K) + nd(g, q, I1, J, K1) + nd(g, q, I1, J, K) + nd(g, q, I, J1, K1) +
            nd(g, q, I, J1, K) + nd(g, q, I, J, K1) + nd(g, q, I, J, K)) / 8.;
}

// atan over [0, 1]: two half-angle reductions atan t = 2 atan(t / (1 + sqrt(1 + t^2))), then the
// odd Taylor series to t^31 (the host set-up's own atan2, so the two agree bit for bit)
__device__ double atan01(double t) {
    for (int r = 0; r < 2; ++r) t = t / (1.0 + sqrt(1.0 + t * t));
    const double t2 = t * t;
    double p = 0.0;
    for (int n = 31; n > 1; n -= 2) p = (1.0 / n - p) * t2;
    return 4.0 * (t - t * p);
}
__device__ double det_atan2(double y, double x) {
    const double PI = 3.141592653589793115997963468544185161590576171875;     // RN(pi)
    const double PIO2 = 1.5707963267948965579989817342720925807952880859375;  // RN(pi/2)
    const double ay = fabs(y), ax = fabs(x);
    const bool big = ay > ax;
    const double num = big ? ax : ay, den = big ? ay : ax;
    const double t = den > 0 ? num / den : 0.0;
    double a = atan01(t);
    if (big) a = PIO2 - a;
    if (x < 0) a = PI - a;
    if (y < 0) a = -a;
    return a;
}

// interior cells: centres, thtc, rad, and the points of the wall distance
__global__ void k_geo_cells(Geo g, double* __restrict__ pts) {
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int NI1 = g.NI - 1, NJ1 = g.NJ - 1, NK1 = g.NK - 1;
    if (n >= (long long)NI1 * NJ1 * NK1) return;
    const int I = (int)(n % NI1) + 1, J = (int)((n / NI1) % NJ1) + 1, K = (int)(n / ((long long)NI1 * NJ1)) + 1;
    const size_t c = gp(g, I, J, K);
    const double zc = cell_centre(g, 2, I, J, K), yc = cell_centre(g, 1, I, J, K), xc = cell_centre(g, 0, I, J, K);
    gf(g, G_XC)[c] = xc; gf(g, G_YC)[c] = yc; gf(g, G_ZC)[c] = zc;
    gf(g, G_THTC)[c] = det_atan2(zc, yc);
    gf(g, G_RAD)[c] = sqrt(yc * yc + zc * zc);
    pts[3 * n] = xc; pts[3 * n + 1] = yc; pts[3 * n + 2] = zc;
}

__global__ void k_geo_dst(Geo g, const double* __restrict__ dst) {
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int NI1 = g.NI - 1, NJ1 = g.NJ - 1, NK1 = g.NK - 1;
    if (n >= (long long)NI1 * NJ1 * NK1) return;
    const int I = (int)(n % NI1) + 1, J = (int)((n / NI1) % NJ1) + 1, K = (int)(n / ((long long)NI1 * NJ1)) + 1;
    gf(g, G_DST)[gp(g, I, J, K)] = dst[n];
}

// half cross product of the two face diagonals of face (I,J,K) of direction d (:180-300)
__device__ void face_cross(const Geo& g, int d, int I, int J, int K, double* xs) {
    double R1[3], R2[3];
    for (int q = 0; q < 3; ++q) {
        if (d == 0) {
            R1[q] = nd(g, q, I, J + 1, K + 1) - nd(g, q, I, J, K);
            R2[q] = nd(g, q, I, J, K + 1) - nd(g, q, I, J + 1, K);
        } else if (d == 1) {
            R1[q] = nd(g, q, I, J, K + 1) - nd(g, q, I + 1, J, K);
            R2[q] = nd(g, q, I + 1, J, K + 1) - nd(g, q, I, J, K);
        } else {
            R1[q] = nd(g, q, I + 1, J, K) - nd(g, q, I, J + 1, K);
            R2[q] = nd(g, q, I + 1, J + 1, K) - nd(g, q, I, J, K);
        }
    }
    xs[0] = (R1[1] * R2[2] - R1[2] * R2[1]) * 0.5;
    xs[1] = (R1[2] * R2[0] - R1[0] * R2[2]) * 0.5;
    xs[2] = (R1[0] * R2[1] - R1[1] * R2[0]) * 0.5;
}

// faces of direction d: SD = the half cross product oriented by the block's handedness (dl),
// Grad = |SD| (+ tiny under the root); face 0 copies face 1
__global__ void k_geo_faces(Geo g, int d, double tiny) {
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int nI = d == 0 ? g.NI : g.NI - 1, nJ = d == 1 ? g.NJ : g.NJ - 1, nK = d == 2 ? g.NK : g.NK - 1;
    if (n >= (long long)nI * nJ * nK) return;
    const int I = (int)(n % nI) + 1, J = (int)((n / nI) % nJ) + 1, K = (int)(n / ((long long)nI * nJ)) + 1;
    // handedness: the first i-face normal against the direction from cell (1,1,1) to (2,1,1)
    double x0[3];
    face_cross(g, 0, 1, 1, 1, x0);
    const double xv = cell_centre(g, 0, 2, 1, 1) - cell_centre(g, 0, 1, 1, 1);
    const double yv = cell_centre(g, 1, 2, 1, 1) - cell_centre(g, 1, 1, 1, 1);
    const double zv = cell_centre(g, 2, 2, 1, 1) - cell_centre(g, 2, 1, 1, 1);
    const double dl = (xv * x0[0] + yv * x0[1] + zv * x0[2] < 0) ? -1.0 : 1.0;
    double xs[3];
    face_cross(g, d, I, J, K, xs);
    const size_t c = gp(g, I, J, K);
    double sd[3];
    for (int q = 0; q < 3; ++q) { sd[q] = xs[q] * dl; gf(g, G_SD + 3 * d + q)[c] = sd[q]; }
    const double gr = sqrt(sd[0] * sd[0] + sd[1] * sd[1] + sd[2] * sd[2] + tiny);
    gf(g, G_GRAD + d)[c] = gr;
    const int e1 = d == 0 ? I : (d == 1 ? J : K);
    if (e1 == 1) {
        const size_t c0 = gp(g, I - (d == 0), J - (d == 1), K - (d == 2));
        for (int q = 0; q < 3; ++q) gf(g, G_SD + 3 * d + q)[c0] = sd[q];
        gf(g, G_GRAD + d)[c0] = gr;
    }
}

// face centre (0.25 of the sum of 4 nodes) of face `f` (w e s n b t) of cell (I,J,K), component q
__device__ double face_centre(const Geo& g, int q, int f, int I, int J, int K) {
    int a[4][3];
    switch (f) {
        case 0: { int t[4][3] = {{0, 0, 0}, {0, 1, 0}, {0, 0, 1}, {0, 1, 1}}; memcpy(a, t, sizeof(a)); break; }
        case 1: { int t[4][3] = {{1, 0, 0}, {1, 1, 0}, {1, 0, 1}, {1, 1, 1}}; memcpy(a, t, sizeof(a)); break; }
        case 2: { int t[4][3] = {{0, 0, 0}, {1, 0, 0}, {0, 0, 1}, {1, 0, 1}}; memcpy(a, t, sizeof(a)); break; }
        case 3: { int t[4][3] = {{0, 1, 0}, {1, 1, 0}, {0, 1, 1}, {1, 1, 1}}; memcpy(a, t, sizeof(a)); break; }
        case 4: { int t[4][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {1, 1, 0}}; memcpy(a, t, sizeof(a)); break; }
        default: { int t[4][3] = {{0, 0, 1}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}}; memcpy(a, t, sizeof(a)); break; }
    }
    double s = nd(g, q, I + a[0][0], J + a[0][1], K + a[0][2]) + nd(g, q, I + a[1][0], J + a[1][1], K + a[1][2]);
    s = s + nd(g, q, I + a[2][0], J + a[2][1], K + a[2][2]);
    s = s + nd(g, q, I + a[3][0], J + a[3][1], K + a[3][2]);
    return 0.25 * s;
}

// Alagm (:322-358): distance between the two opposite face centres of a cell, per direction
__global__ void k_geo_alagm(Geo g) {
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int NI1 = g.NI - 1, NJ1 = g.NJ - 1, NK1 = g.NK - 1;
    if (n >= (long long)NI1 * NJ1 * NK1) return;
    const int I = (int)(n % NI1) + 1, J = (int)((n / NI1) % NJ1) + 1, K = (int)(n / ((long long)NI1 * NJ1)) + 1;
    const size_t c = gp(g, I, J, K);
    for (int d = 0; d < 3; ++d) {
        const double dx = face_centre(g, 0, 2 * d, I, J, K) - face_centre(g, 0, 2 * d + 1, I, J, K);
        const double dy = face_centre(g, 1, 2 * d, I, J, K) - face_centre(g, 1, 2 * d + 1, I, J, K);
        const double dz = face_centre(g, 2, 2 * d, I, J, K) - face_centre(g, 2, 2 * d + 1, I, J, K);
        gf(g, G_ALAGM + d)[c] = sqrt(dx * dx + dy * dy + dz * dz);
    }
}

// centres of the boundary faces stored in the first ghost layer (:370-422): one thread per
// face cell of the six block faces
__global__ void k_geo_bface(Geo g) {
    const int NI1 = g.NI - 1, NJ1 = g.NJ - 1, NK1 = g.NK - 1;
    const long long nI = (long long)NJ1 * NK1, nJ = (long long)NI1 * NK1, nK = (long long)NI1 * NJ1;
    long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= 2 * (nI + nJ + nK)) return;
    int d, side, a, b;
    if (n < 2 * nI) { d = 0; side = (int)(n / nI); n %= nI; a = (int)(n % NJ1) + 1; b = (int)(n / NJ1) + 1; }
    else if ((n -= 2 * nI) < 2 * nJ) { d = 1; side = (int)(n / nJ); n %= nJ; a = (int)(n % NI1) + 1; b = (int)(n / NI1) + 1; }
    else { n -= 2 * nJ; d = 2; side = (int)(n / nK); n %= nK; a = (int)(n % NI1) + 1; b = (int)(n / NI1) + 1; }
    for (int q = 0; q < 3; ++q) {
        double v;
        size_t c;
        if (d == 0) {
            const int ii = side ? g.NI : 1;
            v = (nd(g, q, ii, a, b) + nd(g, q, ii, a + 1, b) + nd(g, q, ii, a, b + 1) + nd(g, q, ii, a + 1, b + 1)) / 4.0;
            c = gp(g, side ? g.NI : 0, a, b);
        } else if (d == 1) {
            const int jj = side ? g.NJ : 1;
            v = (nd(g, q, a, jj, b) + nd(g, q, a + 1, jj, b) + nd(g, q, a, jj, b + 1) + nd(g, q, a + 1, jj, b + 1)) / 4.0;
            c = gp(g, a, side ? g.NJ : 0, b);
        } else {
            const int kk = side ? g.NK : 1;
            v = (nd(g, q, a, b, kk) + nd(g, q, a + 1, b, kk) + nd(g, q, a, b + 1, kk) + nd(g, q, a + 1, b + 1, kk)) / 4.0;
            c = gp(g, a, b, side ? g.NK : 0);
        }
        gf(g, G_XC + q)[c] = v;
    }
}

// aLeng / aSeng (:430-480): largest and smallest distance to the six neighbouring centres
// (boundary face centres at the block faces), directions of 2 cells left out; Vol (:488-521)
__global__ void k_geo_len_vol(Geo g, double tiny, int* __restrict__ bad) {
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int NI1 = g.NI - 1, NJ1 = g.NJ - 1, NK1 = g.NK - 1;
    if (n >= (long long)NI1 * NJ1 * NK1) return;
    const int I = (int)(n % NI1) + 1, J = (int)((n / NI1) % NJ1) + 1, K = (int)(n / ((long long)NI1 * NJ1)) + 1;
    const size_t c = gp(g, I, J, K);
    const double* Xc = gf(g, G_XC);
    const double* Yc = gf(g, G_YC);
    const double* Zc = gf(g, G_ZC);
    const int off[6][3] = {{-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};
    double dd[6];
    for (int m = 0; m < 6; ++m) {
        const size_t o = gp(g, I + off[m][0], J + off[m][1], K + off[m][2]);
        const double dx = Xc[o] - Xc[c], dy = Yc[o] - Yc[c], dz = Zc[o] - Zc[c];
        dd[m] = sqrt(dx * dx + dy * dy + dz * dz);
    }
    int use[6] = {1, 1, 1, 1, 1, 1};
    if (NI1 == 2) { use[0] = 0; use[1] = 0; use[2] = 1; use[3] = 1; use[4] = 1; use[5] = 1; }
    if (NJ1 == 2) { use[0] = 1; use[1] = 1; use[2] = 0; use[3] = 0; use[4] = 1; use[5] = 1; }
    if (NK1 == 2) { use[0] = 1; use[1] = 1; use[2] = 1; use[3] = 1; use[4] = 0; use[5] = 0; }
    double mx = -INFINITY, mn = INFINITY;
    for (int m = 0; m < 6; ++m)
        if (use[m]) { mx = fmax(mx, dd[m]); mn = fmin(mn, dd[m]); }
    gf(g, G_ALENG)[c] = mx;
    gf(g, G_ASENG)[c] = mn;
    // Vol = (1/3) sum over the three min faces of (diagonal node difference) . SD
    const double* SD = gf(g, G_SD);
    auto sd = [&](int d, int q) { return SD[(size_t)(3 * d + q) * g.P + c]; };
    double XR = nd(g, 0, I + 1, J + 1, K + 1) - nd(g, 0, I, J + 1, K + 1);
    double YR = nd(g, 1, I + 1, J + 1, K + 1) - nd(g, 1, I, J + 1, K + 1);
    double ZR = nd(g, 2, I + 1, J + 1, K + 1) - nd(g, 2, I, J + 1, K + 1);
    double OMG = XR * sd(0, 0) + YR * sd(0, 1) + ZR * sd(0, 2);
    XR = nd(g, 0, I + 1, J + 1, K + 1) - nd(g, 0, I + 1, J, K + 1);
    YR = nd(g, 1, I + 1, J + 1, K + 1) - nd(g, 1, I + 1, J, K + 1);
    ZR = nd(g, 2, I + 1, J + 1, K + 1) - nd(g, 2, I + 1, J, K + 1);
    OMG = OMG + XR * sd(1, 0) + YR * sd(1, 1) + ZR * sd(1, 2);
    XR = nd(g, 0, I + 1, J + 1, K + 1) - nd(g, 0, I + 1, J + 1, K);
    YR = nd(g, 1, I + 1, J + 1, K + 1) - nd(g, 1, I + 1, J + 1, K);
    ZR = nd(g, 2, I + 1, J + 1, K + 1) - nd(g, 2, I + 1, J + 1, K);
    OMG = OMG + XR * sd(2, 0) + YR * sd(2, 1) + ZR * sd(2, 2);
    const double vol = (1.0 / 3.0) * OMG;
    gf(g, G_VOL)[c] = vol;
    if (vol < tiny) atomicExch(bad, 1);
}

int wd_fail(int code, const std::string& msg) {
    g_stateless_err = msg;
    return code;
}

}  // namespace
}  // namespace tg

namespace tg {
namespace {

// panel centres of the wall surfaces (the reference's expression, in its order), their FP32
// copies, the surface offsets and the largest coordinate magnitude
struct Panels {
    std::vector<long long> soff{0};
    std::vector<double> p64;
    std::vector<float> p32;
    double R = 0.0;
};

int make_panels(int nsurf, const int* dims, const double* nodes, Panels& P) {
    for (int s = 0; s < nsurf; ++s) {
        const int ni = dims[2 * s], nj = dims[2 * s + 1];
        if (ni < 1 || nj < 1) return wd_fail(TRANS_E_ARG, "bad surface dimensions");
        P.soff.push_back(P.soff.back() + (long long)(ni - 1) * (nj - 1));
    }
    const long long np = P.soff.back();
    P.p64.assign((size_t)(3 * np), 0.0);
    P.p32.assign((size_t)(4 * np), 0.0f);
    size_t base = 0;
    long long p = 0;
    for (int s = 0; s < nsurf; ++s) {
        const int ni = dims[2 * s], nj = dims[2 * s + 1];
        const size_t plane = (size_t)ni * nj;
        const double* X = nodes + base;
        const double* Y = X + plane;
        const double* Z = Y + plane;
        for (int J = 0; J < nj - 1; ++J)
            for (int I = 0; I < ni - 1; ++I, ++p) {
                const size_t a = (size_t)I + (size_t)ni * J, b = a + 1, cc = a + ni, dd = cc + 1;
                const double xs = (X[a] + X[b] + X[cc] + X[dd]) / 4.0;
                const double ys = (Y[a] + Y[b] + Y[cc] + Y[dd]) / 4.0;
                const double zs = (Z[a] + Z[b] + Z[cc] + Z[dd]) / 4.0;
                if (!std::isfinite(xs) || !std::isfinite(ys) || !std::isfinite(zs))
                    return wd_fail(TRANS_E_ARG, "surface coordinates not finite");
                P.p64[3 * p] = xs; P.p64[3 * p + 1] = ys; P.p64[3 * p + 2] = zs;
                P.p32[4 * p] = (float)xs; P.p32[4 * p + 1] = (float)ys; P.p32[4 * p + 2] = (float)zs;
                P.R = std::max(P.R, std::max(std::fabs(xs), std::max(std::fabs(ys), std::fabs(zs))));
            }
        base += 3 * plane;
    }
    return TRANS_OK;
}

// device memory released at scope exit
struct DevBufs {
    std::vector<void*> v;
    ~DevBufs() { for (void* p : v) cudaFree(p); }
    template <typename T> cudaError_t get(T** p, size_t bytes) {
        cudaError_t e = cudaMalloc((void**)p, std::max<size_t>(bytes, 16));
        if (e == cudaSuccess) v.push_back((void*)*p);
        return e;
    }
};

// the wall distance of n device points (x y z interleaved) into d_dst, on stream st
int run_wall_distance(cudaStream_t st, long long n, const double* d_pts, int nsurf, const Panels& P, double R, double tiny,
                      double* d_dst, DevBufs& bufs) {
    if (R > 1.0e18) return wd_fail(TRANS_E_ARG, "coordinates beyond 1e18");   // FP32 squares stay finite
    const float eabs = std::max((float)(1.0e-6 * R), 1.0e-37f);
    const long long np = P.soff.back();
    double* d_p64 = nullptr;
    float4* d_p32 = nullptr;
    long long* d_off = nullptr;
    cudaError_t e;
    if ((e = bufs.get(&d_p64, sizeof(double) * P.p64.size())) != cudaSuccess ||
        (e = bufs.get(&d_p32, sizeof(float4) * (size_t)np)) != cudaSuccess ||
        (e = bufs.get(&d_off, sizeof(long long) * P.soff.size())) != cudaSuccess ||
        (e = cudaMemcpyAsync(d_p64, P.p64.data(), sizeof(double) * P.p64.size(), cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(d_p32, P.p32.data(), sizeof(float) * P.p32.size(), cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(d_off, P.soff.data(), sizeof(long long) * P.soff.size(), cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return wd_fail(TRANS_E_CUDA, std::string("wall distance set-up: ") + cudaGetErrorString(e));
    const unsigned grid = (unsigned)((n + WD_THREADS - 1) / WD_THREADS);
    k_wall_distance<<<grid, WD_THREADS, 0, st>>>(n, d_pts, d_p32, d_p64, d_off, nsurf, eabs, tiny, d_dst);
    if ((e = cudaGetLastError()) != cudaSuccess) return wd_fail(TRANS_E_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    return TRANS_OK;
}

struct StreamGuard {
    cudaStream_t s = nullptr;
    ~StreamGuard() { if (s) cudaStreamDestroy(s); }
};

}  // namespace
}  // namespace tg

using namespace tg;

extern "C" int trans_wall_distance(long long n, const double* xyz, int nsurf, const int* dims, const double* nodes,
                                   double tiny, double* dst) {
    g_stateless_err.clear();
    if (n < 0 || nsurf < 0 || (n > 0 && (!xyz || !dst)) || (nsurf > 0 && (!dims || !nodes)))
        return wd_fail(TRANS_E_ARG, "bad argument");
    if (n == 0) return TRANS_OK;
    if (n > (long long)2147483647 * WD_THREADS) return wd_fail(TRANS_E_ARG, "too many points");
    Panels P;
    int rc = make_panels(nsurf, dims, nodes, P);
    if (rc) return rc;
    double R = P.R;
    for (long long q = 0; q < 3 * n; ++q) {
        if (!std::isfinite(xyz[q])) return wd_fail(TRANS_E_ARG, "point coordinates not finite");
        R = std::max(R, std::fabs(xyz[q]));
    }
    StreamGuard sg;
    DevBufs bufs;
    double *d_pts = nullptr, *d_dst = nullptr;
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&sg.s, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = bufs.get(&d_pts, sizeof(double) * 3 * (size_t)n)) != cudaSuccess ||
        (e = bufs.get(&d_dst, sizeof(double) * (size_t)n)) != cudaSuccess ||
        (e = cudaMemcpyAsync(d_pts, xyz, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice, sg.s)) != cudaSuccess)
        return wd_fail(TRANS_E_CUDA, std::string("set-up: ") + cudaGetErrorString(e));
    if ((rc = run_wall_distance(sg.s, n, d_pts, nsurf, P, R, tiny, d_dst, bufs))) { cudaStreamSynchronize(sg.s); return rc; }
    if ((e = cudaMemcpyAsync(dst, d_dst, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, sg.s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(sg.s)) != cudaSuccess)
        return wd_fail(TRANS_E_CUDA, std::string("wall distance: ") + cudaGetErrorString(e));
    return TRANS_OK;
}

extern "C" int trans_block_metrics(int ni, int nj, int nk, const double* xyz, int nsurf, const int* dims,
                                   const double* nodes, double tiny, double* out) {
    g_stateless_err.clear();
    if (ni < 3 || nj < 3 || nk < 3 || !xyz || !out || nsurf < 0 || (nsurf > 0 && (!dims || !nodes)))
        return wd_fail(TRANS_E_ARG, "bad argument");
    const size_t nn = (size_t)ni * nj * nk;
    const size_t P = (size_t)(ni + 5) * (nj + 5) * (nk + 5);
    if (P * GEO_NF > ((size_t)1 << 33)) return wd_fail(TRANS_E_ARG, "block too large");
    Panels pan;
    int rc = make_panels(nsurf, dims, nodes, pan);
    if (rc) return rc;
    double R = pan.R;
    for (size_t q = 0; q < 3 * nn; ++q) {
        if (!std::isfinite(xyz[q])) return wd_fail(TRANS_E_ARG, "node coordinates not finite");
        R = std::max(R, std::fabs(xyz[q]));          // cell centres lie within the nodes' bound
    }
    const long long ncell = (long long)(ni - 1) * (nj - 1) * (nk - 1);
    StreamGuard sg;
    DevBufs bufs;
    double *d_x = nullptr, *d_out = nullptr, *d_pts = nullptr, *d_dst = nullptr;
    int* d_bad = nullptr;
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&sg.s, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = bufs.get(&d_x, sizeof(double) * 3 * nn)) != cudaSuccess ||
        (e = bufs.get(&d_out, sizeof(double) * GEO_NF * P)) != cudaSuccess ||
        (e = bufs.get(&d_pts, sizeof(double) * 3 * (size_t)ncell)) != cudaSuccess ||
        (e = bufs.get(&d_dst, sizeof(double) * (size_t)ncell)) != cudaSuccess ||
        (e = bufs.get(&d_bad, sizeof(int))) != cudaSuccess ||
        (e = cudaMemcpyAsync(d_x, xyz, sizeof(double) * 3 * nn, cudaMemcpyHostToDevice, sg.s)) != cudaSuccess ||
        (e = cudaMemsetAsync(d_out, 0, sizeof(double) * GEO_NF * P, sg.s)) != cudaSuccess ||
        (e = cudaMemsetAsync(d_bad, 0, sizeof(int), sg.s)) != cudaSuccess)
        return wd_fail(TRANS_E_CUDA, std::string("set-up: ") + cudaGetErrorString(e));
    Geo g{ni, nj, nk, ni + 5, nj + 5, d_x, d_out, P};
    const unsigned T = 256;
    auto blocks = [&](long long n) { return (unsigned)((n + T - 1) / T); };
    k_geo_cells<<<blocks(ncell), T, 0, sg.s>>>(g, d_pts);
    for (int d = 0; d < 3; ++d) {
        const long long nf = (long long)(d == 0 ? ni : ni - 1) * (d == 1 ? nj : nj - 1) * (d == 2 ? nk : nk - 1);
        k_geo_faces<<<blocks(nf), T, 0, sg.s>>>(g, d, tiny);
    }
    k_geo_alagm<<<blocks(ncell), T, 0, sg.s>>>(g);
    const long long nb = 2LL * ((long long)(nj - 1) * (nk - 1) + (long long)(ni - 1) * (nk - 1) + (long long)(ni - 1) * (nj - 1));
    k_geo_bface<<<blocks(nb), T, 0, sg.s>>>(g);
    k_geo_len_vol<<<blocks(ncell), T, 0, sg.s>>>(g, tiny, d_bad);
    if ((e = cudaGetLastError()) != cudaSuccess) return wd_fail(TRANS_E_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    if ((rc = run_wall_distance(sg.s, ncell, d_pts, nsurf, pan, R, tiny, d_dst, bufs))) { cudaStreamSynchronize(sg.s); return rc; }
    k_geo_dst<<<blocks(ncell), T, 0, sg.s>>>(g, d_dst);
    int bad = 0;
    if ((e = cudaGetLastError()) != cudaSuccess ||
        (e = cudaMemcpyAsync(out, d_out, sizeof(double) * GEO_NF * P, cudaMemcpyDeviceToHost, sg.s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, sg.s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(sg.s)) != cudaSuccess)
        return wd_fail(TRANS_E_CUDA, std::string("metrics: ") + cudaGetErrorString(e));
    if (bad) return wd_fail(TRANS_E_ARG, "negative volume");
    return TRANS_OK;
}
