// k_walldist.cu -- wall distance of GEOM_CalcDST (Geom/CalcDst.F90:127-164) on the device.
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

int wd_fail(int code, const std::string& msg) {
    g_stateless_err = msg;
    return code;
}

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
    // panel centres (the reference's expression, in its order) and the coordinate bound R
    std::vector<long long> soff(1, 0);
    for (int s = 0; s < nsurf; ++s) {
        const int ni = dims[2 * s], nj = dims[2 * s + 1];
        if (ni < 1 || nj < 1) return wd_fail(TRANS_E_ARG, "bad surface dimensions");
        soff.push_back(soff.back() + (long long)(ni - 1) * (nj - 1));
    }
    const long long np = soff.back();
    std::vector<double> pan64((size_t)(3 * np));
    std::vector<float> pan32((size_t)(4 * np));
    double R = 0.0;
    {
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
                    pan64[3 * p] = xs; pan64[3 * p + 1] = ys; pan64[3 * p + 2] = zs;
                    pan32[4 * p] = (float)xs; pan32[4 * p + 1] = (float)ys; pan32[4 * p + 2] = (float)zs; pan32[4 * p + 3] = 0.0f;
                    if (!std::isfinite(xs) || !std::isfinite(ys) || !std::isfinite(zs))
                        return wd_fail(TRANS_E_ARG, "surface coordinates not finite");
                    R = std::max(R, std::max(std::fabs(xs), std::max(std::fabs(ys), std::fabs(zs))));
                }
            base += 3 * plane;
        }
    }
    for (long long q = 0; q < 3 * n; ++q) {
        if (!std::isfinite(xyz[q])) return wd_fail(TRANS_E_ARG, "point coordinates not finite");
        R = std::max(R, std::fabs(xyz[q]));
    }
    if (R > 1.0e18) return wd_fail(TRANS_E_ARG, "coordinates beyond 1e18");   // FP32 squares stay finite
    const float eabs = std::max((float)(1.0e-6 * R), 1.0e-37f);

    cudaStream_t st = nullptr;
    double *d_pts = nullptr, *d_p64 = nullptr, *d_dst = nullptr;
    float4* d_p32 = nullptr;
    long long* d_off = nullptr;
    int rc = TRANS_OK;
    auto ck = [&](cudaError_t e, const char* what) {
        if (e != cudaSuccess && rc == TRANS_OK) rc = wd_fail(TRANS_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
        return rc == TRANS_OK;
    };
    if (ck(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream") &&
        ck(cudaMalloc(&d_pts, sizeof(double) * 3 * (size_t)n), "malloc") &&
        ck(cudaMalloc(&d_dst, sizeof(double) * (size_t)n), "malloc") &&
        ck(cudaMalloc(&d_p64, sizeof(double) * std::max<size_t>(1, pan64.size())), "malloc") &&
        ck(cudaMalloc(&d_p32, sizeof(float4) * std::max<size_t>(1, (size_t)np)), "malloc") &&
        ck(cudaMalloc(&d_off, sizeof(long long) * soff.size()), "malloc") &&
        ck(cudaMemcpyAsync(d_pts, xyz, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice, st), "copy") &&
        ck(cudaMemcpyAsync(d_p64, pan64.data(), sizeof(double) * pan64.size(), cudaMemcpyHostToDevice, st), "copy") &&
        ck(cudaMemcpyAsync(d_p32, pan32.data(), sizeof(float) * pan32.size(), cudaMemcpyHostToDevice, st), "copy") &&
        ck(cudaMemcpyAsync(d_off, soff.data(), sizeof(long long) * soff.size(), cudaMemcpyHostToDevice, st), "copy")) {
        const unsigned grid = (unsigned)((n + WD_THREADS - 1) / WD_THREADS);
        k_wall_distance<<<grid, WD_THREADS, 0, st>>>(n, d_pts, d_p32, d_p64, d_off, nsurf, eabs, tiny, d_dst);
        if (ck(cudaGetLastError(), "launch"))
            ck(cudaMemcpyAsync(dst, d_dst, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, st), "copy");
        ck(cudaStreamSynchronize(st), "sync");
    }
    cudaFree(d_pts); cudaFree(d_dst); cudaFree(d_p64); cudaFree(d_p32); cudaFree(d_off);
    if (st) cudaStreamDestroy(st);
    return rc;
}
