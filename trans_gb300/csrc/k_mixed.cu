// k_mixed.cu -- FP32 instantiation of the flux, source and sweep kernels (mixed-precision mode).
// Compiled with fused multiply-add enabled.
#define TG_R float
#define TG_NAME flux_launchers_f32
#include "flux_inst.cuh"
#include "kernels_mixed.cuh"
#include "resid_tma.cuh"

namespace tg {
cudaError_t prepare_resid_tma() {
    cudaError_t e = cudaFuncSetAttribute(k_resid_tma<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rt_smem_bytes(1));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_resid_tma<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rt_smem_bytes(2));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_resid_tma<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rt_smem_bytes(3));
    return e;
}
// cluster-barrier sweeps: cs CTAs of bs threads per solver block
static cudaLaunchConfig_t cluster_cfg(cudaStream_t s, int nblk, int cs, int bs, cudaLaunchAttribute* attr) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(nblk * cs));
    cfg.blockDim = dim3((unsigned)bs);
    cfg.stream = s;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)cs;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cfg;
}
int sweep_cluster_fits(int cs, int bs) {
    if (cs > 8 && cudaFuncSetAttribute(k_sweep_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = cluster_cfg(nullptr, 1, cs, bs, attr);
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, k_sweep_cluster, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}
cudaError_t launch_sweep_cluster(cudaStream_t s, const SweepView& v, const int* pb_off, int nh, int nblk, int turb, int cs, int bs,
                                 int pf) {
    if (nblk <= 0 || v.n <= 0) return cudaSuccess;
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = cluster_cfg(s, nblk, cs, bs, attr);
    return cudaLaunchKernelEx(&cfg, k_sweep_cluster, (const int*)v.nbp, (const float*)v.rec, (float*)v.dq, pb_off, nh, nblk,
                              turb, pf);
}
void launch_resid_tma(int dir, cudaStream_t s, const DevBlock* blks, const ResidTile* tiles, int nt, const CaseDev* cdev,
                      const void* maps, int* err, unsigned limit) {
    if (nt <= 0) return;
    const CUtensorMap* m = (const CUtensorMap*)maps;
    if (dir == 1) k_resid_tma<1><<<nt, 32 * RT_R1, rt_smem_bytes(1), s>>>(blks, tiles, cdev, m, err, limit);
    else if (dir == 2) k_resid_tma<2><<<nt, RT_FACES, rt_smem_bytes(2), s>>>(blks, tiles, cdev, m, err, limit);
    else k_resid_tma<3><<<nt, RT_FACES, rt_smem_bytes(3), s>>>(blks, tiles, cdev, m, err, limit);
}
void launch_specrad_mixed(cudaStream_t s, const DevBlock* blks, const Tile* tiles, int nt, const CaseDev* cdev) {
    if (nt > 0) k_specrad_mixed<<<nt, CELL_TILE, 0, s>>>(blks, tiles, cdev);
}
void launch_bc_outlet_mixed(cudaStream_t s, const DevBlock* blks, const BCEntry* ent, const OutletLine* lines, int nl,
                            const CaseDev* cdev) {
    if (nl > 0) k_bc_outlet_mixed<<<(nl + 3) / 4, 128, 0, s>>>(blks, ent, lines, nl, cdev);     // a warp per line
}
void launch_prims_mixed(cudaStream_t s, const DevBlock* blks, int nblk, long long total, const long long* off) {
    if (total > 0) k_prims_mixed<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(blks, nblk, total, off);
}
void launch_update_mixed(cudaStream_t s, const DevBlock* blks, const Tile* tiles, int nt, const CaseDev* cdev, NormPart* parts) {
    if (nt > 0) k_update_mixed<<<nt, CELL_TILE, 0, s>>>(blks, tiles, cdev, parts);
}
}  // namespace tg

// Throughput probes of the FP64 and FP32 pipes (independent fused multiply-add chains in
// every thread of a grid covering all SMs); used to state the compute roof of the kernels.
namespace tg {
template <typename T>
__global__ void k_fma_probe(T* out, int iters, T a, T b) {
    T x0 = (T)threadIdx.x, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3;
    T x4 = x0 + (T)4, x5 = x0 + (T)5, x6 = x0 + (T)6, x7 = x0 + (T)7;
    for (int q = 0; q < iters; ++q) {
        x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
        x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
    }
    T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == (T)-1.2345) out[blockIdx.x] = s;      // keeps the chains alive
}

double probe_fma_gflops(int fp64) {
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    int blocks = nsm * 8, threads = 256, iters = fp64 ? 2000 : 40000;
    void* out = nullptr;
    if (cudaMalloc(&out, sizeof(double) * blocks) != cudaSuccess) return -1.0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0); cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0);
        if (fp64) k_fma_probe<double><<<blocks, threads>>>((double*)out, iters, 0.999999, 1e-7);
        else k_fma_probe<float><<<blocks, threads>>>((float*)out, iters, 0.999999f, 1e-7f);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0) best = ms < best ? ms : best;
    }
    cudaEventDestroy(e0); cudaEventDestroy(e1);
    cudaFree(out);
    double flops = 2.0 * 8.0 * (double)iters * blocks * threads;
    return flops / (best * 1e-3) / 1e9;
}

// Floor of one dependent step of the hyperplane sweeps: a chain of launches of `grid` CTAs of
// SWEEP_CTA threads where each thread reads, after the previous launch completed, a value the
// previous launch wrote (through L2) and writes it back incremented -- the kernel boundary,
// one dependent L2 round trip and the launch, without the sweep arithmetic.  Replayed as a
// CUDA graph like the sweeps, with programmatic dependent launch when `chained`.
__global__ void k_chain_probe(int* buf, int chained) {
    if (chained) asm volatile("griddepcontrol.wait;" ::: "memory");
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int x = __ldcg(buf + t);
    if (chained) asm volatile("griddepcontrol.launch_dependents;");
    buf[t] = x + 1;
}

double probe_chain_us(int chained, int grid) {
    const int n = 512;
    if (grid < 1) grid = 1;
    int* buf = nullptr;
    if (cudaMalloc(&buf, sizeof(int) * (size_t)grid * SWEEP_CTA) != cudaSuccess) return -1.0;
    cudaMemset(buf, 0, sizeof(int) * (size_t)grid * SWEEP_CTA);
    cudaStream_t s;
    cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    double us = -1.0;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(SWEEP_CTA);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = chained ? 1 : 0;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        for (int q = 0; q < n; ++q) cudaLaunchKernelEx(&cfg, k_chain_probe, buf, chained);
        if (cudaStreamEndCapture(s, &g) == cudaSuccess && cudaGraphInstantiate(&ge, g, 0) == cudaSuccess) {
            cudaEvent_t e0, e1;
            cudaEventCreate(&e0); cudaEventCreate(&e1);
            float best = 1e30f;
            for (int rep = 0; rep < 4; ++rep) {
                cudaEventRecord(e0, s);
                cudaGraphLaunch(ge, s);
                cudaEventRecord(e1, s);
                cudaEventSynchronize(e1);
                float ms = 0;
                cudaEventElapsedTime(&ms, e0, e1);
                if (rep > 0) best = ms < best ? ms : best;
            }
            cudaEventDestroy(e0); cudaEventDestroy(e1);
            us = best * 1e3 / n;
        }
    }
    if (ge) cudaGraphExecDestroy(ge);
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    cudaStreamDestroy(s);
    cudaFree(buf);
    return us;
}
}  // namespace tg

// ---------------------------------------------------------------------------------------
// Check of the integer-pipe conversions (cvt.cuh) against the hardware conversions: n bit
// patterns from a counter-based generator (seed), a quarter each uniform over all doubles,
// with exponents around the float range, at and next to rounding ties, and float patterns for
// float -> double; the first CVT_NSPECIAL indices take the fixed patterns below.  NaN results
// compare equal to NaN results.
// ---------------------------------------------------------------------------------------
namespace tg {
namespace {
constexpr int CVT_NSPECIAL = 16;
__constant__ unsigned long long cvt_special[CVT_NSPECIAL] = {
    0x0000000000000000ull, 0x8000000000000000ull,    // +-0
    0x7ff0000000000000ull, 0xfff0000000000000ull,    // +-inf
    0x7ff8000000000000ull, 0x0000000000000001ull,    // NaN, the smallest double
    0x47efffffe0000000ull, 0x47efffffefffffffull,    // the largest float; just below its rounding tie
    0x47effffff0000000ull, 0x3810000000000000ull,    // the tie to infinity; the smallest normal float
    0x380fffffffffffffull, 0x3690000000000000ull,    // just below it (a float subnormal); 2^-150
    0x3ff0000010000000ull, 0x3ff0000030000000ull,    // 1 + half an ulp (to even: 1), 1 + 1.5 ulp (up)
    0xbff0000010000001ull, 0x3fefffffffffffffull};   // -(1 + just above half an ulp), 1 - 2^-53
__device__ __forceinline__ unsigned long long cvt_mix(unsigned long long z) {
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
__global__ void k_check_cvt(long long n, unsigned long long seed, unsigned long long* __restrict__ bad) {
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n) return;
    const unsigned long long z = cvt_mix((unsigned long long)g ^ (seed * 0x2545f4914f6cdd1dull));
    unsigned long long u;
    const int kind = (int)(g & 3);
    if (g < CVT_NSPECIAL) {
        u = cvt_special[g];
        const unsigned f = (unsigned)(u >> 32) ^ (unsigned)u;     // a float pattern from it too
        const double a = f64_of(__uint_as_float(f)), h = (double)__uint_as_float(f);
        if (__double_as_longlong(a) != __double_as_longlong(h) && !(isnan(a) && isnan(h))) atomicAdd(bad + 1, 1ull);
    } else if (kind == 0) {
        u = z;
    } else if (kind == 1) {                                       // exponents 880..1170
        u = (z & 0x800fffffffffffffull) | ((880ull + (z >> 55) % 291ull) << 52);
    } else if (kind == 2) {                                       // the tie, one below, one or two above
        const unsigned long long m = ((z & 0xfffffe0000000ull) | 0x10000000ull) + ((z >> 40) & 3ull) - 1ull;
        u = (z & 0x8000000000000000ull) | ((890ull + (z >> 55) % 270ull) << 52) | (m & 0xfffffffffffffull);
    } else {                                                      // float -> double
        const unsigned f = (unsigned)z;
        const double a = f64_of(__uint_as_float(f)), h = (double)__uint_as_float(f);
        if (__double_as_longlong(a) != __double_as_longlong(h) && !(isnan(a) && isnan(h))) atomicAdd(bad + 1, 1ull);
        return;
    }
    const double x = __longlong_as_double((long long)u);
    const float a = f32_rn(x), h = (float)x;
    if (__float_as_uint(a) != __float_as_uint(h) && !(isnan(a) && isnan(h))) atomicAdd(bad, 1ull);
}
}  // namespace

cudaError_t check_conversions(long long n, unsigned long long seed, long long* mismatches) {
    unsigned long long* d = nullptr;
    cudaError_t e = cudaMalloc(&d, 2 * sizeof(unsigned long long));
    if (e != cudaSuccess) return e;
    unsigned long long h[2] = {0, 0};
    e = cudaMemset(d, 0, sizeof(h));
    if (e == cudaSuccess) {
        k_check_cvt<<<(unsigned)((n + 255) / 256), 256>>>(n, seed, d);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    mismatches[0] = (long long)h[0];
    mismatches[1] = (long long)h[1];
    return e;
}
}  // namespace tg
