// noalloc.cu -- TIME_Update_V with its per-tile norm partials in a fixed device buffer.
//
// The buffer is a file-scope __device__ array, part of the loaded library image: the call
// makes no device or page-locked host allocation of any kind.  Its address is taken once per
// device with cudaGetSymbolAddress, with that device current, on the first call made on it
// (that lookup may load the library's device code on the device if nothing has yet, so the
// first call should come before any stream capture), and handed to the kernel as a plain
// pointer.  All contexts and calls share the array and it keeps the last call's contents;
// every entry a call reads is written earlier in the same call, so nothing needs clearing.
// Calls that overlap (two host threads, or two contexts whose streams run concurrently) race
// on it.  The context must already be built (by trans_prepare, a stage or an iteration):
// building it allocates its work lists, so an unbuilt context is refused, not built here.
#include <algorithm>
#include <mutex>
#include <string>

#include "engine.h"

using namespace tg;
using namespace tg::eng;

namespace {
constexpr int kStaticNormTiles = 65536;              // 16,777,216 interior cells; 4 MiB
static __device__ __align__(256) NormPart g_norm_scratch[kStaticNormTiles];
constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
NormPart* g_scratch_ptr[kMaxDevices] = {};

int static_norm_scratch(Ctx* c, NormPart** out) {
    int dev = -1;
    CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(c, TRANS_E_ARG, "device ordinal beyond the static scratch table");
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_norm_scratch);
        if (e != cudaSuccess)
            return fail(c, TRANS_E_CUDA, std::string("cudaGetSymbolAddress(static norm scratch): ") + cudaGetErrorString(e));
        g_scratch_ptr[dev] = static_cast<NormPart*>(ptr);
    }
    *out = g_scratch_ptr[dev];
    return TRANS_OK;
}
}  // namespace

extern "C" int trans_update_static_scratch(void* ctx, int ki, trans_norms* norms) {
    Ctx* c = static_cast<Ctx*>(ctx);
    if (!c || c->cases.empty()) return TRANS_E_ARG;
    if (c->cases[0]->p.IF_RK == 1) return fail(c, TRANS_E_ARG, "trans_update_static_scratch is TIME_Update_V: LU-SGS cases only");
    int rc;
    if (!c->built)      // building the work lists would allocate device memory
        return fail(c, TRANS_E_ARG, "trans_update_static_scratch: the context is not built yet; call trans_prepare, "
                                    "trans_run_stage or trans_iterate first");
    if (c->cell_tiles.size() > (size_t)kStaticNormTiles)
        return fail(c, TRANS_E_ARG, "trans_update_static_scratch: " + std::to_string(c->cell_tiles.size()) +
                    " cell tiles exceed the static scratch of 65536 tiles (16,777,216 interior cells)");
    NormPart* scratch = nullptr;
    if ((rc = static_norm_scratch(c, &scratch))) return rc;
    for (CaseRec* cs : c->cases) cs->KI = ki;
    if ((rc = finalize_geometry(c))) return rc;
    if ((rc = upload_cdev(c))) return rc;
    if (c->mixed) launch_update_mixed(c->stream, c->d_blk, c->d_cell, (int)c->cell_tiles.size(), c->d_cdev, scratch);
    else launch_update(c->stream, c->d_blk, c->d_cell, (int)c->cell_tiles.size(), c->d_cdev, scratch, 0);
    c->launches++;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(c->h_parts.data(), scratch, sizeof(NormPart) * c->h_parts.size(), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    // a cooperative sweep of this iteration that gave up on a bounded wait left DeltaQ partial
    if (c->sweep_mode >= 1 && c->sweep_mode <= 3 && c->h_sync->err) return fail(c, TRANS_E_TIMEOUT, "LU-SGS sweep wait timed out");
    rc = reduce_norms(c);
    if (norms) std::copy(c->cases[0]->norms.begin(), c->cases[0]->norms.end(), norms);
    return rc;
}
