// flux_inst.cuh -- instantiation of the templated flux/source/sweep kernels for one type R.
// Included once per precision translation unit with TG_R and TG_NAME defined.
#include "kernels.cuh"
#include "launch.h"

namespace tg {
namespace {
template <int DIR>
void ff(cudaStream_t s, const DevBlock* b, const Tile* t, int nt, const Params& p, int turb) {
    if (nt > 0) k_face_flux<TG_R, DIR><<<nt, FACE_TILE, 0, s>>>(b, t, p, turb);
}
void ga(cudaStream_t s, const DevBlock* b, const Tile* t, int nt, int turb) {
    if (nt > 0) k_gather<TG_R><<<nt, CELL_TILE, 0, s>>>(b, t, turb);
}
void fc(cudaStream_t s, const DevBlock* b, const Tile* t, int nt, const Params& p) {
    if (nt > 0) k_sst_fc1<TG_R><<<nt, CELL_TILE, 0, s>>>(b, t, p);
}
void rh(cudaStream_t s, const DevBlock* b, const Tile* t, int nt, const Params& p, int turb) {
    if (nt > 0) k_lusgs_rhs<TG_R><<<nt, CELL_TILE, 0, s>>>(b, t, p, turb);
}
void swl(cudaStream_t s, const DevBlock* b, const SweepCell* c, int first, int count, int turb) {
    if (count > 0) k_sweep<TG_R, true><<<(count + 31) / 32, 32, 0, s>>>(b, c, first, count, turb);
}
void swu(cudaStream_t s, const DevBlock* b, const SweepCell* c, int first, int count, int turb) {
    if (count > 0) k_sweep<TG_R, false><<<(count + 31) / 32, 32, 0, s>>>(b, c, first, count, turb);
}
}  // namespace

const FluxLaunchers& TG_NAME() {
    static const FluxLaunchers L = {{ff<1>, ff<2>, ff<3>}, ga, fc, rh, swl, swu};
    return L;
}
}  // namespace tg
