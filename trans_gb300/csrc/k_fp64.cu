// k_fp64.cu -- FP64 kernels of the hot path.  Compiled with -fmad=false so that every FP64
// expression rounds exactly as the reference's (built with -fp-model strict) would.
#define TG_R double
#define TG_NAME flux_launchers_f64
#define TG_COMMON_KERNELS
#include "flux_inst.cuh"

namespace tg {
void launch_specrad(cudaStream_t s, const DevBlock* blks, const Tile* tiles, int nt, const CaseDev* cdev) {
    if (nt > 0) k_specrad<<<nt, CELL_TILE, 0, s>>>(blks, tiles, cdev);
}
void launch_bc_state(cudaStream_t s, const DevBlock* blks, const BCEntry* ent, int n, const CaseDev* cdev) {
    if (n > 0) k_bc_state<<<(n + 127) / 128, 128, 0, s>>>(blks, ent, n, cdev);
}
void launch_bc_outlet(cudaStream_t s, const DevBlock* blks, const BCEntry* ent, const OutletLine* lines, int nl,
                      const CaseDev* cdev) {
    if (nl > 0) k_bc_outlet<<<(nl + 3) / 4, 128, 0, s>>>(blks, ent, lines, nl, cdev);     // a warp per line
}
void launch_prims(cudaStream_t s, const DevBlock* blks, int nblk, long long total, const long long* off) {
    if (total > 0) k_prims<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(blks, nblk, total, off);
}
void launch_update(cudaStream_t s, const DevBlock* blks, const Tile* tiles, int nt, const CaseDev* cdev, NormPart* parts,
                   int d_fp32) {
    if (nt > 0) k_update<<<nt, CELL_TILE, 0, s>>>(blks, tiles, cdev, parts, d_fp32);
}
void launch_rk_update(cudaStream_t s, const DevBlock* blks, const Tile* tiles, int nt, NormPart* parts, int d_fp32, int itr) {
    if (nt > 0) k_rk_update<<<nt, CELL_TILE, 0, s>>>(blks, tiles, parts, d_fp32, itr);
}
void launch_rk_vupdate(cudaStream_t s, const DevBlock* blks, const Tile* tiles, int nt, const CaseDev* cdev, NormPart* parts,
                       int d_fp32) {
    if (nt > 0) k_rk_vupdate<<<nt, CELL_TILE, 0, s>>>(blks, tiles, cdev, parts, d_fp32);
}
void launch_mirror(cudaStream_t s, const DevBlock* blks, int nblk, long long total, const long long* off, const MirrorList& ml) {
    if (total > 0) k_mirror<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(blks, nblk, total, off, ml);
}
void launch_block_norms(cudaStream_t s, const DevBlock* blks, int nblk, const NormPart* parts, const int* tile_first,
                        BlockNorms* out) {
    if (nblk > 0) k_block_norms<<<nblk, 256, 0, s>>>(blks, parts, tile_first, out);
}
void launch_update_u(cudaStream_t s, const DevBlock* blks, const Tile* tiles, int nt, const CaseDev* cdev) {
    if (nt > 0) k_update_u<<<nt, CELL_TILE, 0, s>>>(blks, tiles, cdev);
}
void launch_geom_static(cudaStream_t s, const DevBlock* blks, int nblk, long long total, const long long* off) {
    if (total > 0) k_geom_static<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(blks, nblk, total, off);
}
}  // namespace tg

namespace tg {
void launch_halo_pack(cudaStream_t s, const DevBlock& b, const int* cells, int n, int sweep, int dq_fp32, double* out) {
    if (n > 0) k_halo_pack<<<(n + 127) / 128, 128, 0, s>>>(b, cells, n, sweep, dq_fp32, out);
}
void launch_fields_xfer(cudaStream_t s, const XferBatch& x, long long total, int to_slots, int chunk) {
    if (total > 0) k_fields_xfer<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(x, total, to_slots, chunk);
}
void launch_field_xfer(cudaStream_t s, const DevBlock& b, int slot0, int ncomp, int lb, int is_sd, double* stage, int to_slots) {
    long long n = (long long)(b.NI + 3 - lb) * (b.NJ + 3 - lb) * (b.NK + 3 - lb) * ncomp;
    if (n > 0) k_field_xfer<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(b, slot0, ncomp, lb, is_sd, stage, to_slots);
}
}  // namespace tg
