// k_mixed.cu -- FP32 instantiation of the flux, source and sweep kernels (mixed-precision mode).
// Compiled with fused multiply-add enabled.
#define TG_R float
#define TG_NAME flux_launchers_f32
#include "flux_inst.cuh"
