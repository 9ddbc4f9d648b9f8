// Kernel instantiations for one source count S = PM_INST_S (the build
// compiles this file once per S so the variants compile in parallel).
#include "pm_kernels.h"
#include "pm_sweep.cuh"

#ifndef PM_INST_S
#error "PM_INST_S must be defined"
#endif

namespace pm {

namespace {
template <class Img>
cudaError_t tile_launch(dim3 grid, cudaStream_t st, const SweepArgs &a) {
    tile_kernel<PM_INST_S, Img><<<grid, kThreads, kTileSmemBytes, st>>>(a);
    return cudaGetLastError();
}
}  // namespace

// Opt both image variants in to > 48 KB of dynamic shared memory (called for
// the current device when a context is created).
template <int S>
cudaError_t configure_tile();
template <>
cudaError_t configure_tile<PM_INST_S>() {
    cudaError_t e = cudaFuncSetAttribute(tile_kernel<PM_INST_S, QuadU8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kTileSmemBytes);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(tile_kernel<PM_INST_S, QuadF16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)kTileSmemBytes);
}

template <>
cudaError_t launch_tile<PM_INST_S>(int fmt, dim3 grid, cudaStream_t st, const SweepArgs &a) {
    return fmt == PM_IMAGE_F16 ? tile_launch<QuadF16>(grid, st, a) : tile_launch<QuadU8>(grid, st, a);
}

template <>
cudaError_t launch_hyp<PM_INST_S>(int fmt, int n, cudaStream_t st, const HypArgs &a) {
    const int blocks = (n + 255) / 256;
    if (fmt == PM_IMAGE_F16)
        hyp_kernel<PM_INST_S, QuadF16><<<blocks, 256, 0, st>>>(a);
    else
        hyp_kernel<PM_INST_S, QuadU8><<<blocks, 256, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace pm
