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
    if (a.propagation == PM_PROPAGATION_PLAIN)
        tile_kernel<PM_INST_S, Img, true><<<grid, kThreads, kTileSmemBytes, st>>>(a);
    else
        tile_kernel<PM_INST_S, Img, false><<<grid, kThreads, kTileSmemBytes, st>>>(a);
    return cudaGetLastError();
}
}  // namespace

namespace {
template <class Img>
cudaError_t tile_smem_attr() {
    cudaError_t e = cudaFuncSetAttribute(tile_kernel<PM_INST_S, Img, false>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTileSmemBytes);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(tile_kernel<PM_INST_S, Img, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)kTileSmemBytes);
}
template <class Img>
cudaError_t hyp_launch(int n, cudaStream_t st, const HypArgs &a) {
    hyp_kernel<PM_INST_S, Img><<<(n + 255) / 256, 256, 0, st>>>(a);
    return cudaGetLastError();
}
}  // namespace

// Set the dynamic shared memory limit of every image variant (called for the
// current device when a context is created).
template <int S>
cudaError_t configure_tile();
template <>
cudaError_t configure_tile<PM_INST_S>() {
    cudaError_t e = tile_smem_attr<QuadU8>();
    e = e ? e : tile_smem_attr<QuadF16>();
    e = e ? e : tile_smem_attr<TexU8>();
    return e ? e : tile_smem_attr<TexF16>();
}

// kind: kImageQuadU8, kImageQuadF16, kImageTexU8, kImageTexF16
template <>
cudaError_t launch_tile<PM_INST_S>(int kind, dim3 grid, cudaStream_t st, const SweepArgs &a) {
    switch (kind) {
        case kImageQuadF16: return tile_launch<QuadF16>(grid, st, a);
        case kImageTexU8: return tile_launch<TexU8>(grid, st, a);
        case kImageTexF16: return tile_launch<TexF16>(grid, st, a);
        default: return tile_launch<QuadU8>(grid, st, a);
    }
}

template <>
cudaError_t launch_hyp<PM_INST_S>(int kind, int n, cudaStream_t st, const HypArgs &a) {
    switch (kind) {
        case kImageQuadF16: return hyp_launch<QuadF16>(n, st, a);
        case kImageTexU8: return hyp_launch<TexU8>(n, st, a);
        case kImageTexF16: return hyp_launch<TexF16>(n, st, a);
        default: return hyp_launch<QuadU8>(n, st, a);
    }
}

}  // namespace pm
