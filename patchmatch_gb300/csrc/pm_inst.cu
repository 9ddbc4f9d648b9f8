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
cudaError_t tile_launch(dim3 grid, cudaStream_t st, const SweepArgs &a, const BandArgs *band) {
    if (band) {
        if (a.propagation == PM_PROPAGATION_PLAIN)
            tile_kernel_banded<PM_INST_S, Img, true><<<band->blocks, kThreads, tile_kernel_smem<PM_INST_S>(), st>>>(
                a, *band);
        else
            tile_kernel_banded<PM_INST_S, Img, false><<<band->blocks, kThreads, tile_kernel_smem<PM_INST_S>(), st>>>(
                a, *band);
        return cudaGetLastError();
    }
    if (a.propagation == PM_PROPAGATION_PLAIN)
        tile_kernel<PM_INST_S, Img, true><<<grid, kThreads, tile_kernel_smem<PM_INST_S>(), st>>>(a);
    else
        tile_kernel<PM_INST_S, Img, false><<<grid, kThreads, tile_kernel_smem<PM_INST_S>(), st>>>(a);
    return cudaGetLastError();
}

template <class Img>
cudaError_t tile_smem_attr() {
    constexpr int dyn = (int)tile_kernel_smem<PM_INST_S>();
    constexpr int blocks = tile_min_blocks<PM_INST_S>(), pblocks = persistent_min_blocks<PM_INST_S>();
    cudaError_t e = cudaFuncSetAttribute(tile_kernel<PM_INST_S, Img, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn);
    e = e ? e : cudaFuncSetAttribute(tile_kernel<PM_INST_S, Img, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn);
    e = e ? e : prefer_l1(tile_kernel<PM_INST_S, Img, false>, dyn, blocks);
    e = e ? e : prefer_l1(tile_kernel<PM_INST_S, Img, true>, dyn, blocks);
    e = e ? e : cudaFuncSetAttribute(batch_kernel<PM_INST_S, Img, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn);
    e = e ? e : cudaFuncSetAttribute(batch_kernel<PM_INST_S, Img, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn);
    e = e ? e : prefer_l1(batch_kernel<PM_INST_S, Img, false>, dyn, pblocks);
    e = e ? e : prefer_l1(batch_kernel<PM_INST_S, Img, true>, dyn, pblocks);
    e = e ? e : cudaFuncSetAttribute(tile_kernel_banded<PM_INST_S, Img, false>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, dyn);
    e = e ? e : cudaFuncSetAttribute(tile_kernel_banded<PM_INST_S, Img, true>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, dyn);
    e = e ? e : prefer_l1(tile_kernel_banded<PM_INST_S, Img, false>, dyn, pblocks);
    return e ? e : prefer_l1(tile_kernel_banded<PM_INST_S, Img, true>, dyn, pblocks);
}

template <class Img>
int banded_occ() {
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, tile_kernel_banded<PM_INST_S, Img, false>, kThreads,
                                                  tile_kernel_smem<PM_INST_S>());
    return n;
}
template <class Img>
cudaError_t hyp_launch(int n, cudaStream_t st, const HypArgs &a) {
    hyp_kernel<PM_INST_S, Img><<<(n + 255) / 256, 256, 0, st>>>(a);
    return cudaGetLastError();
}

template <class Img>
cudaError_t batch_launch_img(bool plain, int blocks, cudaStream_t st, const BatchArgs &b) {
    if (plain)
        batch_kernel<PM_INST_S, Img, true><<<blocks, kThreads, tile_kernel_smem<PM_INST_S>(), st>>>(b);
    else
        batch_kernel<PM_INST_S, Img, false><<<blocks, kThreads, tile_kernel_smem<PM_INST_S>(), st>>>(b);
    return cudaGetLastError();
}

template <class Img>
int batch_occ(bool plain) {
    int n = 0;
    if (plain)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_kernel<PM_INST_S, Img, true>, kThreads, tile_kernel_smem<PM_INST_S>());
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_kernel<PM_INST_S, Img, false>, kThreads,
                                                      tile_kernel_smem<PM_INST_S>());
    return n;
}

}  // namespace (helpers are per translation unit: each compiles one S)

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
cudaError_t launch_tile<PM_INST_S>(int kind, dim3 grid, cudaStream_t st, const SweepArgs &a, const BandArgs *band) {
    switch (kind) {
        case kImageQuadF16: return tile_launch<QuadF16>(grid, st, a, band);
        case kImageTexU8: return tile_launch<TexU8>(grid, st, a, band);
        case kImageTexF16: return tile_launch<TexF16>(grid, st, a, band);
        default: return tile_launch<QuadU8>(grid, st, a, band);
    }
}

template <>
int tile_blocks_per_sm<PM_INST_S>(int kind) {
    switch (kind) {
        case kImageQuadF16: return banded_occ<QuadF16>();
        case kImageTexU8: return banded_occ<TexU8>();
        case kImageTexF16: return banded_occ<TexF16>();
        default: return banded_occ<QuadU8>();
    }
}

template <>
cudaError_t launch_batch<PM_INST_S>(int kind, bool plain, int blocks, cudaStream_t st, const BatchArgs &b) {
    switch (kind) {
        case kImageQuadF16: return batch_launch_img<QuadF16>(plain, blocks, st, b);
        case kImageTexU8: return batch_launch_img<TexU8>(plain, blocks, st, b);
        case kImageTexF16: return batch_launch_img<TexF16>(plain, blocks, st, b);
        default: return batch_launch_img<QuadU8>(plain, blocks, st, b);
    }
}

template <>
int batch_blocks_per_sm<PM_INST_S>(int kind, bool plain) {
    switch (kind) {
        case kImageQuadF16: return batch_occ<QuadF16>(plain);
        case kImageTexU8: return batch_occ<TexU8>(plain);
        case kImageTexF16: return batch_occ<TexF16>(plain);
        default: return batch_occ<QuadU8>(plain);
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
