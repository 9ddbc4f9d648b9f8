// The batched executor's mixed kernel: one persistent launch per phase over
// requests of any source count.  Each work item carries its request's source
// count and the CTA dispatches to the tile visit compiled for it.  The kernel
// is compiled once per image variant (PM_MIXED_KIND) and holds all ten
// source-count bodies, so its register budget is that of the largest.
#include <type_traits>

#include "pm_kernels.h"
#include "pm_sweep.cuh"

#ifndef PM_MIXED_KIND
#error "PM_MIXED_KIND must be defined"
#endif

namespace pm {

namespace {

using MixedImg = typename std::conditional<
    PM_MIXED_KIND == kImageQuadF16, QuadF16,
    typename std::conditional<PM_MIXED_KIND == kImageTexU8, TexU8,
                              typename std::conditional<PM_MIXED_KIND == kImageTexF16, TexF16, QuadU8>::type>::type>::type;

template <int S, bool Plain>
__device__ __forceinline__ void visit(const SweepArgs &sa, int bx, int by, float4 *tile) {
    tile_body<S, MixedImg, Plain, SharedAccess>(sa, bx, by, tile);
}

template <bool Plain>
__global__ void __launch_bounds__(kThreads, 2 * kCtaScale) batch_mixed_kernel(const __grid_constant__ BatchArgs b) {
    extern __shared__ float4 tile[];
    __shared__ SweepArgs sa;
    __shared__ int s_item;
    for (;;) {
        if (threadIdx.x == 0) s_item = (int)atomicAdd(b.counter, 1u);
        __syncthreads();
        const int it = s_item;
        if (it >= b.n_items) return;
        const int4 w = b.items[it];  // (request, tile x, tile y, source count)
        const int4 *src = reinterpret_cast<const int4 *>(b.args + w.x);
        int4 *dst = reinterpret_cast<int4 *>(&sa);
        for (int k = threadIdx.x; k < (int)(sizeof(SweepArgs) / 16); k += blockDim.x) dst[k] = src[k];
        __syncthreads();
        if (threadIdx.x == 0) {
            sa.mode = b.mode;
            sa.colour = b.colour;
            sa.sweep = b.sweep;
        }
        __syncthreads();
        switch (w.w) {
            case 1: visit<1, Plain>(sa, w.y, w.z, tile); break;
            case 2: visit<2, Plain>(sa, w.y, w.z, tile); break;
            case 3: visit<3, Plain>(sa, w.y, w.z, tile); break;
            case 4: visit<4, Plain>(sa, w.y, w.z, tile); break;
            case 5: visit<5, Plain>(sa, w.y, w.z, tile); break;
            case 6: visit<6, Plain>(sa, w.y, w.z, tile); break;
            case 7: visit<7, Plain>(sa, w.y, w.z, tile); break;
            case 8: visit<8, Plain>(sa, w.y, w.z, tile); break;
            case 9: visit<9, Plain>(sa, w.y, w.z, tile); break;
            default: visit<10, Plain>(sa, w.y, w.z, tile); break;
        }
        __syncthreads();  // before the next item replaces the arguments and the tile
    }
}

}  // namespace

template <>
cudaError_t launch_batch_mixed<PM_MIXED_KIND>(bool plain, int blocks, cudaStream_t st, const BatchArgs &b) {
    if (plain)
        batch_mixed_kernel<true><<<blocks, kThreads, tile_kernel_smem_max(), st>>>(b);
    else
        batch_mixed_kernel<false><<<blocks, kThreads, tile_kernel_smem_max(), st>>>(b);
    return cudaGetLastError();
}

template <>
cudaError_t configure_batch_mixed<PM_MIXED_KIND>() {
    constexpr int dyn = (int)tile_kernel_smem_max();
    cudaError_t e = cudaFuncSetAttribute(batch_mixed_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn);
    return e ? e : cudaFuncSetAttribute(batch_mixed_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn);
}

template <>
int batch_mixed_blocks_per_sm<PM_MIXED_KIND>(bool plain) {
    int n = 0;
    if (plain)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_mixed_kernel<true>, kThreads, tile_kernel_smem_max());
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_mixed_kernel<false>, kThreads, tile_kernel_smem_max());
    return n;
}

}  // namespace pm
