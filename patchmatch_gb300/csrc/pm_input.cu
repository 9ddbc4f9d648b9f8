// Input preparation on the GPU: the keyframe thumbnails the densifier reads
// (data/frame.cc:53-54,136-138: gray and mask resized to the densification
// size, colour thumbnail via set_rgb_thumb) and the FP16 image pyramid of the
// precision form.  All buffers are caller-owned device memory; work is
// enqueued on the context's stream.
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "pm_gb300.h"

namespace {

// Colour -> gray with the BT.601 weights in 14-bit fixed point, rounded
// (0.299, 0.587, 0.114 -> 4899, 9617, 1868 of 16384; the published
// fixed-point form of COLOR_BGR2GRAY, util/image_converter.cc:8-39).
__global__ void to_gray_kernel(const uint8_t *src, int W, int H, size_t pitch, int ch, int rgb, uint8_t *dst,
                               size_t dpitch) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    const uint8_t *p = src + (size_t)y * pitch + (size_t)x * ch;
    uint8_t g;
    if (ch == 1) {
        g = p[0];
    } else {
        const uint32_t b = rgb ? p[2] : p[0], gg = p[1], r = rgb ? p[0] : p[2];
        g = (uint8_t)((r * 4899u + gg * 9617u + b * 1868u + 8192u) >> 14);
    }
    dst[(size_t)y * dpitch + x] = g;
}

// Bilinear resize with pixel-centre alignment (source coordinate
// (x + 0.5) * sw / dw - 0.5, clamped to the image) and 11-bit fixed-point
// weights, rounded once at the end: the scheme of an 8-bit linear resize
// (cv::resize INTER_LINEAR).  ch interleaved channels.
__global__ void resize_kernel(const uint8_t *src, int sw, int sh, size_t spitch, int ch, uint8_t *dst, int dw, int dh,
                              size_t dpitch) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= dw || y >= dh) return;
    // separately rounded operations (no contraction), as the restatement computes them
    const float fx0 = __fsub_rn(__fmul_rn(__fadd_rn((float)x, 0.5f), __fdiv_rn((float)sw, (float)dw)), 0.5f);
    const float fy0 = __fsub_rn(__fmul_rn(__fadd_rn((float)y, 0.5f), __fdiv_rn((float)sh, (float)dh)), 0.5f);
    int sx = (int)floorf(fx0), sy = (int)floorf(fy0);
    float fx = fx0 - (float)sx, fy = fy0 - (float)sy;
    if (sx < 0) { sx = 0; fx = 0.f; }
    if (sx >= sw - 1) { sx = sw - 1; fx = 0.f; }
    if (sy < 0) { sy = 0; fy = 0.f; }
    if (sy >= sh - 1) { sy = sh - 1; fy = 0.f; }
    const int cx1 = __float2int_rn(fx * 2048.f), cx0 = 2048 - cx1;
    const int cy1 = __float2int_rn(fy * 2048.f), cy0 = 2048 - cy1;
    const int sx1 = min(sx + 1, sw - 1), sy1 = min(sy + 1, sh - 1);
    const uint8_t *r0 = src + (size_t)sy * spitch, *r1 = src + (size_t)sy1 * spitch;
    for (int c = 0; c < ch; ++c) {
        const int a = r0[(size_t)sx * ch + c] * cx0 + r0[(size_t)sx1 * ch + c] * cx1;
        const int b = r1[(size_t)sx * ch + c] * cx0 + r1[(size_t)sx1 * ch + c] * cx1;
        const int v = (a * cy0 + b * cy1 + (1 << 21)) >> 22;
        dst[(size_t)y * dpitch + (size_t)x * ch + c] = (uint8_t)min(max(v, 0), 255);
    }
}

// FP16 pyramid: level 0 = the image; level k+1 entry (y, x) = mean of the 2x2
// block (2y, 2x) of level k (rows/columns past the edge repeat the last one),
// summed in FP32 (exact for FP16 inputs) and rounded once to FP16.
__global__ void u8_to_half_kernel(const uint8_t *src, int W, int H, size_t pitch, __half *dst) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    dst[(size_t)y * W + x] = __float2half_rn((float)src[(size_t)y * pitch + x]);
}

__global__ void half_down_kernel(const __half *src, int sw, int sh, __half *dst, int dw, int dh) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= dw || y >= dh) return;
    const int x0 = min(2 * x, sw - 1), x1 = min(2 * x + 1, sw - 1);
    const int y0 = min(2 * y, sh - 1), y1 = min(2 * y + 1, sh - 1);
    const float s = __half2float(src[(size_t)y0 * sw + x0]) + __half2float(src[(size_t)y0 * sw + x1]) +
                    __half2float(src[(size_t)y1 * sw + x0]) + __half2float(src[(size_t)y1 * sw + x1]);
    dst[(size_t)y * dw + x] = __float2half_rn(0.25f * s);
}

dim3 grid2(int W, int H) { return dim3((W + 31) / 32, (H + 7) / 8); }

}  // namespace

extern "C" {

void *pm_stream(const pm_ctx *ctx);

int pm_image_to_gray(pm_ctx *ctx, const void *src, int W, int H, size_t pitch, int channels, int order, void *gray,
                     size_t gray_pitch) {
    if (!ctx || !src || !gray || W < 1 || H < 1 || (channels != 1 && channels != 3 && channels != 4) ||
        (order != PM_ORDER_BGR && order != PM_ORDER_RGB) || pitch < (size_t)W * channels || gray_pitch < (size_t)W)
        return PM_EINVAL;
    cudaStream_t st = (cudaStream_t)pm_stream(ctx);
    to_gray_kernel<<<grid2(W, H), dim3(32, 8), 0, st>>>((const uint8_t *)src, W, H, pitch, channels,
                                                        order == PM_ORDER_RGB, (uint8_t *)gray, gray_pitch);
    return cudaGetLastError() == cudaSuccess ? PM_OK : PM_ECUDA;
}

int pm_image_resize(pm_ctx *ctx, const void *src, int sw, int sh, size_t spitch, int channels, void *dst, int dw,
                    int dh, size_t dpitch) {
    if (!ctx || !src || !dst || sw < 1 || sh < 1 || dw < 1 || dh < 1 || channels < 1 || channels > 4 ||
        spitch < (size_t)sw * channels || dpitch < (size_t)dw * channels)
        return PM_EINVAL;
    cudaStream_t st = (cudaStream_t)pm_stream(ctx);
    resize_kernel<<<grid2(dw, dh), dim3(32, 8), 0, st>>>((const uint8_t *)src, sw, sh, spitch, channels,
                                                         (uint8_t *)dst, dw, dh, dpitch);
    return cudaGetLastError() == cudaSuccess ? PM_OK : PM_ECUDA;
}

int pm_build_pyramid_f16(pm_ctx *ctx, const void *src, int W, int H, size_t pitch, int src_format, int levels,
                         void *const *out) {
    const size_t es = src_format == PM_IMAGE_F16 ? 2 : 1;
    if (!ctx || !src || !out || W < 1 || H < 1 || levels < 1 || levels > 16 || pitch < (size_t)W * es ||
        (src_format != PM_IMAGE_U8 && src_format != PM_IMAGE_F16))
        return PM_EINVAL;
    for (int k = 0; k < levels; ++k)
        if (!out[k]) return PM_EINVAL;
    cudaStream_t st = (cudaStream_t)pm_stream(ctx);
    if (src_format == PM_IMAGE_U8) {
        u8_to_half_kernel<<<grid2(W, H), dim3(32, 8), 0, st>>>((const uint8_t *)src, W, H, pitch, (__half *)out[0]);
    } else if (out[0] != src || pitch != (size_t)W * 2) {
        if (cudaMemcpy2DAsync(out[0], (size_t)W * 2, src, pitch, (size_t)W * 2, H, cudaMemcpyDeviceToDevice, st) !=
            cudaSuccess)
            return PM_ECUDA;
    }
    int w = W, h = H;
    for (int k = 1; k < levels; ++k) {
        const int dw = (w + 1) / 2, dh = (h + 1) / 2;
        half_down_kernel<<<grid2(dw, dh), dim3(32, 8), 0, st>>>((const __half *)out[k - 1], w, h, (__half *)out[k],
                                                               dw, dh);
        w = dw;
        h = dh;
    }
    return cudaGetLastError() == cudaSuccess ? PM_OK : PM_ECUDA;
}

}  // extern "C"
