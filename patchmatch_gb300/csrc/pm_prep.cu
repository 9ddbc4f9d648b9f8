// View preparation and random initialisation kernels.
#include <cuda_fp16.h>

#include "pm_device.cuh"
#include "pm_kernels.h"

namespace pm {

// Raw view (u8 or f16, pitched) -> float reference intensities.
__global__ void ref_to_float_kernel(const uint8_t *raw, size_t pitch, int fmt, int W, int H, float *out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= H || j >= W) return;
    const uint8_t *row = raw + (size_t)i * pitch;
    out[(size_t)i * W + j] =
        fmt == PM_IMAGE_U8 ? (float)row[j] : __half2float(reinterpret_cast<const __half *>(row)[j]);
}

// Raw view -> quad-packed sampling image of (H+1) x (W+1) entries holding the
// 2x2 bilinear footprint with the border policy baked in.
__global__ void build_quad_kernel(const uint8_t *raw, size_t pitch, int fmt, int W, int H, int seam, void *quad) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (y > H || x > W) return;
    // columns: x and x + 1 with x = W meaning the coordinate u = W
    int xa, xb;
    if (seam == PM_SEAM_WRAP) {
        xa = x % W;
        xb = (x + 1) % W;
    } else {
        xa = min(x, W - 1);
        xb = min(x + 1, W - 1);
    }
    const int ya = min(y, H - 1), yb = min(y + 1, H - 1);
    const size_t qi = (size_t)y * (W + 1) + x;
    if (seam == PM_SEAM_ZERO && (x >= W - 1 || y >= H - 1)) {
        // a sample whose footprint leaves [0, W-1) x [0, H-1) reads 0
        // (LinearInterpolation, depthmap.cc:34-38): the whole cell is 0
        if (fmt == PM_IMAGE_U8) static_cast<uint32_t *>(quad)[qi] = 0u;
        else static_cast<uint2 *>(quad)[qi] = make_uint2(0u, 0u);
        return;
    }
    if (fmt == PM_IMAGE_U8) {
        const uint8_t *r0 = raw + (size_t)ya * pitch, *r1 = raw + (size_t)yb * pitch;
        const uint32_t w = (uint32_t)r0[xa] | ((uint32_t)r0[xb] << 8) | ((uint32_t)r1[xa] << 16) |
                           ((uint32_t)r1[xb] << 24);
        static_cast<uint32_t *>(quad)[qi] = w;
    } else {
        const __half *r0 = reinterpret_cast<const __half *>(raw + (size_t)ya * pitch);
        const __half *r1 = reinterpret_cast<const __half *>(raw + (size_t)yb * pitch);
        __half2 lo = __halves2half2(r0[xa], r0[xb]);
        __half2 hi = __halves2half2(r1[xa], r1[xb]);
        uint2 w;
        w.x = *reinterpret_cast<uint32_t *>(&lo);
        w.y = *reinterpret_cast<uint32_t *>(&hi);
        static_cast<uint2 *>(quad)[qi] = w;
    }
}

// Random plane per pixel (Philox tag 0).  Log-uniform depth and a uniform
// unit normal on the camera-facing hemisphere, or the reference's uniform
// depth with U[-1,1]^3 normal components (PatchMatchCuda.cu:210-244); plane
// = n / (n . (d b)) (PlaneFromDepthNormal, PatchMatchCuda.cu:31-43).
__global__ void init_planes_kernel(const float2 *row_trig, const float2 *col_trig, int W, int H, uint32_t seed,
                                   uint32_t kf, int mode, float dmin, float dmax, float4 *plane, float *score,
                                   int8_t *best) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= H || j >= W) return;
    const size_t idx = (size_t)i * W + j;
    const uint4 q = philox_block(seed, kf, (uint32_t)idx, 0u, 0u);
    const float2 rt = row_trig[i], ct = col_trig[j];
    const float bx = rt.x * ct.x, by = -rt.y, bz = rt.x * ct.y;
    float d, nx, ny, nz;
    if (mode == PM_INIT_REF_UNIFORM) {
        d = __fadd_rn(__fmul_rn(u24(q.x), __fsub_rn(dmax, dmin)), dmin);
        nx = __fsub_rn(__fmul_rn(u24(q.y), 2.0f), 1.0f);
        ny = __fsub_rn(__fmul_rn(u24(q.z), 2.0f), 1.0f);
        nz = __fsub_rn(__fmul_rn(u24(q.w), 2.0f), 1.0f);
    } else {
        const float lmin = logf(dmin), lmax = logf(dmax);
        d = expf(__fadd_rn(lmin, __fmul_rn(u24(q.x), __fsub_rn(lmax, lmin))));
        const float z = __fsub_rn(1.0f, __fmul_rn(2.0f, u24(q.y)));
        const float rxy = sqrtf(fmaxf(0.0f, __fsub_rn(1.0f, __fmul_rn(z, z))));
        const float ph = __fmul_rn(6.28318530717958647692f, u24(q.z));
        nx = __fmul_rn(rxy, cosf(ph));
        ny = __fmul_rn(rxy, sinf(ph));
        nz = z;
        const float dot = __fadd_rn(__fadd_rn(__fmul_rn(nx, bx), __fmul_rn(ny, by)), __fmul_rn(nz, bz));
        if (dot > 0.0f) { nx = -nx; ny = -ny; nz = -nz; }
    }
    const float px = __fmul_rn(d, bx), py = __fmul_rn(d, by), pz = __fmul_rn(d, bz);
    const float nom = __fdiv_rn(1.0f, __fadd_rn(__fadd_rn(__fmul_rn(nx, px), __fmul_rn(ny, py)), __fmul_rn(nz, pz)));
    plane[idx] = make_float4(__fmul_rn(nx, nom), __fmul_rn(ny, nom), __fmul_rn(nz, nom), d);
    score[idx] = -1.0f;
    best[idx] = 0;
}

// Caller-provided planes (H x W x 3) -> state (depth = 1 / max(1e-6, |pi . b|)).
__global__ void set_planes_kernel(const float *planes3, const float *scores, const float2 *row_trig,
                                  const float2 *col_trig, int W, int H, float4 *plane, float *score, int8_t *best) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= H || j >= W) return;
    const size_t idx = (size_t)i * W + j;
    const float2 rt = row_trig[i], ct = col_trig[j];
    const float bx = rt.x * ct.x, by = -rt.y, bz = rt.x * ct.y;
    const float x = planes3[3 * idx], y = planes3[3 * idx + 1], z = planes3[3 * idx + 2];
    const float den = __fadd_rn(__fadd_rn(__fmul_rn(bx, x), __fmul_rn(by, y)), __fmul_rn(bz, z));
    plane[idx] = make_float4(x, y, z, __fdiv_rn(1.0f, fmaxf(1e-6f, fabsf(den))));
    score[idx] = scores ? scores[idx] : -1.0f;
    best[idx] = 0;
}

void launch_ref_to_float(cudaStream_t st, const uint8_t *raw, size_t pitch, int fmt, int W, int H, float *out) {
    dim3 b(32, 8), g((W + 31) / 32, (H + 7) / 8);
    ref_to_float_kernel<<<g, b, 0, st>>>(raw, pitch, fmt, W, H, out);
}

void launch_build_quad(cudaStream_t st, const uint8_t *raw, size_t pitch, int fmt, int W, int H, int seam,
                       void *quad) {
    dim3 b(32, 8), g((W + 1 + 31) / 32, (H + 1 + 7) / 8);
    build_quad_kernel<<<g, b, 0, st>>>(raw, pitch, fmt, W, H, seam, quad);
}

void launch_init_planes(cudaStream_t st, const float2 *row_trig, const float2 *col_trig, int W, int H, uint32_t seed,
                        uint32_t kf, int mode, float dmin, float dmax, float4 *plane, float *score, int8_t *best) {
    dim3 b(32, 8), g((W + 31) / 32, (H + 7) / 8);
    init_planes_kernel<<<g, b, 0, st>>>(row_trig, col_trig, W, H, seed, kf, mode, dmin, dmax, plane, score, best);
}

void launch_set_planes(cudaStream_t st, const float *planes3, const float *scores, const float2 *row_trig,
                       const float2 *col_trig, int W, int H, float4 *plane, float *score, int8_t *best) {
    dim3 b(32, 8), g((W + 31) / 32, (H + 7) / 8);
    set_planes_kernel<<<g, b, 0, st>>>(planes3, scores, row_trig, col_trig, W, H, plane, score, best);
}

}  // namespace pm
