// Seeding a keyframe from a previous keyframe's result: the GPU form of the
// reference's PreInitResultWarp (depthmap.cc:434-516).  Each valid pixel of
// the prior result is lifted onto its plane, transformed into the new camera
// and splatted to the nearest pixel; when several land on one pixel the
// nearest (then lowest index) wins, so the outcome does not depend on thread
// order.  The candidates are then scored by the tile kernel (kModeSeed) and
// kept where they beat the random initialisation.
#include <cuda_runtime.h>

#include "pm_device.cuh"
#include "pm_kernels.h"

namespace pm {

namespace {

constexpr float kPiF = 3.14159265358979323846f;

struct Splat {
    bool ok;
    int target;
    unsigned long long key;
    float r, Xx, Xy, Xz;
};

// Lift prior pixel (i, j) onto its plane (PosPatchPartOnPlane, depthmap.cc:163-177),
// move it into the new camera and project it (ReprojectEquirect, :143-161).
__device__ __forceinline__ Splat splat(const WarpArgs &a, int i, int j) {
    Splat s;
    s.ok = false;
    const size_t idx = (size_t)i * a.Wp + j;
    const float d = a.prev_depth[idx];
    if (!(d >= 1e-4f)) return s;  // depthmap.cc:451-453
    const float4 pl = a.prev_plane[idx];
    const float2 rt = a.prow[i], ct = a.pcol[j];
    const float bx = rt.x * ct.x, by = -rt.y, bz = rt.x * ct.y;
    float sc = pl.x * bx + pl.y * by + pl.z * bz;
    if (sc < 1e-6f && sc >= 0.0f) sc = 1e-6f;
    else if (sc > -1e-6f && sc < 0.0f) sc = -1e-6f;
    const float Px = bx / sc, Py = by / sc, Pz = bz / sc;
    const float X = a.M[0] * Px + a.M[1] * Py + a.M[2] * Pz + a.c[0];
    const float Y = a.M[3] * Px + a.M[4] * Py + a.M[5] * Pz + a.c[1];
    const float Z = a.M[6] * Px + a.M[7] * Py + a.M[8] * Pz + a.c[2];
    const float r = sqrtf(X * X + Y * Y + Z * Z);
    if (!(r >= 1e-4f) || !isfinite(r)) return s;
    const float lon = atan2f(X, Z), lat = -asinf(fminf(1.0f, fmaxf(-1.0f, Y / r)));
    const float x = a.Wf * (0.5f + lon / (2.0f * kPiF)), y = a.Hf * (0.5f - lat / kPiF);
    const int ti = (int)(y + 0.5f), tj = (int)(x + 0.5f);  // depthmap.cc:460-461
    if (ti < 0 || tj < 0 || ti >= a.H || tj >= a.W) return s;
    s.ok = true;
    s.target = ti * a.W + tj;
    s.key = ((unsigned long long)__float_as_uint(r) << 32) | (unsigned long long)(unsigned)idx;
    s.r = r;
    s.Xx = X;
    s.Xy = Y;
    s.Xz = Z;
    return s;
}

__global__ void warp_scatter_kernel(const __grid_constant__ WarpArgs a) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= a.Hp || j >= a.Wp) return;
    const Splat s = splat(a, i, j);
    if (s.ok) atomicMin(a.zbuf + s.target, s.key);
}

__global__ void warp_gather_kernel(const __grid_constant__ WarpArgs a) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= a.Hp || j >= a.Wp) return;
    const Splat s = splat(a, i, j);
    if (!s.ok || a.zbuf[s.target] != s.key) return;
    // the prior plane's unit normal, rotated into the new camera, through the
    // splatted point (PlanePosFromDepthAndNormal_equirect, depthmap.cc:130-141)
    const float4 pl = a.prev_plane[(size_t)i * a.Wp + j];
    const float nn = rsqrtf(pl.x * pl.x + pl.y * pl.y + pl.z * pl.z);
    const float nx = (a.M[0] * pl.x + a.M[1] * pl.y + a.M[2] * pl.z) * nn;
    const float ny = (a.M[3] * pl.x + a.M[4] * pl.y + a.M[5] * pl.z) * nn;
    const float nz = (a.M[6] * pl.x + a.M[7] * pl.y + a.M[8] * pl.z) * nn;
    const int ti = s.target / a.W, tj = s.target - ti * a.W;
    const float2 rt = a.row[ti], ct = a.col[tj];
    const float bx = rt.x * ct.x, by = -rt.y, bz = rt.x * ct.y;
    float den = s.r * (nx * bx + ny * by + nz * bz);
    if (den < 1e-5f && den >= 0.0f) den = 1e-5f;
    else if (den > -1e-5f && den < 0.0f) den = -1e-5f;
    a.seed[s.target] = make_float4(nx / den, ny / den, nz / den, s.r);
}

}  // namespace

void launch_warp_prior(cudaStream_t st, const WarpArgs &a) {
    cudaMemsetAsync(a.zbuf, 0xFF, sizeof(unsigned long long) * (size_t)a.W * a.H, st);
    cudaMemsetAsync(a.seed, 0, sizeof(float4) * (size_t)a.W * a.H, st);
    dim3 b(32, 8), g((a.Wp + 31) / 32, (a.Hp + 7) / 8);
    warp_scatter_kernel<<<g, b, 0, st>>>(a);
    warp_gather_kernel<<<g, b, 0, st>>>(a);
}

}  // namespace pm

// ---------------------------------------------------------------------------
// Seeding from SLAM landmarks: the GPU half of the reference's
// PreInitSparsePCL2 (depthmap.cc:361-432).  The host projects the landmarks
// in FP64 and keeps the nearest landmark per pixel; here each one becomes the
// candidate plane of its pixel with the normal facing the camera
// (normal = -bearing, PlanePosFromDepthAndNormal_equirect, depthmap.cc:130-141).
// ---------------------------------------------------------------------------
namespace pm {
namespace {

__global__ void landmark_cand_kernel(const int2 *lm, int n, const uint8_t *mask, const float2 *row, const float2 *col,
                                     int W, float4 *cand) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int idx = lm[k].x;
    const float d = __int_as_float(lm[k].y);
    if (mask && !mask[idx]) return;  // depthmap.cc:384-386
    const int i = idx / W, j = idx - i * W;
    const float2 rt = row[i], ct = col[j];
    const float bx = rt.x * ct.x, by = -rt.y, bz = rt.x * ct.y;
    // plane = n / (n . (d b)) with n = -b, |denominator| clamped to 1e-5
    float den = -d * (bx * bx + by * by + bz * bz);
    if (den < 1e-5f && den >= 0.0f) den = 1e-5f;
    else if (den > -1e-5f && den < 0.0f) den = -1e-5f;
    cand[idx] = make_float4(-bx / den, -by / den, -bz / den, d);
}

}  // namespace

void launch_landmark_cands(cudaStream_t st, const int2 *lm, int n, const uint8_t *mask, const float2 *row,
                           const float2 *col, int W, int H, float4 *cand) {
    cudaMemsetAsync(cand, 0, (size_t)W * H * sizeof(float4), st);
    if (n > 0) landmark_cand_kernel<<<(n + 255) / 256, 256, 0, st>>>(lm, n, mask, row, col, W, cand);
}

}  // namespace pm
