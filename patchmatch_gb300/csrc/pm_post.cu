// Post-filter, export, geometric-consistency filter and point fusion kernels.
#include <cuda_runtime.h>

#include "pm_device.cuh"
#include "pm_kernels.h"

namespace pm {

namespace {

constexpr float kPiF = 3.14159265358979323846f;

__device__ __forceinline__ void cswap(float &a, float &b) {
    const float lo = fminf(a, b), hi = fmaxf(a, b);
    a = lo;
    b = hi;
}
__device__ __forceinline__ float med3(float a, float b, float c) {
    return fmaxf(fminf(a, b), fminf(fmaxf(a, b), c));
}

// 3x3 median with replicated borders (OpenCV medianBlur ksize 3 on CV_32F):
// sort each row, then median(max of minima, median of medians, min of maxima).
__device__ __forceinline__ float median3x3(const float *m, int W, int H, int i, int j) {
    float r[3][3];
#pragma unroll
    for (int di = 0; di < 3; ++di) {
        const int y = min(max(i + di - 1, 0), H - 1);
#pragma unroll
        for (int dj = 0; dj < 3; ++dj) {
            const int x = min(max(j + dj - 1, 0), W - 1);
            r[di][dj] = m[(size_t)y * W + x];
        }
        cswap(r[di][0], r[di][1]);
        cswap(r[di][1], r[di][2]);
        cswap(r[di][0], r[di][1]);
    }
    const float lo = fmaxf(fmaxf(r[0][0], r[1][0]), r[2][0]);
    const float mid = med3(r[0][1], r[1][1], r[2][1]);
    const float hi = fminf(fminf(r[0][2], r[1][2]), r[2][2]);
    return med3(lo, mid, hi);
}

// Window of the host copy-back (depthmap.cc:731-760): rows/cols
// [patch_half, N - patch_half - 4); mask; low-variance mask over the taps
// (PatchVariance, depthmap.cc:963-973, averaged over the taps it fills).
__global__ void post_window_kernel(const PostArgs a) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= a.H || j >= a.W) return;
    const size_t idx = (size_t)i * a.W + j;
    const int ph = a.patch_half;
    float d = 0.0f, s = -1.0f;
    if (i >= ph && i < a.H - ph - 4 && j >= ph && j < a.W - ph - 4 && (!a.mask || a.mask[idx])) {
        bool low = false;
        if (a.min_var > 0.0f) {
            float sum = 0.0f;
            int n = 0;
            for (int u = -ph; u <= ph; u += 2)
                for (int v = -ph; v <= ph; v += 2, ++n) sum = __fadd_rn(sum, a.ref[(size_t)(i + u) * a.W + (j + v)]);
            const float mean = __fdiv_rn(sum, (float)n);
            float sum2 = 0.0f;
            for (int u = -ph; u <= ph; u += 2)
                for (int v = -ph; v <= ph; v += 2) {
                    const float dd = __fsub_rn(a.ref[(size_t)(i + u) * a.W + (j + v)], mean);
                    sum2 = __fadd_rn(sum2, __fmul_rn(dd, dd));
                }
            low = __fdiv_rn(sum2, (float)n) < a.min_var;
        }
        if (low) {
            d = 0.0f;
            s = 0.0f;
        } else {
            d = a.plane[idx].w;
            s = a.score[idx];
        }
    }
    a.d0[idx] = d;
    a.s0[idx] = s;
}

__global__ void median_kernel(const float *in, float *out, int W, int H) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= H || j >= W) return;
    out[(size_t)i * W + j] = median3x3(in, W, H, i, j);
}

// Second median + PostProcess thresholds (depthmap.cc:1176-1197).
__global__ void post_threshold_kernel(const PostArgs a) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= a.H || j >= a.W) return;
    const size_t idx = (size_t)i * a.W + j;
    const float m = median3x3(a.m1, a.W, a.H, i, j);
    const float d = a.d0[idx], s = a.s0[idx];
    // (float) q > 0.05 (double) is q >= 0.05f for a float q
    const bool reject = d == 0.0f || __fdiv_rn(fabsf(__fsub_rn(d, m)), d) >= 0.05f || d < a.min_depth ||
                        d > a.max_depth || s <= a.min_score;
    a.out_depth[idx] = reject ? 0.0f : m;
    a.out_score[idx] = reject ? -1.0f : s;
}

__global__ void export_kernel(const float4 *plane, const float *score, const int8_t *best, const float *fd,
                              const float *fs, const float2 *row_trig, const float2 *col_trig, int W, int H, int raw,
                              float *depth, float *score_out, float *plane3, float *normal3, int32_t *best32) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= H || j >= W) return;
    const size_t idx = (size_t)i * W + j;
    const float4 p = plane[idx];
    const float d = raw ? p.w : fd[idx];
    if (depth) depth[idx] = d;
    if (score_out) score_out[idx] = raw ? score[idx] : fs[idx];
    if (plane3) {
        plane3[3 * idx] = p.x;
        plane3[3 * idx + 1] = p.y;
        plane3[3 * idx + 2] = p.z;
    }
    if (normal3) {
        // unit normal facing the camera: -pi / |pi| (pi . b = 1 / depth > 0)
        const float n = sqrtf(p.x * p.x + p.y * p.y + p.z * p.z);
        const float2 rt = row_trig[i], ct = col_trig[j];
        const float s = p.x * rt.x * ct.x - p.y * rt.y + p.z * rt.x * ct.y;
        const float k = (d > 0.0f && n > 0.0f) ? (s > 0.0f ? -1.0f : 1.0f) / n : 0.0f;
        normal3[3 * idx] = p.x * k;
        normal3[3 * idx + 1] = p.y * k;
        normal3[3 * idx + 2] = p.z * k;
    }
    if (best32) best32[idx] = best[idx];
}

// Equirect projection of a camera-frame point (ReprojectEquirect,
// depthmap.cc:143-161, in float).  Returns false when nearer than 1e-4.
__device__ __forceinline__ bool project(float X, float Y, float Z, float Wf, float Hf, float &x, float &y, float &r) {
    r = sqrtf(X * X + Y * Y + Z * Z);
    if (r < 1e-4f) return false;
    const float lat = -asinf(fminf(1.0f, fmaxf(-1.0f, Y / r)));
    const float lon = atan2f(X, Z);
    x = Wf * (0.5f + lon / (2.0f * kPiF));
    y = Hf * (0.5f - lat / kPiF);
    return true;
}

// LinearInterpolation<float> (depthmap.cc:34-50)
__device__ __forceinline__ float interp_depth(const float *img, int W, int H, float y, float x) {
    if (x < 0.0f || x >= (float)(W - 1) || y < 0.0f || y >= (float)(H - 1)) return 0.0f;
    const int ix = (int)x, iy = (int)y;
    const float dx = x - ix, dy = y - iy;
    const float *r0 = img + (size_t)iy * W + ix, *r1 = r0 + W;
    const float im0 = (1 - dx) * r0[0] + dx * r0[1];
    const float im1 = (1 - dx) * r1[0] + dx * r1[1];
    return (1 - dy) * im0 + dy * im1;
}

// DepthmapCleaner::Clean (depthmap.cc:1337-1373) for every pixel of view 0.
__global__ void clean_kernel(const __grid_constant__ CleanArgs a) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= a.H || j >= a.W) return;
    const size_t idx = (size_t)i * a.W + j;
    const float d = a.depths[0][idx];
    float out = 0.0f;
    // depth < 1e-6 (double) is depth <= 1e-6f for a float depth
    if (!(d <= 1e-6f)) {
        const float2 rt = a.row_trig[i], ct = a.col_trig[j];
        const float Xc = d * rt.x * ct.x, Yc = -d * rt.y, Zc = d * rt.x * ct.y;
        const float Wf = (float)a.W, Hf = (float)a.H;
        int consistent = 1;
        for (int k = 1; k < a.n; ++k) {
            const float *M = a.M[k], *c = a.c[k];
            const float X = M[0] * Xc + M[1] * Yc + M[2] * Zc + c[0];
            const float Y = M[3] * Xc + M[4] * Yc + M[5] * Zc + c[1];
            const float Z = M[6] * Xc + M[7] * Yc + M[8] * Zc + c[2];
            float x, y, dop;
            if (!project(X, Y, Z, Wf, Hf, x, y, dop)) continue;
            const int ix = (int)x, iy = (int)y;
            if (!(iy >= 0 && iy < a.H && ix >= 0 && ix < a.W)) continue;
            const float dat = interp_depth(a.depths[k], a.W, a.H, y, x);
            if (!(fabsf(dat - dop) < dop * a.thr)) continue;
            if (a.reproj_px > 0.0f) {
                // round trip through view k's depth back into view 0
                const float lon = 2.0f * kPiF * (x / Wf - 0.5f), lat = -kPiF * (y / Hf - 0.5f);
                float sl, cl, sn, cn;
                sincosf(lat, &sl, &cl);
                sincosf(lon, &sn, &cn);
                const float qx = dat * cl * sn, qy = -dat * sl, qz = dat * cl * cn;
                const float *Mi = a.Minv[k], *ci = a.cinv[k];
                const float X0 = Mi[0] * qx + Mi[1] * qy + Mi[2] * qz + ci[0];
                const float Y0 = Mi[3] * qx + Mi[4] * qy + Mi[5] * qz + ci[1];
                const float Z0 = Mi[6] * qx + Mi[7] * qy + Mi[8] * qz + ci[2];
                float x0, y0, r0;
                if (!project(X0, Y0, Z0, Wf, Hf, x0, y0, r0)) continue;
                float ex = fabsf(x0 - (float)j);
                const float ey = fabsf(y0 - (float)i);
                if (ex > 0.5f * Wf) ex = Wf - ex;
                if (ex > a.reproj_px || ey > a.reproj_px) continue;
            }
            ++consistent;
        }
        if (consistent >= a.min_consistent) out = d;
    }
    a.out[idx] = out;
}

// ---------------------------------------------------------------------------
// Point fusion (DepthmapPruner::Prune, depthmap.cc:1556-1695).  The reference
// walks the head map in raster order and, per pixel, visits views 1..n-1 in
// order; a nearer head pixel zeroes the matching pixel of a later view, which
// later head pixels then see as empty.  Within view k, a target pixel q is
// therefore zeroed by the first (raster order) head pixel that reaches view k
// and qualifies; head pixels after it see 0, head pixels before it see the
// original value.  Processing views in order with an atomicMin per target
// reproduces that exactly, independent of thread scheduling.
// ---------------------------------------------------------------------------
enum : int8_t { kSkip = 0, kZero = 1, kDrop = 2 };

__global__ void fuse_init_kernel(const __grid_constant__ FuseArgs a) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= a.H || j >= a.W) return;
    const size_t idx = (size_t)i * a.W + j;
    const float *D0 = a.depths[0];
    const float d = D0[idx];
    bool f = d == 0.0f;
    if (i - 1 > 0 && i - 1 < a.H) f = f || D0[idx - a.W] == 0.0f;
    if (j - 1 > 0 && j - 1 < a.W) f = f || D0[idx - 1] == 0.0f;
    if (i + 1 > 0 && i + 1 < a.H) f = f || D0[idx + a.W] == 0.0f;
    if (j + 1 > 0 && j + 1 < a.W) f = f || D0[idx + 1] == 0.0f;
    a.alive[idx] = f ? 0 : 1;
    a.pruned[idx] = f ? 0.0f : d;
}

__global__ void fuse_classify_kernel(const __grid_constant__ FuseArgs a, int k) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= a.H || j >= a.W) return;
    const size_t idx = (size_t)i * a.W + j;
    int8_t cls = kSkip;
    if (a.alive[idx]) {
        const float d = a.depths[0][idx];
        const float2 rt = a.row_trig[i], ct = a.col_trig[j];
        const float Xc = d * rt.x * ct.x, Yc = -d * rt.y, Zc = d * rt.x * ct.y;
        const float *M = a.M[k], *c = a.c[k];
        const float X = M[0] * Xc + M[1] * Yc + M[2] * Zc + c[0];
        const float Y = M[3] * Xc + M[4] * Yc + M[5] * Zc + c[1];
        const float Z = M[6] * Xc + M[7] * Yc + M[8] * Zc + c[2];
        float x, y, dop;
        if (project(X, Y, Z, (float)a.W, (float)a.H, x, y, dop)) {
            const int iu = (int)x, iv = (int)y;
            if (iv >= 0 && iv < a.H && iu >= 0 && iu < a.W && !(dop < 1e-5f)) {
                const int q = iv * a.W + iu;
                const float dat = a.depths[k][q];
                if (!(dat == 0.0f || fabsf(dat - dop) > a.thr * dop)) {
                    cls = d < dat ? kZero : kDrop;
                    a.target[idx] = q;
                    if (cls == kZero) atomicMin(a.first + q, (unsigned)idx);
                }
            }
        }
    }
    a.cls[idx] = cls;
}

__global__ void fuse_resolve_kernel(const __grid_constant__ FuseArgs a, int k) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= a.H || j >= a.W) return;
    const size_t idx = (size_t)i * a.W + j;
    const int8_t cls = a.cls[idx];
    if (cls == kSkip) return;
    const int q = a.target[idx];
    const unsigned f = a.first[q];
    if ((unsigned)idx > f) return;          // target already zeroed: skipped
    if ((unsigned)idx == f) {               // first qualifying nearer pixel zeroes it
        a.depths[k][q] = 0.0f;
        return;
    }
    if (cls == kDrop) {                     // sees the original, farther-or-equal: dropped
        a.alive[idx] = 0;
        a.pruned[idx] = 0.0f;
    }
}

__global__ void compact_count_kernel(const uint8_t *alive, size_t N, unsigned *counts) {
    const size_t i = (size_t)blockIdx.x * kCompactBlock + threadIdx.x;
    const int keep = (i < N) ? alive[i] : 0;
    const int c = __syncthreads_count(keep);
    if (threadIdx.x == 0) counts[blockIdx.x] = (unsigned)c;
}

// exclusive scan of nb block counts (single block); counts[nb] = total
__global__ void compact_scan_kernel(unsigned *counts, int nb, unsigned *total) {
    __shared__ unsigned s[1024];
    __shared__ unsigned carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nb; base += 1024) {
        const int i = base + threadIdx.x;
        const unsigned v = i < nb ? counts[i] : 0u;
        s[threadIdx.x] = v;
        __syncthreads();
        for (int off = 1; off < 1024; off <<= 1) {
            const unsigned t = threadIdx.x >= off ? s[threadIdx.x - off] : 0u;
            __syncthreads();
            s[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < nb) counts[i] = carry + s[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry += s[1023];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        counts[nb] = carry;
        *total = carry;
    }
}

__global__ void compact_scatter_kernel(const __grid_constant__ FuseArgs a) {
    __shared__ unsigned warp_tot[32];
    const size_t N = (size_t)a.W * a.H;
    const size_t i = (size_t)blockIdx.x * kCompactBlock + threadIdx.x;
    const int keep = (i < N) ? a.alive[i] : 0;
    const unsigned lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const unsigned bal = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) warp_tot[wid] = __popc(bal);
    __syncthreads();
    if (wid == 0) {
        unsigned v = warp_tot[lane];
        for (int off = 1; off < 32; off <<= 1) {
            const unsigned t = __shfl_up_sync(0xffffffffu, v, off);
            if (lane >= (unsigned)off) v += t;
        }
        warp_tot[lane] = v - warp_tot[lane];  // exclusive
    }
    __syncthreads();
    if (!keep) return;
    const unsigned pos = a.block_counts[blockIdx.x] + warp_tot[wid] + __popc(bal & ((1u << lane) - 1u));
    const int row = (int)(i / a.W), col = (int)(i - (size_t)row * a.W);
    const float d = a.depths[0][i];
    const float2 rt = a.row_trig[row], ct = a.col_trig[col];
    const float Xc = d * rt.x * ct.x, Yc = -d * rt.y, Zc = d * rt.x * ct.y;
    a.xyz[3 * (size_t)pos] = a.Rinv[0] * Xc + a.Rinv[1] * Yc + a.Rinv[2] * Zc + a.tw[0];
    a.xyz[3 * (size_t)pos + 1] = a.Rinv[3] * Xc + a.Rinv[4] * Yc + a.Rinv[5] * Zc + a.tw[1];
    a.xyz[3 * (size_t)pos + 2] = a.Rinv[6] * Xc + a.Rinv[7] * Yc + a.Rinv[8] * Zc + a.tw[2];
    if (a.bgr_out && a.bgr) {
        a.bgr_out[3 * (size_t)pos] = a.bgr[3 * i];
        a.bgr_out[3 * (size_t)pos + 1] = a.bgr[3 * i + 1];
        a.bgr_out[3 * (size_t)pos + 2] = a.bgr[3 * i + 2];
    }
    if (a.ij_out) {
        a.ij_out[2 * (size_t)pos] = row;
        a.ij_out[2 * (size_t)pos + 1] = col;
    }
}

}  // namespace

void launch_postprocess(cudaStream_t st, const PostArgs &a) {
    dim3 b(32, 8), g((a.W + 31) / 32, (a.H + 7) / 8);
    post_window_kernel<<<g, b, 0, st>>>(a);
    median_kernel<<<g, b, 0, st>>>(a.d0, a.m1, a.W, a.H);
    post_threshold_kernel<<<g, b, 0, st>>>(a);
}

void launch_export(cudaStream_t st, const float4 *plane, const float *score, const int8_t *best,
                   const float *filt_depth, const float *filt_score, const float2 *row_trig, const float2 *col_trig,
                   int W, int H, int raw, float *depth, float *score_out, float *plane3, float *normal3,
                   int32_t *best32) {
    dim3 b(32, 8), g((W + 31) / 32, (H + 7) / 8);
    export_kernel<<<g, b, 0, st>>>(plane, score, best, filt_depth, filt_score, row_trig, col_trig, W, H, raw, depth,
                                   score_out, plane3, normal3, best32);
}

void clean_set_poses(CleanArgs &a, int n, const double *R, const double *t, int center, int *order) {
    order[0] = center;
    for (int k = 0, s = 1; k < n; ++k)
        if (k != center) order[s++] = k;
    const double *R0 = R + 9 * center, *t0 = t + 3 * center;
    for (int s = 1; s < n; ++s) {
        const int k = order[s];
        compose_pose(R0, t0, R + 9 * k, t + 3 * k, a.M[s], a.c[s]);
        compose_pose(R + 9 * k, t + 3 * k, R0, t0, a.Minv[s], a.cinv[s]);
    }
    a.n = n;
}

void launch_clean(cudaStream_t st, const CleanArgs &a) {
    dim3 b(32, 8), g((a.W + 31) / 32, (a.H + 7) / 8);
    clean_kernel<<<g, b, 0, st>>>(a);
}

namespace {
inline size_t al256(size_t x) { return (x + 255) & ~size_t(255); }
inline int compact_blocks(int W, int H) { return (int)(((size_t)W * H + kCompactBlock - 1) / kCompactBlock); }
}  // namespace

size_t fuse_workspace_bytes(int W, int H) {
    const size_t N = (size_t)W * H;
    return al256(N) + al256(N * 4) + al256(N) + al256(N * 4) + al256((size_t)(compact_blocks(W, H) + 1) * 4);
}

void fuse_bind_workspace(FuseArgs &a, void *ws) {
    const size_t N = (size_t)a.W * a.H;
    char *p = static_cast<char *>(ws);
    auto take = [&](size_t b) { char *q = p; p += al256(b); return q; };
    a.alive = reinterpret_cast<uint8_t *>(take(N));
    a.target = reinterpret_cast<int *>(take(N * 4));
    a.cls = reinterpret_cast<int8_t *>(take(N));
    a.first = reinterpret_cast<unsigned *>(take(N * 4));
    a.block_counts = reinterpret_cast<unsigned *>(take((size_t)(compact_blocks(a.W, a.H) + 1) * 4));
}

void fuse_set_poses(FuseArgs &a, int n, const double *R, const double *t) {
    for (int k = 1; k < n; ++k) compose_pose(R, t, R + 9 * k, t + 3 * k, a.M[k], a.c[k]);
    for (int r0 = 0; r0 < 3; ++r0) {
        for (int c0 = 0; c0 < 3; ++c0) a.Rinv[3 * r0 + c0] = (float)R[3 * c0 + r0];
        a.tw[r0] = (float)(-(R[r0] * t[0] + R[3 + r0] * t[1] + R[6 + r0] * t[2]));
    }
    a.n = n;
}

cudaError_t launch_fuse(cudaStream_t st, const FuseArgs &a) {
    dim3 b(32, 8), g((a.W + 31) / 32, (a.H + 7) / 8);
    const size_t N = (size_t)a.W * a.H;
    fuse_init_kernel<<<g, b, 0, st>>>(a);
    for (int k = 1; k < a.n; ++k) {
        const cudaError_t e = cudaMemsetAsync(a.first, 0xFF, N * sizeof(unsigned), st);
        if (e != cudaSuccess) return e;
        fuse_classify_kernel<<<g, b, 0, st>>>(a, k);
        fuse_resolve_kernel<<<g, b, 0, st>>>(a, k);
    }
    const int nb = compact_blocks(a.W, a.H);
    compact_count_kernel<<<nb, kCompactBlock, 0, st>>>(a.alive, N, a.block_counts);
    compact_scan_kernel<<<1, 1024, 0, st>>>(a.block_counts, nb, a.count);
    compact_scatter_kernel<<<nb, kCompactBlock, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace pm
