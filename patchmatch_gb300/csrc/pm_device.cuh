// Device-side building blocks of the densifier: counter-based random numbers,
// equirectangular angle evaluation, quad-packed bilinear sampling and the
// per-tap NCC moment accumulation shared by every cost kernel.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "pm_types.h"

namespace pm {

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC'11).  Key = (seed, keyframe); counter = (pixel, tag, draw,
// constant).  tag 0 = initialisation, tag s+1 = the pixel's visit in sweep s.
// Replaces the clock-seeded cuRAND XORWOW states of the reference
// (PatchMatchCuda.cu:246-252), which made runs irreproducible.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) { k.x += 0x9E3779B9u; k.y += 0xBB67AE85u; }
        const uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    }
    return c;
}

__device__ __forceinline__ uint4 philox_block(uint32_t seed, uint32_t kf, uint32_t pixel, uint32_t tag,
                                              uint32_t draw) {
    return philox4x32_10(make_uint4(pixel, tag, draw, 0x504d4742u), make_uint2(seed, kf));
}

// 24-bit uniform in (0, 1), exactly representable.
__device__ __forceinline__ float u24(uint32_t x) {
    return __fmul_rn(__fadd_rn((float)(x >> 8), 0.5f), 1.0f / 16777216.0f);
}

// Box-Muller pair from two words.
__device__ __forceinline__ float2 box_muller(uint32_t a, uint32_t b) {
    const float u1 = u24(a), u2 = u24(b);
    const float r = sqrtf(__fmul_rn(-2.0f, logf(u1)));
    const float th = __fmul_rn(6.28318530717958647692f, u2);
    return make_float2(__fmul_rn(r, cosf(th)), __fmul_rn(r, sinf(th)));
}

// ---------------------------------------------------------------------------
// atan on [0, 1]: atan(t) ~ t * P(t^2), P of degree 7, a minimax (Remez
// exchange) fit made for this project (max error 3.7e-8 rad before float
// rounding).  The two coefficient sets below are that polynomial scaled to
// turns (1/2pi, longitude) and half turns (1/pi, latitude) so the angles come
// out directly in image-fraction units.
// ---------------------------------------------------------------------------
#define PM_ATAN_C0 0.9999993443489075f
#define PM_ATAN_C1 -0.33329859375953674f
#define PM_ATAN_C2 0.19946566224098206f
#define PM_ATAN_C3 -0.1390862911939621f
#define PM_ATAN_C4 0.0964219719171524f
#define PM_ATAN_C5 -0.0559123270213604f
#define PM_ATAN_C6 0.021862957626581192f
#define PM_ATAN_C7 -0.004054567310959101f

template <int kScaleInvPi>  // 1: scale by 1/pi; 2: scale by 1/(2 pi)
__device__ __forceinline__ float atan_poly_scaled(float x2) {
    constexpr float s = kScaleInvPi == 1 ? 0.318309886183790671538f : 0.159154943091895335769f;
    float p = PM_ATAN_C7 * s;
    p = fmaf(p, x2, PM_ATAN_C6 * s);
    p = fmaf(p, x2, PM_ATAN_C5 * s);
    p = fmaf(p, x2, PM_ATAN_C4 * s);
    p = fmaf(p, x2, PM_ATAN_C3 * s);
    p = fmaf(p, x2, PM_ATAN_C2 * s);
    p = fmaf(p, x2, PM_ATAN_C1 * s);
    return fmaf(p, x2, PM_ATAN_C0 * s);
}

// Both angles use atan2(a, b) = pi/4 + atan((a - b) / (a + b)) for a, b >= 0,
// whose argument lies in [-1, 1] without an octant select.  The approximate
// division can leave |t| an ulp or two above 1; with kBound each angle is
// clamped to keep |lon| <= 1/2 and |lat| <= 1/2 exactly, so sample
// coordinates stay in [0, W] x [0, H], which the quad samplers index without
// further checks (texture reads clamp in hardware and skip the two clamps).

// atan2(x, z) / (2 pi) in [-1/2, 1/2]: the equirectangular longitude of
// direction (x, ., z) as a fraction of the image width (PatchMatchCuda.cu:140,143).
// x = z = 0 gives t = -1 and an angle of 0, like atan2(0, 0).
template <bool kBound>
__device__ __forceinline__ float lon_turns(float x, float z) {
    const float ax = fabsf(x), az = fabsf(z) + 1e-30f;
    const float t = __fdividef(ax - az, ax + az);
    float a = fmaf(atan_poly_scaled<2>(t * t), t, 0.125f);
    if (kBound) a = fmaxf(a, 0.0f);
    a = (z < 0.0f) ? 0.5f - a : a;
    return copysignf(a, x);
}

// asin(y / |(x, y, z)|) / pi in [-1/2, 1/2]: minus the equirectangular
// latitude as a fraction of the image height (PatchMatchCuda.cu:139,144),
// evaluated as atan2(|y|, sqrt(x^2 + z^2)) with the sign of y.
template <bool kBound>
__device__ __forceinline__ float lat_halfturns(float x, float y, float z) {
    const float r2 = fmaxf(fmaf(x, x, z * z), 1e-30f);
    const float rho = r2 * rsqrtf(r2);
    const float ay = fabsf(y);
    const float t = __fdividef(ay - rho, ay + rho);
    float a = fmaf(atan_poly_scaled<1>(t * t), t, 0.25f);
    if (kBound) a = fminf(a, 0.5f);
    return copysignf(a, y);
}

// ---------------------------------------------------------------------------
// Quad-packed source images.  Entry (y, x) of a (H+1) x (W+1) array holds the
// 2x2 bilinear footprint {T(x,y), T(x+1,y), T(x,y+1), T(x+1,y+1)} with the
// border policy baked in (x+1 clamps at W-1 or wraps to 0; y+1 clamps), so a
// sample is one aligned load.  Texel k sits at coordinate k, matching the
// reference's texture reads at u + 0.5 (PatchMatchCuda.cu:146).
// ---------------------------------------------------------------------------
// Split a sample coordinate c in [0, N] into cell index k = floor(c) and
// weight a = c - k.  A NaN coordinate (a degenerate plane hypothesis) gives
// k = 0, so every index stays inside the (N+1)-entry quad array.
__device__ __forceinline__ void split_coord(float c, int &k, float &a) {
    const float f = floorf(c);
    k = (int)f;
    a = c - f;
}

struct QuadU8 {
    // sample coordinates: texel k at coordinate k, indexed unchecked
    static constexpr float kCoordOffset = 0.0f;
    static constexpr bool kBound = true;
    // shift: value subtracted from every texel, given as 2^23 + I_c so the
    // byte-to-float conversion and the centring are one subtraction.
    static __device__ __forceinline__ float shift_for(float centre) { return 8388608.0f + centre; }
    static __device__ __forceinline__ float sample(const void *quad, unsigned long long, int qpitch, float u, float v,
                                                   float shift) {
        // u in [0, W], v in [0, H] by construction of the angle functions
        int x0, y0;
        float ax, ay;
        split_coord(u, x0, ax);
        split_coord(v, y0, ay);
        const uint32_t w = __ldg(static_cast<const uint32_t *>(quad) + (y0 * qpitch + x0));
        // bytes -> floats minus the centre intensity: (2^23 + byte) - (2^23 + c)
        // texels as 2^23 + byte; differences are exact, the shift is applied once per row
        const float m00 = __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7540));
        const float m01 = __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7541));
        const float m10 = __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7542));
        const float m11 = __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7543));
        const float a = fmaf(ax, m01 - m00, m00 - shift);
        const float b = fmaf(ax, m11 - m10, m10 - shift);
        return fmaf(ay, b - a, a);
    }
};

struct QuadF16 {
    static constexpr float kCoordOffset = 0.0f;
    static constexpr bool kBound = true;
    static __device__ __forceinline__ float shift_for(float centre) { return centre; }
    static __device__ __forceinline__ float sample(const void *quad, unsigned long long, int qpitch, float u, float v,
                                                   float shift) {
        int x0, y0;
        float ax, ay;
        split_coord(u, x0, ax);
        split_coord(v, y0, ay);
        const uint2 w = __ldg(static_cast<const uint2 *>(quad) + (y0 * qpitch + x0));
        const float2 r0 = __half22float2(*reinterpret_cast<const __half2 *>(&w.x));
        const float2 r1 = __half22float2(*reinterpret_cast<const __half2 *>(&w.y));
        const float t00 = r0.x - shift, t01 = r0.y - shift, t10 = r1.x - shift, t11 = r1.y - shift;
        const float a = fmaf(ax, t01 - t00, t00);
        const float b = fmaf(ax, t11 - t10, t10);
        return fmaf(ay, b - a, a);
    }
};

// Texture sampling (PM_SAMPLER_TEXTURE): the texture unit's bilinear filter
// over the source image, read at the texel-centre convention of the
// reference (coordinate + 0.5, PatchMatchCuda.cu:146), clamped at the border.
// u8 images are bound as normalised 8-bit textures (value / 255).
struct TexU8 {
    static constexpr float kCoordOffset = 0.5f;
    static constexpr bool kBound = false;
    static __device__ __forceinline__ float shift_for(float centre) { return centre; }
    static __device__ __forceinline__ float sample(const void *, unsigned long long tex, int, float u, float v,
                                                   float shift) {
        return fmaf(tex2D<float>((cudaTextureObject_t)tex, u, v), 255.0f, -shift);
    }
};

struct TexF16 {
    static constexpr float kCoordOffset = 0.5f;
    static constexpr bool kBound = false;
    static __device__ __forceinline__ float shift_for(float centre) { return centre; }
    static __device__ __forceinline__ float sample(const void *, unsigned long long tex, int, float u, float v,
                                                   float shift) {
        return tex2D<float>((cudaTextureObject_t)tex, u, v) - shift;
    }
};

// Bilateral window weight exp(-dI^2 / (2 sigma_c^2) - d^2 / (2 sigma_x^2))
// (PatchMatchCuda.cu:148-149) as exp2 of a pre-scaled exponent:
// ncf = -log2(e) / (2 sigma_c^2), dk = -log2(e) (dx^2 + dy^2) / (2 sigma_x^2).
__device__ __forceinline__ float bilateral_weight(float xs, float ncf, float dk) {
    return exp2f(fmaf(xs * xs, ncf, dk));
}

// The three standard normals of refinement t (0..5) of one pixel visit:
// normals 3t..3t+2 of the Box-Muller stream whose pair p uses Philox block
// p / 2, words (x, y) for even p and (z, w) for odd p.
__device__ __forceinline__ void refine_normals(uint32_t seed, uint32_t kf, uint32_t pix, uint32_t tag, int t,
                                               float &ra, float &rb, float &rc) {
    const int p0 = (3 * t) >> 1;
    float z[4];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const int p = p0 + q;
        const uint4 blk = philox_block(seed, kf, pix, tag, (uint32_t)(p >> 1));
        const float2 bm = (p & 1) ? box_muller(blk.z, blk.w) : box_muller(blk.x, blk.y);
        z[2 * q] = bm.x;
        z[2 * q + 1] = bm.y;
    }
    const bool odd = (3 * t) & 1;
    ra = odd ? z[1] : z[0];
    rb = odd ? z[2] : z[1];
    rc = odd ? z[3] : z[2];
}

// The four standard normals of refinement t of the plain (host-variant)
// propagation: Philox block t, words (x, y) and (z, w), one depth draw
// followed by three normal draws (depthmap.cc:1041-1050).
__device__ __forceinline__ void refine_normals4(uint32_t seed, uint32_t kf, uint32_t pix, uint32_t tag, int t,
                                                float &z0, float &z1, float &z2, float &z3) {
    const uint4 blk = philox_block(seed, kf, pix, tag, (uint32_t)t);
    const float2 a = box_muller(blk.x, blk.y), b = box_muller(blk.z, blk.w);
    z0 = a.x;
    z1 = a.y;
    z2 = b.x;
    z3 = b.y;
}

// ---------------------------------------------------------------------------
// One tap of the plane-induced warp for all S sources (PatchMatchCuda.cu:107-157,
// restructured).  The reference maps X_c = b / (pi . b) through
// R_r (R_1^T X_c - R_1^T t_1) + t_r and normalises.  Only the direction of the
// source-frame point matters, so with M_r = R_r R_1^T and c_r = t_r - M_r t_1
// (composed in FP64 on the host) we evaluate |s| * X_r = sign(s) M_r b + |s| c_r,
// s = pi . b, which has the same direction and no division.  M_r b does not
// depend on the hypothesis: the tile kernels stage its row and column factors.
// Moments are accumulated shifted by the centre intensity (y - I_c), which is
// exact algebra for the NCC and avoids float cancellation in the variances.
// ---------------------------------------------------------------------------
// Where the per-source constants of the sample loop come from.  ParamAccess:
// kernel parameters (constant bank, usable directly as instruction operands).
// SharedAccess: a request's arguments staged in shared memory by the batched
// executor, re-read at every use: the loads are volatile so that the compiler
// does not hoist all sources' rows into registers (that spills).
struct ParamAccess {
    static __device__ __forceinline__ float val(const float &x) { return x; }
    static __device__ __forceinline__ float4 row(const float4 &g) { return g; }
    static __device__ __forceinline__ unsigned long long tex(const unsigned long long &t) { return t; }
    static __device__ __forceinline__ const void *ptr(const void *const &p) { return p; }
};
struct SharedAccess {
    static __device__ __forceinline__ float val(const float &x) {
        float v;
        const unsigned a = (unsigned)__cvta_generic_to_shared(&x);
        asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(a));
        return v;
    }
    static __device__ __forceinline__ float4 row(const float4 &g) {
        float4 v;
        const unsigned a = (unsigned)__cvta_generic_to_shared(&g);
        asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(a));
        return v;
    }
    static __device__ __forceinline__ unsigned long long tex(const unsigned long long &t) {
        unsigned long long v;
        const unsigned a = (unsigned)__cvta_generic_to_shared(&t);
        asm volatile("ld.shared.u64 %0, [%1];" : "=l"(v) : "r"(a));
        return v;
    }
    static __device__ __forceinline__ const void *ptr(const void *const &p) {
        unsigned long long v;
        const unsigned a = (unsigned)__cvta_generic_to_shared(&p);
        asm volatile("ld.shared.u64 %0, [%1];" : "=l"(v) : "r"(a));
        return reinterpret_cast<const void *>(v);
    }
};

// M b for the pose rows g0, g1, g2 (their xyz; w holds c), the
// hypothesis-independent part of the warp, evaluated directly.
__device__ __forceinline__ float3 rotate(const float4 &g0, const float4 &g1, const float4 &g2, float bx, float by,
                                         float bz) {
    return make_float3(fmaf(g0.x, bx, fmaf(g0.y, by, g0.z * bz)), fmaf(g1.x, bx, fmaf(g1.y, by, g1.z * bz)),
                       fmaf(g2.x, bx, fmaf(g2.y, by, g2.z * bz)));
}

// Factored form over the equirectangular grid: with b = (cos lat sin lon,
// -sin lat, cos lat cos lon),  M b = cos(lat) A(lon) + B(lat),
//   A = sin(lon) M e_x + cos(lon) M e_z   (per image column and source),
//   B = -sin(lat) M e_y                   (per image row and source),
// so a tile kernel stages A per column and B per row once and a tap costs
// three FMAs and two shared-memory reads per source instead of nine FMAs.
// Used from PM_FACTOR_MIN_SOURCES to PM_FACTOR_MAX_SOURCES sources: with
// fewer sources the shared-memory reads cost as much as the FMAs they
// replace and the staged factors take L1 from the texture samples (measured,
// 8 sweeps: 1920x960 u8 - 4-6 sources faster direct, 8 even, 10 sources 4 %
// faster factored; 3840x1920 - 8 sources FP16 4 % faster direct, 9-10
// sources 0-3 % faster factored).  The staged factors take 1760 bytes of
// shared memory per source.
#ifndef PM_FACTOR_MIN_SOURCES
#define PM_FACTOR_MIN_SOURCES 9
#endif
#ifndef PM_FACTOR_MAX_SOURCES
#define PM_FACTOR_MAX_SOURCES 10
#endif
template <int S>
__host__ __device__ constexpr bool factored_warp() {
    return S >= PM_FACTOR_MIN_SOURCES && S <= PM_FACTOR_MAX_SOURCES;
}
__device__ __forceinline__ float3 col_factor(const float4 &g0, const float4 &g1, const float4 &g2, float sin_lon,
                                             float cos_lon) {
    return make_float3(fmaf(sin_lon, g0.x, cos_lon * g0.z), fmaf(sin_lon, g1.x, cos_lon * g1.z),
                       fmaf(sin_lon, g2.x, cos_lon * g2.z));
}
__device__ __forceinline__ float3 row_factor(const float4 &g0, const float4 &g1, const float4 &g2, float sin_lat) {
    return make_float3(-sin_lat * g0.y, -sin_lat * g1.y, -sin_lat * g2.y);
}

// x with its sign bit flipped when sg (0 or 0x80000000) is set.
__device__ __forceinline__ float flip_sign(float x, uint32_t sg) { return __uint_as_float(__float_as_uint(x) ^ sg); }

template <int S, class Img, class Acc = ParamAccess>
struct TapAccum {
    float swy[S], swyy[S], swxy[S];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int r = 0; r < S; ++r) swy[r] = swyy[r] = swxy[r] = 0.0f;
    }
    // One tap given |s| (s = pi . b) and the sources' signed rotated
    // bearings mb(r) = sign(s) M_r b (a float3): X_r = sign(s) M_r b + |s| c_r.
    // P and src live in kernel parameter space (or shared memory, through
    // Acc); w: bilateral weight, xs: tap intensity minus centre; halfW/halfH
    // include the sampler's coordinate offset.
    template <class MB>
    __device__ __forceinline__ void add_rot(const PmPoses &P, const SrcSet &src, float Wf, float Hf, float halfW,
                                            float halfH, float shift, float as, MB mb, float w, float xs) {
        // phase 1: all S sample coordinates, so the S footprint loads issue
        // back to back; phase 2: bilinear + moments as they arrive
        float u[S], v[S];
#pragma unroll
        for (int r = 0; r < S; ++r) {
            const float3 m = mb(r);
            const float X = fmaf(as, Acc::val(P.G[r][0].w), m.x);
            const float Y = fmaf(as, Acc::val(P.G[r][1].w), m.y);
            const float Z = fmaf(as, Acc::val(P.G[r][2].w), m.z);
            u[r] = fmaf(Wf, lon_turns<Img::kBound>(X, Z), halfW);
            v[r] = fmaf(Hf, lat_halfturns<Img::kBound>(X, Y, Z), halfH);
        }
#pragma unroll
        for (int r = 0; r < S; ++r) {
            const float y = Img::sample(Acc::ptr(src.quad[r]), Acc::tex(src.tex[r]), src.qpitch, u[r], v[r], shift);
            const float wy = w * y;
            swy[r] += wy;
            swyy[r] = fmaf(wy, y, swyy[r]);
            swxy[r] = fmaf(wy, xs, swxy[r]);
        }
    }
    // One tap with bearing b = (bx, by, bz), rotated per source directly.
    __device__ __forceinline__ void add_bearing(const PmPoses &P, const SrcSet &src, float Wf, float Hf, float halfW,
                                                float halfH, float shift, float px, float py, float pz, float bx,
                                                float by, float bz, float w, float xs) {
        const float s = fmaf(px, bx, fmaf(py, by, pz * bz));
        const uint32_t sg = __float_as_uint(s) & 0x80000000u;
        const float sbx = flip_sign(bx, sg), sby = flip_sign(by, sg), sbz = flip_sign(bz, sg);
        add_rot(P, src, Wf, Hf, halfW, halfH, shift, fabsf(s),
                [&](int r) { return rotate(Acc::row(P.G[r][0]), Acc::row(P.G[r][1]), Acc::row(P.G[r][2]), sbx, sby, sbz); },
                w, xs);
    }
    // One tap at the grid point with row trig rt = (cos lat, sin lat) and
    // column trig ct = (sin lon, cos lon): the factored form when
    // factored_warp<S>() (the arithmetic of the staged tile factors), the
    // direct rotation of the bearing otherwise; the bearing is
    // (cos lat sin lon, -sin lat, cos lat cos lon), as in the staged tile.
    __device__ __forceinline__ void add_trig(const PmPoses &P, const SrcSet &src, float Wf, float Hf, float halfW,
                                             float halfH, float shift, float px, float py, float pz, float2 rt,
                                             float2 ct, float w, float xs) {
        const float bx = rt.x * ct.x, by = -rt.y, bz = rt.x * ct.y;
        if constexpr (factored_warp<S>()) {
            const float s = fmaf(px, bx, fmaf(py, by, pz * bz));
            const uint32_t sg = __float_as_uint(s) & 0x80000000u;
            const float sc = flip_sign(rt.x, sg);
            add_rot(P, src, Wf, Hf, halfW, halfH, shift, fabsf(s),
                    [&](int r) {
                        const float4 g0 = Acc::row(P.G[r][0]), g1 = Acc::row(P.G[r][1]), g2 = Acc::row(P.G[r][2]);
                        const float3 A = col_factor(g0, g1, g2, ct.x, ct.y);
                        const float3 B = row_factor(g0, g1, g2, rt.y);
                        return make_float3(fmaf(sc, A.x, flip_sign(B.x, sg)), fmaf(sc, A.y, flip_sign(B.y, sg)),
                                           fmaf(sc, A.z, flip_sign(B.z, sg)));
                    },
                    w, xs);
        } else {
            add_bearing(P, src, Wf, Hf, halfW, halfH, shift, px, py, pz, bx, by, bz, w, xs);
        }
    }
};

// NCC from shifted moments (PatchMatchCuda.cu:161-170): -1 when either
// weighted variance is below 0.1.
__device__ __forceinline__ float ncc_from_moments(float sw, float swx, float swxx, float swy, float swyy,
                                                  float swxy) {
    const float prob = 1.0f / sw;
    const float mx = swx * prob, my = swy * prob;
    const float vx = fmaf(-mx, mx, swxx * prob);
    const float vy = fmaf(-my, my, swyy * prob);
    const float cov = fmaf(-mx, my, swxy * prob);
    const float ncc = cov / sqrtf(vx * vy);
    return (vx < 0.1f || vy < 0.1f) ? -1.0f : ncc;
}

// View combination; best = argmax of the per-source NCCs (sep).
//  PM_COMBINE_FOLD: the reference GPU kernel: NCC of the moments accumulated
//    over sources 0..r (cum[r], the reference never resets its sums between
//    views, PatchMatchCuda.cu:57-62,100-176), folded from -1 with "average
//    when within 25 %, else max" (PatchMatchCuda.cu:93,171);
//  PM_COMBINE_FOLD_SEPARATE: the same fold over the per-source NCCs;
//  PM_COMBINE_MAX: maximum (the reference CPU path, depthmap.cc:1104-1127);
//  PM_COMBINE_TOPK: mean of the top_k best sources (per-pixel view selection).
template <int S>
__device__ __forceinline__ float fold_scores(const float (&v)[S]) {
    float score = -1.0f;
#pragma unroll
    for (int r = 0; r < S; ++r) {
        const float s2 = v[r];
        score = (fabsf(__fdiv_rn(__fsub_rn(score, s2), s2)) < 0.25f) ? __fmul_rn(0.5f, __fadd_rn(score, s2))
                                                                     : fmaxf(score, s2);
    }
    return score;
}

template <int S>
__device__ __forceinline__ float combine_scores(const float (&sep)[S], const float (&cum)[S], int mode, int top_k,
                                                int *best) {
    int b = 0;
#pragma unroll
    for (int r = 1; r < S; ++r) b = (sep[r] > sep[b]) ? r : b;
    *best = b;
    if (mode == PM_COMBINE_FOLD) return fold_scores<S>(cum);
    if (mode == PM_COMBINE_FOLD_SEPARATE) return fold_scores<S>(sep);
    if (mode == PM_COMBINE_MAX) {
        float m = sep[0];
#pragma unroll
        for (int r = 1; r < S; ++r) m = fmaxf(m, sep[r]);
        return m;
    }
    // PM_COMBINE_TOPK: sum of the k largest by repeated selection
    float v[S];
#pragma unroll
    for (int r = 0; r < S; ++r) v[r] = sep[r];
    const int k = top_k < 1 ? 1 : (top_k > S ? S : top_k);
    float accf = 0.0f;  // summed in descending order
    for (int a = 0; a < k; ++a) {
        int bi = 0;
#pragma unroll
        for (int r = 1; r < S; ++r) bi = (v[r] > v[bi]) ? r : bi;
        float m = v[0];
#pragma unroll
        for (int r = 0; r < S; ++r) m = (r == bi) ? v[r] : m;
        accf += m;
#pragma unroll
        for (int r = 0; r < S; ++r) v[r] = (r == bi) ? -3.0e38f : v[r];
    }
    return accf / (float)k;
}

// Per-source and cumulative NCCs of one hypothesis from the window moments.
template <int S, class Img, class Acc>
__device__ __forceinline__ void source_nccs(const TapAccum<S, Img, Acc> &acc, float sw, float swx, float swxx, int mode,
                                            float (&sep)[S], float (&cum)[S]) {
#pragma unroll
    for (int r = 0; r < S; ++r) sep[r] = ncc_from_moments(sw, swx, swxx, acc.swy[r], acc.swyy[r], acc.swxy[r]);
    if (mode == PM_COMBINE_FOLD) {
        float cy = 0.f, cyy = 0.f, cxy = 0.f;
#pragma unroll
        for (int r = 0; r < S; ++r) {
            cy += acc.swy[r];
            cyy += acc.swyy[r];
            cxy += acc.swxy[r];
            const float n = (float)(r + 1);
            cum[r] = ncc_from_moments(n * sw, n * swx, n * swxx, cy, cyy, cxy);
        }
    } else {
#pragma unroll
        for (int r = 0; r < S; ++r) cum[r] = sep[r];
    }
}

}  // namespace pm
