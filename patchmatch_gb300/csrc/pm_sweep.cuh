// Tile kernel of the densifier: scores each pixel's own plane (init scoring,
// PatchMatchCuda.cu:255-270) or performs one red/black half-sweep of
// propagation + random refinement (PatchMatchCuda.cu:273-407).
//
// Layout: a CTA of 256 threads owns an 8-row x 64-column image tile and
// updates its 256 pixels of the active colour (one warp per row, one lane per
// pixel).  All window taps of a pixel of colour c are themselves pixels of
// colour c, so the CTA stages only those: an 18 x 37 shared-memory tile of
// (bearing, intensity) float4 including the 5-pixel halo, indexed so that the
// 32 lanes of a warp read 32 consecutive entries.  The hypothesis-independent
// reference moments are computed once per visit; the inner loop then
// evaluates each hypothesis over the 36 taps and S sources with S independent
// accumulation chains (recomputing each tap's bilateral weight, one MUFU.EX2
// shared by the sources).  From 9 sources the CTA also stages the row and
// column factors of the warp (see stage_factors).
#pragma once

#include "pm_device.cuh"

namespace pm {

#ifndef PM_TILE_H
#define PM_TILE_H 8
#endif
constexpr int kTileW = 64;
constexpr int kTileH = PM_TILE_H;  // rows per tile = warps per CTA
constexpr int kThreads = kTileH * 32;
constexpr int kCtaScale = 8 / kTileH;  // CTAs per SM scale inversely with the CTA size
constexpr int kHaloMax = 5;                       // largest supported patch_half
constexpr int kTileRows = kTileH + 2 * kHaloMax;  // 18
constexpr int kTileCols = (kTileW + 2 * kHaloMax) / 2;  // 37 same-colour entries per row
constexpr int kMaxTaps = (kHaloMax + 1) * (kHaloMax + 1);

constexpr int kTilePos = kTileRows * kTileCols;

// Stage the same-colour (bearing, intensity) tile.  Entry (tr, cc) holds image
// pixel (R, C) = (i0 - 5 + tr, x0 - 5 + 2 cc + ((R + colour + 1) & 1)); the
// bearing is (cos lat sin lon, -sin lat, cos lat cos lon).  Entries off the
// image are 0.
__device__ __forceinline__ void load_tile(float4 *tile, const float2 *row_trig, const float2 *col_trig,
                                          const float *ref, int W, int H, int i0, int x0, int colour) {
    for (int e = threadIdx.x; e < kTilePos; e += blockDim.x) {
        const int tr = e / kTileCols, cc = e - tr * kTileCols;
        const int R = i0 - kHaloMax + tr;
        const int C = x0 - kHaloMax + 2 * cc + ((R + colour + 1) & 1);
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (R >= 0 && R < H && C >= 0 && C < W) {
            const float2 rt = row_trig[R], ct = col_trig[C];
            v = make_float4(rt.x * ct.x, -rt.y, rt.x * ct.y, ref[(size_t)R * W + C]);
        }
        tile[e] = v;
    }
}

// While a hypothesis is scored, the rest of a pixel visit's state (current
// and candidate planes, score, depths, reference moments, packed counters
// and coordinates) is parked in shared memory, one 4-byte slot per value and
// thread, so that the scoring loop keeps its S accumulation chains in
// registers without spilling.  The centre bearing is re-read from the tile.
constexpr int kParkSlots = 17;

// Propagation candidates of a pixel visit: the neighbours (0,1), (1,0),
// (0,-1), (-1,0), (0,3), (3,0), (0,-3), (-3,0) (PatchMatchCuda.cu:305).
constexpr int kNbr = 8;

// Dynamic shared memory of tile_kernel: the staged tile, the parked state,
// the scratch of the speculative propagation pass (see tile_body) and the
// warp factors (per source: A of both column parities, B of both signs); the
// rest of the SM's unified L1/shared storage stays L1 for the texture
// samples, whose hit rate sets the kernel's speed.
constexpr int kFactorA = 2 * kTileCols;  // (column parity, same-colour column)
constexpr int kFactorB = 2 * kTileRows;  // (sign, row)
// Byte offsets: tile, parked state, speculative pass (reference moments per
// pixel, candidate scores and best sources per (candidate, pixel), the
// (pixel, candidate) work list, per-warp scan totals), factors.
constexpr size_t kSmemPark = sizeof(float4) * kTilePos;
constexpr size_t kSpecMom = kSmemPark + sizeof(float) * kParkSlots * kThreads;
constexpr size_t kSpecRes = kSpecMom + sizeof(float) * 3 * kThreads;
constexpr size_t kSpecBest = kSpecRes + sizeof(float) * kNbr * kThreads;
constexpr size_t kSpecList = kSpecBest + sizeof(int8_t) * kNbr * kThreads;
constexpr size_t kSpecTot = kSpecList + sizeof(uint16_t) * kNbr * kThreads;
constexpr size_t kSmemFactors = (kSpecTot + sizeof(int) * (kThreads / 32) + 15) / 16 * 16;
constexpr size_t kTileSmemBytes = kSmemFactors;
template <int S>
__host__ __device__ constexpr size_t tile_kernel_smem() {
    return kSmemFactors + (factored_warp<S>() ? sizeof(float4) * S * (kFactorA + kFactorB) : 0);
}
// Largest of the above over the source counts (the mixed batch kernel).
__host__ __device__ constexpr size_t tile_kernel_smem_max() {
    return tile_kernel_smem<PM_MAX_SOURCES>() > tile_kernel_smem<PM_FACTOR_MAX_SOURCES>()
               ? tile_kernel_smem<PM_MAX_SOURCES>()
               : tile_kernel_smem<PM_FACTOR_MAX_SOURCES>();
}
// Three CTAs of the largest layout fit one SM's 228 KB of shared memory.
static_assert(3 * kCtaScale * (tile_kernel_smem<8>() + 1024) <= 228 * 1024 &&
                  2 * kCtaScale * (tile_kernel_smem_max() + 1024) <= 228 * 1024,
              "tile layout exceeds the per-SM shared memory");

// Ask for the smallest shared-memory carveout that holds `blocks` CTAs of
// `kernel` with `dyn` bytes of dynamic shared memory, leaving the rest of the
// SM's unified storage to L1, where the texture samples hit (the driver's
// default keeps a larger carveout).  The driver rounds the percentage up to
// a supported size.
template <class K>
cudaError_t prefer_l1(K kernel, int dyn, int blocks) {
    int dev = 0, per_sm = 0, reserved = 0;
    cudaError_t e = cudaGetDevice(&dev);
    e = e ? e : cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    e = e ? e : cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
    cudaFuncAttributes fa{};
    e = e ? e : cudaFuncGetAttributes(&fa, kernel);
    if (e != cudaSuccess || per_sm <= 0) return e;
    const long long need = (long long)blocks * ((long long)dyn + (long long)fa.sharedSizeBytes + reserved);
    const int pct = (int)((need * 100 + per_sm - 1) / per_sm);
    return cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, pct < 100 ? pct : 100);
}

// Stage the warp factors of the tile: A(r, parity, cc) for image column
// x0 - 5 + 2 cc + parity and B(r, sign, tr) for image row i0 - 5 + tr, the
// latter as (sign B, sign cos lat) so that a tap reads sign(s) M_r b as
// fma(B.w, A, B) with B picked by the sign of s.  Entries off the image are 0.
template <int S, class Acc, class A>
__device__ __forceinline__ void stage_factors(float4 *fac, const A &a, int i0, int x0) {
    float4 *fa = fac, *fb = fac + S * kFactorA;
    for (int e = threadIdx.x; e < S * (kFactorA + kFactorB); e += blockDim.x) {
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (e < S * kFactorA) {
            const int r = e / kFactorA, q = e - r * kFactorA;
            const int pa = q / kTileCols, cc = q - pa * kTileCols;
            const int C = x0 - kHaloMax + 2 * cc + pa;
            if (C >= 0 && C < a.W) {
                const float2 ct = a.col_trig[C];
                const float3 f = col_factor(Acc::row(a.P.G[r][0]), Acc::row(a.P.G[r][1]), Acc::row(a.P.G[r][2]), ct.x,
                                            ct.y);
                v = make_float4(f.x, f.y, f.z, 0.0f);
            }
            fa[e] = v;
        } else {
            const int eb = e - S * kFactorA;
            const int r = eb / kFactorB, q = eb - r * kFactorB;
            const int neg = q / kTileRows, tr = q - neg * kTileRows;
            const int R = i0 - kHaloMax + tr;
            if (R >= 0 && R < a.H) {
                const float2 rt = a.row_trig[R];
                const float3 f = row_factor(Acc::row(a.P.G[r][0]), Acc::row(a.P.G[r][1]), Acc::row(a.P.G[r][2]), rt.y);
                const uint32_t sg = neg ? 0x80000000u : 0u;
                v = make_float4(flip_sign(f.x, sg), flip_sign(f.y, sg), flip_sign(f.z, sg), flip_sign(rt.x, sg));
            }
            fb[eb] = v;
        }
    }
}

// Per-thread slots of the parked state.  The accesses are volatile so that
// the compiler does not keep the values in registers across the scoring loop.
struct Park {
    unsigned base;
    __device__ __forceinline__ explicit Park(const unsigned char *smem)
        : base((unsigned)__cvta_generic_to_shared(reinterpret_cast<const float *>(smem + kSmemPark) + threadIdx.x)) {}
    __device__ __forceinline__ void put(int k, float v) const {
        asm volatile("st.shared.f32 [%0], %1;" ::"r"(base + 4u * kThreads * k), "f"(v) : "memory");
    }
    __device__ __forceinline__ float getf(int k) const {
        float v;
        asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(base + 4u * kThreads * k) : "memory");
        return v;
    }
    __device__ __forceinline__ void put(int k, int v) const { put(k, __int_as_float(v)); }
    __device__ __forceinline__ void put(int k, bool v) const { put(k, __int_as_float(v ? 1 : 0)); }
    __device__ __forceinline__ void get(int k, float &v) const { v = getf(k); }
    __device__ __forceinline__ void get(int k, int &v) const { v = __float_as_int(getf(k)); }
    __device__ __forceinline__ void get(int k, bool &v) const { v = __float_as_int(getf(k)) != 0; }
    template <class... T>
    __device__ __forceinline__ void save(const T &...v) const {
        int k = 0;
        (put(k++, v), ...);
    }
    template <class... T>
    __device__ __forceinline__ void load(T &...v) const {
        int k = 0;
        (get(k++, v), ...);
    }
};

// Resident CTAs per SM the register allocation targets: 3 (80 registers)
// up to 7 sources with the visit state parked; from 8 sources 2 (128
// registers), which also leaves each CTA a larger share of L1 for the
// texture samples (measured, 8 sweeps, 8 sources: 3840x1920 FP16 banded
// 444 -> 384 ms, u8 at 960x480 to 3840x1920 1-3 % faster; 7 sources at
// 1920x960 u8 1 % slower with 2).  The one-CTA-per-tile kernel runs 4 (64
// registers, no spills) up to 4 sources, where the extra warps hide more
// texture latency (measured, 8 sweeps at 1920x960: 2 sources 3 %, 3 sources
// 1 %, 4 sources 3 % faster; 5-6 sources spill and run 1-3 % slower).  The
// persistent kernels (banded, batched) keep 3 there: at 64 registers they
// spill.
template <int S>
constexpr int persistent_min_blocks() { return (S <= 7 ? 3 : 2) * kCtaScale; }
template <int S>
constexpr int tile_min_blocks() { return S <= 4 ? 4 * kCtaScale : persistent_min_blocks<S>(); }

// Smoothness factor f in [0, 1] of a propagated plane p against the pixel's
// current plane h and its depth before propagation (PatchMatchCuda.cu:322-337).
__device__ __forceinline__ float smoothness_factor(float px, float py, float pz, float hx, float hy, float hz,
                                                   float bxc, float byc, float bzc, float curr_depth) {
    const float scale = __fadd_rn(__fadd_rn(__fmul_rn(px, bxc), __fmul_rn(py, byc)), __fmul_rn(pz, bzc));
    const float denom = __fdiv_rn(1.0f, fmaxf(1e-6f, fabsf(scale)));
    const float dq = __fdiv_rn(__fsub_rn(curr_depth, denom), curr_depth);
    const float dsf = expf(__fmul_rn(-__fmul_rn(dq, dq), 1250.0f));
    const float prod = __fadd_rn(__fadd_rn(__fmul_rn(hx, px), __fmul_rn(hy, py)), __fmul_rn(hz, pz));
    const float ex = __fsub_rn(hx, px), ey = __fsub_rn(hy, py), ez = __fsub_rn(hz, pz);
    const float nrm = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(ex, ex), __fmul_rn(ey, ey)), __fmul_rn(ez, ez)));
    const float ac = acosf(__fdiv_rn(prod, nrm));
    const float psf = expf(__fmul_rn(-__fmul_rn(ac, ac), 8.0f));
    return __fmul_rn(__fsub_rn(1.0f, dsf), __fsub_rn(1.0f, psf));
}

// Geometry of same-colour pixel p (0..255) of the tile at (i0, x0): image
// position, its centre entry in the staged tile, the first tap row and column
// of its window in the tile, and the column parity of the staged entries on
// its tap rows (rows rbase + 2 m1 of the tile: image rows i0 - 5 + rbase + 2 m1).
struct TilePixel {
    int i, j, ctr_e, rbase, cbase, pa;
    __device__ __forceinline__ TilePixel(int p, int i0, int x0, int colour, int ph) {
        const int ty = p >> 5, lane = p & 31;
        i = i0 + ty;
        const int par = (i + colour) & 1;
        j = x0 + 2 * lane + par;
        ctr_e = (ty + kHaloMax) * kTileCols + ((2 * lane + par + kHaloMax) >> 1);
        rbase = ty + kHaloMax - ph;
        cbase = lane + ((kHaloMax - ph) >> 1);
        pa = (i0 + rbase + colour) & 1;
    }
};

// Image index of propagation candidate n of pixel (i, j).
__device__ __forceinline__ size_t nbr_index(int n, int i, int j, int W) {
    const int sel = n & 3, far = (n >> 2) ? 3 : 1;
    const int di = (sel == 1) ? far : (sel == 3 ? -far : 0);
    const int dj = (sel == 0) ? far : (sel == 2 ? -far : 0);
    return (size_t)(i + di) * W + (j + dj);
}

// Whether propagation candidate n of pixel (i, j) lies inside the W x H image;
// one outside is not a candidate.  Active pixels sit patch_half + 1 from every
// edge (PatchMatchCuda.cu:283), so with patch_half >= 3 all eight are inside;
// with patch_half = 1 the candidates 3 pixels out from the border pixels are not.
__device__ __forceinline__ bool nbr_inside(int n, int i, int j, int W, int H) {
    const int sel = n & 3, far = (n >> 2) ? 3 : 1;
    const int di = (sel == 1) ? far : (sel == 3 ? -far : 0);
    const int dj = (sel == 0) ? far : (sel == 2 ? -far : 0);
    return (unsigned)(i + di) < (unsigned)H && (unsigned)(j + dj) < (unsigned)W;
}

// Window moments of plane (px, py, pz) at a pixel: the 36 taps x S sources of
// the plane-induced warp (PatchMatchCuda.cu:100-157), one tap row and column
// at a time from the staged tile.
template <int S, class Img, class Acc, class A>
__device__ __forceinline__ void accumulate_plane(TapAccum<S, Img, Acc> &acc, const A &a, const float4 *tile,
                                                 const float4 *fac, int rbase, int cbase, int pa, float Ic, float px,
                                                 float py, float pz) {
    const int nt = a.patch_half + 1, ph = a.patch_half;
    const float shift = Img::shift_for(Ic);
    const float halfW = fmaf(0.5f, Acc::val(a.Wf), Img::kCoordOffset);
    const float halfH = fmaf(0.5f, Acc::val(a.Hf), Img::kCoordOffset);
    acc.zero();
#pragma unroll 1
    for (int m1 = 0; m1 < nt; ++m1) {
        const int tr = rbase + 2 * m1;
        const float4 *trow = tile + tr * kTileCols + cbase;
        const int k1 = 2 * m1 - ph;
        const float dk1 = (float)(k1 * k1) * Acc::val(a.ndf);
#pragma unroll 1
        for (int m2 = 0; m2 < nt; ++m2) {
            const float4 e = trow[m2];
            const int k2 = 2 * m2 - ph;
            const float xs = e.w - Ic;
            const float w = bilateral_weight(xs, Acc::val(a.ncf), fmaf((float)(k2 * k2), Acc::val(a.ndf), dk1));
            if constexpr (factored_warp<S>()) {
                const float s = fmaf(px, e.x, fmaf(py, e.y, pz * e.z));
                const float4 *fa = fac + pa * kTileCols + cbase + m2;
                const float4 *fb = fac + S * kFactorA + (s < 0.0f ? kTileRows : 0) + tr;
                acc.add_rot(a.P, a.src, Acc::val(a.Wf), Acc::val(a.Hf), halfW, halfH, shift, fabsf(s),
                            [&](int r) {
                                const float4 ca = fa[r * kFactorA], rb = fb[r * kFactorB];
                                return make_float3(fmaf(rb.w, ca.x, rb.x), fmaf(rb.w, ca.y, rb.y),
                                                   fmaf(rb.w, ca.z, rb.z));
                            },
                            w, xs);
            } else {
                acc.add_bearing(a.P, a.src, Acc::val(a.Wf), Acc::val(a.Hf), halfW, halfH, shift, px, py, pz, e.x, e.y,
                                e.z, w, xs);
            }
        }
    }
}

// Exclusive prefix sum of one count per thread over the CTA; *total gets the
// sum.  tot: one int per warp in shared memory.  Contains one barrier; the
// caller separates consecutive calls by at least one more.
__device__ __forceinline__ int cta_exclusive_scan(int cnt, int *tot, int *total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = cnt;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) tot[wid] = x;
    __syncthreads();
    int off = 0, sum = 0;
#pragma unroll
    for (int w = 0; w < kThreads / 32; ++w) {
        const int t = tot[w];
        off += (w < wid) ? t : 0;
        sum += t;
    }
    *total = sum;
    return off + x - cnt;
}

// One speculative round of the propagation pass: every thread lists the
// candidates in `need` (bit n = candidate n of its pixel), the CTA scores all
// listed (pixel, candidate) pairs with every thread taking the next pair, and
// the scores (NCC combination before the smoothness factor) and best sources
// land in res/res_best[n][pixel].  All threads of the CTA call it together.
template <int S, class Img, class Acc, class A>
__device__ __forceinline__ void spec_round(const A &a, const float4 *tile, const float4 *fac, unsigned char *smem,
                                           int i0, int x0, unsigned need) {
    const float *mom = reinterpret_cast<const float *>(smem + kSpecMom);
    float *res = reinterpret_cast<float *>(smem + kSpecRes);
    int8_t *res_best = reinterpret_cast<int8_t *>(smem + kSpecBest);
    uint16_t *list = reinterpret_cast<uint16_t *>(smem + kSpecList);
    int total;
    int k = cta_exclusive_scan(__popc(need), reinterpret_cast<int *>(smem + kSpecTot), &total);
    for (unsigned m = need; m; m &= m - 1) list[k++] = (uint16_t)((threadIdx.x << 3) | (__ffs(m) - 1));
    __syncthreads();
#pragma unroll 1
    for (int base = 0; base < total; base += kThreads) {
        const int q = base + (int)threadIdx.x;
        if (q < total) {
            const int e = list[q], p = e >> 3, n = e & 7;
            const TilePixel g(p, i0, x0, a.colour, a.patch_half);
            const float4 np = a.plane[nbr_index(n, g.i, g.j, a.W)];
            TapAccum<S, Img, Acc> acc;
            accumulate_plane(acc, a, tile, fac, g.rbase, g.cbase, g.pa, tile[g.ctr_e].w, np.x, np.y, np.z);
            float sep[S], cum[S];
            source_nccs(acc, mom[p], mom[kThreads + p], mom[2 * kThreads + p], a.combine, sep, cum);
            int hb;
            res[n * kThreads + p] = combine_scores<S>(sep, cum, a.combine, a.top_k, &hb);
            res_best[n * kThreads + p] = (int8_t)hb;
        }
    }
    __syncthreads();
}

// One tile visit: CTA-wide tile staging (one barrier), then per-thread work.
// `a` is the kernel's parameter block (single-request launches) or a copy in
// shared memory (the batched executor); (bx, by) is the tile index.
//
// Red-black sweeps (PatchMatchCuda.cu:287-404) visit each pixel's eight
// propagation candidates in order, then six refinements.  The refinements are
// scored for every pixel, but a candidate is scored only while it can still
// be accepted (2 f > score, see below), so pixels need 0-8 propagation costs
// and a warp that walks its lanes' candidates in step spends as long as its
// busiest lane.  The sweep therefore scores propagation speculatively: the
// CTA lists every (pixel, candidate) pair that passes the test in the pixel's
// state before propagation and scores the list with all its threads; each
// pixel then replays its candidates in order with those scores.  A candidate
// that passes only after an earlier one was taken (the test depends on the
// current plane and score) is listed in a further round, together with every
// later candidate that passes in the new state; rounds repeat until no pixel
// waits.  Every decision is the one the in-order walk takes, so results are
// unchanged; only the assignment of costs to threads differs.
template <int S, class Img, bool Plain, class Acc, class A>
__device__ __forceinline__ void tile_body(const A &a, int bx, int by, float4 *tile) {
    const int tid = threadIdx.x;
    const int x0 = bx * kTileW, i0 = by * kTileH;
    unsigned char *const smem = reinterpret_cast<unsigned char *>(tile);
    float4 *const fac = reinterpret_cast<float4 *>(smem + kSmemFactors);
    load_tile(tile, a.row_trig, a.col_trig, a.ref, a.W, a.H, i0, x0, a.colour);
    if constexpr (factored_warp<S>()) stage_factors<S, Acc>(fac, a, i0, x0);
    __syncthreads();

    const int W = a.W, H = a.H, ph = a.patch_half;
    const TilePixel g(tid, i0, x0, a.colour, ph);
    int i = g.i, j = g.j;
    const bool active = !(i < ph + 1 || i > H - ph - 1 || j < ph + 1 || j > W - ph - 1);  // PatchMatchCuda.cu:283
    constexpr bool plain = Plain;  // PM_PROPAGATION_PLAIN (a separate instantiation)
    const bool spec = a.mode == kModeSweep && !plain;
    if (!active && !spec) return;

    const int ctr_e = g.ctr_e;
    const int rbase = g.rbase, cbase = g.cbase, pa = g.pa;
    const float4 ctr = tile[ctr_e];
    float bxc = ctr.x, byc = ctr.y, bzc = ctr.z;
    const float Ic = ctr.w;
    const int nt = ph + 1;

    // hypothesis-independent moments of the reference window; the bilateral
    // weights are recomputed per tap in the hypothesis loop (one MUFU.EX2 per
    // tap, shared by all sources) rather than held in shared memory
    float sw = 0.f, swx = 0.f, swxx = 0.f;
    if (active) {
        for (int m1 = 0; m1 < nt; ++m1) {
            const int k1 = 2 * m1 - ph;
            for (int m2 = 0; m2 < nt; ++m2) {
                const int k2 = 2 * m2 - ph;
                const float xs = tile[(rbase + 2 * m1) * kTileCols + cbase + m2].w - Ic;
                const float w = bilateral_weight(xs, a.ncf, (float)(k1 * k1 + k2 * k2) * a.ndf);
                sw += w;
                swx = fmaf(w, xs, swx);
                swxx = fmaf(w * xs, xs, swxx);
            }
        }
    }

    size_t idx = (size_t)i * W + j;
    float4 cand = make_float4(0.f, 0.f, 0.f, 0.f);
    if (a.mode == kModeSeed) {
        cand = a.cand[idx];
        if (!(cand.w > 0.0f)) return;  // no candidate for this pixel
    }
    const float4 cur = active ? a.plane[idx] : make_float4(0.f, 0.f, 0.f, 0.f);
    if (a.mode == kModeSweep && plain && cur.w == 0.0f) return;  // ignored pixel (depthmap.cc:1007-1010)
    float score = active ? a.score[idx] : 0.0f;
    int best = active ? a.best[idx] : 0;
    float hx = cur.x, hy = cur.y, hz = cur.z;   // plane_*_hyp of the reference
    float curr_depth = cur.w;
    float cand_w = cand.w;
    bool moved = false;    // plain propagation: a neighbour's plane was taken
    int h = 0;

    if (spec) {
        // ---- speculative propagation pass (see above) ----
        float *mom = reinterpret_cast<float *>(smem + kSpecMom);
        mom[tid] = sw;
        mom[kThreads + tid] = swx;
        mom[2 * kThreads + tid] = swxx;
        const float *res = reinterpret_cast<const float *>(smem + kSpecRes);
        const int8_t *res_best = reinterpret_cast<const int8_t *>(smem + kSpecBest);
        // candidates passing 2 f > score (the in-order walk's test) for m >= from
        // in the current state that are not scored yet
        auto passing = [&](int from, unsigned have) {
            unsigned m = 0;
            if (active)
                for (int n = from; n < kNbr; ++n) {
                    if (((have >> n) & 1u) || !nbr_inside(n, i, j, W, H)) continue;
                    const float4 np = a.plane[nbr_index(n, i, j, W)];
                    const float f = smoothness_factor(np.x, np.y, np.z, hx, hy, hz, bxc, byc, bzc, curr_depth);
                    if (2.0f * f > score) m |= 1u << n;
                }
            return m;
        };
        unsigned need = passing(0, 0u), avail = 0;
        int n = 0;
        const Park park(smem);
#pragma unroll 1
        while (__syncthreads_or(need != 0)) {
            park.save(hx, hy, hz, score, best | (n << 8) | (int)(avail << 16) | (int)(need << 24), curr_depth);
            spec_round<S, Img, Acc>(a, tile, fac, smem, i0, x0, need);
            {
                int st;
                park.load(hx, hy, hz, score, st, curr_depth);
                best = (int)(int8_t)(st & 0xff);
                n = (st >> 8) & 0xff;
                avail = ((unsigned)st >> 16) & 0xffu;
                avail |= ((unsigned)st >> 24) & 0xffu;
                const float4 c = tile[ctr_e];
                bxc = c.x;
                byc = c.y;
                bzc = c.z;
            }
            need = 0;
            if (active) {
                // replay in order with the scores at hand (PatchMatchCuda.cu:305-337)
#pragma unroll 1
                for (; n < kNbr; ++n) {
                    if (!nbr_inside(n, i, j, W, H)) continue;
                    const float4 np = a.plane[nbr_index(n, i, j, W)];
                    const float f = smoothness_factor(np.x, np.y, np.z, hx, hy, hz, bxc, byc, bzc, curr_depth);
                    if (!(2.0f * f > score)) continue;  // cannot be accepted (also when f is NaN)
                    if (!((avail >> n) & 1u)) break;   // passes only in the state reached so far
                    const float sc = __fmul_rn(res[n * kThreads + tid], f);
                    if (sc > score) { hx = np.x; hy = np.y; hz = np.z; score = sc; best = res_best[n * kThreads + tid]; }
                }
                if (n < kNbr) need = (1u << n) | passing(n + 1, avail);
            }
        }
        if (!active) return;
        h = kNbr;  // refinements follow
    }

    float cx = hx, cy = hy, cz = hz, current_depth = curr_depth;
    float depth_hyp = 0.f;
    const int nh = a.mode == kModeSweep ? 14 : 1;

    // Propagated planes are scored as NCC x f with a smoothness factor
    // f in [0, 1] that does not depend on the cost (PatchMatchCuda.cu:322-337).
    // A candidate with 2 f <= score cannot be accepted by any combined score
    // <= 2 (the exact NCC is bounded by 1), so its cost is not evaluated.
    // In the plain (host-variant) propagation every neighbour is scored
    // unless its depth is 0, in order, by each lane for its own pixel.
    int kr = 0;            // plain propagation: refinements tried so far (their ranges shrink only when tried)
#pragma unroll 1
    while (true) {
        float px = 0.f, py = 0.f, pz = 0.f, f = 1.0f;
        bool found = false;
#pragma unroll 1
        for (; h < nh; ++h) {
            if (a.mode == kModeScore) {
                px = hx; py = hy; pz = hz;
            } else if (a.mode == kModeSeed) {
                px = cand.x; py = cand.y; pz = cand.z;
            } else if (h < kNbr) {
                if (!nbr_inside(h, i, j, W, H)) continue;
                const float4 np = a.plane[nbr_index(h, i, j, W)];
                px = np.x; py = np.y; pz = np.z;
                if (plain) {
                    if (np.w == 0.0f) continue;  // ignored neighbour (depthmap.cc:1018-1021)
                } else {
                    f = smoothness_factor(px, py, pz, hx, hy, hz, bxc, byc, bzc, curr_depth);
                    if (!(2.0f * f > score)) continue;  // cannot be accepted (also when f is NaN)
                }
            } else {
                const int t = h - kNbr;
                if (t == 0) {
                    // current depth after propagation (PatchMatchCuda.cu:340-341); the
                    // host variant keeps the stored depth unless a neighbour was taken
                    const float dn = __fadd_rn(__fadd_rn(__fmul_rn(bxc, hx), __fmul_rn(byc, hy)), __fmul_rn(bzc, hz));
                    current_depth = (plain && !moved) ? curr_depth : __fdiv_rn(1.0f, fmaxf(1e-6f, fabsf(dn)));
                    cx = hx; cy = hy; cz = hz;
                }
                if (plain) {
                    // refinement of the host variant (depthmap.cc:1035-1059): current
                    // plane and depth, skipped without shrinking the ranges when
                    // the plane's z is 0; plane from depth and normal with the
                    // 1e-5 clamp (PlanePosFromDepthAndNormal_equirect, :130-141)
                    if (cz == 0.0f) continue;
                    float z0, z1, z2, z3;
                    refine_normals4(a.seed, a.keyframe, (uint32_t)idx, (uint32_t)(a.sweep + 1), t, z0, z1, z2, z3);
                    depth_hyp = __fmul_rn(current_depth, expf(__fmul_rn(a.depth_range[kr], z0)));
                    const float nr = a.normal_range[kr];
                    ++kr;
                    const float nhx = __fadd_rn(cx, __fmul_rn(nr, z1));
                    const float nhy = __fadd_rn(cy, __fmul_rn(nr, z2));
                    const float nhz = __fadd_rn(cz, __fmul_rn(nr, z3));
                    const float qx = __fmul_rn(depth_hyp, bxc), qy = __fmul_rn(depth_hyp, byc), qz = __fmul_rn(depth_hyp, bzc);
                    float den = __fadd_rn(__fadd_rn(__fmul_rn(nhx, qx), __fmul_rn(nhy, qy)), __fmul_rn(nhz, qz));
                    if (den < 1e-5f && den >= 0.0f) den = 1e-5f;
                    else if (den > -1e-5f && den < 0.0f) den = -1e-5f;
                    px = __fdiv_rn(nhx, den); py = __fdiv_rn(nhy, den); pz = __fdiv_rn(nhz, den);
                } else {
                    // refinement t (PatchMatchCuda.cu:364-382) with Philox normals (tag sweep + 1)
                    float ra, rb, rc;
                    refine_normals(a.seed, a.keyframe, (uint32_t)idx, (uint32_t)(a.sweep + 1), t, ra, rb, rc);
                    depth_hyp = __fmul_rn(current_depth, expf(__fmul_rn(a.depth_range[t], ra)));
                    const float nr = a.normal_range[t];
                    const float nhx = __fadd_rn(cx, __fmul_rn(nr, ra));
                    const float nhy = __fadd_rn(cy, __fmul_rn(nr, rb));
                    const float nhz = __fadd_rn(cz, __fmul_rn(nr, rc));
                    const float qx = __fmul_rn(depth_hyp, bxc), qy = __fmul_rn(depth_hyp, byc), qz = __fmul_rn(depth_hyp, bzc);
                    const float den = __fadd_rn(__fadd_rn(__fmul_rn(nhx, qx), __fmul_rn(nhy, qy)), __fmul_rn(nhz, qz));
                    px = __fdiv_rn(nhx, den); py = __fdiv_rn(nhy, den); pz = __fdiv_rn(nhz, den);
                }
            }
            found = true;
            break;
        }
        if (!found) break;

        const Park park(smem);
        // h < 16, kr < 8, i < 2^15, j < 2^15 (image sizes are validated)
        park.save(hx, hy, hz, cx, cy, cz, score, current_depth, depth_hyp, f, sw, swx, swxx, curr_depth, cand_w,
                  h | (kr << 4) | ((int)moved << 7) | (best << 8), i | (j << 16));

        // ---- cost of hypothesis (px, py, pz) ----
        TapAccum<S, Img, Acc> acc;
        accumulate_plane(acc, a, tile, fac, rbase, cbase, pa, Ic, px, py, pz);
        {
            int st, ij;
            park.load(hx, hy, hz, cx, cy, cz, score, current_depth, depth_hyp, f, sw, swx, swxx, curr_depth, cand_w, st,
                      ij);
            h = st & 15;
            kr = (st >> 4) & 7;
            moved = (st >> 7) & 1;
            best = st >> 8;
            i = ij & 0xffff;
            j = ij >> 16;
            const float4 c = tile[ctr_e];
            bxc = c.x;
            byc = c.y;
            bzc = c.z;
        }
        idx = (size_t)i * W + j;
        float sep[S], cum[S];
        source_nccs(acc, sw, swx, swxx, a.combine, sep, cum);
        int hb;
        float sc = combine_scores<S>(sep, cum, a.combine, a.top_k, &hb);

        if (a.mode == kModeScore) {
            score = sc;
            best = hb;
        } else if (a.mode == kModeSeed) {
            if (sc > score) {  // the host seeding rule (depthmap.cc:483-487)
                cx = px; cy = py; cz = pz; score = sc; current_depth = cand_w; best = hb;
            }
        } else if (h < kNbr) {
            sc = __fmul_rn(sc, f);
            if (sc > score) { hx = px; hy = py; hz = pz; score = sc; best = hb; moved = true; }
        } else {
            if (sc > score) {
                cx = px; cy = py; cz = pz; score = sc; best = hb;
                if (plain) {
                    // the host variant stores the plane's own depth (CheckPlaneCandidate, depthmap.cc:1074-1076)
                    const float dn = __fadd_rn(__fadd_rn(__fmul_rn(bxc, px), __fmul_rn(byc, py)), __fmul_rn(bzc, pz));
                    current_depth = __fdiv_rn(1.0f, fmaxf(1e-6f, fabsf(dn)));
                } else {
                    current_depth = depth_hyp;
                }
            }
        }
        ++h;
    }

    a.score[idx] = score;
    a.best[idx] = (int8_t)best;
    if (a.mode == kModeSweep) {
        const float den = __fadd_rn(__fadd_rn(__fmul_rn(bxc, cx), __fmul_rn(byc, cy)), __fmul_rn(bzc, cz));
        a.plane[idx] = make_float4(cx, cy, cz, __fdiv_rn(1.0f, fmaxf(1e-6f, fabsf(den))));
    } else if (a.mode == kModeSeed) {
        a.plane[idx] = make_float4(cx, cy, cz, current_depth);
    }
}

template <int S, class Img, bool Plain>
__global__ void __launch_bounds__(kThreads, tile_min_blocks<S>()) tile_kernel(const __grid_constant__ SweepArgs a) {
    extern __shared__ float4 tile[];
    tile_body<S, Img, Plain, ParamAccess>(a, blockIdx.x, blockIdx.y, tile);
}

// Banded tile order (BandArgs): the same tile visit in a persistent grid.
// Tiles of one half-sweep never depend on each other, so any order gives
// the same result; no CTA waits on another (one atomic per tile taken, at
// most n_bands more when bands run out).
template <int S, class Img, bool Plain>
__global__ void __launch_bounds__(kThreads, persistent_min_blocks<S>())
    tile_kernel_banded(const __grid_constant__ SweepArgs a, const __grid_constant__ BandArgs b) {
    extern __shared__ float4 tile[];
    __shared__ int s_tile;
    unsigned smid;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
    int band = (int)(smid % (unsigned)b.n_home), exhausted = 0;
    for (;;) {
        if (threadIdx.x == 0) {
            int t = -1;
            while (exhausted < b.n_bands) {
                const int k = (int)atomicAdd(b.ctr + band, 1u);
                const int col = band % b.tiles_x, row = (band / b.tiles_x) * b.per_band + k;
                if (k < b.per_band && row < b.tiles_y) {
                    t = row * b.tiles_x + col;
                    break;
                }
                band = band + 1 == b.n_bands ? 0 : band + 1;
                ++exhausted;
            }
            s_tile = t;
        }
        __syncthreads();
        const int t = s_tile;
        if (t < 0) return;
        const int ty = t / b.tiles_x;
        tile_body<S, Img, Plain, ParamAccess>(a, t - ty * b.tiles_x, ty, tile);
        __syncthreads();  // before the next tile replaces the staged tile and s_tile
    }
}

// Batched executor: a persistent grid walks a device queue of (request,
// tile) work items of one phase (init scoring or one red/black half-sweep)
// over many requests with the same source count and image variant.  Each CTA
// takes the next item with one atomic, copies that request's arguments into
// shared memory and visits the tile.  Items of one phase never depend on each
// other (a half-sweep reads only the other colour), so no CTA waits on
// another; phases are separated by kernel boundaries.
template <int S, class Img, bool Plain>
__global__ void __launch_bounds__(kThreads, persistent_min_blocks<S>()) batch_kernel(const __grid_constant__ BatchArgs b) {
    extern __shared__ float4 tile[];
    __shared__ SweepArgs sa;
    __shared__ int s_item;
    for (;;) {
        if (threadIdx.x == 0) s_item = (int)atomicAdd(b.counter, 1u);
        __syncthreads();
        const int it = s_item;
        if (it >= b.n_items) return;
        const int4 w = b.items[it];
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
        tile_body<S, Img, Plain, SharedAccess>(sa, w.y, w.z, tile);
        __syncthreads();  // before the next item replaces the arguments and the tile
    }
}

// Fixed-hypothesis scoring: one thread per (pixel, plane); taps read straight
// from global memory (L1-resident) instead of a staged tile.  Same per-tap
// arithmetic (TapAccum) as the tile kernel.
template <int S, class Img>
__global__ void __launch_bounds__(256) hyp_kernel(const __grid_constant__ HypArgs a) {
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= a.n) return;
    const int2 ij = a.ij[h];
    const int i = ij.x, j = ij.y, W = a.W, ph = a.patch_half;
    const float Ic = a.ref[(size_t)i * W + j];
    const float px = a.planes[3 * h], py = a.planes[3 * h + 1], pz = a.planes[3 * h + 2];
    const float shift = Img::shift_for(Ic);
    const float halfW = fmaf(0.5f, a.Wf, Img::kCoordOffset), halfH = fmaf(0.5f, a.Hf, Img::kCoordOffset);
    float sw = 0.f, swx = 0.f, swxx = 0.f;
    TapAccum<S, Img> acc;
    acc.zero();
    for (int k1 = -ph; k1 <= ph; k1 += 2) {
        const int R = i + k1;
        const float2 rt = a.row_trig[R];
        for (int k2 = -ph; k2 <= ph; k2 += 2) {
            const int C = j + k2;
            const float2 ct = a.col_trig[C];
            const float x = a.ref[(size_t)R * W + C];
            const float xs = x - Ic;
            const float w = bilateral_weight(xs, a.ncf, fmaf((float)(k2 * k2), a.ndf, (float)(k1 * k1) * a.ndf));
            sw += w;
            swx = fmaf(w, xs, swx);
            swxx = fmaf(w * xs, xs, swxx);
            acc.add_trig(a.P, a.src, a.Wf, a.Hf, halfW, halfH, shift, px, py, pz, rt, ct, w, xs);
        }
    }
    float sep[S], cum[S];
    source_nccs(acc, sw, swx, swxx, a.combine, sep, cum);
    if (a.per_source)
#pragma unroll
        for (int r = 0; r < S; ++r) a.per_source[(size_t)h * S + r] = sep[r];
    int hb;
    const float sc = combine_scores<S>(sep, cum, a.combine, a.top_k, &hb);
    if (a.scores) a.scores[h] = sc;
    if (a.best) a.best[h] = hb;
}

}  // namespace pm
