// C ABI of the densifier (include/pm_gb300.h): contexts, device-resident
// requests, the captured init/sweep/post-filter graph, fixed-hypothesis
// scoring, the consistency filter and point fusion.  The batched executor
// is in pm_batch.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "pm_gb300.h"
#include "pm_internal.h"
#include "pm_kernels.h"
#include "pm_sweep.cuh"

namespace pm {
template <int S>
cudaError_t configure_tile();
}

using pmi::fail;
using pmi::align256;
using pmi::fill_args;
using pmi::check_views;
using pmi::enqueue_post;
using pmi::link_prior;
using pmi::unlink_dependents;

namespace {

// FFMA-bound probe: 8 independent chains per thread, 1 FMA = 2 flop.
__global__ void fp32_probe_kernel(float *out, int iters, float a, float b) {
    float x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int k = 0; k < iters; ++k) {
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
            x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
        }
    }
    const float s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == 1.2345f) out[0] = s;  // keeps the chains alive
}

// Special-function-unit probe: 8 independent chains of x <- 2^-x per thread
// (ex2.approx: one MUFU instruction, the unit whose reciprocal, reciprocal
// square root and exponential the cost kernel issues; the negation folds
// into the operand).  The chains converge to a fixed point near 0.64 and
// cannot be simplified away.
__global__ void sfu_probe_kernel(float *out, int iters) {
    float x[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) x[c] = 0.5f + 1e-3f * (float)threadIdx.x + 0.1f * (float)c;
    for (int k = 0; k < iters; ++k) {
#pragma unroll
        for (int u = 0; u < 16; ++u)
#pragma unroll
            for (int c = 0; c < 8; ++c) asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(x[c]) : "f"(-x[c]));
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < 8; ++c) s += x[c];
    if (s == 1.2345f) out[0] = s;
}

// Texture probe: independent bilinear fetches (8 per step) from a small u8
// texture that stays in L1, at coordinates that move by a non-integer step so
// every fetch filters four texels, as the cost kernel's samples do.
__global__ void tex_probe_kernel(cudaTextureObject_t tex, float *out, int iters) {
    const float u0 = 0.37f * (float)(threadIdx.x & 63) + 0.5f, v0 = 0.61f * (float)(threadIdx.x >> 6) + 0.5f;
    float s[8] = {};
    for (int k = 0; k < iters; ++k) {
        const float du = 0.013f * (float)(k & 255);
#pragma unroll
        for (int c = 0; c < 8; ++c) s[c] += tex2D<float>(tex, u0 + du + 3.3f * c, v0 + 1.7f * c);
    }
    float t = 0.f;
#pragma unroll
    for (int c = 0; c < 8; ++c) t += s[c];
    if (t == 1.2345f) out[0] = t;
}

}  // namespace

namespace {





int __float_as_int_host(float f) {
    int i;
    std::memcpy(&i, &f, sizeof i);
    return i;
}

// Start alignment of the per-source sampling buffers: texture objects bound
// to pitched linear memory need the device's texture alignment (512 bytes).
constexpr int kMaxBands = 1024;  // counters of the banded tile order (one per SM)
// The banded tile order (BandArgs) pays when the sources' texture rows are
// wide: the CTAs resident on an SM then overflow L1 with unrelated tiles'
// footprints.  Measured, 8 sweeps: 3840x1920 FP16 textures 4-8 sources
// 1-5 % faster, 2880x1440 FP16 6 sources 1 % faster, 3840x1920 u8 8 sources
// 2 % faster; below 30 KB of source row bytes at 1920x960 (any format and
// count) even or 1-4 % slower, where L1 already holds the footprints (95 %
// hit rate at 1920x960 u8).  From 2880 wide it pays from 21 KB with up to 7
// sources (3 CTAs per SM): 3840x1920 u8 6 sources 2.6 % and 7 sources 0.8 %,
// 2880x1440 FP16 4 sources 13 % and 5 sources 3.5 % faster; 2880x1440 u8
// with 7 sources (20 KB) was even, and with 8 sources (2 CTAs per SM, 23 KB)
// 1.4 % slower.
constexpr size_t kBandedMinRowBytes = 30000;
constexpr size_t kBandedMinRowBytesWide = 21000;  // W >= 2880, up to 7 sources
constexpr int kBandedWideW = 2880;
constexpr size_t kTexAlign = 512;

int get_trig(pm_ctx *ctx, int W, int H, Trig *out) {
    for (const Trig &t : ctx->trig)
        if (t.W == W && t.H == H) {
            *out = t;
            return PM_OK;
        }
    // lat = -pi (i/H - 1/2), lon = 2 pi (j/W - 1/2), evaluated in FP64 and rounded
    std::vector<float2> row(H), col(W);
    for (int i = 0; i < H; ++i) {
        const double lat = -M_PI * ((double)i / H - 0.5);
        row[i] = make_float2((float)std::cos(lat), (float)std::sin(lat));
    }
    for (int j = 0; j < W; ++j) {
        const double lon = 2.0 * M_PI * ((double)j / W - 0.5);
        col[j] = make_float2((float)std::sin(lon), (float)std::cos(lon));
    }
    Trig t;
    t.W = W;
    t.H = H;
    PM_CUDA(ctx, cudaMalloc(&t.row, sizeof(float2) * H));
    PM_CUDA(ctx, cudaMalloc(&t.col, sizeof(float2) * W));
    PM_CUDA(ctx, cudaMemcpy(t.row, row.data(), sizeof(float2) * H, cudaMemcpyHostToDevice));
    PM_CUDA(ctx, cudaMemcpy(t.col, col.data(), sizeof(float2) * W, cudaMemcpyHostToDevice));
    ctx->trig.push_back(t);
    *out = t;
    return PM_OK;
}

int ensure_scratch(pm_ctx *ctx, size_t bytes) {
    if (ctx->scratch_bytes >= bytes) return PM_OK;
    if (ctx->scratch) cudaFree(ctx->scratch);
    ctx->scratch = nullptr;
    ctx->scratch_bytes = 0;
    if (cudaMalloc(&ctx->scratch, bytes) != cudaSuccess) {
        cudaGetLastError();
        return fail(ctx, PM_ENOMEM, "scratch allocation of %zu bytes failed", bytes);
    }
    ctx->scratch_bytes = bytes;
    return PM_OK;
}

bool finite_pose(const double *R, const double *t) {
    for (int a = 0; a < 9; ++a)
        if (!std::isfinite(R[a])) return false;
    for (int a = 0; a < 3; ++a)
        if (!std::isfinite(t[a])) return false;
    return true;
}

// X_k = M X_0 + c with M = R_k R_0^T, c = t_k - M t_0 (FP64, then rounded)
void compose(const double *R0, const double *t0, const double *Rk, const double *tk, float *M, float *c) {
    pm::compose_pose(R0, t0, Rk, tk, M, c);
}

int validate_params(pm_ctx *ctx, const pm_params *p) {
    if (!p) return fail(ctx, PM_EINVAL, "params is NULL");
    if (p->patch_half != 1 && p->patch_half != 3 && p->patch_half != 5)
        return fail(ctx, PM_EINVAL, "patch_half must be 1, 3 or 5 (got %d)", p->patch_half);
    if (p->iterations < 0 || p->iterations > 1000) return fail(ctx, PM_EINVAL, "iterations out of range");
    if (p->combine < PM_COMBINE_FOLD || p->combine > PM_COMBINE_FOLD_SEPARATE) return fail(ctx, PM_EINVAL, "bad combine");
    if (p->top_k < 1) return fail(ctx, PM_EINVAL, "top_k must be >= 1");
    if (p->seam != PM_SEAM_CLAMP && p->seam != PM_SEAM_WRAP && p->seam != PM_SEAM_ZERO)
        return fail(ctx, PM_EINVAL, "bad seam");
    if (p->init_mode != PM_INIT_LOGUNIFORM_HEMI && p->init_mode != PM_INIT_REF_UNIFORM)
        return fail(ctx, PM_EINVAL, "bad init_mode");
    if (p->image_format != PM_IMAGE_U8 && p->image_format != PM_IMAGE_F16)
        return fail(ctx, PM_EINVAL, "bad image_format");
    if (p->sampler != PM_SAMPLER_EXACT && p->sampler != PM_SAMPLER_TEXTURE) return fail(ctx, PM_EINVAL, "bad sampler");
    if (p->propagation != PM_PROPAGATION_SMOOTH && p->propagation != PM_PROPAGATION_PLAIN)
        return fail(ctx, PM_EINVAL, "bad propagation");
    if (p->sampler == PM_SAMPLER_TEXTURE && p->seam != PM_SEAM_CLAMP)
        return fail(ctx, PM_EINVAL, "the texture sampler clamps at the seam (needs PM_SEAM_CLAMP)");
    if (!(p->min_depth > 0.0f) || !(p->max_depth > p->min_depth) || !std::isfinite(p->max_depth))
        return fail(ctx, PM_EINVAL, "need 0 < min_depth < max_depth");
    if (!(p->sigma_color > 0.0f) || !(p->sigma_x > 0.0f)) return fail(ctx, PM_EINVAL, "sigmas must be > 0");
    if (!std::isfinite(p->min_score) || !(p->min_patch_sd >= 0.0f)) return fail(ctx, PM_EINVAL, "bad thresholds");
    return PM_OK;
}

int validate_size(pm_ctx *ctx, int W, int H, int S) {
    if (W < 16 || H < 16 || W > 32768 || H > 16384)
        return fail(ctx, PM_EINVAL, "image size %dx%d out of range (16..32768 x 16..16384)", W, H);
    if ((size_t)(W + 1) * (H + 1) >= (size_t)1 << 31) return fail(ctx, PM_EINVAL, "image too large");
    if (S < 1 || S > PM_MAX_SOURCES) return fail(ctx, PM_EINVAL, "n_sources must be 1..%d (got %d)", PM_MAX_SOURCES, S);
    return PM_OK;
}

}  // namespace

int pmi::tile_band(pm_request *r, dim3 grid, cudaStream_t st, pm::BandArgs *band, const pm::BandArgs **out) {
    *out = nullptr;
    if (r->banded_blocks <= 0) return PM_OK;
    const int n_sm = r->ctx->n_sm, segs = (n_sm + (int)grid.x - 1) / (int)grid.x;
    band->ctr = r->band_ctr;
    band->tiles_x = (int)grid.x;
    band->tiles_y = (int)grid.y;
    band->per_band = ((int)grid.y + segs - 1) / segs;
    band->n_bands = (int)grid.x * segs;  // < tiles_x + n_sm <= kMaxBands
    band->n_home = n_sm;
    band->blocks = r->banded_blocks;
    PM_CUDA(r->ctx, cudaMemsetAsync(r->band_ctr, 0, sizeof(unsigned) * band->n_bands, st));
    *out = band;
    return PM_OK;
}

void pmi::link_prior(pm_request *r, const pm_request *prior, const pm_result *res) {
    const auto drop = [r](std::vector<pm_request *> &v) { v.erase(std::remove(v.begin(), v.end(), r), v.end()); };
    if (r->prior) drop(r->prior->dependents);
    if (r->prior_res) drop(r->prior_res->dependents);
    r->prior = prior;
    r->prior_res = res;
    if (prior) prior->dependents.push_back(r);
    if (res) res->dependents.push_back(r);
    r->graph_dirty = true;
}

void pmi::unlink_dependents(std::vector<pm_request *> &deps, bool from_request) {
    for (pm_request *d : deps) {
        cudaStreamSynchronize(d->stream);
        if (from_request)
            d->prior = nullptr;
        else
            d->prior_res = nullptr;
        d->graph_dirty = true;
    }
    deps.clear();
}

void pmi::fill_args(pm_request *r) {
    pm::SweepArgs &a = r->args;
    const pm_params &p = r->prm;
    for (int k = 0; k < r->S; ++k) {
        float M[9], c[3];
        compose(r->R[0], r->t[0], r->R[k + 1], r->t[k + 1], M, c);
        for (int row = 0; row < 3; ++row)
            a.P.G[k][row] = make_float4(M[3 * row], M[3 * row + 1], M[3 * row + 2], c[row]);
        a.src.quad[k] = r->quad[k];
        a.src.tex[k] = (unsigned long long)r->tex[k];
    }
    a.src.qpitch = r->W + 1;
    a.row_trig = r->trig.row;
    a.col_trig = r->trig.col;
    a.ref = r->ref;
    a.plane = r->plane;
    a.cand = r->seed;
    a.score = r->score;
    a.best = r->best;
    a.W = r->W;
    a.H = r->H;
    a.Wf = (float)r->W;
    a.Hf = (float)r->H;
    a.patch_half = p.patch_half;
    a.combine = p.combine;
    a.top_k = p.top_k;
    a.propagation = p.propagation;
    a.seed = p.seed;
    a.keyframe = p.keyframe_id;
    a.color_factor = 1.0f / (2 * p.sigma_color * p.sigma_color);
    a.dist_factor = 1.0f / (2 * p.sigma_x * p.sigma_x);
    a.ncf = (float)(-1.4426950408889634 * a.color_factor);
    a.ndf = (float)(-1.4426950408889634 * a.dist_factor);
    float dr = 0.02f, nr = 0.5f;  // PatchMatchCuda.cu:348-349,393-394 (float *= double)
    for (int t = 0; t < 6; ++t) {
        a.depth_range[t] = dr;
        a.normal_range[t] = nr;
        dr = (float)(dr * 0.3);
        nr = (float)(nr * 0.8);
    }
}

namespace {

void destroy_textures(pm_request *r) {
    for (int k = 0; k < r->S; ++k)
        if (r->tex[k]) {
            cudaDestroyTextureObject(r->tex[k]);
            r->tex[k] = 0;
        }
    r->tex_format = -1;
}

// Texture objects over the sources' sampling buffers, which then hold the
// images themselves at a texture-aligned pitch (the buffers are sized for
// quads, (W+1)(H+1) x 4 or 8 bytes, which is always enough).  Bilinear
// filter, clamp addressing, unnormalised coordinates; u8 texels read as
// value / 255, half texels as values.
int ensure_textures(pm_request *r) {
    if (r->tex_format == r->prm.image_format) return PM_OK;
    destroy_textures(r);
    pm_ctx *ctx = r->ctx;
    int align = 0, base_align = 0;
    PM_CUDA(ctx, cudaDeviceGetAttribute(&align, cudaDevAttrTexturePitchAlignment, ctx->device));
    PM_CUDA(ctx, cudaDeviceGetAttribute(&base_align, cudaDevAttrTextureAlignment, ctx->device));
    for (int k = 0; k < r->S; ++k)
        if (base_align > 0 && (uintptr_t)r->quad[k] % (uintptr_t)base_align)
            return fail(ctx, PM_ECUDA, "sampling buffer not aligned to the texture alignment (%d bytes)", base_align);
    const bool f16 = r->prm.image_format == PM_IMAGE_F16;
    const size_t es = f16 ? 2 : 1;
    const size_t a = (size_t)std::max(align, 32);
    r->tex_pitch = ((size_t)r->W * es + a - 1) / a * a;
    if (r->tex_pitch * r->H > (size_t)(r->W + 1) * (r->H + 1) * 4)
        return fail(ctx, PM_EINVAL, "texture pitch %zu does not fit the sampling buffer", r->tex_pitch);
    for (int k = 0; k < r->S; ++k) {
        cudaResourceDesc res{};
        res.resType = cudaResourceTypePitch2D;
        res.res.pitch2D.devPtr = r->quad[k];
        res.res.pitch2D.desc = f16 ? cudaCreateChannelDescHalf() : cudaCreateChannelDesc<uint8_t>();
        res.res.pitch2D.width = r->W;
        res.res.pitch2D.height = r->H;
        res.res.pitch2D.pitchInBytes = r->tex_pitch;
        cudaTextureDesc td{};
        td.addressMode[0] = cudaAddressModeClamp;
        td.addressMode[1] = cudaAddressModeClamp;
        td.filterMode = cudaFilterModeLinear;
        td.readMode = f16 ? cudaReadModeElementType : cudaReadModeNormalizedFloat;
        td.normalizedCoords = 0;
        if (cudaCreateTextureObject(&r->tex[k], &res, &td, nullptr) != cudaSuccess) {
            cudaGetLastError();
            destroy_textures(r);
            return fail(ctx, PM_ECUDA, "texture object creation failed");
        }
    }
    r->tex_format = r->prm.image_format;
    return PM_OK;
}

// Choose the tile order of a request: banded (persistent grid) for texture
// sampling when the sources' row bytes W x bytes per texel x S reach
// kBandedMinRowBytes (kBandedMinRowBytesWide from kBandedWideW pixels wide
// with up to 7 sources), else one CTA per tile (the quad samplers measured
// 4-6 % slower banded at 1920x960).
void set_tile_order(pm_request *r) {
    r->banded_blocks = 0;
    if (r->ctx->n_sm <= 0 || r->ctx->n_sm > kMaxBands / 2 || r->prm.sampler != PM_SAMPLER_TEXTURE) return;
    const size_t texel = r->prm.image_format == PM_IMAGE_F16 ? 2 : 1;
    const size_t min_row = (r->W >= kBandedWideW && r->S <= 7) ? kBandedMinRowBytesWide : kBandedMinRowBytes;
    if ((size_t)r->W * texel * (size_t)r->S < min_row) return;
    const int bps = pm::dispatch_tile_blocks_per_sm(r->S, pm::image_kind(r->prm.image_format, r->prm.sampler));
    r->banded_blocks = bps > 0 ? bps * r->ctx->n_sm : 0;
}

int launch_tile(pm_request *r, int mode, int colour, int sweep, cudaStream_t st = nullptr) {
    if (!st) st = r->stream;
    pm::SweepArgs a = r->args;
    a.mode = mode;
    a.colour = colour;
    a.sweep = sweep;
    const int kind = pm::image_kind(r->prm.image_format, r->prm.sampler);
    const dim3 grid = pm::tile_grid(r->W, r->H);
    pm::BandArgs band{};
    const pm::BandArgs *bp = nullptr;
    const int rc = pmi::tile_band(r, grid, st, &band, &bp);
    if (rc) return rc;
    cudaError_t e = pm::dispatch_tile(r->S, kind, grid, st, a, bp);
    r->ctx->launches++;
    if (e != cudaSuccess) return fail(r->ctx, PM_ECUDA, "tile kernel launch: %s", cudaGetErrorString(e));
    return PM_OK;
}

}  // namespace

int pmi::check_views(pm_request *r) {
    for (int k = 0; k <= r->S; ++k)
        if (!r->have[k]) return fail(r->ctx, PM_EINVAL, "view %d has not been set", k);
    return PM_OK;
}

namespace {

int enqueue_init(pm_request *r) {
    const pm_params &p = r->prm;
    pm::launch_init_planes(r->stream, r->trig.row, r->trig.col, r->W, r->H, p.seed, p.keyframe_id, p.init_mode,
                           p.min_depth, p.max_depth, r->plane, r->score, r->best);
    r->ctx->launches++;
    for (int c = 0; c < 2; ++c) {
        int rc = launch_tile(r, pm::kModeScore, c, 0);
        if (rc) return rc;
    }
    return PM_OK;
}

int enqueue_sweeps(pm_request *r, int first_half, int n_half) {
    for (int h = first_half; h < first_half + n_half; ++h) {
        int rc = launch_tile(r, pm::kModeSweep, h & 1, h >> 1);
        if (rc) return rc;
    }
    return PM_OK;
}

}  // namespace

int pmi::enqueue_post(pm_request *r, cudaStream_t st) {
    pm::PostArgs a{};
    a.plane = r->plane;
    a.score = r->score;
    a.ref = r->ref;
    a.mask = r->has_mask ? r->mask : nullptr;
    a.W = r->W;
    a.H = r->H;
    a.patch_half = r->prm.patch_half;
    a.min_var = r->prm.min_patch_sd * r->prm.min_patch_sd;
    a.min_depth = r->prm.min_depth;
    a.max_depth = r->prm.max_depth;
    a.min_score = r->prm.min_score;
    a.d0 = r->d0;
    a.s0 = r->s0;
    a.m1 = r->m1;
    a.out_depth = r->fdepth;
    a.out_score = r->fscore;
    pm::launch_postprocess(st ? st : r->stream, a);
    r->ctx->launches += 3;
    return PM_OK;
}

// Splat the prior result into this keyframe and keep candidates that score
// higher than the random initialisation.
namespace {

// Where a seeding prior comes from: a request's state or a retained result.
struct PriorSrc {
    const float4 *plane;
    const float *fdepth;
    int W, H;
    Trig trig;
    const double *R, *t;
};

int enqueue_seed_from(pm_request *r, const PriorSrc &prior, cudaStream_t st) {
    pm::WarpArgs w{};
    w.prev_plane = prior.plane;
    w.prev_depth = prior.fdepth;
    w.Wp = prior.W;
    w.Hp = prior.H;
    w.prow = prior.trig.row;
    w.pcol = prior.trig.col;
    compose(prior.R, prior.t, r->R[0], r->t[0], w.M, w.c);
    w.W = r->W;
    w.H = r->H;
    w.Wf = (float)r->W;
    w.Hf = (float)r->H;
    w.row = r->trig.row;
    w.col = r->trig.col;
    w.zbuf = r->zbuf;
    w.seed = r->seed;
    pm::launch_warp_prior(st, w);
    r->ctx->launches += 2;
    for (int c = 0; c < 2; ++c) {
        int rc = launch_tile(r, pm::kModeSeed, c, 0, st);
        if (rc) return rc;
    }
    return PM_OK;
}

// `postprocessed` is false for a prior that runs later in the same batch
// (its post-filter is enqueued before this seeding there).
int enqueue_seed(pm_request *r, const pm_request *prior, cudaStream_t st = nullptr, bool in_batch = false) {
    if (!prior->postprocessed && !(in_batch && prior->prm.postprocess))
        return fail(r->ctx, PM_EINVAL, "prior request has no post-filtered result");
    return enqueue_seed_from(r, PriorSrc{prior->plane, prior->fdepth, prior->W, prior->H, prior->trig, prior->R[0],
                                         prior->t[0]}, st ? st : r->stream);
}

int enqueue_seed_result(pm_request *r, const pm_result *res, cudaStream_t st = nullptr) {
    if (!res->valid) return fail(r->ctx, PM_EINVAL, "prior result holds no snapshot");
    return enqueue_seed_from(r, PriorSrc{res->plane, res->fdepth, res->W, res->H, res->trig, res->R, res->t},
                             st ? st : r->stream);
}

int enqueue_landmarks(pm_request *r, cudaStream_t st = nullptr) {
    if (!st) st = r->stream;
    pm::launch_landmark_cands(st, r->lm, r->n_lm, r->has_mask ? r->mask : nullptr, r->trig.row, r->trig.col,
                              r->W, r->H, r->seed);
    r->ctx->launches += r->n_lm > 0 ? 1 : 0;
    for (int c = 0; c < 2; ++c) {
        int rc = launch_tile(r, pm::kModeSeed, c, 0, st);
        if (rc) return rc;
    }
    return PM_OK;
}

// Project world points into the reference view (FP64, ReprojectEquirect,
// depthmap.cc:143-161), round to the nearest pixel (depthmap.cc:380-381) and
// keep the nearest landmark per pixel (then the lowest index); upload the
// list.  Points nearer than 1e-4 or rounding outside the image are skipped.
int stage_landmarks(pm_request *r, const double *xyz, int n) {
    pm_ctx *ctx = r->ctx;
    if (n < 0 || (n > 0 && !xyz)) return fail(ctx, PM_EINVAL, "bad landmark array");
    if (!r->have[0]) return fail(ctx, PM_EINVAL, "set the reference view before its landmarks");
    const double *R = r->R[0], *t = r->t[0];
    const double kPi = 3.14159265358979323846;
    std::vector<std::pair<int, float>> best;  // (pixel, depth) after dedupe
    std::vector<long long> key;               // per pixel in `best`: index into best
    std::vector<std::pair<long long, std::pair<float, int>>> all;
    all.reserve(n);
    for (int k = 0; k < n; ++k) {
        const double *p = xyz + 3 * (size_t)k;
        if (!(std::isfinite(p[0]) && std::isfinite(p[1]) && std::isfinite(p[2])))
            return fail(ctx, PM_EINVAL, "landmark %d is not finite", k);
        const double X = R[0] * p[0] + R[1] * p[1] + R[2] * p[2] + t[0];
        const double Y = R[3] * p[0] + R[4] * p[1] + R[5] * p[2] + t[1];
        const double Z = R[6] * p[0] + R[7] * p[1] + R[8] * p[2] + t[2];
        const double d = std::sqrt(X * X + Y * Y + Z * Z);
        if (d < 1e-4) continue;
        const double lat = -std::asin(std::max(-1.0, std::min(1.0, Y / d)));
        const double lon = std::atan2(X, Z);
        const double x = r->W * (0.5 + lon / (2.0 * kPi)), y = r->H * (0.5 - lat / kPi);
        const int x0 = (int)(x + 0.5), y0 = (int)(y + 0.5);
        if (x0 < 0 || y0 < 0 || x0 >= r->W || y0 >= r->H) continue;
        all.push_back({(long long)y0 * r->W + x0, {(float)d, k}});
    }
    std::sort(all.begin(), all.end());  // by pixel, then depth, then landmark index
    std::vector<int2> list;
    for (size_t q = 0; q < all.size(); ++q)
        if (q == 0 || all[q].first != all[q - 1].first)
            list.push_back(make_int2((int)all[q].first, __float_as_int_host(all[q].second.first)));
    if ((int)list.size() > r->lm_cap) {
        if (r->lm) cudaFree(r->lm);
        r->lm = nullptr;
        r->lm_cap = 0;
        if (cudaMalloc(&r->lm, list.size() * sizeof(int2)) != cudaSuccess) {
            cudaGetLastError();
            return fail(ctx, PM_ENOMEM, "landmark buffer of %zu entries", list.size());
        }
        r->lm_cap = (int)list.size();
        r->graph_dirty = true;
    }
    if (!list.empty())
        PM_CUDA(ctx, cudaMemcpyAsync(r->lm, list.data(), list.size() * sizeof(int2), cudaMemcpyHostToDevice,
                                     r->stream));
    // the run graph is shaped by the count (one kernel more or less)
    if ((int)list.size() != r->n_lm) r->graph_dirty = true;
    r->n_lm = (int)list.size();
    return PM_OK;
}

}  // namespace

int pmi::enqueue_seeding(pm_request *r, cudaStream_t st, bool in_batch) {
    int rc = PM_OK;
    if (r->n_lm > 0) rc = enqueue_landmarks(r, st);
    if (!rc && r->prior) rc = enqueue_seed(r, r->prior, st, in_batch);
    else if (!rc && r->prior_res) rc = enqueue_seed_result(r, r->prior_res, st);
    return rc;
}

int pmi::wait_prior_ready(pm_request *r, cudaStream_t st) {
    if (r->prior && r->prior->stream != st) {
        PM_CUDA(r->ctx, cudaEventRecord(r->prior->ready, r->prior->stream));
        PM_CUDA(r->ctx, cudaStreamWaitEvent(st, r->prior->ready, 0));
    }
    if (r->prior_res) PM_CUDA(r->ctx, cudaStreamWaitEvent(st, r->prior_res->ready, 0));
    return PM_OK;
}

namespace {

int enqueue_run(pm_request *r) {
    int rc = enqueue_init(r);
    if (!rc && r->n_lm > 0) rc = enqueue_landmarks(r);
    if (!rc && r->prior) rc = enqueue_seed(r, r->prior);
    else if (!rc && r->prior_res) rc = enqueue_seed_result(r, r->prior_res);
    if (!rc) rc = enqueue_sweeps(r, 0, 2 * r->prm.iterations);
    if (!rc && r->prm.postprocess) rc = enqueue_post(r);
    return rc;
}

}  // namespace

namespace pm {
dim3 tile_grid(int W, int H) { return dim3((W + kTileW - 1) / kTileW, (H + kTileH - 1) / kTileH); }

cudaError_t dispatch_tile(int S, int kind, dim3 grid, cudaStream_t st, const SweepArgs &a, const BandArgs *band) {
    switch (S) {
        case 1: return launch_tile<1>(kind, grid, st, a, band);
        case 2: return launch_tile<2>(kind, grid, st, a, band);
        case 3: return launch_tile<3>(kind, grid, st, a, band);
        case 4: return launch_tile<4>(kind, grid, st, a, band);
        case 5: return launch_tile<5>(kind, grid, st, a, band);
        case 6: return launch_tile<6>(kind, grid, st, a, band);
        case 7: return launch_tile<7>(kind, grid, st, a, band);
        case 8: return launch_tile<8>(kind, grid, st, a, band);
        case 9: return launch_tile<9>(kind, grid, st, a, band);
        case 10: return launch_tile<10>(kind, grid, st, a, band);
        default: return cudaErrorInvalidValue;
    }
}

int dispatch_tile_blocks_per_sm(int S, int kind) {
    switch (S) {
        case 1: return tile_blocks_per_sm<1>(kind);
        case 2: return tile_blocks_per_sm<2>(kind);
        case 3: return tile_blocks_per_sm<3>(kind);
        case 4: return tile_blocks_per_sm<4>(kind);
        case 5: return tile_blocks_per_sm<5>(kind);
        case 6: return tile_blocks_per_sm<6>(kind);
        case 7: return tile_blocks_per_sm<7>(kind);
        case 8: return tile_blocks_per_sm<8>(kind);
        case 9: return tile_blocks_per_sm<9>(kind);
        case 10: return tile_blocks_per_sm<10>(kind);
        default: return 0;
    }
}

cudaError_t dispatch_batch(int S, int kind, bool plain, int blocks, cudaStream_t st, const BatchArgs &b) {
    switch (S) {
        case 1: return launch_batch<1>(kind, plain, blocks, st, b);
        case 2: return launch_batch<2>(kind, plain, blocks, st, b);
        case 3: return launch_batch<3>(kind, plain, blocks, st, b);
        case 4: return launch_batch<4>(kind, plain, blocks, st, b);
        case 5: return launch_batch<5>(kind, plain, blocks, st, b);
        case 6: return launch_batch<6>(kind, plain, blocks, st, b);
        case 7: return launch_batch<7>(kind, plain, blocks, st, b);
        case 8: return launch_batch<8>(kind, plain, blocks, st, b);
        case 9: return launch_batch<9>(kind, plain, blocks, st, b);
        case 10: return launch_batch<10>(kind, plain, blocks, st, b);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t dispatch_batch_mixed(int kind, bool plain, int blocks, cudaStream_t st, const BatchArgs &b) {
    switch (kind) {
        case kImageQuadF16: return launch_batch_mixed<kImageQuadF16>(plain, blocks, st, b);
        case kImageTexU8: return launch_batch_mixed<kImageTexU8>(plain, blocks, st, b);
        case kImageTexF16: return launch_batch_mixed<kImageTexF16>(plain, blocks, st, b);
        default: return launch_batch_mixed<kImageQuadU8>(plain, blocks, st, b);
    }
}

int dispatch_batch_mixed_blocks_per_sm(int kind, bool plain) {
    switch (kind) {
        case kImageQuadF16: return batch_mixed_blocks_per_sm<kImageQuadF16>(plain);
        case kImageTexU8: return batch_mixed_blocks_per_sm<kImageTexU8>(plain);
        case kImageTexF16: return batch_mixed_blocks_per_sm<kImageTexF16>(plain);
        default: return batch_mixed_blocks_per_sm<kImageQuadU8>(plain);
    }
}

int dispatch_batch_blocks_per_sm(int S, int kind, bool plain) {
    switch (S) {
        case 1: return batch_blocks_per_sm<1>(kind, plain);
        case 2: return batch_blocks_per_sm<2>(kind, plain);
        case 3: return batch_blocks_per_sm<3>(kind, plain);
        case 4: return batch_blocks_per_sm<4>(kind, plain);
        case 5: return batch_blocks_per_sm<5>(kind, plain);
        case 6: return batch_blocks_per_sm<6>(kind, plain);
        case 7: return batch_blocks_per_sm<7>(kind, plain);
        case 8: return batch_blocks_per_sm<8>(kind, plain);
        case 9: return batch_blocks_per_sm<9>(kind, plain);
        case 10: return batch_blocks_per_sm<10>(kind, plain);
        default: return 0;
    }
}

cudaError_t dispatch_hyp(int S, int kind, int n, cudaStream_t st, const HypArgs &a) {
    switch (S) {
        case 1: return launch_hyp<1>(kind, n, st, a);
        case 2: return launch_hyp<2>(kind, n, st, a);
        case 3: return launch_hyp<3>(kind, n, st, a);
        case 4: return launch_hyp<4>(kind, n, st, a);
        case 5: return launch_hyp<5>(kind, n, st, a);
        case 6: return launch_hyp<6>(kind, n, st, a);
        case 7: return launch_hyp<7>(kind, n, st, a);
        case 8: return launch_hyp<8>(kind, n, st, a);
        case 9: return launch_hyp<9>(kind, n, st, a);
        case 10: return launch_hyp<10>(kind, n, st, a);
        default: return cudaErrorInvalidValue;
    }
}
}  // namespace pm

// ===========================================================================
extern "C" {

void pm_params_default(pm_params *p) {
    if (!p) return;
    std::memset(p, 0, sizeof *p);
    p->patch_half = 5;
    p->iterations = 8;
    p->combine = PM_COMBINE_FOLD;
    p->top_k = 3;
    p->seam = PM_SEAM_CLAMP;
    p->init_mode = PM_INIT_LOGUNIFORM_HEMI;
    p->image_format = PM_IMAGE_U8;
    p->postprocess = 1;
    p->min_depth = 0.3f;
    p->max_depth = 20.0f;
    p->min_score = 0.1f;
    p->min_patch_sd = 0.0f;
    p->sigma_color = 50.0f;
    p->sigma_x = 5.0f;
    p->seed = 0;
    p->keyframe_id = 0;
    p->sampler = PM_SAMPLER_TEXTURE;
    p->propagation = PM_PROPAGATION_SMOOTH;
}

const char *pm_status_string(int s) {
    switch (s) {
        case PM_OK: return "ok";
        case PM_EINVAL: return "invalid argument";
        case PM_ENOMEM: return "out of device memory";
        case PM_EBUDGET: return "HBM budget exceeded";
        case PM_ETIMEOUT: return "timed out";
        case PM_ECUDA: return "CUDA error";
        case PM_ENOTREADY: return "not ready";
        case PM_ECANCELLED: return "cancelled";
        case PM_ENOTBUILT: return "configuration not built";
        default: return "unknown status";
    }
}

int pm_create(int device, size_t hbm_budget_bytes, pm_ctx **out) {
    if (!out) return PM_EINVAL;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return PM_ECUDA;
    }
    if (device < 0 || device >= n) return PM_EINVAL;
    if (cudaSetDevice(device) != cudaSuccess) return PM_ECUDA;
    pm_ctx *ctx = new pm_ctx();
    ctx->device = device;
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete ctx;
        return PM_ECUDA;
    }
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    ctx->budget = hbm_budget_bytes ? hbm_budget_bytes : (size_t)(0.9 * (double)fr);
    if (cudaDeviceGetAttribute(&ctx->n_sm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
        cudaGetLastError();
        ctx->n_sm = 0;  // one CTA per tile
    }
    // opt every tile-kernel variant in to its dynamic shared memory up front,
    // so graph capture never meets a first-use attribute call
    cudaError_t e = cudaSuccess;
    e = e ? e : pm::configure_tile<1>();
    e = e ? e : pm::configure_tile<2>();
    e = e ? e : pm::configure_tile<3>();
    e = e ? e : pm::configure_tile<4>();
    e = e ? e : pm::configure_tile<5>();
    e = e ? e : pm::configure_tile<6>();
    e = e ? e : pm::configure_tile<7>();
    e = e ? e : pm::configure_tile<8>();
    e = e ? e : pm::configure_tile<9>();
    e = e ? e : pm::configure_tile<10>();
    e = e ? e : pm::configure_batch_mixed<pm::kImageQuadU8>();
    e = e ? e : pm::configure_batch_mixed<pm::kImageQuadF16>();
    e = e ? e : pm::configure_batch_mixed<pm::kImageTexU8>();
    e = e ? e : pm::configure_batch_mixed<pm::kImageTexF16>();
    if (e != cudaSuccess) {
        cudaStreamDestroy(ctx->stream);
        delete ctx;
        return PM_ECUDA;
    }
    *out = ctx;
    return PM_OK;
}

int pm_destroy(pm_ctx *ctx) {
    if (!ctx) return PM_EINVAL;
    if (ctx->live > (ctx->cached ? 1 : 0))
        return fail(ctx, PM_EINVAL, "%d request(s), result(s) or batch(es) of this context are still alive",
                    ctx->live - (ctx->cached ? 1 : 0));
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (ctx->cached) pm_request_destroy(ctx->cached);
    for (Trig &t : ctx->trig) {
        cudaFree(t.row);
        cudaFree(t.col);
    }
    if (ctx->scratch) cudaFree(ctx->scratch);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return PM_OK;
}

const char *pm_last_error(const pm_ctx *ctx) { return ctx ? ctx->err.c_str() : "no context"; }

uint64_t pm_launch_count(const pm_ctx *ctx) { return ctx ? ctx->launches : 0; }

void *pm_stream(const pm_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

int pm_probe_fp32_peak(pm_ctx *ctx, double *tflops) {
    if (!ctx || !tflops) return fail(ctx, PM_EINVAL, "NULL argument");
    PM_CUDA(ctx, cudaSetDevice(ctx->device));
    int sms = 0;
    PM_CUDA(ctx, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    int rc = ensure_scratch(ctx, 256);
    if (rc) return rc;
    cudaEvent_t e0, e1;
    PM_CUDA(ctx, cudaEventCreate(&e0));
    PM_CUDA(ctx, cudaEventCreate(&e1));
    const int iters = 2048, threads = 256, blocks = sms * 8;
    double best = 0.0;
    for (int rep = 0; rep < 4; ++rep) {
        PM_CUDA(ctx, cudaEventRecord(e0, ctx->stream));
        fp32_probe_kernel<<<blocks, threads, 0, ctx->stream>>>((float *)ctx->scratch, iters, 0.999999f, 1e-7f);
        PM_CUDA(ctx, cudaEventRecord(e1, ctx->stream));
        PM_CUDA(ctx, cudaEventSynchronize(e1));
        float ms = 0.f;
        PM_CUDA(ctx, cudaEventElapsedTime(&ms, e0, e1));
        const double flop = 2.0 * 8 * 16 * (double)iters * threads * blocks;
        if (rep > 0) best = std::max(best, flop / (ms * 1e-3) / 1e12);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *tflops = best;
    return PM_OK;
}

// Time `launch` (one launch on the context's stream) four times and return
// the best rate of `ops` operations per launch, in ops/s, over the last three.
extern "C++" template <class F>
int best_rate(pm_ctx *ctx, double ops, F launch, double *rate) {
    cudaEvent_t e0, e1;
    PM_CUDA(ctx, cudaEventCreate(&e0));
    PM_CUDA(ctx, cudaEventCreate(&e1));
    double best = 0.0;
    for (int rep = 0; rep < 4; ++rep) {
        PM_CUDA(ctx, cudaEventRecord(e0, ctx->stream));
        launch();
        PM_CUDA(ctx, cudaGetLastError());
        PM_CUDA(ctx, cudaEventRecord(e1, ctx->stream));
        PM_CUDA(ctx, cudaEventSynchronize(e1));
        float ms = 0.f;
        PM_CUDA(ctx, cudaEventElapsedTime(&ms, e0, e1));
        if (rep > 0) best = std::max(best, ops / (ms * 1e-3));
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *rate = best;
    return PM_OK;
}

int pm_probe_sfu_peak(pm_ctx *ctx, double *gops) {
    if (!ctx || !gops) return fail(ctx, PM_EINVAL, "NULL argument");
    PM_CUDA(ctx, cudaSetDevice(ctx->device));
    int sms = 0;
    PM_CUDA(ctx, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    int rc = ensure_scratch(ctx, 256);
    if (rc) return rc;
    const int iters = 512, threads = 256, blocks = sms * 8;
    double r = 0.0;
    rc = best_rate(ctx, 8.0 * 16 * iters * threads * blocks, [&] {
        sfu_probe_kernel<<<blocks, threads, 0, ctx->stream>>>((float *)ctx->scratch, iters);
    }, &r);
    *gops = r / 1e9;
    return rc;
}

int pm_probe_tex_peak(pm_ctx *ctx, double *gfetches) {
    if (!ctx || !gfetches) return fail(ctx, PM_EINVAL, "NULL argument");
    PM_CUDA(ctx, cudaSetDevice(ctx->device));
    int sms = 0, align = 0;
    PM_CUDA(ctx, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    PM_CUDA(ctx, cudaDeviceGetAttribute(&align, cudaDevAttrTexturePitchAlignment, ctx->device));
    const int TW = 128, TH = 128;
    const size_t pitch = ((size_t)TW + std::max(align, 32) - 1) / std::max(align, 32) * std::max(align, 32);
    int rc = ensure_scratch(ctx, 512 + pitch * TH);
    if (rc) return rc;
    uint8_t *img = (uint8_t *)ctx->scratch + 512;  // the scratch block is 256-byte aligned
    PM_CUDA(ctx, cudaMemsetAsync(img, 0x5A, pitch * TH, ctx->stream));
    cudaResourceDesc res{};
    res.resType = cudaResourceTypePitch2D;
    res.res.pitch2D.devPtr = img;
    res.res.pitch2D.desc = cudaCreateChannelDesc<uint8_t>();
    res.res.pitch2D.width = TW;
    res.res.pitch2D.height = TH;
    res.res.pitch2D.pitchInBytes = pitch;
    cudaTextureDesc td{};
    td.addressMode[0] = cudaAddressModeClamp;
    td.addressMode[1] = cudaAddressModeClamp;
    td.filterMode = cudaFilterModeLinear;
    td.readMode = cudaReadModeNormalizedFloat;
    cudaTextureObject_t tex = 0;
    PM_CUDA(ctx, cudaCreateTextureObject(&tex, &res, &td, nullptr));
    const int iters = 256, threads = 256, blocks = sms * 8;
    double r = 0.0;
    rc = best_rate(ctx, 8.0 * iters * threads * blocks, [&] {
        tex_probe_kernel<<<blocks, threads, 0, ctx->stream>>>(tex, (float *)ctx->scratch, iters);
    }, &r);
    cudaDestroyTextureObject(tex);
    *gfetches = r / 1e9;
    return rc;
}

size_t pm_request_bytes(int W, int H, int S, int fmt) {
    const size_t N = (size_t)W * H, NQ = (size_t)(W + 1) * (H + 1);
    const size_t qb = fmt == PM_IMAGE_F16 ? 8 : 4;
    size_t b = 0;
    b += align256(N * 4);                 // ref
    b += align256(N * 2);                 // raw staging
    b += (size_t)S * (align256(NQ * qb) + kTexAlign);  // quads (texture-aligned starts)
    b += align256(N);                     // mask
    b += align256(N * 16);                // plane
    b += align256(N * 4);                 // score
    b += align256(N);                     // best
    b += 5 * align256(N * 4);             // d0 s0 m1 fdepth fscore
    b += 2 * align256(N * 4) + 2 * align256(N * 12) + align256(N * 4);  // export staging
    b += align256(N * 16) + align256(N * 8);                            // seeding
    b += align256(sizeof(unsigned) * kMaxBands);                        // banded tile counters
    return b;
}

int pm_request_create(pm_ctx *ctx, int W, int H, int S, const pm_params *params, pm_request **out) {
    if (!ctx || !out) return fail(ctx, PM_EINVAL, "NULL argument");
    *out = nullptr;
    int rc = validate_size(ctx, W, H, S);
    if (rc) return rc;
    rc = validate_params(ctx, params);
    if (rc) return rc;
    PM_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t bytes = pm_request_bytes(W, H, S, params->image_format);
    if (ctx->used + bytes > ctx->budget)
        return fail(ctx, PM_EBUDGET, "request needs %zu bytes, %zu of %zu in use", bytes, ctx->used, ctx->budget);
    pm_request *r = new pm_request();
    r->ctx = ctx;
    r->W = W;
    r->H = H;
    r->S = S;
    r->prm = *params;
    r->bytes = bytes;
    rc = get_trig(ctx, W, H, &r->trig);
    if (rc) {
        delete r;
        return rc;
    }
    if (cudaMalloc(&r->block, bytes) != cudaSuccess) {
        cudaGetLastError();
        delete r;
        return fail(ctx, PM_ENOMEM, "device allocation of %zu bytes failed", bytes);
    }
    if (cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&r->ready, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        if (r->stream) cudaStreamDestroy(r->stream);
        cudaFree(r->block);
        delete r;
        return fail(ctx, PM_ECUDA, "stream creation failed");
    }
    const size_t N = (size_t)W * H, NQ = (size_t)(W + 1) * (H + 1);
    const size_t qb = params->image_format == PM_IMAGE_F16 ? 8 : 4;
    char *p = static_cast<char *>(r->block);
    auto take = [&](size_t n) { void *q = p; p += align256(n); return q; };
    r->ref = (float *)take(N * 4);
    r->raw = (uint8_t *)take(N * 2);
    for (int k = 0; k < S; ++k) {
        // texture objects over these buffers need kTexAlign-aligned addresses
        p = (char *)(((uintptr_t)p + kTexAlign - 1) / kTexAlign * kTexAlign);
        r->quad[k] = take(NQ * qb);
    }
    r->mask = (uint8_t *)take(N);
    r->plane = (float4 *)take(N * 16);
    r->score = (float *)take(N * 4);
    r->best = (int8_t *)take(N);
    r->d0 = (float *)take(N * 4);
    r->s0 = (float *)take(N * 4);
    r->m1 = (float *)take(N * 4);
    r->fdepth = (float *)take(N * 4);
    r->fscore = (float *)take(N * 4);
    r->x_depth = (float *)take(N * 4);
    r->x_score = (float *)take(N * 4);
    r->x_plane3 = (float *)take(N * 12);
    r->x_normal3 = (float *)take(N * 12);
    r->x_best = (int32_t *)take(N * 4);
    r->seed = (float4 *)take(N * 16);
    r->zbuf = (unsigned long long *)take(N * 8);
    r->band_ctr = (unsigned *)take(sizeof(unsigned) * kMaxBands);
    set_tile_order(r);
    ctx->used += bytes;
    ++ctx->live;
    *out = r;
    return PM_OK;
}

int pm_request_destroy(pm_request *r) {
    if (!r) return PM_EINVAL;
    pm_ctx *ctx = r->ctx;
    if (r->batch_refs > 0)
        return fail(ctx, PM_EINVAL, "request is in %d batch(es): clear or destroy them first", r->batch_refs);
    cudaSetDevice(ctx->device);
    unlink_dependents(r->dependents, true);
    link_prior(r, nullptr, nullptr);
    cudaStreamSynchronize(r->stream);
    if (r->gexec) cudaGraphExecDestroy(r->gexec);
    if (r->graph) cudaGraphDestroy(r->graph);
    destroy_textures(r);
    if (r->lm) cudaFree(r->lm);
    cudaEventDestroy(r->ready);
    cudaStreamDestroy(r->stream);
    cudaFree(r->block);
    ctx->used -= r->bytes;
    --ctx->live;
    if (ctx->cached == r) ctx->cached = nullptr;
    delete r;
    return PM_OK;
}

int pm_request_set_params(pm_request *r, const pm_params *params) {
    if (!r) return PM_EINVAL;
    int rc = validate_params(r->ctx, params);
    if (rc) return rc;
    if (params->image_format != r->prm.image_format || params->seam != r->prm.seam ||
        params->sampler != r->prm.sampler) {
        for (int k = 0; k <= r->S; ++k) r->have[k] = false;  // sampling images must be rebuilt
    }
    r->prm = *params;
    set_tile_order(r);
    r->graph_dirty = true;
    return PM_OK;
}

int pm_request_set_view(pm_request *r, int k, const pm_view *v) {
    if (!r) return PM_EINVAL;
    pm_ctx *ctx = r->ctx;
    if (k < 0 || k > r->S) return fail(ctx, PM_EINVAL, "view index %d out of range 0..%d", k, r->S);
    if (!v || !v->gray) return fail(ctx, PM_EINVAL, "view %d has no image", k);
    if (!finite_pose(v->R_cw, v->t_cw)) return fail(ctx, PM_EINVAL, "view %d pose is not finite", k);
    PM_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t es = r->prm.image_format == PM_IMAGE_F16 ? 2 : 1;
    const size_t row = (size_t)r->W * es;
    const size_t pitch = v->pitch_bytes ? v->pitch_bytes : row;
    if (pitch < row) return fail(ctx, PM_EINVAL, "pitch %zu smaller than a row (%zu)", pitch, row);
    if (k > 0 && r->prm.sampler == PM_SAMPLER_TEXTURE) {
        // texture sampler: the source image itself, pitched for the texture unit
        int rc = ensure_textures(r);
        if (rc) return rc;
        PM_CUDA(ctx, cudaMemcpy2DAsync(r->quad[k - 1], r->tex_pitch, v->gray, pitch, row, r->H, cudaMemcpyDefault,
                                       r->stream));
        std::memcpy(r->R[k], v->R_cw, sizeof(double) * 9);
        std::memcpy(r->t[k], v->t_cw, sizeof(double) * 3);
        r->have[k] = true;
        r->graph_dirty = true;
        return PM_OK;
    }
    PM_CUDA(ctx, cudaMemcpy2DAsync(r->raw, row, v->gray, pitch, row, r->H, cudaMemcpyDefault, r->stream));
    if (k == 0) {
        pm::launch_ref_to_float(r->stream, r->raw, row, r->prm.image_format, r->W, r->H, r->ref);
        ctx->launches++;
        r->has_mask = v->mask != nullptr;
        if (v->mask)
            PM_CUDA(ctx, cudaMemcpyAsync(r->mask, v->mask, (size_t)r->W * r->H, cudaMemcpyDefault, r->stream));
    } else {
        pm::launch_build_quad(r->stream, r->raw, row, r->prm.image_format, r->W, r->H, r->prm.seam, r->quad[k - 1]);
        ctx->launches++;
    }
    PM_CUDA(ctx, cudaGetLastError());
    std::memcpy(r->R[k], v->R_cw, sizeof(double) * 9);
    std::memcpy(r->t[k], v->t_cw, sizeof(double) * 3);
    r->have[k] = true;
    r->graph_dirty = true;
    return PM_OK;
}

int pm_request_init(pm_request *r) {
    if (!r) return PM_EINVAL;
    int rc = check_views(r);
    if (rc) return rc;
    PM_CUDA(r->ctx, cudaSetDevice(r->ctx->device));
    fill_args(r);
    r->postprocessed = false;
    return enqueue_init(r);
}

int pm_request_set_state(pm_request *r, const float *planes, const float *scores) {
    if (!r || !planes) return fail(r ? r->ctx : nullptr, PM_EINVAL, "NULL argument");
    int rc = check_views(r);
    if (rc) return rc;
    pm_ctx *ctx = r->ctx;
    PM_CUDA(ctx, cudaSetDevice(ctx->device));
    fill_args(r);
    const size_t N = (size_t)r->W * r->H;
    rc = ensure_scratch(ctx, N * 16);
    if (rc) return rc;
    float *dpl = (float *)ctx->scratch, *dsc = dpl + 3 * N;
    PM_CUDA(ctx, cudaMemcpyAsync(dpl, planes, N * 12, cudaMemcpyHostToDevice, r->stream));
    if (scores) PM_CUDA(ctx, cudaMemcpyAsync(dsc, scores, N * 4, cudaMemcpyHostToDevice, r->stream));
    pm::launch_set_planes(r->stream, dpl, scores ? dsc : nullptr, r->trig.row, r->trig.col, r->W, r->H, r->plane,
                          r->score, r->best);
    ctx->launches++;
    if (!scores)
        for (int c = 0; c < 2; ++c) {
            rc = launch_tile(r, pm::kModeScore, c, 0);
            if (rc) return rc;
        }
    PM_CUDA(ctx, cudaStreamSynchronize(r->stream));
    r->postprocessed = false;
    return PM_OK;
}

int pm_request_sweep(pm_request *r, int first_half, int n_half) {
    if (!r) return PM_EINVAL;
    if (first_half < 0 || n_half < 0) return fail(r->ctx, PM_EINVAL, "negative half-sweep index");
    int rc = check_views(r);
    if (rc) return rc;
    PM_CUDA(r->ctx, cudaSetDevice(r->ctx->device));
    fill_args(r);
    r->postprocessed = false;
    return enqueue_sweeps(r, first_half, n_half);
}

// Order this request's stream after all work enqueued so far on the prior's.
static int wait_for_prior(pm_request *r, const pm_request *prior) {
    if (!prior || prior->stream == r->stream) return PM_OK;
    PM_CUDA(r->ctx, cudaEventRecord(prior->ready, prior->stream));
    PM_CUDA(r->ctx, cudaStreamWaitEvent(r->stream, prior->ready, 0));
    return PM_OK;
}

int pm_request_set_prior(pm_request *r, const pm_request *prior) {
    if (!r) return PM_EINVAL;
    if (prior && prior->ctx != r->ctx) return fail(r->ctx, PM_EINVAL, "prior belongs to another context");
    if (prior == r) return fail(r->ctx, PM_EINVAL, "a request cannot seed itself");
    link_prior(r, prior, nullptr);
    return PM_OK;
}

int pm_request_set_prior_result(pm_request *r, const pm_result *res) {
    if (!r) return PM_EINVAL;
    if (res && res->ctx != r->ctx) return fail(r->ctx, PM_EINVAL, "result belongs to another context");
    link_prior(r, nullptr, res);
    return PM_OK;
}

size_t pm_result_bytes(int W, int H) { return align256((size_t)W * H * 16) + align256((size_t)W * H * 4); }

int pm_result_create(pm_ctx *ctx, int W, int H, pm_result **out) {
    if (!ctx || !out) return fail(ctx, PM_EINVAL, "NULL argument");
    *out = nullptr;
    int rc = validate_size(ctx, W, H, 1);
    if (rc) return rc;
    PM_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t bytes = pm_result_bytes(W, H);
    if (ctx->used + bytes > ctx->budget)
        return fail(ctx, PM_EBUDGET, "result needs %zu bytes, %zu of %zu in use", bytes, ctx->used, ctx->budget);
    pm_result *r = new pm_result();
    r->ctx = ctx;
    r->W = W;
    r->H = H;
    r->bytes = bytes;
    rc = get_trig(ctx, W, H, &r->trig);
    if (!rc && cudaMalloc(&r->block, bytes) != cudaSuccess) {
        cudaGetLastError();
        rc = fail(ctx, PM_ENOMEM, "device allocation of %zu bytes failed", bytes);
    }
    if (!rc && cudaEventCreateWithFlags(&r->ready, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(r->block);
        rc = fail(ctx, PM_ECUDA, "event creation failed");
    }
    if (rc) {
        delete r;
        return rc;
    }
    r->plane = (float4 *)r->block;
    r->fdepth = (float *)((char *)r->block + align256((size_t)W * H * 16));
    ctx->used += bytes;
    ++ctx->live;
    *out = r;
    return PM_OK;
}

int pm_result_snapshot(pm_result *res, pm_request *r) {
    if (!res || !r) return PM_EINVAL;
    if (res->ctx != r->ctx || res->W != r->W || res->H != r->H)
        return fail(r->ctx, PM_EINVAL, "result and request differ in context or size");
    if (!r->postprocessed) return fail(r->ctx, PM_EINVAL, "request has no post-filtered result");
    PM_CUDA(r->ctx, cudaSetDevice(r->ctx->device));
    const size_t N = (size_t)r->W * r->H;
    PM_CUDA(r->ctx, cudaMemcpyAsync(res->plane, r->plane, N * 16, cudaMemcpyDeviceToDevice, r->stream));
    PM_CUDA(r->ctx, cudaMemcpyAsync(res->fdepth, r->fdepth, N * 4, cudaMemcpyDeviceToDevice, r->stream));
    PM_CUDA(r->ctx, cudaEventRecord(res->ready, r->stream));
    std::memcpy(res->R, r->R[0], sizeof res->R);
    std::memcpy(res->t, r->t[0], sizeof res->t);
    res->valid = true;
    return PM_OK;
}

int pm_result_destroy(pm_result *res) {
    if (!res) return PM_EINVAL;
    cudaSetDevice(res->ctx->device);
    unlink_dependents(res->dependents, false);
    cudaEventSynchronize(res->ready);
    cudaEventDestroy(res->ready);
    cudaFree(res->block);
    res->ctx->used -= res->bytes;
    --res->ctx->live;
    delete res;
    return PM_OK;
}

int pm_request_set_landmarks(pm_request *r, const double *xyz_world, int n) {
    if (!r) return PM_EINVAL;
    PM_CUDA(r->ctx, cudaSetDevice(r->ctx->device));
    return stage_landmarks(r, xyz_world, n);
}

int pm_request_seed_landmarks(pm_request *r, const double *xyz_world, int n) {
    if (!r) return PM_EINVAL;
    int rc = check_views(r);
    if (rc) return rc;
    PM_CUDA(r->ctx, cudaSetDevice(r->ctx->device));
    rc = stage_landmarks(r, xyz_world, n);
    if (rc) return rc;
    fill_args(r);
    r->postprocessed = false;
    return enqueue_landmarks(r);
}

int pm_request_seed(pm_request *r, const pm_request *prior) {
    if (!r || !prior) return fail(r ? r->ctx : nullptr, PM_EINVAL, "NULL argument");
    if (prior->ctx != r->ctx) return fail(r->ctx, PM_EINVAL, "prior belongs to another context");
    int rc = check_views(r);
    if (rc) return rc;
    PM_CUDA(r->ctx, cudaSetDevice(r->ctx->device));
    fill_args(r);
    r->postprocessed = false;
    rc = wait_for_prior(r, prior);
    if (rc) return rc;
    return enqueue_seed(r, prior);
}

int pm_request_postprocess(pm_request *r) {
    if (!r) return PM_EINVAL;
    PM_CUDA(r->ctx, cudaSetDevice(r->ctx->device));
    int rc = enqueue_post(r);
    if (!rc) r->postprocessed = true;
    return rc;
}

int pm_request_run(pm_request *r) {
    if (!r) return PM_EINVAL;
    pm_ctx *ctx = r->ctx;
    NvtxRange range("pm_request_run %dx%d S=%d sweeps=%d", r->W, r->H, r->S, r->prm.iterations);
    int rc = check_views(r);
    if (rc) return rc;
    PM_CUDA(ctx, cudaSetDevice(ctx->device));
    if (r->graph_dirty || !r->gexec) {
        NvtxRange capture("capture sweep graph");
        fill_args(r);
        cudaGraph_t g = nullptr;
        PM_CUDA(ctx, cudaStreamBeginCapture(r->stream, cudaStreamCaptureModeThreadLocal));
        const uint64_t before = ctx->launches;
        rc = enqueue_run(r);
        cudaError_t ce = cudaStreamEndCapture(r->stream, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (ce != cudaSuccess) return fail(ctx, PM_ECUDA, "graph capture: %s", cudaGetErrorString(ce));
        ctx->launches = before;  // counted again on replay below
        bool updated = false;
        if (r->gexec) {
            cudaGraphExecUpdateResultInfo info;
            if (cudaGraphExecUpdate(r->gexec, g, &info) == cudaSuccess) updated = true;
            else cudaGetLastError();
        }
        if (!updated) {
            if (r->gexec) cudaGraphExecDestroy(r->gexec);
            r->gexec = nullptr;
            PM_CUDA(ctx, cudaGraphInstantiate(&r->gexec, g, 0));
        }
        if (r->graph) cudaGraphDestroy(r->graph);
        r->graph = g;
        r->graph_dirty = false;
    }
    rc = wait_for_prior(r, r->prior);
    if (rc) return rc;
    if (r->prior_res) PM_CUDA(ctx, cudaStreamWaitEvent(r->stream, r->prior_res->ready, 0));
    PM_CUDA(ctx, cudaGraphLaunch(r->gexec, r->stream));
    ctx->launches += 3 + 2 * (uint64_t)r->prm.iterations + (r->prm.postprocess ? 3 : 0) +
                     ((r->prior || r->prior_res) ? 4 : 0) + (r->n_lm > 0 ? 3 : 0);
    r->postprocessed = r->prm.postprocess != 0;
    return PM_OK;
}

static int enqueue_read(pm_request *r, pm_maps *out, int raw) {
    if (!r || !out) return fail(r ? r->ctx : nullptr, PM_EINVAL, "NULL argument");
    pm_ctx *ctx = r->ctx;
    PM_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t N = (size_t)r->W * r->H;
    const int use_raw = raw || !r->postprocessed;
    pm::launch_export(r->stream, r->plane, r->score, r->best, r->fdepth, r->fscore, r->trig.row, r->trig.col, r->W,
                      r->H, use_raw, r->x_depth, r->x_score, r->x_plane3, r->x_normal3, r->x_best);
    ctx->launches++;
    // host or device destinations
    if (out->depth) PM_CUDA(ctx, cudaMemcpyAsync(out->depth, r->x_depth, N * 4, cudaMemcpyDefault, r->stream));
    if (out->score) PM_CUDA(ctx, cudaMemcpyAsync(out->score, r->x_score, N * 4, cudaMemcpyDefault, r->stream));
    if (out->plane) PM_CUDA(ctx, cudaMemcpyAsync(out->plane, r->x_plane3, N * 12, cudaMemcpyDefault, r->stream));
    if (out->normal) PM_CUDA(ctx, cudaMemcpyAsync(out->normal, r->x_normal3, N * 12, cudaMemcpyDefault, r->stream));
    if (out->best_view)
        PM_CUDA(ctx, cudaMemcpyAsync(out->best_view, r->x_best, N * 4, cudaMemcpyDefault, r->stream));
    return PM_OK;
}

int pm_request_read(pm_request *r, pm_maps *out, int raw) {
    int rc = enqueue_read(r, out, raw);
    if (rc) return rc;
    PM_CUDA(r->ctx, cudaStreamSynchronize(r->stream));
    return PM_OK;
}

int pm_request_read_async(pm_request *r, pm_maps *out, int raw) { return enqueue_read(r, out, raw); }

int pm_request_synchronize(pm_request *r) {
    if (!r) return PM_EINVAL;
    PM_CUDA(r->ctx, cudaStreamSynchronize(r->stream));
    return PM_OK;
}

const float *pm_request_depth_device(const pm_request *r) { return r ? r->fdepth : nullptr; }

const float *pm_result_depth_device(const pm_result *res) { return res ? res->fdepth : nullptr; }

void *pm_request_stream(const pm_request *r) { return r ? (void *)r->stream : nullptr; }

int pm_request_query(const pm_request *r) {
    if (!r) return PM_EINVAL;
    const cudaError_t e = cudaStreamQuery(r->stream);
    if (e == cudaSuccess) return PM_OK;
    if (e == cudaErrorNotReady) return PM_ENOTREADY;
    return PM_ECUDA;
}

int pm_densify(pm_ctx *ctx, int W, int H, const pm_view *views, int n_views, const pm_params *params, pm_maps *out) {
    if (!ctx || !views || !out || !out->depth) return fail(ctx, PM_EINVAL, "NULL argument");
    const int S = n_views - 1;
    int rc = validate_size(ctx, W, H, S);
    if (rc) return rc;
    rc = validate_params(ctx, params);
    if (rc) return rc;
    pm_request *r = ctx->cached;
    if (r && (r->W != W || r->H != H || r->S != S || r->prm.image_format != params->image_format)) {
        pm_request_destroy(r);
        r = nullptr;
    }
    if (!r) {
        rc = pm_request_create(ctx, W, H, S, params, &r);
        if (rc) return rc;
        ctx->cached = r;
    }
    rc = pm_request_set_params(r, params);
    for (int k = 0; !rc && k < n_views; ++k) rc = pm_request_set_view(r, k, &views[k]);
    if (!rc) rc = pm_request_run(r);
    if (!rc) rc = pm_request_read(r, out, 0);
    return rc;
}

int pm_score_hypotheses(pm_request *r, int n, const int32_t *ij, const float *planes, float *scores, int32_t *best,
                        float *per_source) {
    if (!r) return PM_EINVAL;
    pm_ctx *ctx = r->ctx;
    if (n < 0 || (n > 0 && (!ij || !planes))) return fail(ctx, PM_EINVAL, "bad hypothesis arrays");
    if (n == 0) return PM_OK;
    int rc = check_views(r);
    if (rc) return rc;
    const int ph = r->prm.patch_half;
    for (int h = 0; h < n; ++h) {
        const int i = ij[2 * h], j = ij[2 * h + 1];
        if (i < ph || i >= r->H - ph || j < ph || j >= r->W - ph)
            return fail(ctx, PM_EINVAL, "hypothesis %d at (%d, %d) has taps outside the image", h, i, j);
    }
    PM_CUDA(ctx, cudaSetDevice(ctx->device));
    fill_args(r);
    const size_t S = (size_t)r->S;
    const size_t need = align256((size_t)n * 8) + align256((size_t)n * 12) + align256((size_t)n * 4) * 2 +
                        align256((size_t)n * 4 * S);
    rc = ensure_scratch(ctx, need);
    if (rc) return rc;
    char *p = (char *)ctx->scratch;
    int2 *dij = (int2 *)p;
    p += align256((size_t)n * 8);
    float *dpl = (float *)p;
    p += align256((size_t)n * 12);
    float *dsc = (float *)p;
    p += align256((size_t)n * 4);
    int *dbest = (int *)p;
    p += align256((size_t)n * 4);
    float *dper = (float *)p;
    PM_CUDA(ctx, cudaMemcpyAsync(dij, ij, (size_t)n * 8, cudaMemcpyHostToDevice, r->stream));
    PM_CUDA(ctx, cudaMemcpyAsync(dpl, planes, (size_t)n * 12, cudaMemcpyHostToDevice, r->stream));
    pm::HypArgs a{};
    a.P = r->args.P;
    for (int k = 0; k < r->S; ++k) {
        a.src.quad[k] = r->quad[k];
        a.src.tex[k] = (unsigned long long)r->tex[k];
    }
    a.src.qpitch = r->W + 1;
    a.row_trig = r->trig.row;
    a.col_trig = r->trig.col;
    a.ref = r->ref;
    a.W = r->W;
    a.H = r->H;
    a.Wf = (float)r->W;
    a.Hf = (float)r->H;
    a.patch_half = ph;
    a.combine = r->prm.combine;
    a.top_k = r->prm.top_k;
    a.color_factor = r->args.color_factor;
    a.dist_factor = r->args.dist_factor;
    a.ncf = r->args.ncf;
    a.ndf = r->args.ndf;
    a.n = n;
    a.ij = dij;
    a.planes = dpl;
    a.scores = dsc;
    a.best = dbest;
    a.per_source = per_source ? dper : nullptr;
    cudaError_t e = pm::dispatch_hyp(r->S, pm::image_kind(r->prm.image_format, r->prm.sampler), n, r->stream, a);
    ctx->launches++;
    if (e != cudaSuccess) return fail(ctx, PM_ECUDA, "hypothesis kernel: %s", cudaGetErrorString(e));
    if (scores) PM_CUDA(ctx, cudaMemcpyAsync(scores, dsc, (size_t)n * 4, cudaMemcpyDeviceToHost, r->stream));
    if (best) PM_CUDA(ctx, cudaMemcpyAsync(best, dbest, (size_t)n * 4, cudaMemcpyDeviceToHost, r->stream));
    if (per_source)
        PM_CUDA(ctx, cudaMemcpyAsync(per_source, dper, (size_t)n * 4 * S, cudaMemcpyDeviceToHost, r->stream));
    PM_CUDA(ctx, cudaStreamSynchronize(r->stream));
    return PM_OK;
}

// Arguments shared by the host- and device-buffer filter calls.
static int filter_check(pm_ctx *ctx, int W, int H, int n, const float *const *depths, const double *R,
                        const double *t, int center, float thr, const float *out) {
    if (!ctx || !depths || !R || !t || !out) return fail(ctx, PM_EINVAL, "NULL argument");
    if (W < 2 || H < 2 || n < 1 || n > pm::kMaxFilterViews || center < 0 || center >= n)
        return fail(ctx, PM_EINVAL, "bad sizes (W=%d H=%d n=%d center=%d)", W, H, n, center);
    for (int k = 0; k < n; ++k)
        if (!depths[k] || !finite_pose(R + 9 * k, t + 3 * k)) return fail(ctx, PM_EINVAL, "view %d invalid", k);
    if (!(thr > 0.0f)) return fail(ctx, PM_EINVAL, "same_depth_threshold must be > 0");
    return PM_OK;
}

// Enqueue the filter on device maps (depths in caller order) on st.
static int enqueue_filter(pm_ctx *ctx, int W, int H, int n, const float *const *depths, const double *R,
                          const double *t, int center, float thr, int min_consistent, float reproj_px, float *out,
                          cudaStream_t st) {
    NvtxRange range("consistency filter %dx%d views=%d", W, H, n);
    Trig tr;
    int rc = get_trig(ctx, W, H, &tr);
    if (rc) return rc;
    pm::CleanArgs a{};
    int order[pm::kMaxFilterViews];
    pm::clean_set_poses(a, n, R, t, center, order);
    for (int s = 0; s < n; ++s) a.depths[s] = depths[order[s]];
    a.W = W;
    a.H = H;
    a.row_trig = tr.row;
    a.col_trig = tr.col;
    a.thr = thr;
    a.min_consistent = min_consistent;
    a.reproj_px = reproj_px;
    a.out = out;
    pm::launch_clean(st, a);
    ctx->launches++;
    PM_CUDA(ctx, cudaGetLastError());
    return PM_OK;
}

int pm_filter_consistency(pm_ctx *ctx, int W, int H, int n, const float *const *depths, const double *R,
                          const double *t, int center, float thr, int min_consistent, float reproj_px, float *out) {
    int rc = filter_check(ctx, W, H, n, depths, R, t, center, thr, out);
    if (rc) return rc;
    PM_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t N = (size_t)W * H;
    rc = ensure_scratch(ctx, (size_t)(n + 1) * align256(N * 4));
    if (rc) return rc;
    char *base = (char *)ctx->scratch;
    const float *dptr[pm::kMaxFilterViews];
    for (int k = 0; k < n; ++k) {
        float *d = (float *)(base + (size_t)k * align256(N * 4));
        PM_CUDA(ctx, cudaMemcpyAsync(d, depths[k], N * 4, cudaMemcpyHostToDevice, ctx->stream));
        dptr[k] = d;
    }
    float *dout = (float *)(base + (size_t)n * align256(N * 4));
    rc = enqueue_filter(ctx, W, H, n, dptr, R, t, center, thr, min_consistent, reproj_px, dout, ctx->stream);
    if (rc) return rc;
    PM_CUDA(ctx, cudaMemcpyAsync(out, dout, N * 4, cudaMemcpyDeviceToHost, ctx->stream));
    PM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return PM_OK;
}

int pm_filter_consistency_device(pm_ctx *ctx, int W, int H, int n, const float *const *depths, const double *R,
                                 const double *t, int center, float thr, int min_consistent, float reproj_px,
                                 float *out, void *stream) {
    int rc = filter_check(ctx, W, H, n, depths, R, t, center, thr, out);
    if (rc) return rc;
    PM_CUDA(ctx, cudaSetDevice(ctx->device));
    return enqueue_filter(ctx, W, H, n, depths, R, t, center, thr, min_consistent, reproj_px, out,
                          stream ? (cudaStream_t)stream : ctx->stream);
}

static int fuse_check(pm_ctx *ctx, int W, int H, int n, float *const *depths, const double *R, const double *t,
                      float thr, const void *pruned) {
    if (!ctx || !depths || !R || !t || !pruned) return fail(ctx, PM_EINVAL, "NULL argument");
    if (W < 2 || H < 2 || n < 1 || n > pm::kMaxFilterViews) return fail(ctx, PM_EINVAL, "bad sizes");
    for (int k = 0; k < n; ++k)
        if (!depths[k] || !finite_pose(R + 9 * k, t + 3 * k)) return fail(ctx, PM_EINVAL, "view %d invalid", k);
    if (!(thr > 0.0f)) return fail(ctx, PM_EINVAL, "same_depth_threshold must be > 0");
    return PM_OK;
}

// Enqueue the fusion on device maps with a caller workspace on st.
static int enqueue_fuse(pm_ctx *ctx, int W, int H, int n, float *const *depths, const double *R, const double *t,
                        const uint8_t *bgr, float thr, float *pruned, float *xyz, uint8_t *bgr_out, int32_t *ij,
                        unsigned *count, void *ws, cudaStream_t st) {
    NvtxRange range("fusion %dx%d views=%d", W, H, n);
    Trig tr;
    int rc = get_trig(ctx, W, H, &tr);
    if (rc) return rc;
    pm::FuseArgs a{};
    a.W = W;
    a.H = H;
    for (int k = 0; k < n; ++k) a.depths[k] = depths[k];
    pm::fuse_set_poses(a, n, R, t);
    pm::fuse_bind_workspace(a, ws);
    a.row_trig = tr.row;
    a.col_trig = tr.col;
    a.thr = thr;
    a.pruned = pruned;
    a.bgr = bgr;
    a.xyz = xyz;
    a.bgr_out = bgr ? bgr_out : nullptr;
    a.ij_out = ij;
    a.count = count;
    const cudaError_t e = pm::launch_fuse(st, a);
    ctx->launches += 1 + 2 * (uint64_t)(n - 1) + 3;
    if (e != cudaSuccess) return fail(ctx, PM_ECUDA, "fusion: %s", cudaGetErrorString(e));
    return PM_OK;
}

size_t pm_fuse_workspace_bytes(int W, int H) {
    if (W < 2 || H < 2) return 0;
    return pm::fuse_workspace_bytes(W, H);
}

int pm_fuse_device(pm_ctx *ctx, int W, int H, int n, float *const *depths, const double *R, const double *t,
                   const uint8_t *bgr, float thr, float *pruned, float *xyz, uint8_t *bgr_out, int32_t *ij,
                   unsigned *count, void *workspace, size_t workspace_bytes, void *stream) {
    int rc = fuse_check(ctx, W, H, n, depths, R, t, thr, pruned);
    if (rc) return rc;
    if (!xyz || !count || !workspace) return fail(ctx, PM_EINVAL, "NULL argument");
    if (workspace_bytes < pm::fuse_workspace_bytes(W, H) || ((uintptr_t)workspace & 255))
        return fail(ctx, PM_EINVAL, "workspace must be 256-byte aligned and hold pm_fuse_workspace_bytes");
    PM_CUDA(ctx, cudaSetDevice(ctx->device));
    return enqueue_fuse(ctx, W, H, n, depths, R, t, bgr, thr, pruned, xyz, bgr_out, ij, count, workspace,
                        stream ? (cudaStream_t)stream : ctx->stream);
}

int pm_fuse(pm_ctx *ctx, int W, int H, int n, float *const *depths, const double *R, const double *t,
            const uint8_t *bgr, float thr, float *pruned, pm_points *out) {
    int rc = fuse_check(ctx, W, H, n, depths, R, t, thr, pruned);
    if (rc) return rc;
    if (!out) return fail(ctx, PM_EINVAL, "NULL argument");
    PM_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t N = (size_t)W * H;
    const size_t need = (size_t)n * align256(N * 4) + align256(pm::fuse_workspace_bytes(W, H)) + align256(N * 4) +
                        align256(N * 3) + align256(N * 12) + align256(N * 3) + align256(N * 8) + 256;
    rc = ensure_scratch(ctx, need);
    if (rc) return rc;
    char *p = (char *)ctx->scratch;
    auto take = [&](size_t b) { void *q = p; p += align256(b); return q; };
    float *dptr[pm::kMaxFilterViews];
    for (int k = 0; k < n; ++k) {
        dptr[k] = (float *)take(N * 4);
        PM_CUDA(ctx, cudaMemcpyAsync(dptr[k], depths[k], N * 4, cudaMemcpyHostToDevice, ctx->stream));
    }
    void *ws = take(pm::fuse_workspace_bytes(W, H));
    float *dpruned = (float *)take(N * 4);
    uint8_t *dbgr = (uint8_t *)take(N * 3);
    float *dxyz = (float *)take(N * 12);
    uint8_t *dbgr_out = (uint8_t *)take(N * 3);
    int32_t *dij = (int32_t *)take(N * 8);
    unsigned *dcount = (unsigned *)take(4);
    if (bgr) PM_CUDA(ctx, cudaMemcpyAsync(dbgr, bgr, N * 3, cudaMemcpyHostToDevice, ctx->stream));
    rc = enqueue_fuse(ctx, W, H, n, dptr, R, t, bgr ? dbgr : nullptr, thr, dpruned, dxyz, dbgr_out, dij, dcount, ws,
                      ctx->stream);
    if (rc) return rc;
    unsigned count = 0;
    PM_CUDA(ctx, cudaMemcpyAsync(&count, dcount, 4, cudaMemcpyDeviceToHost, ctx->stream));
    PM_CUDA(ctx, cudaMemcpyAsync(pruned, dpruned, N * 4, cudaMemcpyDeviceToHost, ctx->stream));
    for (int k = 1; k < n; ++k)
        PM_CUDA(ctx, cudaMemcpyAsync(depths[k], dptr[k], N * 4, cudaMemcpyDeviceToHost, ctx->stream));
    PM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const int m = (int)std::min<unsigned>(count, out->capacity > 0 ? (unsigned)out->capacity : 0u);
    if (m > 0) {
        std::vector<float> xyz((size_t)m * 3);
        PM_CUDA(ctx, cudaMemcpy(xyz.data(), dxyz, (size_t)m * 12, cudaMemcpyDeviceToHost));
        if (out->xyz)
            for (size_t q = 0; q < (size_t)m * 3; ++q) out->xyz[q] = xyz[q];
        if (out->bgr && bgr) PM_CUDA(ctx, cudaMemcpy(out->bgr, dbgr_out, (size_t)m * 3, cudaMemcpyDeviceToHost));
        if (out->ij) PM_CUDA(ctx, cudaMemcpy(out->ij, dij, (size_t)m * 8, cudaMemcpyDeviceToHost));
    }
    out->count = (int)count;
    if ((int)count > out->capacity)
        return fail(ctx, PM_EINVAL, "point capacity %d too small for %u points", out->capacity, count);
    return PM_OK;
}

}  // extern "C"

