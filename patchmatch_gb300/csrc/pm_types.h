// Internal types shared by the host code and the kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "pm_gb300.h"

namespace pm {

constexpr int kMaxSrc = PM_MAX_SOURCES;

// Composed reference-camera -> source-camera poses, FP64-composed on the
// host and rounded to float: X_r = M_r X_c + c_r, stored as three rows
// (M_r[k][0..2], c_r[k]) per source so a row is one 16-byte load.
struct PmPoses {
    float4 G[kMaxSrc][3];
};

// Per-source sampling images: quad-packed footprints (exact sampler) or
// texture objects (texture sampler).
struct SrcSet {
    const void *quad[kMaxSrc];
    unsigned long long tex[kMaxSrc];
    int qpitch;  // quads per row (W + 1)
};

// Kernel arguments of the tile kernels (init scoring and red-black sweeps).
struct SweepArgs {
    PmPoses P;
    SrcSet src;
    const float2 *row_trig;     // H entries: (cos lat, sin lat)
    const float2 *col_trig;     // W entries: (sin lon, cos lon)
    const float *ref;           // H x W reference intensities (float)
    float4 *plane;              // H x W: plane (x, y, z) and depth (w)
    const float4 *cand;         // H x W seeding candidates (w = depth, 0 = none), mode kModeSeed
    float *score;               // H x W
    int8_t *best;               // H x W
    int W, H;
    float Wf, Hf;
    int patch_half;
    int colour;                 // 0 = red, 1 = black: pixels with (i + j + colour) even
    int sweep;                  // sweep index (Philox tag = sweep + 1)
    int mode;                   // 0 = score own plane, 1 = red-black update
    int combine, top_k;
    int propagation;            // PM_PROPAGATION_*
    uint32_t seed, keyframe;
    float color_factor;         // 1 / (2 sigma_color^2)
    float dist_factor;          // 1 / (2 sigma_x^2)
    float ncf, ndf;             // -log2(e) * color_factor, -log2(e) * dist_factor
    float depth_range[6];       // refinement depth ranges 0.02 * 0.3^t (float, reference rounding)
    float normal_range[6];      // refinement normal ranges 0.5 * 0.8^t
};

static_assert(sizeof(SweepArgs) % 16 == 0, "SweepArgs is copied as 16-byte words");

// Tile order of the banded (persistent) tile kernel.  Band b is a segment of
// one tile column: column b % tiles_x, rows [seg * per_band, (seg + 1) *
// per_band) with seg = b / tiles_x, the column split into as many segments
// as make at least one band per SM.  A CTA starts on band smid % n_home and
// takes its next tile with one atomic, so the CTAs resident on an SM walk
// down vertically adjacent tiles and share their source footprints in L1,
// while all SMs stay near the same rows of their segments (the sources stay
// L2-resident); exhausted bands pass the CTA on to the following ones.  ctr
// holds one counter per band, zero before the launch.
struct BandArgs {
    unsigned int *ctr;
    int n_bands, per_band, tiles_x, tiles_y, n_home;
    int blocks;  // persistent grid: SMs x resident CTAs per SM
};

// Arguments of the batched executor (one phase over many requests).
struct BatchArgs {
    const SweepArgs *args;   // per request (mode/colour/sweep taken from here)
    const int4 *items;       // (request, tile x, tile y, 0), request-major
    int n_items;
    unsigned int *counter;   // next item; zero before the launch
    int mode, colour, sweep;
};

// kModeScore: score each pixel's own plane; kModeSweep: red-black update;
// kModeSeed: score the seeding candidate and keep it when it scores higher.
enum { kModeScore = 0, kModeSweep = 1, kModeSeed = 2 };

// Arguments of the fixed-hypothesis scoring kernel.
struct HypArgs {
    PmPoses P;
    SrcSet src;
    const float2 *row_trig;
    const float2 *col_trig;
    const float *ref;
    int W, H;
    float Wf, Hf;
    int patch_half;
    int combine, top_k;
    float color_factor, dist_factor;
    float ncf, ndf;
    int n;
    const int2 *ij;
    const float *planes;  // n x 3
    float *scores;        // n
    int *best;            // n
    float *per_source;    // n x S or null
};

}  // namespace pm
