// Host-side launch wrappers of the densifier kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "pm_types.h"

namespace pm {

// pm_prep.cu
void launch_ref_to_float(cudaStream_t st, const uint8_t *raw, size_t pitch, int fmt, int W, int H, float *out);
void launch_build_quad(cudaStream_t st, const uint8_t *raw, size_t pitch, int fmt, int W, int H, int seam,
                       void *quad);
void launch_init_planes(cudaStream_t st, const float2 *row_trig, const float2 *col_trig, int W, int H, uint32_t seed,
                        uint32_t kf, int mode, float dmin, float dmax, float4 *plane, float *score, int8_t *best);
void launch_set_planes(cudaStream_t st, const float *planes3, const float *scores, const float2 *row_trig,
                       const float2 *col_trig, int W, int H, float4 *plane, float *score, int8_t *best);

// Source-image variants of the tile and hypothesis kernels: image format x
// sampler (quad-packed footprints or texture objects).
enum { kImageQuadU8 = 0, kImageQuadF16 = 1, kImageTexU8 = 2, kImageTexF16 = 3 };
inline int image_kind(int image_format, int sampler) {
    return (sampler == PM_SAMPLER_TEXTURE ? 2 : 0) + (image_format == PM_IMAGE_F16 ? 1 : 0);
}

// pm_inst.cu (one translation unit per source count S)
// band: null for one CTA per tile over `grid`, else the banded persistent order
template <int S>
cudaError_t launch_tile(int kind, dim3 grid, cudaStream_t st, const SweepArgs &a, const BandArgs *band);
template <int S>
int tile_blocks_per_sm(int kind);
template <int S>
cudaError_t launch_hyp(int kind, int n, cudaStream_t st, const HypArgs &a);
template <int S>
cudaError_t launch_batch(int kind, bool plain, int blocks, cudaStream_t st, const BatchArgs &b);
template <int S>
int batch_blocks_per_sm(int kind, bool plain);
// pm_batch_mixed.cu (one translation unit per image variant)
template <int Kind>
cudaError_t launch_batch_mixed(bool plain, int blocks, cudaStream_t st, const BatchArgs &b);
template <int Kind>
int batch_mixed_blocks_per_sm(bool plain);
template <int Kind>
cudaError_t configure_batch_mixed();  // dynamic shared-memory limit of the current device
cudaError_t dispatch_batch_mixed(int kind, bool plain, int blocks, cudaStream_t st, const BatchArgs &b);
int dispatch_batch_mixed_blocks_per_sm(int kind, bool plain);
cudaError_t dispatch_tile(int S, int kind, dim3 grid, cudaStream_t st, const SweepArgs &a, const BandArgs *band);
int dispatch_tile_blocks_per_sm(int S, int kind);
cudaError_t dispatch_batch(int S, int kind, bool plain, int blocks, cudaStream_t st, const BatchArgs &b);
int dispatch_batch_blocks_per_sm(int S, int kind, bool plain);
cudaError_t dispatch_hyp(int S, int kind, int n, cudaStream_t st, const HypArgs &a);
dim3 tile_grid(int W, int H);

// pm_seed.cu: prior result -> seeding candidates of a new keyframe
struct WarpArgs {
    const float4 *prev_plane;     // prior plane state (prior camera frame)
    const float *prev_depth;      // prior filtered depth (0 = invalid)
    int Wp, Hp;
    const float2 *prow, *pcol;    // prior bearing tables
    float M[9], c[3];             // prior camera -> new camera (FP64-composed)
    int W, H;
    float Wf, Hf;
    const float2 *row, *col;      // new bearing tables
    unsigned long long *zbuf;     // W*H scratch: (range bits, prior index) of the nearest splat
    float4 *seed;                 // W*H candidates (w = range, 0 = none)
};
void launch_warp_prior(cudaStream_t st, const WarpArgs &a);
// landmark seeds: lm[k] = (pixel index, depth bits), one per pixel
void launch_landmark_cands(cudaStream_t st, const int2 *lm, int n, const uint8_t *mask, const float2 *row,
                           const float2 *col, int W, int H, float4 *cand);

// pm_post.cu
struct PostArgs {
    const float4 *plane;
    const float *score;
    const float *ref;
    const uint8_t *mask;  // may be null
    int W, H, patch_half;
    float min_var, min_depth, max_depth, min_score;
    float *d0, *s0, *m1;  // scratch: windowed depth, score, first median
    float *out_depth, *out_score;
};
void launch_postprocess(cudaStream_t st, const PostArgs &a);
// raw = 1: export the sweep state instead of the filtered maps
void launch_export(cudaStream_t st, const float4 *plane, const float *score, const int8_t *best,
                   const float *filt_depth, const float *filt_score, const float2 *row_trig, const float2 *col_trig,
                   int W, int H, int raw, float *depth, float *score_out, float *plane3, float *normal3,
                   int32_t *best32);

// Depth maps a consistency filter or a fusion call takes at most.
constexpr int kMaxFilterViews = PM_MAX_SOURCES + 6;

// Camera k relative to camera 0 from world->camera poses, composed in FP64
// and rounded to float: X_k = M X_0 + c with M = R_k R_0^T, c = t_k - M t_0.
inline void compose_pose(const double *R0, const double *t0, const double *Rk, const double *tk, float *M, float *c) {
    double Md[9];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
            Md[3 * a + b] = Rk[3 * a] * R0[3 * b] + Rk[3 * a + 1] * R0[3 * b + 1] + Rk[3 * a + 2] * R0[3 * b + 2];
    for (int a = 0; a < 9; ++a) M[a] = (float)Md[a];
    for (int a = 0; a < 3; ++a) c[a] = (float)(tk[a] - (Md[3 * a] * t0[0] + Md[3 * a + 1] * t0[1] + Md[3 * a + 2] * t0[2]));
}

struct CleanArgs {
    const float *depths[kMaxFilterViews];  // device pointers, view 0 = centre (passed by value)
    int n, W, H;
    float M[kMaxFilterViews][9];  // centre camera -> view k (k >= 1)
    float c[kMaxFilterViews][3];
    float Minv[kMaxFilterViews][9];  // view k -> centre camera (round trip)
    float cinv[kMaxFilterViews][3];
    const float2 *row_trig, *col_trig;
    float thr;
    int min_consistent;
    float reproj_px;
    float *out;
};
// Poses of a filter call: view `center` of R/t (world->camera) becomes view 0,
// the others follow in order (order[s] = original index of view s).
void clean_set_poses(CleanArgs &a, int n, const double *R, const double *t, int center, int *order);
void launch_clean(cudaStream_t st, const CleanArgs &a);

struct FuseArgs {
    float *depths[kMaxFilterViews];  // device pointers, view 0 = head (passed by value)
    int n, W, H;
    float M[kMaxFilterViews][9];  // head camera -> view k
    float c[kMaxFilterViews][3];
    float Rinv[9], tw[3];          // head camera -> world: X_w = R0^T (X_c - t0)
    const float2 *row_trig, *col_trig;
    float thr;
    uint8_t *alive;                // H*W scratch
    int *target;                   // H*W scratch
    int8_t *cls;                   // H*W scratch
    unsigned *first;               // H*W scratch
    float *pruned;                 // H*W out
    // compaction
    unsigned *block_counts;        // ceil(H*W / 1024) + 1
    const uint8_t *bgr;            // H*W*3 or null
    float *xyz;                    // out, capacity*3
    uint8_t *bgr_out;              // out
    int *ij_out;                   // out
    unsigned *count;               // out (device)
};
// Pixels per block of the fusion's output compaction (count, scan, scatter).
constexpr int kCompactBlock = 1024;
// Working memory of one fusion (alive, target, cls, first, block counts) as one
// device block of fuse_workspace_bytes(W, H) bytes, 256-byte aligned.
size_t fuse_workspace_bytes(int W, int H);
void fuse_bind_workspace(FuseArgs &a, void *ws);
// Poses of a fusion (R/t world->camera, view 0 = head): head camera -> view k
// and head camera -> world.
void fuse_set_poses(FuseArgs &a, int n, const double *R, const double *t);
// Every scratch entry a launch reads is written earlier in the same call, so
// nothing from a previous call on the same workspace leaks in.
cudaError_t launch_fuse(cudaStream_t st, const FuseArgs &a);

}  // namespace pm
