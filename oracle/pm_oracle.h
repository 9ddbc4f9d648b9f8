/*
 * pm_oracle.h -- CPU restatement of the PatchMatch-Stereo densification path
 * of RoblabWh/PatchMatch, used ONLY as test infrastructure: the parity checker
 * for tests/, __graft_entry__.smoke() and the cpu_baseline / reference arm of
 * bench.py.  Nothing in the product (patchmatch_gb300/) links, loads or calls
 * this code.
 *
 * What it restates (paths relative to the reference project):
 *   - equirectangular bearing        src/openvslam/PatchMatchCuda.cu:183-208,
 *                                    src/openvslam/depthmap.cc:113-128
 *   - plane <-> depth                PatchMatchCuda.cu:31-43, depthmap.cc:97-104
 *   - plane-induced warp + bilateral-weighted NCC cost
 *                                    PatchMatchCuda.cu:46-180, depthmap.cc:1129-1167,66-94
 *   - view combination               PatchMatchCuda.cu:161-171 (fold), depthmap.cc:1104-1127 (max)
 *   - random initialisation + init scoring  PatchMatchCuda.cu:210-270
 *   - red-black propagation + refinement    PatchMatchCuda.cu:273-407,568-615
 *   - host window / low-variance mask / post-filter  depthmap.cc:731-767,963-973,1169-1208
 *   - geometric-consistency filter   depthmap.cc:1320-1377
 *   - point fusion (pruning)         depthmap.cc:1535-1696
 *
 * Parity status: pinned against outputs of the reference's own CUDA kernels,
 * compiled unmodified from its sources and run on a GB300 (fixtures under
 * tests/golden/, generated by tests/golden/make_golden.py), and against the
 * reference's own host stages (PostProcess, DepthmapCleaner::Clean,
 * DepthmapPruner::Prune of depthmap.cc, compiled unmodified against a
 * minimal OpenCV stand-in by oracle/refhost.py; fixtures from
 * tests/golden/make_golden_host.py): bit-exact.
 *
 * Random numbers: the reference seeds cuRAND XORWOW from clock64() and is not
 * reproducible.  This restatement (and the product) instead draws from
 * Philox4x32-10 keyed by (seed, keyframe) with counter (pixel, sweep, draw),
 * restated here from Salmon et al., "Parallel random numbers: as easy as
 * 1, 2, 3", SC'11.
 */
#ifndef PM_ORACLE_H
#define PM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OR_MAX_VIEWS 17

/* Views of one request.  Images are H*W row-major float intensities (0..255
 * scale).  Poses are world->camera (R_cw row-major, t_cw), index 0 = the
 * reference (centre) keyframe, 1..n_src = sources. */
typedef struct {
    int W, H, n_src;
    const float *ref;
    const float *src[OR_MAX_VIEWS - 1];
    double R[OR_MAX_VIEWS][9];
    double t[OR_MAX_VIEWS][3];
} or_views;

/* OR_COMBINE_FOLD is the reference kernel's rule exactly: its moment sums are
 * never reset between views (PatchMatchCuda.cu:57-62,100-176), so view r's
 * NCC covers the samples of views 1..r, folded with the 25 % rule.
 * OR_COMBINE_FOLD_SEPARATE folds independent per-view NCCs instead. */
enum { OR_COMBINE_FOLD = 0, OR_COMBINE_MAX = 1, OR_COMBINE_TOPK = 2, OR_COMBINE_FOLD_SEPARATE = 3 };
/* OR_SEAM_ZERO is the reference host cost (ComputePlaneImageScoreUnoptimized_equirect,
 * depthmap.cc:1129-1157): LinearInterpolation returns 0 for a sample outside
 * [0, W-1) x [0, H-1) (depthmap.cc:34-38), and a sample whose point lies within
 * 1e-4 of the source camera is skipped (ReprojectEquirect, depthmap.cc:143-150). */
enum { OR_SEAM_CLAMP = 0, OR_SEAM_WRAP = 1, OR_SEAM_ZERO = 2 };
/* OR_ARITH_F64: exact (double) arithmetic and exact bilinear interpolation.
 * OR_ARITH_F32_REF: the reference kernel's own float arithmetic, step by step
 * (PatchMatchCuda.cu:97-178): normalised float bearing table, two-step pose
 * transform, unshifted float moments. */
enum { OR_ARITH_F64 = 0, OR_ARITH_F32_REF = 1 };
/* Bilinear weights: exact, or the texture unit's 8-bit fixed-point weights
 * (round-to-nearest or truncation of the sample coordinate to 1/256 texel). */
enum { OR_INTERP_EXACT = 0, OR_INTERP_TEX8_RN = 1, OR_INTERP_TEX8_RZ = 2 };
enum { OR_INIT_LOGUNIFORM_HEMI = 0, OR_INIT_REF_UNIFORM = 1 };

typedef struct {
    int patch_half;   /* 5 = PatchSize 7 - 2 (depthmap.cc:725, config.cc:183) */
    int combine;      /* OR_COMBINE_* */
    int top_k;        /* for OR_COMBINE_TOPK */
    int seam;         /* OR_SEAM_* */
    int arith;        /* OR_ARITH_* */
    int interp;       /* OR_INTERP_* */
    float sigma_color;/* 50 (PatchMatchCuda.cu:897) */
    float sigma_x;    /* 5  (PatchMatchCuda.cu:898) */
} or_cost_params;

typedef struct {
    or_cost_params cp;
    int iterations;       /* red-black sweeps */
    float min_depth, max_depth;
    uint32_t seed, keyframe;
    int init_mode;        /* OR_INIT_* */
    int row_lo, row_hi;   /* restrict updates to rows [row_lo, row_hi); -1,-1 = all */
    int threads;          /* OpenMP threads, 0 = default */
    int propagation;      /* OR_PROP_* */
} or_run_params;

/* OR_PROP_SMOOTH: the reference GPU update (PatchMatchCuda.cu:287-404);
 * OR_PROP_PLAIN: the reference host update (PatchMatchUpdatePixel,
 * depthmap.cc:1003-1067) with Philox draws in place of mt19937. */
enum { OR_PROP_SMOOTH = 0, OR_PROP_PLAIN = 1 };

/* ---- random numbers ---- */
void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* 18 refinement normals of one pixel visit (tag = sweep + 1). */
void or_refine_normals(uint32_t seed, uint32_t keyframe, uint32_t pixel, uint32_t tag, float out[18]);

/* ---- geometry ---- */
/* Exact (FP64) bearing of pixel (i, j): pixel-corner convention, x = j. */
void or_bearing64(int W, int H, int i, int j, double b[3]);

/* The reference kernel's float bearing (PatchMatchCuda.cu:183-208). */
void or_bearing_ref_f32(int W, int H, int i, int j, float b[3]);

/* ---- cost ---- */
/* Cost of plane hypothesis `plane` (camera frame, plane . X = 1) at pixel
 * (i, j).  Writes per-source NCC (n_src values) if ncc != NULL and the
 * best source index (0-based) if best != NULL.  Returns the combined score. */
double or_cost(const or_views *v, const or_cost_params *p, int i, int j,
               const double plane[3], double *ncc, int *best);
/* Batch of n hypotheses: ij[2n] (row, col), planes[3n]; OpenMP-parallel. */
void or_cost_batch(const or_views *v, const or_cost_params *p, int n,
                   const int32_t *ij, const float *planes, double *scores,
                   int32_t *best, double *ncc_all, int threads);

/* ---- full PatchMatch run (FP32 state maps, like the GPU) ----
 * plane: H*W*3, depth: H*W, score: H*W, best: H*W (may be NULL).
 * Random init of every pixel, init scoring of interior pixels, then
 * `iterations` red-black sweeps.  Returns wall seconds spent. */
double or_patchmatch(const or_views *v, const or_run_params *rp,
                     float *plane, float *depth, float *score, int32_t *best);

/* Apply n_half red/black half-sweeps (even = red, odd = black; sweep =
 * half / 2) to the given state in place. */
void or_sweeps(const or_views *v, const or_run_params *rp, float *plane, float *depth, float *score,
               int32_t *best, int first_half, int n_half);

/* ---- host post-processing of one estimator result (depthmap.cc:727-767) ----
 * depth/score in: raw GPU-equivalent maps; out: filtered maps (in place).
 * mask may be NULL (all valid).  ref_u8 = reference gray image (for the
 * low-variance mask; min_patch_sd 0 disables it). */
void or_postprocess(int W, int H, int patch_half, const float *ref,
                    const uint8_t *mask, float min_patch_sd,
                    float min_depth, float max_depth, float min_score,
                    float *depth, float *score);
/* OpenCV medianBlur(ksize 3, BORDER_REPLICATE) restated, float maps. */
void or_median3(int W, int H, const float *in, float *out);

/* ---- seeding from a prior result (depthmap.cc:434-516) ---- */
void or_warp_prior(int Wp, int Hp, const float *prev_plane, const float *prev_depth, const double *Rp,
                   const double *tp, int W, int H, const double *Rn, const double *tn, float *cand);

/* ---- geometric consistency filter (depthmap.cc:1320-1377) ----
 * depths[n] (n views, H*W each), poses R[n][9], t[n][3]; view `center` is
 * filtered against all others.  reproj_px > 0 adds a round-trip
 * reprojection test (not in the reference; 0 disables). */
void or_clean(int W, int H, int n, const float *const *depths,
              const double *R, const double *t, int center,
              float same_depth_threshold, int min_consistent_views,
              float reproj_px, float *out);

/* ---- fusion / pruning (depthmap.cc:1535-1696) ----
 * depths[0] = head map (pruned), depths[1..n-1] are mutated in place the way
 * the reference mutates the later queue entries.  rgb = head colour image
 * (H*W*3 bytes, may be NULL).  Writes pruned depth (H*W), and returns the
 * number of points; points (3*count doubles), colors (3*count bytes), keypts
 * (2*count ints: i, j) are filled when non-NULL (caller sizes them H*W). */
int or_prune(int W, int H, int n, float *const *depths, const double *R,
             const double *t, const uint8_t *rgb, float same_depth_threshold,
             float *pruned, double *points, uint8_t *colors, int32_t *keypts);

#ifdef __cplusplus
}
#endif
#endif
