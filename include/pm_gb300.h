/*
 * pm_gb300.h -- C ABI of the GB300-native PatchMatch-Stereo densifier for
 * equirectangular keyframes.
 *
 * It sits where RoblabWh/PatchMatch's densification thread calls into its
 * CUDA file: a reference keyframe plus its neighbour keyframes go in; depth,
 * normal, plane, score and best-view maps, a geometric-consistency-filtered
 * depth map and a fused, coloured point cloud come out.  All signatures use
 * plain pointers and sizes.  Every function returns a status code (PM_OK = 0)
 * and records a message retrievable with pm_last_error(); nothing is printed.
 * The reference's launchers return void and only print cudaGetLastError
 * (src/openvslam/PatchMatchCuda.cu:447-451).
 *
 * Conventions (as in the reference):
 *   - images are H x W row-major; pixel (i, j) = (row, column);
 *   - pixel (i, j) has bearing (cos lat sin lon, -sin lat, cos lat cos lon),
 *     lon = 2 pi (j/W - 1/2), lat = -pi (i/H - 1/2)  (PatchMatchCuda.cu:183-208);
 *   - poses are world->camera: X_c = R_cw X_w + t_cw, R_cw row-major;
 *   - a plane hypothesis is the camera-frame vector pi with pi . X = 1, so the
 *     depth (range) of pixel (i, j) is 1 / |pi . b(i, j)|  (PatchMatchCuda.cu:31-43,402-404).
 *
 * Thread safety: one context may be used from one host thread at a time; use
 * one context per thread for concurrency.  No process-global state is kept
 * (the reference kept poses in __constant__ symbols, PatchMatchCuda.cu:11-23).
 */
#ifndef PM_GB300_H
#define PM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PM_MAX_SOURCES 10

/* status codes */
#define PM_OK 0
#define PM_EINVAL 1      /* bad argument (size, pointer, pose, parameter) */
#define PM_ENOMEM 2      /* device allocation failed */
#define PM_EBUDGET 3     /* request does not fit the context's HBM budget */
#define PM_ETIMEOUT 4    /* a bounded wait expired */
#define PM_ECUDA 5       /* CUDA runtime error (message in pm_last_error) */
#define PM_ENOTREADY 6   /* asynchronous work still in flight */
#define PM_ECANCELLED 7  /* request was cancelled */
#define PM_ENOTBUILT 8   /* no kernel variant for this configuration */

/* view combination (how per-source NCC scores become one cost) */
/* PM_COMBINE_FOLD is the reference GPU kernel exactly: its weighted moment
 * sums are declared once outside the per-view loop and never reset
 * (PatchMatchCuda.cu:57-62,100-176), so view r's NCC is taken over the samples
 * of views 1..r together; the running score then averages when within 25 %,
 * else keeps the max (PatchMatchCuda.cu:93,161-171). */
#define PM_COMBINE_FOLD 0
#define PM_COMBINE_MAX 1          /* reference CPU rule: maximum over sources (depthmap.cc:1104-1127) */
#define PM_COMBINE_TOPK 2         /* per-pixel view selection: mean of the top_k sources */
#define PM_COMBINE_FOLD_SEPARATE 3 /* the 25 % fold over independent per-source NCCs */

/* longitude seam handling of bilinear source samples */
#define PM_SEAM_CLAMP 0    /* clamp at the image border (the reference's texture behaviour) */
#define PM_SEAM_WRAP 1     /* wrap around in longitude (360-degree continuity) */
#define PM_SEAM_ZERO 2     /* the reference host cost's border: a sample whose bilinear footprint leaves
                              [0, W-1) x [0, H-1) reads 0 (LinearInterpolation, depthmap.cc:34-38);
                              with PM_SAMPLER_EXACT and PM_COMBINE_MAX this is
                              ComputePlaneImageScoreUnoptimized_equirect + ComputePlaneScore
                              (depthmap.cc:1104-1157) for interior pixels */

/* initialisation */
#define PM_INIT_LOGUNIFORM_HEMI 0 /* log-uniform depth, unit normals on the camera-facing hemisphere */
#define PM_INIT_REF_UNIFORM 1     /* uniform depth, normal components U[-1,1] (PatchMatchCuda.cu:210-244) */

/* image storage */
#define PM_IMAGE_U8 0
#define PM_IMAGE_F16 1

/* Source-image sampling (pm_params.sampler).
 *   PM_SAMPLER_EXACT  : bilinear interpolation with FP32 weights from
 *                       quad-packed footprints (either seam policy).
 *   PM_SAMPLER_TEXTURE: the GPU's texture filter, as the reference samples its
 *                       source images (PatchMatchCuda.cu:146, 754-763): texel
 *                       centres at +0.5, weights quantised to 1/256 of a
 *                       texel, clamped at the image border (PM_SEAM_CLAMP
 *                       only). */
#define PM_SAMPLER_EXACT 0
#define PM_SAMPLER_TEXTURE 1

/* Propagation rule of the red-black sweeps (pm_params.propagation).
 *   PM_PROPAGATION_SMOOTH: the reference GPU kernel (PatchMatchRedBlackPass_,
 *     PatchMatchCuda.cu:273-407): neighbour planes scored x smoothness factor,
 *     refinements around the plane after propagation.
 *   PM_PROPAGATION_PLAIN: the reference's host variant (PatchMatchUpdatePixel,
 *     depthmap.cc:1003-1067): plain score comparison, pixels and neighbours of
 *     depth 0 ignored, each refinement around the current plane and depth with
 *     its own depth draw, skipped (ranges kept) when the plane's z is 0. */
#define PM_PROPAGATION_SMOOTH 0
#define PM_PROPAGATION_PLAIN 1

typedef struct {
    int patch_half;      /* taps at odd offsets -patch_half..patch_half (5 = PatchSize 7 - 2, depthmap.cc:725) */
    int iterations;      /* red-black sweeps (Dense.Iterations, config.cc:172) */
    int combine;         /* PM_COMBINE_* */
    int top_k;           /* sources averaged by PM_COMBINE_TOPK */
    int seam;            /* PM_SEAM_* */
    int init_mode;       /* PM_INIT_* */
    int image_format;    /* PM_IMAGE_* of pm_view.gray */
    int postprocess;     /* 1: host-equivalent window, median and thresholds (depthmap.cc:731-767) */
    float min_depth;     /* initialisation range and accepted depth range */
    float max_depth;
    float min_score;     /* 0.1 (depthmap_computation_module.cc:223) */
    float min_patch_sd;  /* low-texture mask threshold (Dense.MinPatchSD, 0 disables) */
    float sigma_color;   /* bilateral sigmas 50 and 5 (PatchMatchCuda.cu:897-900) */
    float sigma_x;
    uint32_t seed;       /* Philox key, with keyframe_id */
    uint32_t keyframe_id;
    int sampler;         /* PM_SAMPLER_* */
    int propagation;     /* PM_PROPAGATION_* */
} pm_params;

typedef struct {
    const void *gray;     /* H x W intensities, uint8 or IEEE half per pm_params.image_format */
    size_t pitch_bytes;   /* row pitch; 0 = tightly packed */
    const uint8_t *mask;  /* optional H x W (reference view only): 0 = pixel ignored */
    double R_cw[9];       /* world->camera rotation, row-major */
    double t_cw[3];
} pm_view;

typedef struct {
    float *depth;         /* H x W, 0 = invalid (required) */
    float *score;         /* H x W or NULL */
    float *plane;         /* H x W x 3 or NULL */
    float *normal;        /* H x W x 3 or NULL: unit, camera frame, facing the camera */
    int32_t *best_view;   /* H x W or NULL: 0-based index of the best source */
} pm_maps;

typedef struct pm_ctx pm_ctx;
typedef struct pm_request pm_request;
typedef struct pm_result pm_result;
typedef struct pm_batch pm_batch;

/* Defaults of the reference path: patch_half 5, iterations 8, fold
 * combination, clamp seam, log-uniform/hemisphere init in [0.3, 20] m,
 * u8 images, post-processing on, min_score 0.1, sigmas 50/5, texture
 * sampler, smooth (GPU) propagation. */
void pm_params_default(pm_params *p);

/* Context: one CUDA stream on `device`, device buffers owned by the context,
 * an HBM budget for admission (0 = 90 % of free memory).
 * Replaces the per-keyframe cudaMalloc/cudaFree of
 * DepthmapEstimator::ComputePatchMatch (depthmap.cc:557-800) and the global
 * constant-memory state of InitConstantMem (PatchMatchCuda.cu:885-912).
 *
 * Threads and lifetimes: a context and everything made from it (requests,
 * retained results, batches) are used from one host thread at a time; a
 * pm_server works on its context from its own worker thread, so make no
 * other calls on that context while the server exists.  Several contexts
 * may run side by side.  A request held by a batch cannot be destroyed
 * until the batch is cleared or destroyed; destroying a prior (request or
 * retained result) unlinks the requests it seeds.  pm_destroy returns
 * PM_EINVAL while requests, retained results or batches of the context are
 * alive: destroy servers, batches, requests and results first. */
int pm_create(int device, size_t hbm_budget_bytes, pm_ctx **out);
int pm_destroy(pm_ctx *ctx);
const char *pm_last_error(const pm_ctx *ctx);
const char *pm_status_string(int status);
/* Kernel launches issued by this context so far (instrumentation). */
uint64_t pm_launch_count(const pm_ctx *ctx);
/* The context's CUDA stream (a cudaStream_t), for timing with CUDA events. */
void *pm_stream(const pm_ctx *ctx);
/* Measured FP32 FMA throughput of this GPU in TFLOP/s (an FFMA-bound probe
 * kernel on the context's stream; 1 FMA = 2 flop).  The densifier's cost
 * kernel is bounded by the FP32 pipe, so this is its roofline denominator. */
int pm_probe_fp32_peak(pm_ctx *ctx, double *tflops);
/* Measured special-function-unit throughput (approximate exponentials, one
 * MUFU instruction each, like the cost kernel's reciprocals, reciprocal
 * square roots and exponentials) in Gop/s, and bilinear texture-fetch
 * throughput from an L1-resident u8 texture in Gfetch/s: the two other terms
 * of the cost kernel's roofline (40 FP32 flop, 4 special-function operations
 * and 1 bilinear fetch per sample). */
int pm_probe_sfu_peak(pm_ctx *ctx, double *gops);
int pm_probe_tex_peak(pm_ctx *ctx, double *gfetches);

/* One keyframe, host buffers in and out (synchronous).  views[0] is the
 * reference keyframe, views[1..n_views-1] its sources (1..PM_MAX_SOURCES).
 * Replaces DepthmapEstimator::ComputePatchMatch (depthmap.cc:541-806):
 * bearing table, random initialisation, init scoring, red-black sweeps,
 * host post-filter. */
int pm_densify(pm_ctx *ctx, int width, int height, const pm_view *views, int n_views, const pm_params *params,
               pm_maps *out);

/* ---- device-resident requests (the building block of batching/serving) ---- */
/* Allocate device state for one W x H keyframe with n_sources sources.
 * Fails with PM_EBUDGET when the context's HBM budget would be exceeded. */
int pm_request_create(pm_ctx *ctx, int width, int height, int n_sources, const pm_params *params,
                      pm_request **out);
int pm_request_destroy(pm_request *req);
size_t pm_request_bytes(int width, int height, int n_sources, int image_format);
int pm_request_set_params(pm_request *req, const pm_params *params);
/* Upload view k (0 = reference, 1.. = sources) asynchronously and build its
 * sampling form.  Replaces InitTextureImages + InitConstantMem
 * (PatchMatchCuda.cu:697-797,885-912). */
int pm_request_set_view(pm_request *req, int k, const pm_view *view);
/* Random planes (Philox) + scoring of every interior pixel.  Replaces
 * ComputeRandomSeed + RandomInitialization (PatchMatchCuda.cu:621-663). */
int pm_request_init(pm_request *req);
/* Overwrite the plane map (H x W x 3, camera frame) and rescore it: the
 * seeding entry for prior knowledge (replaces the host round trip of
 * depthmap.cc:669-719). scores may be NULL (then every interior pixel is rescored). */
int pm_request_set_state(pm_request *req, const float *planes, const float *scores);
/* Reuse a previous keyframe's post-filtered result as initialisation: its
 * planes are splatted into this view (nearest candidate per pixel) and kept
 * where they score higher than the random planes.  pm_request_seed does it
 * now (after pm_request_init); pm_request_set_prior makes pm_request_run do
 * it after the random initialisation (NULL clears).  The prior must stay
 * alive and unchanged until the work is done.  Replaces the host
 * PreInitResultWarp (depthmap.cc:434-516); the prior's normals are rotated
 * into the new camera (the reference reuses them unrotated). */
/* Seeding from SLAM landmarks (world points, n x 3 FP64): the GPU form of
 * DepthmapEstimator::PreInitSparsePCL2 (depthmap.cc:361-432).  Each point is
 * projected into the reference view in FP64 and rounded to the nearest pixel;
 * the pixel's candidate plane faces the camera (normal = -bearing) at the
 * point's range, and it replaces the current plane where it scores higher.
 * Where several points land on one pixel the nearest is used (the reference
 * resolves that by an OpenMP race).  pm_request_set_landmarks stages the
 * points for pm_request_run (applied after the random initialisation and
 * before the prior result, as in ComputePatchMatch, depthmap.cc:683-684);
 * pm_request_seed_landmarks applies them to the current state now (and
 * stages them too).  The reference view must be set first; n = 0 clears. */
int pm_request_set_landmarks(pm_request *req, const double *xyz_world, int n);
int pm_request_seed_landmarks(pm_request *req, const double *xyz_world, int n);
int pm_request_seed(pm_request *req, const pm_request *prior);
int pm_request_set_prior(pm_request *req, const pm_request *prior);
/* Retained results: a compact copy (plane state + filtered depth + pose,
 * 20 bytes per pixel) of a finished request, kept for seeding later
 * keyframes while the request itself is reused.  pm_result_snapshot enqueues
 * the copy on the request's stream (the request must have been
 * post-processed); pm_request_set_prior_result makes pm_request_run seed from
 * it once the copy has finished.  A prior link (to a request or a result)
 * lasts until it is replaced; destroying the prior waits for its dependents'
 * in-flight work and unlinks them, so their next run starts unseeded. */
size_t pm_result_bytes(int width, int height);
int pm_result_create(pm_ctx *ctx, int width, int height, pm_result **out);
int pm_result_snapshot(pm_result *res, pm_request *req);
int pm_result_destroy(pm_result *res);
int pm_request_set_prior_result(pm_request *req, const pm_result *res);
/* n_half red/black half-sweeps starting at half-sweep index first_half
 * (even = red, odd = black; sweep = first_half / 2).  Replaces
 * PatchMatchRedBlackPass (PatchMatchCuda.cu:568-615). */
int pm_request_sweep(pm_request *req, int first_half, int n_half);
/* Host-equivalent post-filter on the device (depthmap.cc:731-767,1169-1208). */
int pm_request_postprocess(pm_request *req);
/* init + all sweeps + post-filter, replayed from a captured CUDA graph. */
int pm_request_run(pm_request *req);
/* Copy maps out (host or device destinations; synchronous).  raw = 1 returns
 * the unfiltered sweep state.  _async enqueues the copies on the request's
 * stream and returns; completion is visible through pm_request_query. */
int pm_request_read(pm_request *req, pm_maps *out, int raw);
int pm_request_read_async(pm_request *req, pm_maps *out, int raw);
int pm_request_synchronize(pm_request *req);
/* PM_OK when all work enqueued for the request has finished, PM_ENOTREADY
 * while some is in flight. */
int pm_request_query(const pm_request *req);
/* The request's own CUDA stream (a cudaStream_t): every request runs on its
 * own stream, so requests of one context overlap on the device. */
void *pm_request_stream(const pm_request *req);
/* Device pointer of the (filtered) depth map, H x W float, for chaining into
 * pm_filter_consistency_device / pm_fuse_device without a host round trip. */
const float *pm_request_depth_device(const pm_request *req);
/* The same for a retained result (its snapshot of the filtered depth); valid
 * once the snapshot's request stream has passed pm_result_snapshot. */
const float *pm_result_depth_device(const pm_result *res);

/* Score n fixed plane hypotheses at pixels ij[2n] (row, col) against the
 * request's views: the cost kernel in isolation.  scores[n], best[n] and
 * per_source[n * n_sources] may be NULL.  Replaces ScorePlaneDepth
 * (PatchMatchCuda.cu:255-270,528-565) for arbitrary hypotheses. */
int pm_score_hypotheses(pm_request *req, int n, const int32_t *ij, const float *planes, float *scores,
                        int32_t *best, float *per_source);

/* Geometric-consistency filter of depths[center] against the other views
 * (host buffers).  A pixel is kept when at least min_consistent_views views
 * (itself included) see the reprojected depth within same_depth_threshold
 * relative; reproj_px > 0 adds a round-trip reprojection test of that many
 * pixels.  Replaces DepthmapCleaner::Clean (depthmap.cc:1320-1377). */
int pm_filter_consistency(pm_ctx *ctx, int width, int height, int n_views, const float *const *depths,
                          const double *R_cw, const double *t_cw, int center, float same_depth_threshold,
                          int min_consistent_views, float reproj_px, float *out);

typedef struct {
    int capacity;      /* entries available in the arrays below */
    int count;         /* points written */
    double *xyz;       /* capacity x 3 world coordinates (FP64, composed on the host) */
    uint8_t *bgr;      /* capacity x 3 colour of the head keyframe (BGR) or NULL */
    int32_t *ij;       /* capacity x 2 pixel (row, col) or NULL */
} pm_points;

/* Point fusion of the head map depths[0] against depths[1..n_views-1]:
 * duplicate points are resolved in favour of the nearer observation and the
 * later maps are edited in place (pixels zeroed), exactly in the order the
 * reference does it.  pruned (H x W) receives the head's kept depth.
 * Replaces DepthmapPruner::Prune (depthmap.cc:1535-1696). */
int pm_fuse(pm_ctx *ctx, int width, int height, int n_views, float *const *depths, const double *R_cw,
            const double *t_cw, const uint8_t *bgr, float same_depth_threshold, float *pruned, pm_points *out);

/* The same two stages on DEVICE buffers, chained after densification without
 * a host round trip: depths[k] are device pointers (e.g. pm_request_depth_device
 * of finished requests, or caller buffers) and every output is a device
 * buffer.  Work is enqueued on `stream` (a cudaStream_t; NULL = the context's
 * stream) and the call returns without synchronising; order the stream after
 * the work that writes the inputs.  Neither call allocates, except that the
 * context builds its bearing tables for an image size on the first use of that
 * size.  Same kernels and results as the host-buffer calls.
 * Replace DepthmapCleaner::Clean (depthmap.cc:1320-1377) and
 * DepthmapPruner::Prune (depthmap.cc:1535-1696) for device-resident maps (the
 * reference hands host cv::Mat copies between its threads,
 * depthmap_computation_module.cc:396-412, dense_pointcloud_module.cc:115-175). */
int pm_filter_consistency_device(pm_ctx *ctx, int width, int height, int n_views, const float *const *depths,
                                 const double *R_cw, const double *t_cw, int center, float same_depth_threshold,
                                 int min_consistent_views, float reproj_px, float *out, void *stream);
/* Bytes of the fusion workspace for one image size (0 for invalid sizes). */
size_t pm_fuse_workspace_bytes(int width, int height);
/* Fusion on device maps: the later maps are edited in place as by pm_fuse;
 * pruned (H x W), xyz (H*W x 3 floats, world frame), bgr_out (H*W x 3, may be
 * NULL), ij (H*W x 2 int32 (row, col), may be NULL) and count (one unsigned)
 * receive the results; bgr (device, may be NULL) is the head's colour image.
 * workspace: a 256-byte aligned device block of pm_fuse_workspace_bytes bytes
 * that no other call uses until this one has finished on the device. */
int pm_fuse_device(pm_ctx *ctx, int width, int height, int n_views, float *const *depths, const double *R_cw,
                   const double *t_cw, const uint8_t *bgr, float same_depth_threshold, float *pruned, float *xyz,
                   uint8_t *bgr_out, int32_t *ij, unsigned *count, void *workspace, size_t workspace_bytes,
                   void *stream);

/* ---- served densification (a request loop over the calls above) ----
 * Keyframes are submitted as SLAM emits them (any thread).  A worker thread
 * owns the context: it admits keyframes in submission order as in-flight
 * slots and the HBM budget allow, keeps every admitted keyframe's image
 * resident on the device (a cache of cache_capacity keyframes) for reuse as a
 * neighbour, selects as sources the nearest earlier keyframes whose camera
 * baseline lies in [min_baseline, max_baseline] metres (min_sources ..
 * max_sources of them), seeds each keyframe from the newest densified keyframe
 * at least prior_lag submissions back (then runs seeded_iterations sweeps
 * instead of params.iterations), and runs it on its own stream so keyframes
 * that arrive while others are on the GPU overlap with them.  Every choice
 * depends only on submission order, so a keyframe's result is the same
 * whether it ran alone or among others.  Replaces the densification thread's
 * loop (depthmap_computation_module.cc:205-472). */
typedef struct pm_server pm_server;
typedef struct {
    pm_params params;        /* base parameters; params.iterations = sweeps without a prior */
    int cache_capacity;      /* resident keyframes (40) */
    int max_inflight;        /* keyframes on the GPU at once (4) */
    int min_sources;         /* fewer earlier neighbours: the keyframe completes with PM_ENOTREADY */
    int max_sources;
    float min_baseline;      /* metres */
    float max_baseline;
    int seed_from_prior;     /* 1: reuse an earlier result as initialisation */
    int seeded_iterations;   /* sweeps of a seeded keyframe (2) */
    int prior_lag;           /* seed from the newest densified keyframe at least this many back (4) */
    int poll_us;             /* worker polling interval while work is in flight */
    int coarse_to_fine;      /* 1: a keyframe without a prior, at least 1920 wide with even sizes, is
                                densified at half resolution first (params.iterations sweeps) and
                                then refined at full resolution (seeded_iterations sweeps) seeded
                                from that result */
    int dense_output;        /* 1: run the geometric-consistency filter and point fusion over the stream,
                                as the reference's cleaner and pruner queues do
                                (depthmap_computation_module.cc:396-412, dense_pointcloud_module.cc:115-175):
                                keyframe k's depth is cleaned against the two densified keyframes of its size
                                before and after it, and its cleaned map is fused against the next four
                                cleaned maps; results through pm_server_wait_dense */
    float clean_threshold;   /* filter: relative depth agreement (0.01, DepthmapCleaner default) */
    int clean_min_views;     /* filter: consistent views including itself (3) */
    float clean_reproj_px;   /* filter: round-trip reprojection test in pixels (1.0; 0 = off) */
    float fuse_threshold;    /* fusion: relative depth threshold (0.08, Dense.SameDepthThreshold of the
                                reference's example configuration) */
    float min_view_score;    /* keyframes submitted with landmarks join only when score_view against the
                                previous joined keyframe exceeds this (0.25, :334-335) */
} pm_server_config;
typedef struct {
    int status;              /* PM_OK, PM_ENOTREADY (too few neighbours) or an error */
    int n_sources;
    int seeded;              /* 0: random initialisation, 1: an earlier keyframe's result,
                                2: its own half-resolution pass (coarse_to_fine) */
    int iterations;
    double queue_ms;         /* submit -> start on the GPU */
    double latency_ms;       /* submit -> maps on the host */
    float view_score;        /* score_view against the previous joined keyframe (-1: not computed) */
} pm_served_info;
/* Memory: requests and retained results (20 B/px, at most prior_lag + 1 per
 * image size) are admitted against the context's HBM budget; the keyframe
 * cache (cache_capacity images of W*H bytes) and pinned host buffers for the
 * results are allocated outside it, once, and reused. */
void pm_server_config_default(pm_server_config *cfg);
int pm_server_create(pm_ctx *ctx, const pm_server_config *cfg, pm_server **out);
/* Copies the keyframe's gray image (uint8) and pose; returns a ticket. */
int pm_server_submit(pm_server *srv, int width, int height, const pm_view *keyframe, uint64_t *ticket);
/* The same with the keyframe's SLAM landmarks (world points xyz[n x 3], FP64,
 * and their ids), as the reference's densification thread receives them
 * (depthmap_computation_module.cc:328-374): the keyframe joins only when
 * score_view against the previous joined keyframe with landmarks exceeds
 * min_view_score (otherwise it completes with PM_ENOTREADY and is neither
 * cached nor densified), its depth interval's upper bound becomes 1.1 x the
 * 90th percentile of the landmark ranges (compute_depth_intervall, :123-131;
 * the lower bound stays params.min_depth), and it is seeded from the
 * landmarks before any prior result (PreInitSparsePCL2, depthmap.cc:361-432). */
int pm_server_submit_landmarks(pm_server *srv, int width, int height, const pm_view *keyframe,
                               const double *xyz_world, const uint64_t *ids, int n_landmarks, uint64_t *ticket);
/* Blocks until the ticket's keyframe is done (timeout_ms < 0: no limit;
 * PM_ETIMEOUT otherwise), then fills out->depth / out->score (host, may be
 * NULL) and info.  Returns the keyframe's status.  Each ticket is collected
 * once: PM_EINVAL for a ticket this server did not issue or that was already
 * collected (also when another thread collects it while this one waits).
 * All waits must have returned before pm_server_destroy. */
int pm_server_wait(pm_server *srv, uint64_t ticket, int timeout_ms, pm_maps *out, pm_served_info *info);
/* With dense_output: blocks until the ticket's fused output exists (timeout as
 * pm_server_wait), then fills depth (H x W host floats: the keyframe's depth
 * after the consistency filter and fusion, may be NULL) and points (host:
 * xyz world FP64 and ij (row, col) of the points fusion kept;
 * points->count receives their number.  When it exceeds points->capacity
 * nothing is written, the call returns PM_EINVAL with points->count set and
 * the ticket stays collectable with a larger buffer; bgr is not written, the
 * served loop receives gray images).  Returns PM_OK, PM_ENOTREADY for a keyframe that was not densified
 * or whose filter or fusion window never filled (the first two and the last
 * keyframes of each image size, as in the reference), PM_ECANCELLED for one
 * cancelled by pm_server_destroy, or PM_EINVAL (no dense output, unknown or
 * already collected ticket).  Collected once, independently of pm_server_wait. */
int pm_server_wait_dense(pm_server *srv, uint64_t ticket, int timeout_ms, float *depth, pm_points *points);
/* End of the stream: refuses further submissions (PM_ECANCELLED), densifies
 * every keyframe already submitted, completes every dense output (those whose
 * windows never filled with PM_ENOTREADY) and returns when all results exist;
 * they stay collectable until pm_server_destroy.  A pm_server_destroy on
 * another thread while this call blocks returns only after it has. */
int pm_server_finish(pm_server *srv);
/* Finishes the keyframes already on the GPU; keyframes still queued complete
 * with PM_ECANCELLED (and their dense outputs too).  Returns once every thread
 * blocked in pm_server_wait / pm_server_wait_dense has returned; no call may
 * use the server afterwards.  Uncollected results are released. */
int pm_server_destroy(pm_server *srv);

/* ---- fusion for callers that cannot allocate device memory ----
 * Some callers must not allocate at the moment they fuse: a process whose
 * device memory belongs to an external pool or arena, a real-time thread that
 * cannot enter the CUDA allocator (unbounded latency, possible device-wide
 * synchronisation), or code whose HBM is already committed.  This entry point
 * has no counterpart in the reference.  It runs the pm_fuse kernels on
 * caller-owned DEVICE buffers and enqueues on `stream` (a cudaStream_t, NULL =
 * default stream) without synchronising; it never calls cudaMalloc/cudaFree.
 * Its working memory is one file-scope device array (about 20 MB) that every
 * GPU loading the library holds until the process exits, so images are limited
 * to PM_FUSE_NOALLOC_MAX_PIXELS pixels, width <= PM_FUSE_NOALLOC_MAX_WIDTH and
 * height <= PM_FUSE_NOALLOC_MAX_HEIGHT (larger sizes return PM_EINVAL).
 * The first call on each device looks up that array's device address
 * (cudaGetSymbolAddress) with the device current; make that first call before
 * any stream capture.  The first call for each image size on a device also
 * copies that size's bearing tables from host memory into the array.  A launch
 * error left pending by earlier work on the calling thread is cleared on entry
 * (it is not reported as this call's).  All calls on a device share the array: calls whose GPU
 * work overlaps (e.g. on two streams) race and must be serialised by the
 * caller.  depths[k] (device, H x W floats, k = 0 head) are edited in place as
 * by pm_fuse; pruned (H x W), xyz (H*W x 3 floats, world frame), bgr_out
 * (H*W x 3, may be NULL), ij (H*W x 2, may be NULL) and count (one unsigned)
 * are device outputs; bgr (device, may be NULL) is the head's colour image. */
#define PM_FUSE_NOALLOC_MAX_PIXELS (1u << 21)
#define PM_FUSE_NOALLOC_MAX_WIDTH 8192
#define PM_FUSE_NOALLOC_MAX_HEIGHT 4096
int pm_fuse_noalloc(int width, int height, int n_views, float *const *depths, const double *R_cw,
                    const double *t_cw, const uint8_t *bgr, float same_depth_threshold, float *pruned, float *xyz,
                    uint8_t *bgr_out, int32_t *ij, unsigned *count, void *stream);

/* ---- batched form ----
 * Many requests densified together: init scoring, every red/black half-sweep
 * and the post-filter run phase-major over all requests, captured once into a
 * CUDA graph and replayed by pm_batch_run.  Requests are grouped by source
 * count, image variant, propagation rule and sweep count; each phase of a
 * group is one persistent launch over a device queue of (request, 8x64 tile)
 * items (PM_BATCH_PERSISTENT, grid = grid_mult x resident CTAs) or one launch
 * per request (PM_BATCH_LAUNCHES); PM_BATCH_STREAMS instead runs each
 * request's whole chain on one of 8 parallel graph branches (largest request
 * first onto the least-loaded branch) so that requests overlap on the GPU;
 * PM_BATCH_MIXED is one persistent launch per phase over all requests of
 * every source count (items carry their count; the kernel holds the bodies
 * of all counts, at the register budget of the largest).  Every request's maps equal those of
 * pm_request_run bit for bit.  Requests keep their own buffers and streams:
 * set their views before pm_batch_run; read them afterwards with
 * pm_request_read (their streams wait for the batch).  Seeded requests are
 * batched too: landmark seeds and priors (a retained result, a request outside
 * the batch, or a request of the same batch, e.g. a coarse-to-fine chain whose
 * full-size request is seeded from a half-size one) are applied between the
 * init scoring and the sweeps as pm_request_run does; a request seeded from a
 * member runs one level after it (levels run in order, each level
 * phase-major), and priors from outside the batch are waited for before the
 * graph starts.  A cycle of priors within a batch is PM_EINVAL.  A request in a batch cannot be
 * destroyed (pm_request_destroy returns PM_EINVAL) until pm_batch_clear or
 * pm_batch_destroy releases it.  pm_batch_tune runs the batch once
 * per executor candidate, keeps the fastest and reports the timings.
 * No counterpart in the reference (one keyframe at a time,
 * depthmap_computation_module.cc:205-472). */
#define PM_BATCH_PERSISTENT 0
#define PM_BATCH_LAUNCHES 1
#define PM_BATCH_STREAMS 2
#define PM_BATCH_MIXED 3
#define PM_BATCH_CANDIDATES 5
typedef struct {
    int executor;            /* chosen PM_BATCH_* */
    int grid_mult;           /* chosen persistent grid multiple */
    float ms;                /* its time for one pm_batch_run */
    float candidate_ms[PM_BATCH_CANDIDATES];  /* persistent x1, persistent x2, per-request launches,
                                                 parallel branches, mixed persistent */
} pm_batch_tuning;
int pm_batch_create(pm_ctx *ctx, pm_batch **out);
int pm_batch_add(pm_batch *b, pm_request *req);
int pm_batch_clear(pm_batch *b);
int pm_batch_set_executor(pm_batch *b, int executor, int grid_mult);
int pm_batch_run(pm_batch *b);
int pm_batch_synchronize(pm_batch *b);
void *pm_batch_stream(const pm_batch *b);
int pm_batch_tune(pm_batch *b, pm_batch_tuning *out);
int pm_batch_destroy(pm_batch *b);

/* ---- input preparation (device buffers, context stream) ----
 * The keyframe thumbnails the densifier reads (data/frame.cc:53-54,136-138)
 * and the FP16 pyramid of the precision form.  All pointers are device
 * memory; pitches in bytes; work is enqueued on the context's stream.
 * pm_image_to_gray: 1, 3 or 4 interleaved channels in PM_ORDER_BGR or
 *   PM_ORDER_RGB to gray with BT.601 weights in 14-bit fixed point, rounded
 *   (the fixed-point form of the colour conversion in
 *   util/image_converter.cc:8-39); 1 channel is copied.
 * pm_image_resize: bilinear resize of 1-4 interleaved u8 channels, pixel
 *   centres aligned, 11-bit fixed-point weights, one rounding (cv::resize's
 *   linear scheme for thumbnails and masks).
 * pm_build_pyramid_f16: out[0] = the image (u8 or FP16 per src_format) as
 *   FP16 (W x H, tightly packed; may be the FP16 source itself), out[k] =
 *   2x2 means of out[k-1] ((w+1)/2 x (h+1)/2, the last row/column repeated
 *   at odd sizes), summed in FP32 and rounded once. */
#define PM_ORDER_BGR 0
#define PM_ORDER_RGB 1
int pm_image_to_gray(pm_ctx *ctx, const void *src, int width, int height, size_t pitch, int channels, int order,
                     void *gray, size_t gray_pitch);
int pm_image_resize(pm_ctx *ctx, const void *src, int src_w, int src_h, size_t src_pitch, int channels, void *dst,
                    int dst_w, int dst_h, size_t dst_pitch);
int pm_build_pyramid_f16(pm_ctx *ctx, const void *src, int width, int height, size_t pitch, int src_format,
                         int levels, void *const *out);

/* ---- dense map output (host) ----
 * pm_write_ply: the fused points as ASCII PLY (x y z in fixed notation,
 * colours as three uchar in stored order, white without colours), the file of
 * map_database_io::save_point_cloud_dense (io/map_database_io.cc:45-80).
 * pm_write_dense_msgpack: the dense map message of save_message_pack_dense
 * (io/map_database_io.cc:22-43): a MessagePack map {cameras, keyframes,
 * landmarks}, one landmark record per point in the layout of
 * landmark::to_json (data/landmark.cc:370-377) with ids first_id, first_id+1,
 * ... and keyframe_id as first and reference keyframe; the camera and
 * keyframe tables (SLAM map state) are written empty.  Both return
 * PM_EINVAL when the file cannot be written. */
int pm_write_ply(const char *path, const pm_points *pts);
int pm_write_dense_msgpack(const char *path, const pm_points *pts, uint64_t first_id, uint32_t keyframe_id);

/* ---- neighbour geometry (host, FP64) ----
 * pm_score_view: the densification thread's view test (score_view,
 * depthmap_computation_module.cc:147-198; a keyframe joins the window when the
 * score exceeds 0.25, :334-335): the fraction of landmarks common to both
 * keyframes (matched by id) whose triangulation angle between the camera
 * centres lies in (3, 30) degrees.  cur_xyz: n_cur x 3 world positions.
 * No common landmark gives score 0.
 * pm_depth_interval: the 10th / 90th percentile of the landmarks' ranges from
 * the camera (keyframe::computePercentileDepth_10_90, data/keyframe.cc:428-455)
 * and the densifier's depth interval [1e-5, 1.1 p90]
 * (compute_depth_intervall, depthmap_computation_module.cc:123-131). */
int pm_score_view(const double prev_center[3], const double cur_center[3], const uint64_t *prev_ids, int n_prev,
                  const uint64_t *cur_ids, const double *cur_xyz, int n_cur, float *score, int *n_common);
int pm_depth_interval(const double R_cw[9], const double t_cw[3], const double *xyz, int n, double *p10,
                      double *p90, double *min_depth, double *max_depth);

#ifdef __cplusplus
}
#endif
#endif
