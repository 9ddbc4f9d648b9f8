// Internal types and helpers shared by the host-side translation units of the
// densifier (pm_api.cu, pm_batch.cu): the opaque C ABI objects and the few
// request helpers the batched executor reuses.  Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <string>
#include <vector>

#include "pm_gb300.h"
#include "pm_types.h"

#define PM_INTERNAL __attribute__((visibility("hidden")))

#include <nvtx3/nvToolsExt.h>

// An NVTX range over a host-side scope (visible in Nsight timelines; a no-op
// unless a tool is attached).
struct NvtxRange {
    explicit NvtxRange(const char *fmt, ...) {
        char buf[128];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        nvtxRangePushA(buf);
    }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// Bearing tables of one image size (device).
struct Trig {
    int W = 0, H = 0;
    float2 *row = nullptr, *col = nullptr;
};


struct pm_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    size_t budget = 0, used = 0;
    std::string err;
    uint64_t launches = 0;
    std::vector<Trig> trig;
    pm_request *cached = nullptr;
    void *scratch = nullptr;
    size_t scratch_bytes = 0;
    int live = 0;  // requests, retained results and batches made from this context (cached included)
    int n_sm = 0;  // streaming multiprocessors: bands of the banded tile order
};

struct pm_request {
    pm_ctx *ctx = nullptr;
    int W = 0, H = 0, S = 0;
    int batch_refs = 0;  // batches holding this request (it cannot be destroyed meanwhile)
    unsigned *band_ctr = nullptr;  // per-SM tile counters of the banded order (in the block)
    int banded_blocks = 0;         // persistent grid of the banded order (0: one CTA per tile)
    pm_params prm{};
    size_t bytes = 0;
    void *block = nullptr;  // one device allocation holding everything below
    float *ref = nullptr;
    uint8_t *raw = nullptr;
    void *quad[PM_MAX_SOURCES] = {};     // quad-packed footprints, or pitched images for textures
    cudaTextureObject_t tex[PM_MAX_SOURCES] = {};
    int tex_format = -1;                 // image format the texture objects were made for (-1: none)
    size_t tex_pitch = 0;
    uint8_t *mask = nullptr;
    bool has_mask = false;
    float4 *plane = nullptr;
    float *score = nullptr;
    int8_t *best = nullptr;
    float *d0 = nullptr, *s0 = nullptr, *m1 = nullptr, *fdepth = nullptr, *fscore = nullptr;
    float *x_depth = nullptr, *x_score = nullptr, *x_plane3 = nullptr, *x_normal3 = nullptr;
    int32_t *x_best = nullptr;
    float4 *seed = nullptr;              // seeding candidates from a prior result
    unsigned long long *zbuf = nullptr;  // splat depth test of the prior warp
    const pm_request *prior = nullptr;   // result reused as initialisation (may be null)
    const pm_result *prior_res = nullptr;
    // requests whose prior is this one: unlinked when it is destroyed
    mutable std::vector<pm_request *> dependents;
    int2 *lm = nullptr;                  // landmark seeds (pixel index, depth bits), device
    int n_lm = 0, lm_cap = 0;
    double R[PM_MAX_SOURCES + 1][9] = {}, t[PM_MAX_SOURCES + 1][3] = {};
    bool have[PM_MAX_SOURCES + 1] = {};
    Trig trig;
    pm::SweepArgs args{};
    cudaStream_t stream = nullptr;  // the request's own stream: requests overlap on the device
    cudaEvent_t ready = nullptr;    // recorded on this stream for requests seeded from it
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    bool graph_dirty = true;
    bool postprocessed = false;
};

// A retained keyframe result (plane state + filtered depth + pose): the
// compact form in which results are kept for seeding later keyframes.
struct pm_result {
    pm_ctx *ctx = nullptr;
    int W = 0, H = 0;
    size_t bytes = 0;
    void *block = nullptr;
    float4 *plane = nullptr;
    float *fdepth = nullptr;
    double R[9] = {}, t[3] = {};
    Trig trig;
    cudaEvent_t ready = nullptr;  // recorded after the snapshot copies
    bool valid = false;
    // requests whose prior is this result: unlinked when it is destroyed
    mutable std::vector<pm_request *> dependents;
};

namespace pmi {

// Record the message of a failure on the context and return its status code.
inline int fail(pm_ctx *ctx, int code, const char *fmt, ...) {
    if (ctx) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        ctx->err = buf;
    }
    return code;
}

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Kernel arguments of a request from its views, poses and parameters.
PM_INTERNAL void fill_args(pm_request *r);
// PM_EINVAL unless every view of the request has been set.
PM_INTERNAL int check_views(pm_request *r);
// Enqueue the post-filter of a request on `st` (its own stream when null).
PM_INTERNAL int enqueue_post(pm_request *r, cudaStream_t st = nullptr);
// The band arguments of the request's tile order for one launch of `grid`
// on `st`, with the band counters reset there first; *out is null when the
// request runs one CTA per tile.
PM_INTERNAL int tile_band(pm_request *r, dim3 grid, cudaStream_t st, pm::BandArgs *band, const pm::BandArgs **out);
// Enqueue r's seeding on st: landmark seeds, then its prior request or
// retained result (the stage of pm_request_run between the init scoring and
// the sweeps).  in_batch: the prior is a request of the same batch whose
// post-filter is enqueued earlier on that batch's streams.
PM_INTERNAL int enqueue_seeding(pm_request *r, cudaStream_t st, bool in_batch);
// Order st after the work that produces r's prior (a request's stream up to
// now, or a retained result's snapshot).
PM_INTERNAL int wait_prior_ready(pm_request *r, cudaStream_t st);
// Replace the prior links of r (request or retained result, at most one set),
// keeping the priors' dependent lists in step.
PM_INTERNAL void link_prior(pm_request *r, const pm_request *prior, const pm_result *res);
// Unlink every dependent of a prior that is being destroyed, after the
// dependents' in-flight work (which may read the prior) has finished.
PM_INTERNAL void unlink_dependents(std::vector<pm_request *> &deps, bool from_request);

}  // namespace pmi

#define PM_CUDA(ctx, call)                                                                                   \
    do {                                                                                                     \
        cudaError_t e_ = (call);                                                                             \
        if (e_ != cudaSuccess) return pmi::fail((ctx), PM_ECUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)
