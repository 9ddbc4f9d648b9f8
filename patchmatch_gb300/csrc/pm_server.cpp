// Served densification: a request loop over the device-resident request API.
//
// Keyframes arrive through pm_server_submit (any thread).  A worker thread
// owns the CUDA context: it uploads each keyframe once into a device cache of
// resident images, chooses the nearest cached keyframes as sources, admits the
// keyframe when an in-flight slot and the HBM budget allow, seeds it from the
// newest finished result and runs it on its own stream, so keyframes that
// arrive while others are on the GPU overlap with them (continuous batching).
// pm_server_wait returns the maps and the submit-to-result latency.  With
// dense output on, finished keyframes also pass, in ticket order, through the
// reference's cleaner and pruner windows (consistency filter of the centre of
// five, fusion of the head of five cleaned maps) on the context stream;
// pm_server_wait_dense returns the fused depth and points.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include <cuda_runtime.h>

#include <nvtx3/nvToolsExt.h>

#include "pm_gb300.h"

namespace {

using Clock = std::chrono::steady_clock;

// Coarse-to-fine starts only for keyframes at least this wide: with 960 or
// more columns at half size the 11x11 window still resolves the scene
// (measured: same accuracy at 1920x960 in 0.55x the time, +6 points of
// pixels within 1 % at 3840x1920 in 0.53x; at 960x480 it loses 8 points).
constexpr int kCoarseMinWidth = 1920;

double ms_since(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Submission {
    uint64_t ticket;
    int W, H;
    std::vector<uint8_t> gray;
    double R[9], t[3];
    Clock::time_point t_submit;
    bool has_landmarks = false;
    std::vector<double> lm_xyz;     // n x 3 world points
    std::vector<uint64_t> lm_ids;
    bool gated = false;             // the view test has run (admission may be retried)
    float view_score = -1.0f;
};

// A device image buffer of the keyframe cache.  `uses` are events recorded
// after each copy out of it, so an evicted buffer is reused only once every
// copy has finished (no device-wide synchronisation).
struct ImageBuf {
    uint8_t *d = nullptr;
    size_t bytes = 0;
    std::vector<cudaEvent_t> uses;
};

struct CachedKeyframe {
    uint64_t ticket;
    int W, H;
    ImageBuf *img = nullptr;
    ImageBuf *half = nullptr;     // W/2 x H/2 copy for coarse-to-fine passes (or none)
    cudaEvent_t ready = nullptr;  // recorded on the context stream after the upload (and resize)
    double R[9], t[3], C[3];
};

// Idle requests by shape: pm_request_destroy frees device memory, which
// synchronises the whole device, so finished requests are kept and reused.
struct RequestPool {
    struct Idle {
        pm_request *req;
        int W, H, S;
    };
    std::vector<Idle> idle;
    pm_request *take(int W, int H, int S) {
        for (size_t q = 0; q < idle.size(); ++q)
            if (idle[q].W == W && idle[q].H == H && idle[q].S == S) {
                pm_request *r = idle[q].req;
                idle.erase(idle.begin() + q);
                return r;
            }
        return nullptr;
    }
    void give(pm_request *r, int W, int H, int S) { idle.push_back({r, W, H, S}); }
    // free one idle request (oldest first); false when none is left
    bool shrink() {
        if (idle.empty()) return false;
        pm_request_destroy(idle.front().req);
        idle.erase(idle.begin());
        return true;
    }
    ~RequestPool() {
        for (Idle &i : idle) pm_request_destroy(i.req);
    }
};

struct ResultPool;

// A retained result (plane state + filtered depth of one densified keyframe)
// usable as the prior of later keyframes.  Held by the server's prior table,
// by the job that writes it and by every job seeded from it; it returns to the
// pool only when all of them have let go, so a snapshot is never overwritten
// while a copy into it or a read out of it may still be in flight.
struct ResHolder {
    pm_result *res = nullptr;
    int W = 0, H = 0;
    ResultPool *pool = nullptr;
    ~ResHolder();
};

struct ResultPool {
    struct Idle {
        pm_result *res;
        int W, H;
    };
    std::vector<Idle> idle;
    pm_result *take(int W, int H) {
        for (size_t q = 0; q < idle.size(); ++q)
            if (idle[q].W == W && idle[q].H == H) {
                pm_result *r = idle[q].res;
                idle.erase(idle.begin() + q);
                return r;
            }
        return nullptr;
    }
    bool shrink() {
        if (idle.empty()) return false;
        pm_result_destroy(idle.front().res);
        idle.erase(idle.begin());
        return true;
    }
    ~ResultPool() {
        for (Idle &i : idle) pm_result_destroy(i.res);
    }
};

ResHolder::~ResHolder() {
    if (res && pool) pool->idle.push_back({res, W, H});
    else if (res) pm_result_destroy(res);
}

// Pinned host buffers by size (cudaMallocHost/cudaFreeHost synchronise).
struct PinnedPool {
    std::vector<std::pair<size_t, float *>> idle;
    float *take(size_t bytes) {
        for (size_t q = 0; q < idle.size(); ++q)
            if (idle[q].first == bytes) {
                float *p = idle[q].second;
                idle.erase(idle.begin() + q);
                return p;
            }
        float *p = nullptr;
        if (cudaMallocHost(&p, bytes) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        return p;
    }
    void give(size_t bytes, float *p) {
        if (p) idle.push_back({bytes, p});
    }
    ~PinnedPool() {
        for (auto &i : idle) cudaFreeHost(i.second);
    }
};

struct Job {
    uint64_t ticket;
    pm_request *req = nullptr;
    pm_request *coarse = nullptr;  // half-resolution pass of a coarse-to-fine keyframe
    std::shared_ptr<ResHolder> out, prior;
    float *h_depth = nullptr, *h_score = nullptr;  // pinned
    int W, H, S, iterations;
    int seeded;  // 1: from an earlier keyframe's result, 2: from its own half-resolution pass
    float view_score = -1.0f;
    double R[9], t[3];
    Clock::time_point t_submit, t_start;
};

struct Result {
    int status = PM_OK;
    std::vector<float> depth, score;
    pm_served_info info{};
};

// ---- dense output: the reference's cleaner and pruner windows ----
// A densified keyframe in a filter window (its retained result holds the
// filtered depth on the device).
struct DenseView {
    uint64_t ticket = 0;
    std::shared_ptr<ResHolder> res;
    double R[9], t[3];
    bool cleaned = false;  // has been the centre of a filter window
};
// A cleaned map in a fusion window (device, W*H floats, pooled).
struct CleanedView {
    uint64_t ticket = 0;
    float *d = nullptr;
    double R[9], t[3];
};
// The one fusion of an image size in flight: device outputs, pinned copies,
// and the stage of its device->host copies.
struct FuseSlot {
    bool alloc = false;
    void *ws = nullptr;
    size_t ws_bytes = 0;
    float *pruned = nullptr, *xyz = nullptr;
    int32_t *ij = nullptr;
    unsigned *count = nullptr;
    float *h_pruned = nullptr, *h_xyz = nullptr;
    int32_t *h_ij = nullptr;
    unsigned *h_count = nullptr;
    cudaEvent_t ev = nullptr;
    int stage = 0;  // 0 idle, 1 point count on its way to the host, 2 maps and points on their way
    unsigned n = 0;
};
struct SizeWindows {
    int W = 0, H = 0;
    std::deque<DenseView> clean;
    std::deque<CleanedView> fuse;
    std::vector<float *> free_maps;
    FuseSlot slot;
};
// Retained results leaving a filter window stay held until the filter
// launches that read them have run.
struct Retiring {
    cudaEvent_t ev;
    std::shared_ptr<ResHolder> res;
};
struct DenseResult {
    int status = PM_OK;
    std::vector<float> depth, xyz;
    std::vector<int32_t> ij;
};

}  // namespace

struct pm_server {
    pm_ctx *ctx = nullptr;
    pm_server_config cfg{};
    ResultPool respool;  // declared before rpool and priors: destroyed after them
    RequestPool rpool;
    PinnedPool hpool;
    std::vector<ImageBuf *> retired;   // evicted cache buffers awaiting reuse
    std::vector<cudaEvent_t> event_pool;
    std::thread worker;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    bool stop = false;       // destroy: queued keyframes are cancelled
    bool finishing = false;  // pm_server_finish: no more submissions, queued keyframes still run
    bool finished = false;   // the worker has completed every result and exited
    uint64_t next_ticket = 1;
    std::deque<Submission> pending;
    std::deque<CachedKeyframe> cache;
    std::vector<Job> inflight;
    // retained results of started keyframes (ticket -> snapshot); the prior
    // of keyframe k is the newest entry with ticket <= k - prior_lag, so it
    // never depends on timing.  Pruned to what a later keyframe can still use.
    std::map<uint64_t, std::shared_ptr<ResHolder>> priors;
    std::unordered_map<uint64_t, Result> done;
    std::unordered_set<uint64_t> outstanding;  // issued and not yet collected by pm_server_wait
    int waiters = 0;                           // threads inside pm_server_wait / pm_server_wait_dense
    // dense output, results (under mu)
    std::unordered_map<uint64_t, DenseResult> dense_done;
    std::unordered_set<uint64_t> dense_outstanding;
    // dense output, pipeline (worker thread only)
    std::map<uint64_t, int> dense_status;        // decided tickets without a densified result
    std::map<uint64_t, DenseView> dense_ready;   // densified, waiting for earlier tickets
    uint64_t dense_cursor = 1;                   // next ticket to enter the windows
    std::vector<std::unique_ptr<SizeWindows>> windows;
    std::vector<Retiring> retiring;
    // the view test (worker thread only): the previous joined keyframe with landmarks
    bool have_prev_view = false;
    double prev_C[3] = {};
    std::vector<uint64_t> prev_ids;
};

namespace {

cudaEvent_t get_event(pm_server *s) {
    if (!s->event_pool.empty()) {
        cudaEvent_t e = s->event_pool.back();
        s->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return e;
}

bool buffer_idle(pm_server *s, ImageBuf *b) {
    for (cudaEvent_t e : b->uses)
        if (cudaEventQuery(e) != cudaSuccess) return false;
    for (cudaEvent_t e : b->uses) s->event_pool.push_back(e);
    b->uses.clear();
    return true;
}

ImageBuf *get_image_buffer(pm_server *s, size_t bytes) {
    for (size_t q = 0; q < s->retired.size(); ++q)
        if (s->retired[q]->bytes == bytes && buffer_idle(s, s->retired[q])) {
            ImageBuf *b = s->retired[q];
            s->retired.erase(s->retired.begin() + q);
            return b;
        }
    ImageBuf *b = new ImageBuf();
    if (cudaMalloc(&b->d, bytes) != cudaSuccess) {
        cudaGetLastError();
        delete b;
        return nullptr;
    }
    b->bytes = bytes;
    return b;
}

void cache_retire(pm_server *s, CachedKeyframe &k) {
    s->retired.push_back(k.img);
    if (k.half) s->retired.push_back(k.half);
    if (k.ready) s->event_pool.push_back(k.ready);
    k.img = k.half = nullptr;
    k.ready = nullptr;
}

// Upload a submission into the resident cache (retiring the oldest entry) on
// the context stream, with its half-resolution copy when coarse-to-fine is on;
// requests wait for `ready` before reading the images.
int cache_insert(pm_server *s, Submission &sub, CachedKeyframe **out) {
    if ((int)s->cache.size() >= s->cfg.cache_capacity) {
        cache_retire(s, s->cache.front());
        s->cache.pop_front();
    }
    CachedKeyframe k;
    k.ticket = sub.ticket;
    k.W = sub.W;
    k.H = sub.H;
    std::memcpy(k.R, sub.R, sizeof k.R);
    std::memcpy(k.t, sub.t, sizeof k.t);
    for (int a = 0; a < 3; ++a) k.C[a] = -(k.R[a] * k.t[0] + k.R[3 + a] * k.t[1] + k.R[6 + a] * k.t[2]);
    const size_t n = (size_t)k.W * k.H;
    cudaStream_t cs = (cudaStream_t)pm_stream(s->ctx);
    k.img = get_image_buffer(s, n);
    if (!k.img) return PM_ENOMEM;
    // pageable source: staged before the call returns, so `sub` may go away
    if (cudaMemcpyAsync(k.img->d, sub.gray.data(), n, cudaMemcpyHostToDevice, cs) != cudaSuccess) {
        cudaGetLastError();
        cache_retire(s, k);
        return PM_ECUDA;
    }
    if (s->cfg.coarse_to_fine && k.W % 2 == 0 && k.H % 2 == 0 && k.W >= kCoarseMinWidth) {
        k.half = get_image_buffer(s, n / 4);
        if (!k.half) {
            cache_retire(s, k);
            return PM_ENOMEM;
        }
        const int rc = pm_image_resize(s->ctx, k.img->d, k.W, k.H, k.W, 1, k.half->d, k.W / 2, k.H / 2, k.W / 2);
        if (rc) {
            cache_retire(s, k);
            return rc;
        }
    }
    k.ready = get_event(s);
    if (!k.ready || cudaEventRecord(k.ready, cs) != cudaSuccess) {
        cudaGetLastError();
        cache_retire(s, k);
        return PM_ECUDA;
    }
    s->cache.push_back(k);
    *out = &s->cache.back();
    return PM_OK;
}

// Neighbours: cached keyframes with a camera baseline in [min, max] metres,
// nearest first (equirectangular views overlap most when their centres are
// close), at most max_sources.
std::vector<const CachedKeyframe *> select_sources(const pm_server *s, const CachedKeyframe &ref) {
    std::vector<std::pair<double, const CachedKeyframe *>> c;
    for (const CachedKeyframe &k : s->cache) {
        if (k.ticket == ref.ticket || k.W != ref.W || k.H != ref.H) continue;  // one resolution per request
        const double dx = k.C[0] - ref.C[0], dy = k.C[1] - ref.C[1], dz = k.C[2] - ref.C[2];
        const double d = std::sqrt(dx * dx + dy * dy + dz * dz);
        if (d >= s->cfg.min_baseline && d <= s->cfg.max_baseline) c.push_back({d, &k});
    }
    std::sort(c.begin(), c.end(), [](const auto &a, const auto &b) { return a.first < b.first; });
    std::vector<const CachedKeyframe *> out;
    for (size_t q = 0; q < c.size() && (int)out.size() < s->cfg.max_sources; ++q) out.push_back(c[q].second);
    return out;
}

void finish_dense(pm_server *s, uint64_t ticket, DenseResult &&r) {
    std::lock_guard<std::mutex> lk(s->mu);
    s->dense_done[ticket] = std::move(r);
    s->cv_done.notify_all();
}

void finish(pm_server *s, uint64_t ticket, Result &&r) {
    // a keyframe that ends without a densified result never enters the windows
    if (s->cfg.dense_output && r.status != PM_OK) s->dense_status[ticket] = r.status;
    std::lock_guard<std::mutex> lk(s->mu);
    s->done[ticket] = std::move(r);
    s->cv_done.notify_all();
}

// Free idle pooled memory until `create` stops failing for lack of it.
template <class F>
int create_with_room(pm_server *s, F create) {
    int rc = create();
    while ((rc == PM_EBUDGET || rc == PM_ENOMEM) && (s->rpool.shrink() || s->respool.shrink())) rc = create();
    return rc;
}

// The prior of keyframe `ticket`: the newest retained result of the same
// size with ticket <= ticket - prior_lag (a function of the ticket order only).
std::shared_ptr<ResHolder> find_prior(const pm_server *s, uint64_t ticket, int W, int H) {
    const uint64_t lag = (uint64_t)s->cfg.prior_lag;
    if (ticket <= lag) return nullptr;
    for (auto it = s->priors.upper_bound(ticket - lag); it != s->priors.begin();) {
        --it;
        if (it->second->W == W && it->second->H == H) return it->second;
    }
    return nullptr;
}

// Drop retained results that no keyframe from `next` on can select: for each
// size, everything older than the newest entry with ticket <= next - prior_lag.
void prune_priors(pm_server *s, uint64_t next) {
    const uint64_t lag = (uint64_t)s->cfg.prior_lag;
    if (next <= lag) return;
    std::vector<std::pair<int, int>> kept;  // sizes whose newest usable entry was seen
    auto it = s->priors.upper_bound(next - lag);
    while (it != s->priors.begin()) {
        --it;
        const std::pair<int, int> wh{it->second->W, it->second->H};
        if (std::find(kept.begin(), kept.end(), wh) == kept.end()) {
            kept.push_back(wh);
        } else {
            it = s->priors.erase(it);
        }
    }
}

// Start one submission on the GPU; returns PM_EBUDGET when it must wait.
int start_job(pm_server *s, Submission &sub, CachedKeyframe *kf) {
    nvtxRangePushA("served keyframe start");
    struct Pop {
        ~Pop() { nvtxRangePop(); }
    } pop;
    std::vector<const CachedKeyframe *> src = select_sources(s, *kf);
    if ((int)src.size() < s->cfg.min_sources) {
        Result r;
        r.status = PM_ENOTREADY;  // not enough neighbours yet (the first keyframes of a stream)
        r.info.status = PM_ENOTREADY;
        r.info.view_score = sub.view_score;
        r.info.latency_ms = ms_since(sub.t_submit, Clock::now());
        finish(s, sub.ticket, std::move(r));
        return PM_OK;
    }
    const int S = (int)src.size();
    pm_params p = s->cfg.params;
    p.keyframe_id = (uint32_t)sub.ticket;
    std::shared_ptr<ResHolder> prior;
    if (s->cfg.seed_from_prior) prior = find_prior(s, sub.ticket, sub.W, sub.H);
    // without a prior, a keyframe whose images all have half-resolution copies
    // is densified coarse to fine: full sweeps at half resolution, then the
    // seeded sweep count at full resolution, seeded from the half-size result
    bool c2f = !prior && s->cfg.coarse_to_fine && kf->half;
    for (const CachedKeyframe *c : src) c2f = c2f && c->half;
    p.iterations = (prior || c2f) ? s->cfg.seeded_iterations : s->cfg.params.iterations;
    const int n_lm = sub.has_landmarks ? (int)sub.lm_ids.size() : 0;
    if (n_lm > 0) {
        // depth interval from the landmarks (compute_depth_intervall): its upper bound
        double p10 = 0, p90 = 0, dmin = 0, dmax = 0;
        if (pm_depth_interval(sub.R, sub.t, sub.lm_xyz.data(), n_lm, &p10, &p90, &dmin, &dmax) == PM_OK &&
            dmax > p.min_depth)
            p.max_depth = (float)dmax;
    }
    // the snapshot this keyframe leaves for later ones, then the request
    pm_result *res = s->respool.take(sub.W, sub.H);
    int rc = PM_OK;
    if (!res) rc = create_with_room(s, [&] { return pm_result_create(s->ctx, sub.W, sub.H, &res); });
    if (rc == PM_EBUDGET || rc == PM_ENOMEM) return PM_EBUDGET;
    if (rc) return rc;
    auto out = std::make_shared<ResHolder>();
    out->res = res;
    out->W = sub.W;
    out->H = sub.H;
    out->pool = &s->respool;
    // pooled or new requests: the coarse pass (if any), then the keyframe's own
    auto take_request = [&](int W, int H, const pm_params &pp, pm_request **out) {
        *out = s->rpool.take(W, H, S);
        if (*out) return pm_request_set_params(*out, &pp);
        const int c = create_with_room(s, [&] { return pm_request_create(s->ctx, W, H, S, &pp, out); });
        return (c == PM_EBUDGET || c == PM_ENOMEM) ? PM_EBUDGET : c;
    };
    pm_request *coarse = nullptr;
    pm_params pc = p;
    if (c2f) {
        pc.iterations = s->cfg.params.iterations;
        pc.postprocess = 1;  // the full-resolution pass seeds from the filtered half-size depth
        rc = take_request(sub.W / 2, sub.H / 2, pc, &coarse);
        if (rc) return rc;
    }
    pm_request *req = nullptr;
    rc = take_request(sub.W, sub.H, p, &req);
    if (rc) {
        if (coarse) s->rpool.give(coarse, sub.W / 2, sub.H / 2, S);
        return rc;
    }
    // the views (full size or their half-size copies), after their upload
    auto set_views = [&](pm_request *r, bool half) {
        cudaStream_t rs = (cudaStream_t)pm_request_stream(r);
        for (int k = 0; k <= S; ++k) {
            const CachedKeyframe *c = k == 0 ? kf : src[k - 1];
            ImageBuf *b = half ? c->half : c->img;
            if (cudaStreamWaitEvent(rs, c->ready, 0) != cudaSuccess) {
                cudaGetLastError();
                return PM_ECUDA;
            }
            pm_view v{};
            v.gray = b->d;
            std::memcpy(v.R_cw, c->R, sizeof v.R_cw);
            std::memcpy(v.t_cw, c->t, sizeof v.t_cw);
            const int e = pm_request_set_view(r, k, &v);
            if (e) return e;
            // the buffer is reused only after this event: a use that cannot be
            // recorded fails the keyframe (its request is synchronised then)
            cudaEvent_t u = get_event(s);
            if (!u || cudaEventRecord(u, rs) != cudaSuccess) {
                cudaGetLastError();
                if (u) s->event_pool.push_back(u);
                return PM_ECUDA;
            }
            b->uses.push_back(u);
        }
        return PM_OK;
    };
    if (coarse) {
        rc = set_views(coarse, true);
        if (!rc) rc = pm_request_set_prior(coarse, nullptr);
        if (!rc) rc = pm_request_run(coarse);
    }
    if (!rc) rc = set_views(req, false);
    // landmark seeds are applied after the random initialisation, before the prior
    if (!rc) rc = pm_request_set_landmarks(req, n_lm > 0 ? sub.lm_xyz.data() : nullptr, n_lm);
    if (!rc) rc = coarse ? pm_request_set_prior(req, coarse) : pm_request_set_prior_result(req, prior ? prior->res : nullptr);
    if (!rc) rc = pm_request_run(req);
    if (!rc) rc = pm_result_snapshot(res, req);
    Job j;
    j.ticket = sub.ticket;
    j.req = req;
    j.coarse = coarse;
    j.out = out;
    j.prior = prior;
    j.W = sub.W;
    j.H = sub.H;
    j.S = S;
    j.iterations = p.iterations;
    j.seeded = prior ? 1 : (coarse ? 2 : 0);
    j.view_score = sub.view_score;
    std::memcpy(j.R, sub.R, sizeof j.R);
    std::memcpy(j.t, sub.t, sizeof j.t);
    j.t_submit = sub.t_submit;
    j.t_start = Clock::now();
    const size_t n = (size_t)sub.W * sub.H;
    if (!rc) {
        j.h_depth = s->hpool.take(n * 4);
        j.h_score = s->hpool.take(n * 4);
        if (!j.h_depth || !j.h_score) rc = PM_ENOMEM;
    }
    if (!rc) {
        pm_maps m{j.h_depth, j.h_score, nullptr, nullptr, nullptr};
        rc = pm_request_read_async(req, &m, 0);
    }
    if (rc) {
        // nothing was left in flight that reads these buffers past the stream
        pm_request_synchronize(req);
        if (coarse) {
            pm_request_synchronize(coarse);
            s->rpool.give(coarse, sub.W / 2, sub.H / 2, S);
        }
        s->rpool.give(req, sub.W, sub.H, S);
        s->hpool.give(n * 4, j.h_depth);
        s->hpool.give(n * 4, j.h_score);
        Result r;
        r.status = rc;
        r.info.status = rc;
        r.info.view_score = sub.view_score;
        finish(s, sub.ticket, std::move(r));
        return PM_OK;
    }
    s->priors[sub.ticket] = out;
    prune_priors(s, sub.ticket + 1);
    s->inflight.push_back(std::move(j));
    return PM_OK;
}

void poll_inflight(pm_server *s) {
    for (size_t q = 0; q < s->inflight.size();) {
        Job &j = s->inflight[q];
        const int rc = pm_request_query(j.req);
        if (rc == PM_ENOTREADY) {
            ++q;
            continue;
        }
        const auto now = Clock::now();
        Result r;
        r.status = rc;
        r.info.status = rc;
        r.info.n_sources = j.S;
        r.info.seeded = j.seeded;
        r.info.iterations = j.iterations;
        r.info.queue_ms = ms_since(j.t_submit, j.t_start);
        r.info.latency_ms = ms_since(j.t_submit, now);
        r.info.view_score = j.view_score;
        if (rc == PM_OK) {
            const size_t n = (size_t)j.W * j.H;
            r.depth.assign(j.h_depth, j.h_depth + n);
            r.score.assign(j.h_score, j.h_score + n);
            if (s->cfg.dense_output) {
                DenseView v;
                v.ticket = j.ticket;
                v.res = j.out;  // complete: the snapshot ran on the finished request's stream
                std::memcpy(v.R, j.R, sizeof v.R);
                std::memcpy(v.t, j.t, sizeof v.t);
                s->dense_ready[j.ticket] = std::move(v);
            }
        } else {
            s->priors.erase(j.ticket);
        }
        s->hpool.give((size_t)j.W * j.H * 4, j.h_depth);
        s->hpool.give((size_t)j.W * j.H * 4, j.h_score);
        s->rpool.give(j.req, j.W, j.H, j.S);  // reusable at once: later keyframes seed from the snapshot
        if (j.coarse) s->rpool.give(j.coarse, j.W / 2, j.H / 2, j.S);  // finished before j.req
        const uint64_t t = j.ticket;
        s->inflight.erase(s->inflight.begin() + q);
        finish(s, t, std::move(r));
    }
}

// ---- dense output pipeline (worker thread) ----

SizeWindows *windows_for(pm_server *s, int W, int H) {
    for (auto &w : s->windows)
        if (w->W == W && w->H == H) return w.get();
    s->windows.push_back(std::make_unique<SizeWindows>());
    s->windows.back()->W = W;
    s->windows.back()->H = H;
    return s->windows.back().get();
}

float *take_map(SizeWindows &w) {
    if (!w.free_maps.empty()) {
        float *d = w.free_maps.back();
        w.free_maps.pop_back();
        return d;
    }
    float *d = nullptr;
    if (cudaMalloc(&d, (size_t)w.W * w.H * sizeof(float)) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return d;
}

int slot_alloc(SizeWindows &w) {
    FuseSlot &sl = w.slot;
    if (sl.alloc) return PM_OK;
    const size_t N = (size_t)w.W * w.H;
    sl.ws_bytes = pm_fuse_workspace_bytes(w.W, w.H);
    bool ok = cudaMalloc(&sl.ws, sl.ws_bytes) == cudaSuccess && cudaMalloc(&sl.pruned, N * 4) == cudaSuccess &&
              cudaMalloc(&sl.xyz, N * 12) == cudaSuccess && cudaMalloc(&sl.ij, N * 8) == cudaSuccess &&
              cudaMalloc(&sl.count, 4) == cudaSuccess && cudaMallocHost(&sl.h_pruned, N * 4) == cudaSuccess &&
              cudaMallocHost(&sl.h_xyz, N * 12) == cudaSuccess && cudaMallocHost(&sl.h_ij, N * 8) == cudaSuccess &&
              cudaMallocHost(&sl.h_count, 4) == cudaSuccess &&
              cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming) == cudaSuccess;
    sl.alloc = true;  // partial allocations are released with the slot
    if (!ok) cudaGetLastError();
    return ok ? PM_OK : PM_ENOMEM;
}

void slot_free(FuseSlot &sl) {
    cudaFree(sl.ws);
    cudaFree(sl.pruned);
    cudaFree(sl.xyz);
    cudaFree(sl.ij);
    cudaFree(sl.count);
    cudaFreeHost(sl.h_pruned);
    cudaFreeHost(sl.h_xyz);
    cudaFreeHost(sl.h_ij);
    cudaFreeHost(sl.h_count);
    if (sl.ev) cudaEventDestroy(sl.ev);
    sl = FuseSlot{};
}

DenseResult dense_status_result(int status) {
    DenseResult r;
    r.status = status;
    return r;
}

// Tickets enter the windows in ticket order; a keyframe without a densified
// result (too few neighbours, rejected view, cancelled, failed) completes its
// dense output with that status at its turn.
void dense_feed(pm_server *s) {
    for (;;) {
        const uint64_t t = s->dense_cursor;
        auto ir = s->dense_ready.find(t);
        if (ir != s->dense_ready.end()) {
            SizeWindows *w = windows_for(s, ir->second.res->W, ir->second.res->H);
            w->clean.push_back(std::move(ir->second));
            s->dense_ready.erase(ir);
            ++s->dense_cursor;
            continue;
        }
        auto is = s->dense_status.find(t);
        if (is != s->dense_status.end()) {
            finish_dense(s, t, dense_status_result(is->second));
            s->dense_status.erase(is);
            ++s->dense_cursor;
            continue;
        }
        return;
    }
}

// Release retained results whose last filter launch has run.
void dense_retire(pm_server *s, bool wait) {
    for (size_t q = 0; q < s->retiring.size();) {
        if (wait) cudaEventSynchronize(s->retiring[q].ev);
        if (cudaEventQuery(s->retiring[q].ev) == cudaSuccess) {
            s->event_pool.push_back(s->retiring[q].ev);
            s->retiring.erase(s->retiring.begin() + q);
        } else {
            cudaGetLastError();
            ++q;
        }
    }
}

// Consistency filter of every full window's centre (DepthmapCleaner::Clean
// over five maps, depthmap.cc:1320-1377, then PopHeadUnlessOne), and the
// fusion of the head of five cleaned maps (DepthmapPruner::Prune,
// depthmap.cc:1535-1696, then PopHead), all on the context stream.
void dense_step(pm_server *s) {
    const pm_server_config &c = s->cfg;
    for (auto &wp : s->windows) {
        SizeWindows &w = *wp;
        const size_t N = (size_t)w.W * w.H;
        while (w.clean.size() >= 5) {
            const float *ptrs[5];
            double R[45], t[15];
            for (int q = 0; q < 5; ++q) {
                ptrs[q] = pm_result_depth_device(w.clean[q].res->res);
                std::memcpy(R + 9 * q, w.clean[q].R, sizeof(double) * 9);
                std::memcpy(t + 3 * q, w.clean[q].t, sizeof(double) * 3);
            }
            DenseView &centre = w.clean[2];
            float *out = take_map(w);
            int rc = out ? pm_filter_consistency_device(s->ctx, w.W, w.H, 5, ptrs, R, t, 2, c.clean_threshold,
                                                        c.clean_min_views, c.clean_reproj_px, out, nullptr)
                         : PM_ENOMEM;
            centre.cleaned = true;
            if (rc) {
                if (out) w.free_maps.push_back(out);
                finish_dense(s, centre.ticket, dense_status_result(rc));
            } else {
                CleanedView cv;
                cv.ticket = centre.ticket;
                cv.d = out;
                std::memcpy(cv.R, centre.R, sizeof cv.R);
                std::memcpy(cv.t, centre.t, sizeof cv.t);
                w.fuse.push_back(cv);
            }
            DenseView head = std::move(w.clean.front());
            w.clean.pop_front();
            if (!head.cleaned) finish_dense(s, head.ticket, dense_status_result(PM_ENOTREADY));
            cudaEvent_t e = get_event(s);
            if (e && cudaEventRecord(e, (cudaStream_t)pm_stream(s->ctx)) == cudaSuccess) {
                s->retiring.push_back({e, std::move(head.res)});
            } else {  // cannot tell when the launch has run: wait for it
                cudaGetLastError();
                cudaStreamSynchronize((cudaStream_t)pm_stream(s->ctx));
                if (e) s->event_pool.push_back(e);
            }
        }
        FuseSlot &sl = w.slot;
        if (sl.stage == 1 && cudaEventQuery(sl.ev) == cudaSuccess) {
            sl.n = *sl.h_count;
            const size_t m = std::min<size_t>(sl.n, N);
            cudaStream_t cs = (cudaStream_t)pm_stream(s->ctx);
            bool ok = cudaMemcpyAsync(sl.h_pruned, sl.pruned, N * 4, cudaMemcpyDeviceToHost, cs) == cudaSuccess &&
                      cudaMemcpyAsync(sl.h_xyz, sl.xyz, m * 12, cudaMemcpyDeviceToHost, cs) == cudaSuccess &&
                      cudaMemcpyAsync(sl.h_ij, sl.ij, m * 8, cudaMemcpyDeviceToHost, cs) == cudaSuccess &&
                      cudaEventRecord(sl.ev, cs) == cudaSuccess;
            if (!ok) {
                cudaGetLastError();
                cudaStreamSynchronize(cs);
            }
            sl.stage = 2;
        }
        if (sl.stage == 2 && cudaEventQuery(sl.ev) == cudaSuccess) {
            CleanedView head = w.fuse.front();
            w.fuse.pop_front();
            DenseResult r;
            const size_t m = std::min<size_t>(sl.n, N);
            r.depth.assign(sl.h_pruned, sl.h_pruned + N);
            r.xyz.assign(sl.h_xyz, sl.h_xyz + m * 3);
            r.ij.assign(sl.h_ij, sl.h_ij + m * 2);
            finish_dense(s, head.ticket, std::move(r));
            w.free_maps.push_back(head.d);  // every launch that used it has run
            sl.stage = 0;
        }
        if (sl.stage == 0 && w.fuse.size() >= 5) {
            float *ptrs[5];
            double R[45], t[15];
            for (int q = 0; q < 5; ++q) {
                ptrs[q] = w.fuse[q].d;
                std::memcpy(R + 9 * q, w.fuse[q].R, sizeof(double) * 9);
                std::memcpy(t + 3 * q, w.fuse[q].t, sizeof(double) * 3);
            }
            int rc = slot_alloc(w);
            cudaStream_t cs = (cudaStream_t)pm_stream(s->ctx);
            if (!rc)
                rc = pm_fuse_device(s->ctx, w.W, w.H, 5, ptrs, R, t, nullptr, c.fuse_threshold, sl.pruned, sl.xyz,
                                    nullptr, sl.ij, sl.count, sl.ws, sl.ws_bytes, nullptr);
            if (!rc && (cudaMemcpyAsync(sl.h_count, sl.count, 4, cudaMemcpyDeviceToHost, cs) != cudaSuccess ||
                        cudaEventRecord(sl.ev, cs) != cudaSuccess)) {
                cudaGetLastError();
                rc = PM_ECUDA;
            }
            if (rc) {
                cudaStreamSynchronize(cs);
                CleanedView head = w.fuse.front();
                w.fuse.pop_front();
                w.free_maps.push_back(head.d);
                finish_dense(s, head.ticket, dense_status_result(rc));
            } else {
                sl.stage = 1;
            }
        }
    }
    dense_retire(s, false);
}

// Allocate an image size's filter and fusion buffers when its first keyframe
// is admitted: device and pinned allocations synchronise the device, which
// would stall keyframes in flight if it happened later in the stream.  A
// window holds five cleaned maps; one more is produced while the head's
// fusion results travel to the host, and one is being cleaned.
constexpr int kDenseMaps = 8;
void dense_prepare(pm_server *s, int W, int H) {
    if (!s->cfg.dense_output) return;
    for (auto &w : s->windows)
        if (w->W == W && w->H == H) return;
    SizeWindows *w = windows_for(s, W, H);
    slot_alloc(*w);  // a failure shows again at the first fusion
    for (int k = 0; k < kDenseMaps; ++k) {
        float *d = nullptr;
        if (cudaMalloc(&d, (size_t)W * H * sizeof(float)) != cudaSuccess) {
            cudaGetLastError();
            break;  // take_map allocates later, as needed
        }
        w->free_maps.push_back(d);
    }
}

bool dense_busy(const pm_server *s) {
    for (const auto &w : s->windows)
        if (w->slot.stage != 0) return true;
    return false;
}

// End of stream: keyframes whose windows never filled complete with
// PM_ENOTREADY (the reference never cleans or fuses them either).
void dense_close(pm_server *s) {
    cudaStreamSynchronize((cudaStream_t)pm_stream(s->ctx));
    for (auto &wp : s->windows) {
        SizeWindows &w = *wp;
        for (DenseView &v : w.clean)
            if (!v.cleaned) finish_dense(s, v.ticket, dense_status_result(PM_ENOTREADY));
        w.clean.clear();
        for (CleanedView &v : w.fuse) {
            finish_dense(s, v.ticket, dense_status_result(PM_ENOTREADY));
            w.free_maps.push_back(v.d);
        }
        w.fuse.clear();
        for (float *d : w.free_maps) cudaFree(d);
        w.free_maps.clear();
        slot_free(w.slot);
    }
    s->windows.clear();
    dense_retire(s, true);
}

// The reference's view test for a keyframe with landmarks: it joins when
// score_view against the previous joined keyframe exceeds min_view_score
// (depthmap_computation_module.cc:330-340).  Returns false when it is dropped.
bool view_test(pm_server *s, Submission &sub) {
    if (sub.gated || !sub.has_landmarks) return true;
    sub.gated = true;
    double C[3];
    for (int a = 0; a < 3; ++a) C[a] = -(sub.R[a] * sub.t[0] + sub.R[3 + a] * sub.t[1] + sub.R[6 + a] * sub.t[2]);
    if (s->have_prev_view) {
        float score = 0.0f;
        int n_common = 0;
        if (pm_score_view(s->prev_C, C, s->prev_ids.data(), (int)s->prev_ids.size(), sub.lm_ids.data(),
                          sub.lm_xyz.data(), (int)sub.lm_ids.size(), &score, &n_common) != PM_OK)
            score = 0.0f;
        sub.view_score = score;
        if (!(score > s->cfg.min_view_score)) return false;
    }
    s->have_prev_view = true;
    std::memcpy(s->prev_C, C, sizeof C);
    s->prev_ids = sub.lm_ids;
    return true;
}

void worker_main(pm_server *s) {
    std::deque<Submission> waiting;  // dequeued, waiting for a slot / memory (submission order)
    for (;;) {
        bool stopping = false;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            const bool idle = s->pending.empty() && waiting.empty() && s->inflight.empty() && !dense_busy(s);
            if ((s->stop || s->finishing) && idle) break;
            if (idle) s->cv_work.wait_for(lk, std::chrono::milliseconds(50));
            while (!s->pending.empty()) {
                waiting.push_back(std::move(s->pending.front()));
                s->pending.pop_front();
            }
            stopping = s->stop;
        }
        if (stopping) {
            // destroy: keyframes not yet on the GPU are cancelled
            for (Submission &sub : waiting) {
                Result r;
                r.status = r.info.status = PM_ECANCELLED;
                finish(s, sub.ticket, std::move(r));
            }
            waiting.clear();
        }
        poll_inflight(s);
        if (s->cfg.dense_output) {
            dense_feed(s);
            dense_step(s);
        }
        while (!waiting.empty() && (int)s->inflight.size() < s->cfg.max_inflight) {
            Submission &sub = waiting.front();
            if (!view_test(s, sub)) {
                // not enough stereo baseline to the previous keyframe: dropped
                Result r;
                r.status = r.info.status = PM_ENOTREADY;
                r.info.view_score = sub.view_score;
                r.info.latency_ms = ms_since(sub.t_submit, Clock::now());
                finish(s, sub.ticket, std::move(r));
                waiting.pop_front();
                continue;
            }
            // admission happens in submission order, so the cache holds exactly
            // the keyframes before this one: neighbours never depend on timing
            dense_prepare(s, sub.W, sub.H);
            CachedKeyframe *kf = nullptr;
            int rc = cache_insert(s, sub, &kf);
            if (!rc) {
                rc = start_job(s, sub, kf);
                if (rc == PM_EBUDGET && !s->inflight.empty()) {
                    // wait for memory; undo the cache insertion so the retry is identical
                    cache_retire(s, s->cache.back());
                    s->cache.pop_back();
                    break;
                }
            }
            if (rc) {
                Result r;
                r.status = r.info.status = rc;
                r.info.view_score = sub.view_score;
                finish(s, sub.ticket, std::move(r));
            }
            waiting.pop_front();
        }
        if (!s->inflight.empty() || dense_busy(s))
            std::this_thread::sleep_for(std::chrono::microseconds(s->cfg.poll_us));
    }
    if (s->cfg.dense_output) {
        dense_feed(s);
        dense_close(s);
    }
    std::lock_guard<std::mutex> lk(s->mu);
    s->finished = true;
    s->cv_done.notify_all();
}

}  // namespace

extern "C" {

void pm_server_config_default(pm_server_config *c) {
    if (!c) return;
    std::memset(c, 0, sizeof *c);
    pm_params_default(&c->params);
    c->cache_capacity = 40;
    c->max_inflight = 4;
    c->min_sources = 4;
    c->max_sources = 8;
    c->min_baseline = 0.05f;
    c->max_baseline = 3.0f;
    c->seed_from_prior = 1;
    c->seeded_iterations = 2;
    c->prior_lag = 4;
    c->poll_us = 100;
    c->coarse_to_fine = 1;
    c->dense_output = 0;
    c->clean_threshold = 0.01f;
    c->clean_min_views = 3;
    c->clean_reproj_px = 1.0f;
    c->fuse_threshold = 0.08f;
    c->min_view_score = 0.25f;
}

int pm_server_create(pm_ctx *ctx, const pm_server_config *cfg, pm_server **out) {
    if (!ctx || !cfg || !out) return PM_EINVAL;
    if (cfg->cache_capacity < 2 || cfg->max_inflight < 1 || cfg->min_sources < 1 ||
        cfg->max_sources > PM_MAX_SOURCES || cfg->min_sources > cfg->max_sources || cfg->seeded_iterations < 0 ||
        !(cfg->max_baseline > cfg->min_baseline) || cfg->poll_us < 0 || cfg->prior_lag < 1)
        return PM_EINVAL;
    if (cfg->dense_output && (!(cfg->clean_threshold > 0.0f) || cfg->clean_min_views < 1 ||
                              cfg->clean_min_views > 5 || !(cfg->clean_reproj_px >= 0.0f) ||
                              !(cfg->fuse_threshold > 0.0f)))
        return PM_EINVAL;
    if (!std::isfinite(cfg->min_view_score)) return PM_EINVAL;
    pm_server *s = new pm_server();
    s->ctx = ctx;
    s->cfg = *cfg;
    s->worker = std::thread(worker_main, s);
    *out = s;
    return PM_OK;
}

namespace {
int submit(pm_server *s, int W, int H, const pm_view *view, const double *xyz, const uint64_t *ids, int n_lm,
           bool with_landmarks, uint64_t *ticket) {
    if (!s || !view || !view->gray || !ticket || W < 16 || H < 16) return PM_EINVAL;
    if (with_landmarks && (n_lm < 0 || (n_lm > 0 && (!xyz || !ids)))) return PM_EINVAL;
    for (int k = 0; k < 3 * n_lm; ++k)
        if (!std::isfinite(xyz[k])) return PM_EINVAL;
    for (int a = 0; a < 9; ++a)
        if (!std::isfinite(view->R_cw[a])) return PM_EINVAL;
    for (int a = 0; a < 3; ++a)
        if (!std::isfinite(view->t_cw[a])) return PM_EINVAL;
    Submission sub;
    sub.W = W;
    sub.H = H;
    sub.t_submit = Clock::now();
    sub.gray.resize((size_t)W * H);
    const size_t pitch = view->pitch_bytes ? view->pitch_bytes : (size_t)W;
    for (int i = 0; i < H; ++i)
        std::memcpy(sub.gray.data() + (size_t)i * W, static_cast<const uint8_t *>(view->gray) + i * pitch, W);
    std::memcpy(sub.R, view->R_cw, sizeof sub.R);
    std::memcpy(sub.t, view->t_cw, sizeof sub.t);
    if (with_landmarks) {
        sub.has_landmarks = true;
        sub.lm_xyz.assign(xyz, xyz + 3 * (size_t)n_lm);
        sub.lm_ids.assign(ids, ids + n_lm);
    }
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop || s->finishing) return PM_ECANCELLED;
    sub.ticket = s->next_ticket++;
    *ticket = sub.ticket;
    s->outstanding.insert(sub.ticket);
    if (s->cfg.dense_output) s->dense_outstanding.insert(sub.ticket);
    s->pending.push_back(std::move(sub));
    s->cv_work.notify_one();
    return PM_OK;
}

// Counts a thread inside a wait so that destroy can wait for it to leave.
struct WaiterScope {
    pm_server *s;
    explicit WaiterScope(pm_server *srv) : s(srv) { ++s->waiters; }  // under s->mu
    ~WaiterScope() {
        --s->waiters;  // under s->mu: the scope ends before the lock is released
        s->cv_done.notify_all();
    }
};
}  // namespace

int pm_server_submit(pm_server *s, int W, int H, const pm_view *view, uint64_t *ticket) {
    return submit(s, W, H, view, nullptr, nullptr, 0, false, ticket);
}

int pm_server_submit_landmarks(pm_server *s, int W, int H, const pm_view *view, const double *xyz,
                               const uint64_t *ids, int n, uint64_t *ticket) {
    return submit(s, W, H, view, xyz, ids, n, true, ticket);
}

int pm_server_wait(pm_server *s, uint64_t ticket, int timeout_ms, pm_maps *out, pm_served_info *info) {
    if (!s) return PM_EINVAL;
    std::unique_lock<std::mutex> lk(s->mu);
    if (!s->outstanding.count(ticket)) return PM_EINVAL;  // never issued, or already collected
    Result r;
    {
        WaiterScope ws(s);
        // also wakes when another thread collects the ticket first
        const auto pred = [&] { return s->done.count(ticket) > 0 || !s->outstanding.count(ticket); };
        if (timeout_ms < 0)
            s->cv_done.wait(lk, pred);
        else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred))
            return PM_ETIMEOUT;
        if (!s->done.count(ticket)) return PM_EINVAL;
        r = std::move(s->done[ticket]);
        s->done.erase(ticket);
        s->outstanding.erase(ticket);
    }
    lk.unlock();
    if (info) *info = r.info;
    if (out && r.status == PM_OK) {
        if (out->depth) std::memcpy(out->depth, r.depth.data(), r.depth.size() * 4);
        if (out->score) std::memcpy(out->score, r.score.data(), r.score.size() * 4);
    }
    return r.status;
}

int pm_server_wait_dense(pm_server *s, uint64_t ticket, int timeout_ms, float *depth, pm_points *points) {
    if (!s) return PM_EINVAL;
    std::unique_lock<std::mutex> lk(s->mu);
    if (!s->cfg.dense_output || !s->dense_outstanding.count(ticket)) return PM_EINVAL;
    DenseResult r;
    {
        WaiterScope ws(s);
        const auto pred = [&] { return s->dense_done.count(ticket) > 0 || !s->dense_outstanding.count(ticket); };
        if (timeout_ms < 0)
            s->cv_done.wait(lk, pred);
        else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred))
            return PM_ETIMEOUT;
        if (!s->dense_done.count(ticket)) return PM_EINVAL;
        const DenseResult &d = s->dense_done[ticket];
        if (points && d.status == PM_OK && (long long)(d.ij.size() / 2) > (long long)points->capacity) {
            points->count = (int)(d.ij.size() / 2);  // too small: the ticket stays collectable
            return PM_EINVAL;
        }
        r = std::move(s->dense_done[ticket]);
        s->dense_done.erase(ticket);
        s->dense_outstanding.erase(ticket);
    }
    lk.unlock();
    if (r.status != PM_OK) return r.status;
    if (depth) std::memcpy(depth, r.depth.data(), r.depth.size() * sizeof(float));
    if (points) {
        const int n = (int)(r.ij.size() / 2);
        const int m = std::min(n, std::max(points->capacity, 0));
        for (int q = 0; q < m; ++q) {
            if (points->xyz)
                for (int a = 0; a < 3; ++a) points->xyz[3 * q + a] = r.xyz[3 * (size_t)q + a];
            if (points->ij) {
                points->ij[2 * q] = r.ij[2 * (size_t)q];
                points->ij[2 * q + 1] = r.ij[2 * (size_t)q + 1];
            }
        }
        points->count = n;
    }
    return PM_OK;
}

int pm_server_finish(pm_server *s) {
    if (!s) return PM_EINVAL;
    std::unique_lock<std::mutex> lk(s->mu);
    s->finishing = true;
    s->cv_work.notify_all();
    WaiterScope ws(s);  // a concurrent destroy waits until this thread has left
    s->cv_done.wait(lk, [&] { return s->finished; });
    return PM_OK;
}

int pm_server_destroy(pm_server *s) {
    if (!s) return PM_EINVAL;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv_work.notify_all();
    }
    s->worker.join();
    {
        // every ticket has its result now; wait for the threads still collecting
        std::unique_lock<std::mutex> lk(s->mu);
        s->cv_done.notify_all();
        s->cv_done.wait(lk, [&] { return s->waiters == 0; });
    }
    s->priors.clear();
    cudaDeviceSynchronize();
    for (CachedKeyframe &k : s->cache) cache_retire(s, k);
    for (ImageBuf *b : s->retired) {
        for (cudaEvent_t e : b->uses) cudaEventDestroy(e);
        cudaFree(b->d);
        delete b;
    }
    for (cudaEvent_t e : s->event_pool) cudaEventDestroy(e);
    delete s;
    return PM_OK;
}

}  // extern "C"
