// Served densification: a request loop over the device-resident request API.
//
// Keyframes arrive through pm_server_submit (any thread).  A worker thread
// owns the CUDA context: it uploads each keyframe once into a device cache of
// resident images, chooses the nearest cached keyframes as sources, admits the
// keyframe when an in-flight slot and the HBM budget allow, seeds it from the
// newest finished result and runs it on its own stream, so keyframes that
// arrive while others are on the GPU overlap with them (continuous batching).
// pm_server_wait returns the maps and the submit-to-result latency.
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
    Clock::time_point t_submit, t_start;
};

struct Result {
    int status = PM_OK;
    std::vector<float> depth, score;
    pm_served_info info{};
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
    bool stop = false;
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

void finish(pm_server *s, uint64_t ticket, Result &&r) {
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
    std::vector<const CachedKeyframe *> src = select_sources(s, *kf);
    if ((int)src.size() < s->cfg.min_sources) {
        Result r;
        r.status = PM_ENOTREADY;  // not enough neighbours yet (the first keyframes of a stream)
        r.info.status = PM_ENOTREADY;
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
        if (rc == PM_OK) {
            const size_t n = (size_t)j.W * j.H;
            r.depth.assign(j.h_depth, j.h_depth + n);
            r.score.assign(j.h_score, j.h_score + n);
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

void worker_main(pm_server *s) {
    std::deque<Submission> waiting;  // dequeued, waiting for a slot / memory (submission order)
    for (;;) {
        {
            std::unique_lock<std::mutex> lk(s->mu);
            if (s->stop && s->pending.empty() && waiting.empty() && s->inflight.empty()) break;
            if (s->pending.empty() && waiting.empty() && s->inflight.empty())
                s->cv_work.wait_for(lk, std::chrono::milliseconds(50));
            while (!s->pending.empty()) {
                waiting.push_back(std::move(s->pending.front()));
                s->pending.pop_front();
            }
        }
        poll_inflight(s);
        while (!waiting.empty() && (int)s->inflight.size() < s->cfg.max_inflight) {
            Submission &sub = waiting.front();
            // admission happens in submission order, so the cache holds exactly
            // the keyframes before this one: neighbours never depend on timing
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
                finish(s, sub.ticket, std::move(r));
            }
            waiting.pop_front();
        }
        if (!s->inflight.empty()) std::this_thread::sleep_for(std::chrono::microseconds(s->cfg.poll_us));
    }
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
}

int pm_server_create(pm_ctx *ctx, const pm_server_config *cfg, pm_server **out) {
    if (!ctx || !cfg || !out) return PM_EINVAL;
    if (cfg->cache_capacity < 2 || cfg->max_inflight < 1 || cfg->min_sources < 1 ||
        cfg->max_sources > PM_MAX_SOURCES || cfg->min_sources > cfg->max_sources || cfg->seeded_iterations < 0 ||
        !(cfg->max_baseline > cfg->min_baseline) || cfg->poll_us < 0 || cfg->prior_lag < 1)
        return PM_EINVAL;
    pm_server *s = new pm_server();
    s->ctx = ctx;
    s->cfg = *cfg;
    s->worker = std::thread(worker_main, s);
    *out = s;
    return PM_OK;
}

int pm_server_submit(pm_server *s, int W, int H, const pm_view *view, uint64_t *ticket) {
    if (!s || !view || !view->gray || !ticket || W < 16 || H < 16) return PM_EINVAL;
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
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return PM_ECANCELLED;
    sub.ticket = s->next_ticket++;
    *ticket = sub.ticket;
    s->outstanding.insert(sub.ticket);
    s->pending.push_back(std::move(sub));
    s->cv_work.notify_one();
    return PM_OK;
}

int pm_server_wait(pm_server *s, uint64_t ticket, int timeout_ms, pm_maps *out, pm_served_info *info) {
    if (!s) return PM_EINVAL;
    std::unique_lock<std::mutex> lk(s->mu);
    if (!s->outstanding.count(ticket)) return PM_EINVAL;  // never issued, or already collected
    // also wakes when another thread collects the ticket first
    const auto pred = [&] { return s->done.count(ticket) > 0 || !s->outstanding.count(ticket); };
    if (timeout_ms < 0)
        s->cv_done.wait(lk, pred);
    else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred))
        return PM_ETIMEOUT;
    if (!s->done.count(ticket)) return PM_EINVAL;
    Result r = std::move(s->done[ticket]);
    s->done.erase(ticket);
    s->outstanding.erase(ticket);
    lk.unlock();
    s->cv_done.notify_all();
    if (info) *info = r.info;
    if (out && r.status == PM_OK) {
        if (out->depth) std::memcpy(out->depth, r.depth.data(), r.depth.size() * 4);
        if (out->score) std::memcpy(out->score, r.score.data(), r.score.size() * 4);
    }
    return r.status;
}

int pm_server_destroy(pm_server *s) {
    if (!s) return PM_EINVAL;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv_work.notify_all();
    }
    s->worker.join();
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
