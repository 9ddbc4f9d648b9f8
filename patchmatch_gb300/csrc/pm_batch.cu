// Batched executor of the C ABI (pm_batch_*): many requests densified
// together in one captured CUDA graph (see include/pm_gb300.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "pm_gb300.h"
#include "pm_internal.h"
#include "pm_kernels.h"
#include "pm_sweep.cuh"

using pmi::check_views;
using pmi::enqueue_post;
using pmi::fail;
using pmi::fill_args;

// ---------------------------------------------------------------------------
// Batched executor: many requests densified by phase-major launches (init
// scoring, then each red/black half-sweep of every request, then the
// post-filter), captured once into a CUDA graph and replayed.  Requests are
// grouped by (source count, image variant, propagation rule, sweep count);
// each phase of a group is one persistent launch over a device queue of
// (request, tile) items (PM_BATCH_PERSISTENT) or one launch per request
// (PM_BATCH_LAUNCHES).  A tile's update reads only pixels of the other colour,
// so the result of every request is the same as from pm_request_run.
// ---------------------------------------------------------------------------
struct pm_batch {
    struct Group {
        int S = 0, kind = 0, iterations = 0;
        int level = 0;  // seeding level: requests seeded from a batch member run one level after it
        bool plain = false;
        std::vector<pm_request *> members;
        pm::SweepArgs *d_args = nullptr;
        int4 *d_items = nullptr;
        int n_items = 0;
        unsigned int *d_counters = nullptr;
        int n_phases = 0;
        std::vector<pm::SweepArgs> h_args;
    };
    pm_ctx *ctx = nullptr;
    std::vector<pm_request *> reqs;
    std::vector<Group> groups;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    std::vector<cudaEvent_t> req_events;
    static constexpr int kBranches = 8;      // PM_BATCH_STREAMS: parallel chains of requests
    cudaStream_t branch[kBranches] = {};
    cudaEvent_t fork = nullptr, join[kBranches] = {};
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    bool dirty = true;
    std::vector<char> signature;   // what the captured graph depends on
    int executor = PM_BATCH_PERSISTENT;
    int grid_mult = 1;
    uint64_t launches_per_run = 0;
    std::vector<int> level;        // per request (index into reqs)
    int n_levels = 1;
};

namespace {

void batch_free_groups(pm_batch *b) {
    for (auto &g : b->groups) {
        cudaFree(g.d_args);
        cudaFree(g.d_items);
        cudaFree(g.d_counters);
    }
    b->groups.clear();
}

int batch_index(const pm_batch *b, const pm_request *r) {
    for (size_t k = 0; k < b->reqs.size(); ++k)
        if (b->reqs[k] == r) return (int)k;
    return -1;
}

// Seeding levels: 0 for a request without a prior in the batch, else one more
// than its prior's.  A cycle of priors inside the batch is rejected.
int batch_levels(pm_batch *b) {
    const size_t n = b->reqs.size();
    b->level.assign(n, 0);
    b->n_levels = 1;
    for (size_t k = 0; k < n; ++k) {
        int lv = 0;
        const pm_request *r = b->reqs[k];
        for (size_t hop = 0; hop <= n; ++hop) {
            const int p = r->prior ? batch_index(b, r->prior) : -1;
            if (p < 0) break;
            if (hop == n) return fail(b->ctx, PM_EINVAL, "the priors of the batch's requests form a cycle");
            ++lv;
            r = b->reqs[p];
        }
        b->level[k] = lv;
        b->n_levels = std::max(b->n_levels, lv + 1);
    }
    return PM_OK;
}

int batch_build(pm_batch *b) {
    pm_ctx *ctx = b->ctx;
    batch_free_groups(b);
    int rc0 = batch_levels(b);
    if (rc0) return rc0;
    for (size_t k = 0; k < b->reqs.size(); ++k) {
        pm_request *r = b->reqs[k];
        const int kind = pm::image_kind(r->prm.image_format, r->prm.sampler);
        const bool plain = r->prm.propagation == PM_PROPAGATION_PLAIN;
        pm_batch::Group *g = nullptr;
        // the mixed kernel takes every source count in one group (S = 0)
        const int gS = b->executor == PM_BATCH_MIXED ? 0 : r->S;
        for (auto &x : b->groups)
            if (x.S == gS && x.kind == kind && x.plain == plain && x.iterations == r->prm.iterations &&
                x.level == b->level[k])
                g = &x;
        if (!g) {
            b->groups.emplace_back();
            g = &b->groups.back();
            g->S = gS;
            g->kind = kind;
            g->plain = plain;
            g->iterations = r->prm.iterations;
            g->level = b->level[k];
        }
        g->members.push_back(r);
    }
    for (auto &g : b->groups) {
        std::vector<int4> items;
        for (int m = 0; m < (int)g.members.size(); ++m) {
            const dim3 tg = pm::tile_grid(g.members[m]->W, g.members[m]->H);
            for (unsigned y = 0; y < tg.y; ++y)
                for (unsigned x = 0; x < tg.x; ++x) items.push_back(make_int4(m, (int)x, (int)y, g.members[m]->S));
        }
        g.n_items = (int)items.size();
        g.n_phases = 2 + 2 * g.iterations;
        g.h_args.resize(g.members.size());
        if (cudaMalloc(&g.d_args, g.members.size() * sizeof(pm::SweepArgs)) != cudaSuccess ||
            cudaMalloc(&g.d_items, items.size() * sizeof(int4)) != cudaSuccess ||
            cudaMalloc(&g.d_counters, g.n_phases * sizeof(unsigned int)) != cudaSuccess) {
            cudaGetLastError();
            return fail(ctx, PM_ENOMEM, "batch work queues");
        }
        PM_CUDA(ctx, cudaMemcpy(g.d_items, items.data(), items.size() * sizeof(int4), cudaMemcpyHostToDevice));
    }
    return PM_OK;
}

// Seeding of r on st inside the batch's graph; its launches are counted in `launches`.
int seed_in_batch(pm_batch *b, pm_request *r, cudaStream_t st, uint64_t &launches) {
    const uint64_t before = b->ctx->launches;
    const int rc = pmi::enqueue_seeding(r, st, r->prior && batch_index(b, r->prior) >= 0);
    launches += b->ctx->launches - before;
    return rc;
}

int batch_enqueue(pm_batch *b) {
    pm_ctx *ctx = b->ctx;
    const cudaStream_t st = b->stream;
    int sms = 0;
    PM_CUDA(ctx, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    uint64_t launches = 0;
    int max_phases = 0;
    for (auto &g : b->groups) {
        PM_CUDA(ctx, cudaMemsetAsync(g.d_counters, 0, g.n_phases * sizeof(unsigned int), st));
        max_phases = std::max(max_phases, g.n_phases);
    }
    if (b->executor == PM_BATCH_STREAMS) {
        // each request's whole chain on one of the branch streams (largest
        // first onto the least-loaded branch), branches forked from and
        // joined back into the batch stream
        // seeded requests follow their prior (lower level first) on the prior's branch
        std::vector<int> order(b->reqs.size());
        for (size_t k = 0; k < order.size(); ++k) order[k] = (int)k;
        auto work = [&](int k) {
            const pm_request *x = b->reqs[k];
            return (double)x->W * x->H * x->S * (1 + x->prm.iterations);
        };
        std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
            if (b->level[x] != b->level[y]) return b->level[x] < b->level[y];
            return work(x) > work(y);
        });
        double load[pm_batch::kBranches] = {};
        std::vector<int> branch_of(b->reqs.size(), -1);
        const int nb = std::min<int>(pm_batch::kBranches, (int)order.size());
        PM_CUDA(ctx, cudaEventRecord(b->fork, st));
        for (int k = 0; k < nb; ++k) PM_CUDA(ctx, cudaStreamWaitEvent(b->branch[k], b->fork, 0));
        for (int idx : order) {
            pm_request *r = b->reqs[idx];
            const int pi = r->prior ? batch_index(b, r->prior) : -1;
            int k = 0;
            if (pi >= 0) {
                k = branch_of[pi];
            } else {
                for (int q = 1; q < nb; ++q)
                    if (load[q] < load[k]) k = q;
            }
            branch_of[idx] = k;
            load[k] += work(idx);
            const cudaStream_t bs = b->branch[k];
            const pm_params &p = r->prm;
            pm::launch_init_planes(bs, r->trig.row, r->trig.col, r->W, r->H, p.seed, p.keyframe_id, p.init_mode,
                                   p.min_depth, p.max_depth, r->plane, r->score, r->best);
            ++launches;
            const int kind = pm::image_kind(p.image_format, p.sampler);
            for (int ph = 0; ph < 2 + 2 * p.iterations; ++ph) {
                if (ph == 2) {
                    const int rc = seed_in_batch(b, r, bs, launches);
                    if (rc) return rc;
                }
                pm::SweepArgs a = r->args;
                a.mode = ph < 2 ? pm::kModeScore : pm::kModeSweep;
                a.colour = ph < 2 ? ph : (ph - 2) & 1;
                a.sweep = ph < 2 ? 0 : (ph - 2) >> 1;
                const dim3 grid = pm::tile_grid(r->W, r->H);
                pm::BandArgs band{};
                const pm::BandArgs *bp = nullptr;
                const int rc = pmi::tile_band(r, grid, bs, &band, &bp);
                if (rc) return rc;
                cudaError_t e = pm::dispatch_tile(r->S, kind, grid, bs, a, bp);
                if (e != cudaSuccess) return fail(ctx, PM_ECUDA, "tile launch: %s", cudaGetErrorString(e));
                ++launches;
            }
            if (p.iterations == 0) {  // no sweep phase: the seeding follows the init scoring
                const int rc = seed_in_batch(b, r, bs, launches);
                if (rc) return rc;
            }
            if (p.postprocess) {
                enqueue_post(r, bs);
                launches += 3;
            }
        }
        for (int k = 0; k < nb; ++k) {
            PM_CUDA(ctx, cudaEventRecord(b->join[k], b->branch[k]));
            PM_CUDA(ctx, cudaStreamWaitEvent(st, b->join[k], 0));
        }
        b->launches_per_run = launches;
        return PM_OK;
    }
    for (int lv = 0; lv < b->n_levels; ++lv) {
    for (size_t k = 0; k < b->reqs.size(); ++k) {
        if (b->level[k] != lv) continue;
        pm_request *r = b->reqs[k];
        const pm_params &p = r->prm;
        pm::launch_init_planes(st, r->trig.row, r->trig.col, r->W, r->H, p.seed, p.keyframe_id, p.init_mode,
                               p.min_depth, p.max_depth, r->plane, r->score, r->best);
        ++launches;
    }
    for (int ph = 0; ph < max_phases; ++ph) {
        if (ph == 2) {
            // seeding of this level's requests, between the init scoring and the sweeps
            for (size_t k = 0; k < b->reqs.size(); ++k) {
                if (b->level[k] != lv) continue;
                const int rc = seed_in_batch(b, b->reqs[k], st, launches);
                if (rc) return rc;
            }
        }
        const int mode = ph < 2 ? pm::kModeScore : pm::kModeSweep;
        const int colour = ph < 2 ? ph : (ph - 2) & 1;
        const int sweep = ph < 2 ? 0 : (ph - 2) >> 1;
        for (auto &g : b->groups) {
            if (g.level != lv || ph >= g.n_phases) continue;
            if (b->executor == PM_BATCH_PERSISTENT || b->executor == PM_BATCH_MIXED) {
                pm::BatchArgs a{};
                a.args = g.d_args;
                a.items = g.d_items;
                a.n_items = g.n_items;
                a.counter = g.d_counters + ph;
                a.mode = mode;
                a.colour = colour;
                a.sweep = sweep;
                const bool mixed = b->executor == PM_BATCH_MIXED;
                const int occ = std::max(1, mixed ? pm::dispatch_batch_mixed_blocks_per_sm(g.kind, g.plain)
                                                  : pm::dispatch_batch_blocks_per_sm(g.S, g.kind, g.plain));
                const int blocks = std::max(1, std::min(g.n_items, b->grid_mult * occ * sms));
                cudaError_t e = mixed ? pm::dispatch_batch_mixed(g.kind, g.plain, blocks, st, a)
                                      : pm::dispatch_batch(g.S, g.kind, g.plain, blocks, st, a);
                if (e != cudaSuccess) return fail(ctx, PM_ECUDA, "batch launch: %s", cudaGetErrorString(e));
                ++launches;
            } else {
                for (size_t m = 0; m < g.members.size(); ++m) {
                    pm::SweepArgs a = g.h_args[m];
                    a.mode = mode;
                    a.colour = colour;
                    a.sweep = sweep;
                    const dim3 grid = pm::tile_grid(a.W, a.H);
                    pm::BandArgs band{};
                    const pm::BandArgs *bp = nullptr;
                    const int rc = pmi::tile_band(g.members[m], grid, st, &band, &bp);
                    if (rc) return rc;
                    cudaError_t e = pm::dispatch_tile(g.S, g.kind, grid, st, a, bp);
                    if (e != cudaSuccess) return fail(ctx, PM_ECUDA, "tile launch: %s", cudaGetErrorString(e));
                    ++launches;
                }
            }
        }
    }
    if (max_phases <= 2)  // no sweep phase in the batch: the seeding follows the init scoring
        for (size_t k = 0; k < b->reqs.size(); ++k) {
            if (b->level[k] != lv) continue;
            const int rc = seed_in_batch(b, b->reqs[k], st, launches);
            if (rc) return rc;
        }
    for (size_t k = 0; k < b->reqs.size(); ++k)
        if (b->level[k] == lv && b->reqs[k]->prm.postprocess) {
            enqueue_post(b->reqs[k], st);
            launches += 3;
        }
    }  // level
    b->launches_per_run = launches;
    return PM_OK;
}

}  // namespace

extern "C" {

int pm_batch_create(pm_ctx *ctx, pm_batch **out) {
    if (!ctx || !out) return PM_EINVAL;
    *out = nullptr;
    PM_CUDA(ctx, cudaSetDevice(ctx->device));
    pm_batch *b = new pm_batch();
    b->ctx = ctx;
    ++ctx->live;
    bool ok = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming) == cudaSuccess &&
              cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) == cudaSuccess;
    for (int k = 0; ok && k < pm_batch::kBranches; ++k)
        ok = cudaStreamCreateWithFlags(&b->branch[k], cudaStreamNonBlocking) == cudaSuccess &&
             cudaEventCreateWithFlags(&b->join[k], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        pm_batch_destroy(b);
        return fail(ctx, PM_ECUDA, "batch stream creation failed");
    }
    *out = b;
    return PM_OK;
}

int pm_batch_add(pm_batch *b, pm_request *r) {
    if (!b || !r) return PM_EINVAL;
    if (r->ctx != b->ctx) return fail(b->ctx, PM_EINVAL, "request belongs to another context");
    for (pm_request *q : b->reqs)
        if (q == r) return fail(b->ctx, PM_EINVAL, "request already in the batch");
    b->reqs.push_back(r);
    cudaEvent_t e = nullptr;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        b->reqs.pop_back();
        return fail(b->ctx, PM_ECUDA, "event creation failed");
    }
    b->req_events.push_back(e);
    ++r->batch_refs;
    b->dirty = true;
    return PM_OK;
}

int pm_batch_clear(pm_batch *b) {
    if (!b) return PM_EINVAL;
    cudaStreamSynchronize(b->stream);
    for (cudaEvent_t e : b->req_events) cudaEventDestroy(e);
    b->req_events.clear();
    for (pm_request *r : b->reqs) --r->batch_refs;
    b->reqs.clear();
    b->dirty = true;
    return PM_OK;
}

int pm_batch_set_executor(pm_batch *b, int executor, int grid_mult) {
    if (!b || executor < PM_BATCH_PERSISTENT || executor > PM_BATCH_MIXED || grid_mult < 1 || grid_mult > 16)
        return PM_EINVAL;
    if (executor != b->executor || grid_mult != b->grid_mult) b->dirty = true;
    b->executor = executor;
    b->grid_mult = grid_mult;
    return PM_OK;
}

int pm_batch_run(pm_batch *b) {
    if (!b) return PM_EINVAL;
    pm_ctx *ctx = b->ctx;
    NvtxRange range("pm_batch_run requests=%d", (int)b->reqs.size());
    if (b->reqs.empty()) return fail(ctx, PM_EINVAL, "empty batch");
    bool seeded = false;
    for (pm_request *r : b->reqs) {
        int rc = check_views(r);
        if (rc) return rc;
        seeded = seeded || r->prior || r->prior_res || r->n_lm > 0;
    }
    // the graph bakes in each request's shape, parameters and mask use
    std::vector<char> sig;
    for (pm_request *r : b->reqs) {
        const char *p0 = reinterpret_cast<const char *>(&r);
        sig.insert(sig.end(), p0, p0 + sizeof r);
        const int shape[4] = {r->W, r->H, r->S, r->has_mask ? 1 : 0};
        const char *p1 = reinterpret_cast<const char *>(shape);
        sig.insert(sig.end(), p1, p1 + sizeof shape);
        const char *p2 = reinterpret_cast<const char *>(&r->prm);
        sig.insert(sig.end(), p2, p2 + sizeof r->prm);
    }
    for (pm_request *r : b->reqs) fill_args(r);
    // launches bake the poses in; so do the seeding launches (prior pose, landmark count)
    if (seeded || b->executor == PM_BATCH_LAUNCHES || b->executor == PM_BATCH_STREAMS)
        for (pm_request *r : b->reqs) {
            const char *p3 = reinterpret_cast<const char *>(&r->args);
            sig.insert(sig.end(), p3, p3 + sizeof r->args);
            const void *links[3] = {r->prior, r->prior_res, r->lm};
            const char *p4 = reinterpret_cast<const char *>(links);
            sig.insert(sig.end(), p4, p4 + sizeof links);
            const int nlm = r->n_lm;
            const char *p5 = reinterpret_cast<const char *>(&nlm);
            sig.insert(sig.end(), p5, p5 + sizeof nlm);
            if (r->prior) {
                const char *p6 = reinterpret_cast<const char *>(r->prior->R[0]);
                sig.insert(sig.end(), p6, p6 + sizeof(double) * 12);
            }
            if (r->prior_res) {
                const char *p7 = reinterpret_cast<const char *>(r->prior_res->R);
                sig.insert(sig.end(), p7, p7 + sizeof(double) * 12);
            }
        }
    const int ex[2] = {b->executor, b->grid_mult};
    sig.insert(sig.end(), reinterpret_cast<const char *>(ex), reinterpret_cast<const char *>(ex) + sizeof ex);
    if (sig != b->signature) b->dirty = true;
    PM_CUDA(ctx, cudaSetDevice(ctx->device));
    if (b->dirty || !b->gexec) {
        int rc = batch_build(b);
        if (rc) return rc;
        cudaGraph_t g = nullptr;
        for (auto &gr : b->groups)
            for (size_t m = 0; m < gr.members.size(); ++m) gr.h_args[m] = gr.members[m]->args;
        PM_CUDA(ctx, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        const uint64_t before = ctx->launches;
        rc = batch_enqueue(b);
        cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
        ctx->launches = before;
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (ce != cudaSuccess) return fail(ctx, PM_ECUDA, "batch graph capture: %s", cudaGetErrorString(ce));
        if (b->gexec) cudaGraphExecDestroy(b->gexec);
        if (b->graph) cudaGraphDestroy(b->graph);
        b->gexec = nullptr;
        b->graph = g;
        PM_CUDA(ctx, cudaGraphInstantiate(&b->gexec, g, 0));
        b->dirty = false;
        b->signature = sig;
    }
    // the requests' own streams carry their uploads; the batch waits for them,
    // and for the priors from outside the batch
    for (size_t k = 0; k < b->reqs.size(); ++k) {
        PM_CUDA(ctx, cudaEventRecord(b->req_events[k], b->reqs[k]->stream));
        PM_CUDA(ctx, cudaStreamWaitEvent(b->stream, b->req_events[k], 0));
        pm_request *r = b->reqs[k];
        if ((r->prior && batch_index(b, r->prior) < 0) || r->prior_res) {
            const int rc = pmi::wait_prior_ready(r, b->stream);
            if (rc) return rc;
        }
    }
    // per-request arguments (poses may have changed since the graph was built)
    for (auto &g : b->groups) {
        for (size_t m = 0; m < g.members.size(); ++m) g.h_args[m] = g.members[m]->args;
        PM_CUDA(ctx, cudaMemcpyAsync(g.d_args, g.h_args.data(), g.h_args.size() * sizeof(pm::SweepArgs),
                                     cudaMemcpyHostToDevice, b->stream));
    }
    PM_CUDA(ctx, cudaGraphLaunch(b->gexec, b->stream));
    PM_CUDA(ctx, cudaEventRecord(b->done, b->stream));
    for (pm_request *r : b->reqs) {
        PM_CUDA(ctx, cudaStreamWaitEvent(r->stream, b->done, 0));
        r->postprocessed = r->prm.postprocess != 0;
    }
    ctx->launches += b->launches_per_run;
    return PM_OK;
}

int pm_batch_synchronize(pm_batch *b) {
    if (!b) return PM_EINVAL;
    PM_CUDA(b->ctx, cudaStreamSynchronize(b->stream));
    return PM_OK;
}

void *pm_batch_stream(const pm_batch *b) { return b ? (void *)b->stream : nullptr; }

int pm_batch_tune(pm_batch *b, pm_batch_tuning *out) {
    if (!b) return PM_EINVAL;
    pm_ctx *ctx = b->ctx;
    const int cand[][2] = {{PM_BATCH_PERSISTENT, 1}, {PM_BATCH_PERSISTENT, 2}, {PM_BATCH_LAUNCHES, 1},
                           {PM_BATCH_STREAMS, 1}, {PM_BATCH_MIXED, 1}};
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    PM_CUDA(ctx, cudaEventCreate(&e0));
    PM_CUDA(ctx, cudaEventCreate(&e1));
    float best_ms = 1e30f;
    int best = 0;
    int rc = PM_OK;
    for (int c = 0; c < PM_BATCH_CANDIDATES && !rc; ++c) {
        pm_batch_set_executor(b, cand[c][0], cand[c][1]);
        rc = pm_batch_run(b);  // builds the graph (untimed)
        float ms = 0.f;
        if (!rc) {
            cudaEventRecord(e0, b->stream);
            rc = pm_batch_run(b);
            cudaEventRecord(e1, b->stream);
            if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
                rc = fail(ctx, PM_ECUDA, "tuning timer");
        }
        if (!rc && out) out->candidate_ms[c] = ms;
        if (!rc && ms < best_ms) {
            best_ms = ms;
            best = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    pm_batch_set_executor(b, cand[best][0], cand[best][1]);
    if (out) {
        out->executor = cand[best][0];
        out->grid_mult = cand[best][1];
        out->ms = best_ms;
    }
    return PM_OK;
}

int pm_batch_destroy(pm_batch *b) {
    if (!b) return PM_EINVAL;
    cudaSetDevice(b->ctx->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    if (b->graph) cudaGraphDestroy(b->graph);
    batch_free_groups(b);
    for (cudaEvent_t e : b->req_events) cudaEventDestroy(e);
    for (pm_request *r : b->reqs) --r->batch_refs;
    for (int k = 0; k < pm_batch::kBranches; ++k) {
        if (b->branch[k]) cudaStreamDestroy(b->branch[k]);
        if (b->join[k]) cudaEventDestroy(b->join[k]);
    }
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->done) cudaEventDestroy(b->done);
    if (b->stream) cudaStreamDestroy(b->stream);
    --b->ctx->live;
    delete b;
    return PM_OK;
}

}  // extern "C"
