// C++ mirror of the reference's dense::DepthmapEstimator / DepthmapCleaner /
// DepthmapPruner (src/openvslam/depthmap.h:122-291) over the C ABI.
#include "pm_dense.hpp"

#include <algorithm>
#include <cstring>
#include <utility>

namespace dense {

namespace {

struct CtxHolder {
    pm_ctx *ctx = nullptr;
    int device = 0;
    explicit CtxHolder(int dev) : device(dev) {}
    ~CtxHolder() {
        if (ctx) pm_destroy(ctx);
    }
    Status ensure() {
        if (ctx) return Status{};
        int rc = pm_create(device, 0, &ctx);
        if (rc) return Status{rc, pm_status_string(rc)};
        return Status{};
    }
    Status status(int rc) const { return rc ? Status{rc, pm_last_error(ctx)} : Status{}; }
};

void to_double(const Matx33d &R, double *out) { std::memcpy(out, R.data(), 9 * sizeof(double)); }

}  // namespace

// ----------------------------------------------------------------------------
struct DepthmapEstimator::Impl {
    CtxHolder h;
    std::vector<Matx33d> Rs;
    std::vector<Vec3d> ts;
    std::vector<MatU8> images, masks;
    std::vector<std::vector<Vec3d>> landmarks;
    std::vector<double> maxds, minds;
    int min_images_compute = 2;
    int patch_size = 7;
    int iterations = 3;
    float min_patch_sd = 5.0f;
    double min_score = 0.0;
    int combine = PM_COMBINE_FOLD, top_k = 3, seam = PM_SEAM_CLAMP;
    uint32_t seed = 0, keyframe_counter = 0;
    int debug_shifts = 0;
    explicit Impl(int dev) : h(dev) {}
};

DepthmapEstimator::DepthmapEstimator(int device) : d_(new Impl(device)) {}
DepthmapEstimator::~DepthmapEstimator() = default;

void DepthmapEstimator::AddView(const Matx33d &R, const Vec3d &t, const MatU8 &Img, const MatU8 &mask,
                                const std::vector<Vec3d> &landmarks, double maxd, double mind) {
    d_->Rs.push_back(R);
    d_->ts.push_back(t);
    d_->images.push_back(Img);
    d_->masks.push_back(mask);
    d_->landmarks.push_back(landmarks);
    d_->maxds.push_back(maxd);
    d_->minds.push_back(mind);
}

int DepthmapEstimator::PopHeadUnlessOne() {
    if (d_->images.size() > 1) {
        d_->Rs.erase(d_->Rs.begin());
        d_->ts.erase(d_->ts.begin());
        d_->images.erase(d_->images.begin());
        d_->masks.erase(d_->masks.begin());
        d_->landmarks.erase(d_->landmarks.begin());
        d_->maxds.erase(d_->maxds.begin());
        d_->minds.erase(d_->minds.begin());
    }
    return (int)d_->images.size();
}

void DepthmapEstimator::reset() {
    d_->Rs.clear();
    d_->ts.clear();
    d_->images.clear();
    d_->masks.clear();
    d_->landmarks.clear();
    d_->maxds.clear();
    d_->minds.clear();
    d_->debug_shifts = 0;
}

bool DepthmapEstimator::IsReadyForCompute() const {
    return (int)d_->images.size() >= d_->min_images_compute && d_->debug_shifts < (int)d_->images.size();
}

bool DepthmapEstimator::SetMinImagesCompute(int n) {
    const bool ok = n >= 2;
    d_->min_images_compute = ok ? n : 2;
    return ok;
}

void DepthmapEstimator::SetDepthRange(double min_depth, double max_depth, int) {
    // the per-view range passed to AddView wins, as in the reference (depthmap.cc:549-550)
    (void)min_depth;
    (void)max_depth;
}

void DepthmapEstimator::SetPatchMatchIterations(int n) { d_->iterations = n; }
void DepthmapEstimator::SetPatchSize(int size) { d_->patch_size = size; }
void DepthmapEstimator::SetMinPatchSD(float sd) { d_->min_patch_sd = sd; }
void DepthmapEstimator::SetMinScore(double s) { d_->min_score = s; }
void DepthmapEstimator::SetCombine(int mode, int top_k) {
    d_->combine = mode;
    d_->top_k = top_k;
}
void DepthmapEstimator::SetSeam(int seam) { d_->seam = seam; }
void DepthmapEstimator::SetSeed(uint32_t seed) { d_->seed = seed; }

Status DepthmapEstimator::ComputePatchMatch(DepthmapEstimatorResult *result) {
    Impl &d = *d_;
    if (!result) return Status{PM_EINVAL, "result is null"};
    if (d.images.size() < 2) return Status{PM_EINVAL, "need at least two views"};
    Status st = d.h.ensure();
    if (!st) return st;
    const int n = (int)d.images.size();
    const int center = n / 2;  // swapCenter (depthmap.cc:835-845)
    const MatU8 &ref = d.images[center];
    const int H = ref.rows, W = ref.cols;
    std::vector<int> order{center};
    for (int k = 0; k < n; ++k)
        if (k != center) order.push_back(k);
    std::vector<pm_view> views(n);
    for (int s = 0; s < n; ++s) {
        const int k = order[s];
        if (d.images[k].rows != H || d.images[k].cols != W) return Status{PM_EINVAL, "views differ in size"};
        std::memset(&views[s], 0, sizeof(pm_view));
        views[s].gray = d.images[k].data.data();
        views[s].mask = (s == 0 && !d.masks[k].empty()) ? d.masks[k].data.data() : nullptr;
        to_double(d.Rs[k], views[s].R_cw);
        std::memcpy(views[s].t_cw, d.ts[k].data(), 3 * sizeof(double));
    }
    pm_params p;
    pm_params_default(&p);
    p.patch_half = d.patch_size - 2;
    p.iterations = d.iterations;
    p.combine = d.combine;
    p.top_k = d.top_k;
    p.seam = d.seam;
    // depth range of the centre view (depthmap.cc:549-550); the reference
    // initialises from min_depth = 1e-5, which log-uniform sampling cannot use
    p.min_depth = (float)std::max(d.minds[center], 1e-3);
    p.max_depth = (float)std::max(d.maxds[center], (double)p.min_depth * 2.0);
    p.min_score = (float)d.min_score;
    p.min_patch_sd = d.min_patch_sd;
    p.seed = d.seed;
    p.keyframe_id = d.keyframe_counter++;
    result->depth = MatF(H, W);
    result->score = MatF(H, W, -1.0f);
    result->plane = MatF3(H, W);
    result->normal = MatF3(H, W);
    result->nghbr = MatI(H, W);
    pm_maps m{result->depth.data.data(), result->score.data.data(), result->plane.data.data(),
              result->normal.data.data(), result->nghbr.data.data()};
    const int rc = pm_densify(d.h.ctx, W, H, views.data(), n, &p, &m);
    if (rc) return d.h.status(rc);
    // best source as the reference's view index ("other", 1-based over the
    // non-centre views in queue order)
    for (auto &v : result->nghbr.data) v = v + 1;
    result->R = d.Rs[center];
    result->t = d.ts[center];
    return Status{};
}

// ----------------------------------------------------------------------------
struct DepthmapCleaner::Impl {
    CtxHolder h;
    std::vector<DepthmapEstimatorResult> results;
    float same_depth_threshold = 0.01f;
    int min_consistent_views = 2;
    int queue = 1;
    float reproj_px = 0.0f;
    explicit Impl(int dev) : h(dev) {}
};

DepthmapCleaner::DepthmapCleaner(int device) : d_(new Impl(device)) {}
DepthmapCleaner::~DepthmapCleaner() = default;
int DepthmapCleaner::PopHeadUnlessOne() {
    if (d_->results.size() > 1) d_->results.erase(d_->results.begin());
    return (int)d_->results.size();
}
void DepthmapCleaner::reset() { d_->results.clear(); }
void DepthmapCleaner::SetSameDepthThreshold(float t) { d_->same_depth_threshold = t; }
void DepthmapCleaner::SetMinConsistentViews(int n) { d_->min_consistent_views = n; }
void DepthmapCleaner::SetDepthQueueSize(int n) { d_->queue = n; }
void DepthmapCleaner::SetReprojectionPixels(float px) { d_->reproj_px = px; }
void DepthmapCleaner::AddView(const DepthmapEstimatorResult *r) {
    if (r) d_->results.push_back(*r);
}
bool DepthmapCleaner::IsReadyForCompute() const { return (int)d_->results.size() >= d_->queue; }

Status DepthmapCleaner::Clean(DepthmapCleanerResult *result) {
    Impl &d = *d_;
    if (!result) return Status{PM_EINVAL, "result is null"};
    if (!IsReadyForCompute()) return Status{PM_ENOTREADY, "queue not full"};
    Status st = d.h.ensure();
    if (!st) return st;
    const int n = (int)d.results.size(), center = n / 2;
    const int H = d.results[center].depth.rows, W = d.results[center].depth.cols;
    std::vector<const float *> depths(n);
    std::vector<double> R(9 * n), t(3 * n);
    for (int k = 0; k < n; ++k) {
        depths[k] = d.results[k].depth.data.data();
        to_double(d.results[k].R, &R[9 * k]);
        std::memcpy(&t[3 * k], d.results[k].t.data(), 3 * sizeof(double));
    }
    result->cleaned_depth = MatF(H, W);
    const int rc = pm_filter_consistency(d.h.ctx, W, H, n, depths.data(), R.data(), t.data(), center,
                                         d.same_depth_threshold, d.min_consistent_views, d.reproj_px,
                                         result->cleaned_depth.data.data());
    if (rc) return d.h.status(rc);
    result->R = d.results[center].R;
    result->t = d.results[center].t;
    return Status{};
}

// ----------------------------------------------------------------------------
struct DepthmapPruner::Impl {
    CtxHolder h;
    std::vector<DepthmapCleanerResult> results;
    std::vector<MatU8C3> images;
    float same_depth_threshold = 0.01f;
    int min_views = 3;
    int queue = 1;
    explicit Impl(int dev) : h(dev) {}
};

DepthmapPruner::DepthmapPruner(int device) : d_(new Impl(device)) {}
DepthmapPruner::~DepthmapPruner() = default;
void DepthmapPruner::SetSameDepthThreshold(float t) { d_->same_depth_threshold = t; }
void DepthmapPruner::SetMinViews(int n) { d_->min_views = n; }
void DepthmapPruner::SetDepthQueueSize(int n) { d_->queue = n; }
int DepthmapPruner::PopHead() {
    if (!d_->results.empty()) {
        d_->results.erase(d_->results.begin());
        d_->images.erase(d_->images.begin());
    }
    return (int)d_->results.size();
}
void DepthmapPruner::reset() {
    d_->results.clear();
    d_->images.clear();
}
void DepthmapPruner::AddView(const DepthmapCleanerResult *r, const MatU8C3 &rgb) {
    if (!r) return;
    d_->results.push_back(*r);
    d_->images.push_back(rgb);
}
bool DepthmapPruner::IsReadyForCompute() const { return (int)d_->results.size() >= d_->queue; }

Status DepthmapPruner::Prune(DepthmapPrunerResult *result) {
    Impl &d = *d_;
    if (!result) return Status{PM_EINVAL, "result is null"};
    if (d.results.empty()) return Status{};  // depthmap.cc:1537-1539
    Status st = d.h.ensure();
    if (!st) return st;
    const int n = (int)d.results.size();
    const int H = d.results[0].cleaned_depth.rows, W = d.results[0].cleaned_depth.cols;
    std::vector<float *> depths(n);
    std::vector<double> R(9 * n), t(3 * n);
    for (int k = 0; k < n; ++k) {
        depths[k] = d.results[k].cleaned_depth.data.data();  // later maps are edited in place
        to_double(d.results[k].R, &R[9 * k]);
        std::memcpy(&t[3 * k], d.results[k].t.data(), 3 * sizeof(double));
    }
    result->pruned_depth = MatF(H, W);
    const size_t cap = (size_t)W * H;
    std::vector<double> xyz(3 * cap);
    std::vector<uint8_t> bgr(3 * cap);
    std::vector<int32_t> ij(2 * cap);
    pm_points pts{(int)cap, 0, xyz.data(), bgr.data(), ij.data()};
    const uint8_t *rgb = d.images[0].empty() ? nullptr : d.images[0].data.data();
    const int rc = pm_fuse(d.h.ctx, W, H, n, depths.data(), R.data(), t.data(), rgb, d.same_depth_threshold,
                           result->pruned_depth.data.data(), &pts);
    if (rc) return d.h.status(rc);
    result->points3d.resize(pts.count);
    result->colors.resize(rgb ? pts.count : 0);
    result->keypts.resize(pts.count);
    for (int q = 0; q < pts.count; ++q) {
        result->points3d[q] = {xyz[3 * q], xyz[3 * q + 1], xyz[3 * q + 2]};
        if (rgb) result->colors[q] = {bgr[3 * q], bgr[3 * q + 1], bgr[3 * q + 2]};
        result->keypts[q] = {ij[2 * q], ij[2 * q + 1]};
    }
    result->R = d.results[0].R;
    result->t = d.results[0].t;
    return Status{};
}

}  // namespace dense
