// Drives the reference's own host stages (src/openvslam/depthmap.cc,
// compiled unmodified against oracle/refshim_host) through their public
// classes and functions: PostProcess (depthmap.cc:1169-1208),
// DepthmapCleaner::Clean (:1320-1377) and DepthmapPruner::Prune
// (:1535-1696).  TEST INFRASTRUCTURE ONLY: it pins the oracle's
// restatements of those stages; the product never links it.  The CUDA
// launchers depthmap.cc declares are stubs here (none of the driven stages
// calls them).
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "depthmap.h"

#define RH_STUB(name, ...)                                             \
    extern "C" void name(__VA_ARGS__) {                                \
        std::fprintf(stderr, "reference host harness: %s is not available\n", #name); \
        std::abort();                                                  \
    }
RH_STUB(ComputePatchMatchPano, float *, float *, float *, float *, int, int, cv::Mat &, cv::Mat &, float *, float *)
RH_STUB(ComputeBearingsEquirect, float *, const int, const int)
RH_STUB(ComputeRandomSeed, curandState *, const int, const int)
RH_STUB(ComputeRandomPlanemapDepthmap, float *, float *, float *, int, int, float, float, curandState *)
RH_STUB(InitTextureImages, const int, const int, cv::Mat &, cv::Mat &, cv::Mat &, float *, float *, float *,
        cudaTextureObject_t[])
RH_STUB(ScorePlaneDepth, const int, float *, float *, float *, float *, cudaTextureObject_t *, int, int)
RH_STUB(RandomInitialization, const int, float *, float *, float *, float *, cudaTextureObject_t *, int, int, float,
        float, curandState *)
RH_STUB(InitConstantMem, float *, float *, float *, float *, float *, float *)
RH_STUB(PatchMatchRedBlackPass, const int, int, float *, float *, float *, float *, cudaTextureObject_t *, int, int,
        curandState *)

namespace {
cv::Mat map_f32(const float *p, int W, int H) {
    cv::Mat m(H, W, CV_32F);
    std::memcpy(m.data, p, sizeof(float) * (size_t)W * H);
    return m;
}
}  // namespace

extern "C" {

// PostProcess on (depth, score, plane): depth and score are replaced in place.
void rhh_postprocess(int W, int H, float *depth, float *score, const double *plane, float min_depth,
                     float max_depth, float min_score) {
    dense::DepthmapEstimatorResult r;
    r.depth = map_f32(depth, W, H);
    r.score = map_f32(score, W, H);
    r.plane = cv::Mat(H, W, CV_64FC3);
    std::memcpy(r.plane.data, plane, sizeof(double) * 3 * (size_t)W * H);
    cv::Mat bearings(H, W, CV_64FC3, cv::Scalar(0));
    dense::ComputeBearingTable(bearings);
    cv::Matx33d R = cv::Matx33d::eye();
    cv::Vec3d t;
    dense::PostProcess(bearings, &r, R, t, min_depth, max_depth, min_score);
    std::memcpy(depth, r.depth.data, sizeof(float) * (size_t)W * H);
    std::memcpy(score, r.score.data, sizeof(float) * (size_t)W * H);
}

// Clean of the centre (n / 2) of n depth maps with world->camera poses R (n x 9), t (n x 3).
void rhh_clean(int W, int H, int n, const float *const *depths, const double *R, const double *t, float thr,
               int min_views, float *out) {
    dense::DepthmapCleaner c;
    c.SetDepthQueueSize(n);
    c.SetMinConsistentViews(min_views);
    c.SetSameDepthThreshold(thr);
    for (int k = 0; k < n; ++k) {
        dense::DepthmapEstimatorResult r;
        r.depth = map_f32(depths[k], W, H);
        r.R = cv::Matx33d(R + 9 * k);
        r.t = cv::Vec3d(t[3 * k], t[3 * k + 1], t[3 * k + 2]);
        c.AddView(&r);
    }
    dense::DepthmapCleanerResult res;
    c.Clean(&res);
    std::memcpy(out, res.cleaned_depth.data, sizeof(float) * (size_t)W * H);
}

// Prune of the head (map 0) against maps 1..n-1; returns the point count
// (at most cap are written) and the head's pruned depth.
int rhh_prune(int W, int H, int n, const float *const *depths, const double *R, const double *t,
              const unsigned char *bgr, float thr, float *pruned, double *xyz, unsigned char *colors, int *ij,
              int cap) {
    dense::DepthmapPruner p;
    p.SetDepthQueueSize(n);
    p.SetSameDepthThreshold(thr);
    for (int k = 0; k < n; ++k) {
        dense::DepthmapCleanerResult cr;
        cr.cleaned_depth = map_f32(depths[k], W, H);
        cr.R = cv::Matx33d(R + 9 * k);
        cr.t = cv::Vec3d(t[3 * k], t[3 * k + 1], t[3 * k + 2]);
        cv::Mat rgb(H, W, CV_8UC3, cv::Scalar(0));
        if (bgr && k == 0) std::memcpy(rgb.data, bgr, (size_t)W * H * 3);
        p.AddView(&cr, rgb);
    }
    dense::DepthmapPrunerResult res;
    p.Prune(&res);
    std::memcpy(pruned, res.pruned_depth.data, sizeof(float) * (size_t)W * H);
    const int m = (int)res.points3d.size();
    for (int q = 0; q < m && q < cap; ++q) {
        for (int a = 0; a < 3; ++a) {
            xyz[3 * q + a] = res.points3d[q][a];
            colors[3 * q + a] = res.colors[q][a];
        }
        ij[2 * q] = res.keypts[q][0];
        ij[2 * q + 1] = res.keypts[q][1];
    }
    return m;
}

}  // extern "C"
