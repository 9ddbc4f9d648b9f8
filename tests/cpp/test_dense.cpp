// End-to-end test of the C++ mirror of the reference's dense classes
// (include/pm_dense.hpp): keyframes along a path through a textured room go
// through DepthmapEstimator (3-view windows), DepthmapCleaner (5 results) and
// DepthmapPruner (queue of 5), the way depthmap_computation_module.cc:364-414
// and dense_pointcloud_module.cc:115-175 drive the reference classes.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "pm_dense.hpp"
#include "pm_scene.h"

#define CHECK(c)                                                          \
    do {                                                                  \
        if (!(c)) {                                                       \
            std::fprintf(stderr, "CHECK failed %s:%d: %s\n", __FILE__, __LINE__, #c); \
            std::exit(1);                                                 \
        }                                                                 \
    } while (0)

int main() {
    const int W = 512, H = 256, N = 12;
    pm_scene *sc = pm_scene_create(PM_SCENE_ROOM_OBJECTS, 7);
    CHECK(sc);
    std::vector<dense::Matx33d> Rs(N);
    std::vector<dense::Vec3d> ts(N);
    std::vector<dense::MatU8> grays(N);
    std::vector<dense::MatU8C3> rgbs(N);
    std::vector<std::vector<float>> gts(N);
    for (int k = 0; k < N; ++k) {
        double R[9], t[3];
        CHECK(pm_scene_trajectory_pose(sc, 3, 8, 10.0, 0.4 + 0.2 * k, R, t) == 0);
        for (int a = 0; a < 9; ++a) Rs[k][a] = R[a];
        for (int a = 0; a < 3; ++a) ts[k][a] = t[a];
        grays[k] = dense::MatU8(H, W);
        rgbs[k] = dense::MatU8C3(H, W);
        gts[k].resize((size_t)W * H);
        CHECK(pm_scene_render(sc, R, t, W, H, 2, 0.f, 0, nullptr, grays[k].data.data(), rgbs[k].data.data(),
                              gts[k].data(), nullptr) == 0);
    }
    dense::DepthmapEstimator est;
    dense::DepthmapCleaner cleaner;
    dense::DepthmapPruner pruner;
    est.SetMinImagesCompute(3);
    est.SetPatchSize(7);
    est.SetPatchMatchIterations(8);
    est.SetMinPatchSD(0);
    est.SetMinScore(0.1);
    cleaner.SetMinConsistentViews(3);
    cleaner.SetDepthQueueSize(5);
    cleaner.SetSameDepthThreshold(0.02f);
    pruner.SetDepthQueueSize(5);
    pruner.SetSameDepthThreshold(0.02f);

    dense::MatU8 nomask;
    int estimated = 0, cleaned = 0, pruned_sets = 0;
    size_t points = 0;
    double acc_sum = 0;
    for (int k = 0; k < N; ++k) {
        std::vector<dense::Vec3d> lms;
        est.AddView(Rs[k], ts[k], grays[k], nomask, lms, 20.0, 0.3);
        if (est.IsReadyForCompute()) {
            dense::DepthmapEstimatorResult r;
            dense::Status st = est.ComputePatchMatch(&r);
            if (!st) std::fprintf(stderr, "ComputePatchMatch: %s\n", st.message);
            CHECK(st);
            const int c = k - 1;  // centre of the 3-view window
            CHECK(r.R == Rs[c] && r.t == ts[c]);
            size_t valid = 0, good = 0;
            for (size_t q = 0; q < r.depth.data.size(); ++q) {
                const float d = r.depth.data[q];
                if (d > 0) {
                    ++valid;
                    good += std::fabs(d - gts[c][q]) / gts[c][q] < 0.02f;
                }
            }
            CHECK(valid > r.depth.data.size() / 2);
            acc_sum += (double)good / valid;
            ++estimated;
            cleaner.AddView(&r);
            est.PopHeadUnlessOne();
        }
        if (cleaner.IsReadyForCompute()) {
            dense::DepthmapCleanerResult cr;
            CHECK(cleaner.Clean(&cr));
            ++cleaned;
            size_t kept = 0;
            for (float d : cr.cleaned_depth.data) kept += d > 0;
            CHECK(kept > 0);
            cleaner.PopHeadUnlessOne();
            // the centre result's keyframe: window index k-3 (see run() of the reference)
            pruner.AddView(&cr, rgbs[k - 3]);
            if (pruner.IsReadyForCompute()) {
                dense::DepthmapPrunerResult pr;
                CHECK(pruner.Prune(&pr));
                CHECK(pr.points3d.size() == pr.keypts.size() && pr.colors.size() == pr.points3d.size());
                points += pr.points3d.size();
                ++pruned_sets;
                pruner.PopHead();
            }
        }
    }
    CHECK(estimated == N - 2);
    CHECK(cleaned == N - 2 - 4);
    CHECK(pruned_sets == cleaned - 4 && points > 0);
    std::printf("estimated %d cleaned %d pruned %d points %zu mean acc2%% %.3f\n", estimated, cleaned, pruned_sets,
                points, acc_sum / estimated);
    CHECK(acc_sum / estimated > 0.6);
    pm_scene_destroy(sc);
    return 0;
}
