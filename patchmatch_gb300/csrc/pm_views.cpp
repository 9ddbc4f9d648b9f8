// Host-side neighbour geometry of the densification thread: the view test
// that decides whether a new keyframe joins the densification window, and the
// depth interval taken from the keyframe's landmarks.  FP64, no device work.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <unordered_set>
#include <vector>

#include "pm_gb300.h"

extern "C" {

// depthmap_computation_module::score_view (depthmap_computation_module.cc:147-198):
// the fraction of landmarks seen by both keyframes whose triangulation angle
// between the two camera centres lies in (pi/60, pi/6).  Common landmarks are
// matched by id; the reference intersects its two landmark lists with a
// comparator on the squared norm over unsorted ranges, which only approximates
// an identity match.  No common landmark gives 0 (the reference divides 0 by 0).
int pm_score_view(const double prev_center[3], const double cur_center[3], const uint64_t *prev_ids, int n_prev,
                  const uint64_t *cur_ids, const double *cur_xyz, int n_cur, float *score, int *n_common) {
    if (!prev_center || !cur_center || !score || n_prev < 0 || n_cur < 0 || (n_prev && !prev_ids) ||
        (n_cur && (!cur_ids || !cur_xyz)))
        return PM_EINVAL;
    const double theta_min = M_PI / 60, theta_max = M_PI / 6;
    std::unordered_set<uint64_t> prev(prev_ids, prev_ids + n_prev);
    std::unordered_set<uint64_t> seen;
    int common = 0;
    float s = 0.0f;
    for (int k = 0; k < n_cur; ++k) {
        if (!prev.count(cur_ids[k]) || !seen.insert(cur_ids[k]).second) continue;
        const double *lm = cur_xyz + 3 * (size_t)k;
        double dp[3], dc[3];
        for (int a = 0; a < 3; ++a) {
            dp[a] = prev_center[a] - lm[a];
            dc[a] = cur_center[a] - lm[a];
        }
        const double nom = dc[0] * dp[0] + dc[1] * dp[1] + dc[2] * dp[2];
        const double v1 = dc[0] * dc[0] + dc[1] * dc[1] + dc[2] * dc[2];
        const double v2 = dp[0] * dp[0] + dp[1] * dp[1] + dp[2] * dp[2];
        const double theta = std::acos(nom / std::sqrt(v1 * v2));
        if (theta > theta_min && theta < theta_max) s += 1.0f;
        ++common;
    }
    *score = common ? s / (float)common : 0.0f;
    if (n_common) *n_common = common;
    return PM_OK;
}

// keyframe::computePercentileDepth_10_90 (data/keyframe.cc:428-455) and
// depthmap_computation_module::compute_depth_intervall (:123-131): ranges of
// the landmarks from the camera, sorted; p10 = d[n/10], p90 = d[(n/10)*9];
// the densifier's interval is [1e-5, 1.1 p90] (the reference overrides its
// lower bound).  n = 0 is rejected (the reference indexes an empty vector).
int pm_depth_interval(const double R_cw[9], const double t_cw[3], const double *xyz, int n, double *p10,
                      double *p90, double *min_depth, double *max_depth) {
    if (!R_cw || !t_cw || n <= 0 || !xyz) return PM_EINVAL;
    std::vector<float> d;
    d.reserve(n);
    for (int k = 0; k < n; ++k) {
        const double *p = xyz + 3 * (size_t)k;
        const double X = R_cw[0] * p[0] + R_cw[1] * p[1] + R_cw[2] * p[2] + t_cw[0];
        const double Y = R_cw[3] * p[0] + R_cw[4] * p[1] + R_cw[5] * p[2] + t_cw[1];
        const double Z = R_cw[6] * p[0] + R_cw[7] * p[1] + R_cw[8] * p[2] + t_cw[2];
        d.push_back((float)std::sqrt(X * X + Y * Y + Z * Z));  // std::vector<float> in the reference
    }
    std::sort(d.begin(), d.end());
    const double a = d[(size_t)n / 10], b = d[(size_t)n / 10 * 9];
    if (p10) *p10 = a;
    if (p90) *p90 = b;
    if (min_depth) *min_depth = 1e-5;
    if (max_depth) *max_depth = b * 1.1;
    return PM_OK;
}

}  // extern "C"
