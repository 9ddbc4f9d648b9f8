// pm_dense.hpp -- C++ host interface mirroring the reference's dense
// densification classes (src/openvslam/depthmap.h:122-291) on top of the C ABI
// in pm_gb300.h.
//
// Same class and method names, argument meaning and queue semantics as
// dense::DepthmapEstimator, dense::DepthmapCleaner and dense::DepthmapPruner,
// so the reference's densification thread (depthmap_computation_module.cc:
// 364-414) and fusion thread (dense_pointcloud_module.cc:115-143) can drive
// it unchanged apart from the matrix/image types.  OpenCV is not a dependency:
// images are row-major byte buffers and poses are FP64 arrays; an adapter
// from cv::Mat / cv::Matx33d wraps their data pointers without copies.
//
// Differences from the reference, all deliberate:
//   - errors are reported by return values (the reference prints and goes on);
//   - device memory is allocated once per estimator, not per keyframe;
//   - random numbers are Philox keyed by (seed, keyframe), so runs repeat;
//   - the sources are all views other than the centre (the reference's GPU
//     path is limited to exactly two, PatchMatchCuda.cu:11-18).
#pragma once

#include <array>
#include <cstdint>
#include <memory>
#include <vector>

#include "pm_gb300.h"

namespace dense {

using Matx33d = std::array<double, 9>;  // row-major
using Vec3d = std::array<double, 3>;
using Vec3b = std::array<uint8_t, 3>;
using Vec2i = std::array<int, 2>;

// Owned row-major image/map (the part of cv::Mat the path uses).
template <class T, int C = 1>
struct Map {
    int rows = 0, cols = 0;
    std::vector<T> data;
    Map() = default;
    Map(int r, int c, T fill = T()) : rows(r), cols(c), data((size_t)r * c * C, fill) {}
    T &at(int i, int j, int ch = 0) { return data[((size_t)i * cols + j) * C + ch]; }
    const T &at(int i, int j, int ch = 0) const { return data[((size_t)i * cols + j) * C + ch]; }
    bool empty() const { return data.empty(); }
};
using MatU8 = Map<uint8_t>;
using MatU8C3 = Map<uint8_t, 3>;
using MatF = Map<float>;
using MatF3 = Map<float, 3>;
using MatI = Map<int32_t>;

// depthmap.h:71-79
struct DepthmapEstimatorResult {
    MatF depth;    // 0 = invalid
    MatF3 plane;   // camera-frame plane vectors (pi . X = 1)
    MatF score;
    MatI nghbr;    // best source (1-based view index, like the reference's "other")
    MatF3 normal;  // unit normals facing the camera
    Matx33d R{};
    Vec3d t{};
};

// depthmap.h:204-210
struct DepthmapCleanerResult {
    MatF cleaned_depth;
    Matx33d R{};
    Vec3d t{};
};

// depthmap.h:243-252
struct DepthmapPrunerResult {
    MatF pruned_depth;
    std::vector<Vec3d> points3d;
    std::vector<Vec3b> colors;
    std::vector<Vec2i> keypts;
    Matx33d R{};
    Vec3d t{};
};

// Status of the last failing call (pm_* status code and message).
struct Status {
    int code = PM_OK;
    const char *message = "";
    explicit operator bool() const { return code == PM_OK; }
};

class DepthmapEstimator {
   public:
    explicit DepthmapEstimator(int device = 0);
    ~DepthmapEstimator();
    DepthmapEstimator(const DepthmapEstimator &) = delete;
    DepthmapEstimator &operator=(const DepthmapEstimator &) = delete;

    // depthmap.cc:218-236.  Img/mask: rows x cols bytes (mask may be empty).
    void AddView(const Matx33d &R, const Vec3d &t, const MatU8 &Img, const MatU8 &mask,
                 const std::vector<Vec3d> &landmarks, double maxd, double mind);
    int PopHeadUnlessOne();                          // depthmap.cc:241-254
    void reset();                                    // depthmap.cc:256-282
    bool IsReadyForCompute() const;                  // depthmap.cc:312-314
    bool SetMinImagesCompute(int min_images_compute);
    void SetDepthRange(double min_depth, double max_depth, int num_depth_planes);
    void SetPatchMatchIterations(int n);
    void SetPatchSize(int size);                     // patch_half = size - 2
    void SetMinPatchSD(float sd);
    void SetMinScore(double min_score);
    // Extensions: view combination, seam handling and the Philox seed.
    void SetCombine(int mode, int top_k);
    void SetSeam(int seam);
    void SetSeed(uint32_t seed);

    // depthmap.cc:541-806: densify the centre view against the others.
    Status ComputePatchMatch(DepthmapEstimatorResult *result);

   private:
    struct Impl;
    std::unique_ptr<Impl> d_;
};

class DepthmapCleaner {
   public:
    explicit DepthmapCleaner(int device = 0);
    ~DepthmapCleaner();
    DepthmapCleaner(const DepthmapCleaner &) = delete;
    DepthmapCleaner &operator=(const DepthmapCleaner &) = delete;
    int PopHeadUnlessOne();
    void reset();
    void SetSameDepthThreshold(float t);
    void SetMinConsistentViews(int n);
    void SetDepthQueueSize(int n);
    void SetReprojectionPixels(float px);  // extension: round-trip test (0 = off, as the reference)
    void AddView(const DepthmapEstimatorResult *result);
    bool IsReadyForCompute() const;
    Status Clean(DepthmapCleanerResult *result);  // depthmap.cc:1320-1377

   private:
    struct Impl;
    std::unique_ptr<Impl> d_;
};

class DepthmapPruner {
   public:
    explicit DepthmapPruner(int device = 0);
    ~DepthmapPruner();
    DepthmapPruner(const DepthmapPruner &) = delete;
    DepthmapPruner &operator=(const DepthmapPruner &) = delete;
    void SetSameDepthThreshold(float t);
    void SetMinViews(int min_views);
    void SetDepthQueueSize(int n);
    int PopHead();
    void reset();
    void AddView(const DepthmapCleanerResult *cleaned_result, const MatU8C3 &rgb);
    bool IsReadyForCompute() const;
    Status Prune(DepthmapPrunerResult *result);  // depthmap.cc:1535-1696

   private:
    struct Impl;
    std::unique_ptr<Impl> d_;
};

}  // namespace dense
