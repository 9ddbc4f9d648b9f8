// Point fusion without any device allocation: pm_fuse_noalloc.
//
// Some callers cannot allocate device memory at the moment they fuse: a SLAM
// process whose device memory is owned by an external pool or arena, a
// real-time thread that must not enter the CUDA allocator (its latency is
// unbounded and it may synchronise the device), or code that has already
// handed its whole HBM budget to resident keyframes.  For them this entry
// point runs the same fusion kernels as pm_fuse on caller-owned device
// buffers, with its working memory in file-scope device arrays of a fixed
// maximum size (PM_FUSE_NOALLOC_MAX_PIXELS pixels, about 20 MB), which every
// GPU that loads the library holds until the process exits.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "pm_gb300.h"
#include "pm_kernels.h"

namespace {

constexpr size_t kMaxPix = PM_FUSE_NOALLOC_MAX_PIXELS;
constexpr int kMaxW = PM_FUSE_NOALLOC_MAX_WIDTH, kMaxH = PM_FUSE_NOALLOC_MAX_HEIGHT;
// compaction blocks of the largest image, plus the scan's total slot
constexpr size_t kBlocks = (kMaxPix + pm::kCompactBlock - 1) / pm::kCompactBlock + 1;

// All working memory of one fusion, shared by every call on a device.
struct FuseScratch {
    uint8_t alive[kMaxPix];
    int8_t cls[kMaxPix];
    int target[kMaxPix];
    unsigned first[kMaxPix];
    unsigned block_counts[kBlocks];
    float2 row_trig[kMaxH];
    float2 col_trig[kMaxW];
};

static __device__ __align__(256) FuseScratch g_fuse_scratch;

constexpr int kMaxDevices = 64;
std::mutex g_mu;
// per device: the device address of g_fuse_scratch (from cudaGetSymbolAddress)
// and the image size whose bearing tables it holds
FuseScratch *g_scratch_dev[kMaxDevices] = {};
int g_trig_w[kMaxDevices] = {}, g_trig_h[kMaxDevices] = {};
float2 g_row_host[kMaxH], g_col_host[kMaxW];   // host staging of the bearing tables (guarded by g_mu)

}  // namespace

extern "C" int pm_fuse_noalloc(int W, int H, int n, float *const *depths, const double *R, const double *t,
                               const uint8_t *bgr, float thr, float *pruned, float *xyz, uint8_t *bgr_out,
                               int32_t *ij, unsigned *count, void *stream) {
    if (!depths || !R || !t || !pruned || !xyz || !count) return PM_EINVAL;
    if (W < 2 || H < 2 || W > kMaxW || H > kMaxH || (size_t)W * H > kMaxPix) return PM_EINVAL;
    if (n < 1 || n > pm::kMaxFilterViews || !(thr > 0.0f)) return PM_EINVAL;
    for (int k = 0; k < n; ++k) {
        if (!depths[k]) return PM_EINVAL;
        for (int a = 0; a < 9; ++a)
            if (!std::isfinite(R[9 * k + a])) return PM_EINVAL;
        for (int a = 0; a < 3; ++a)
            if (!std::isfinite(t[3 * k + a])) return PM_EINVAL;
    }
    // a launch error left pending by earlier work on this thread is not this call's
    cudaGetLastError();
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return PM_ECUDA;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    std::lock_guard<std::mutex> lock(g_mu);
    // set-up, once per device, with that device current: the host-side name
    // g_fuse_scratch is only a stand-in, the kernels need the device address
    if (!g_scratch_dev[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_fuse_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            return PM_ECUDA;
        }
        g_scratch_dev[dev] = static_cast<FuseScratch *>(p);
    }
    FuseScratch *s = g_scratch_dev[dev];

    // bearing tables (same FP64 rounding as pm_fuse), copied from host memory
    // on the first call of each image size on this device only
    if (g_trig_w[dev] != W || g_trig_h[dev] != H) {
        for (int i = 0; i < H; ++i) {
            const double lat = -M_PI * ((double)i / H - 0.5);
            g_row_host[i] = make_float2((float)std::cos(lat), (float)std::sin(lat));
        }
        for (int j = 0; j < W; ++j) {
            const double lon = 2.0 * M_PI * ((double)j / W - 0.5);
            g_col_host[j] = make_float2((float)std::sin(lon), (float)std::cos(lon));
        }
        // pageable sources: staged before the calls return, so the host tables may change afterwards
        if (cudaMemcpyAsync(s->row_trig, g_row_host, sizeof(float2) * H, cudaMemcpyHostToDevice, st) != cudaSuccess ||
            cudaMemcpyAsync(s->col_trig, g_col_host, sizeof(float2) * W, cudaMemcpyHostToDevice, st) != cudaSuccess) {
            cudaGetLastError();
            g_trig_w[dev] = g_trig_h[dev] = 0;
            return PM_ECUDA;
        }
        g_trig_w[dev] = W;
        g_trig_h[dev] = H;
    }
    pm::FuseArgs a{};
    a.W = W;
    a.H = H;
    for (int k = 0; k < n; ++k) a.depths[k] = depths[k];  // by value, in the kernel parameters
    pm::fuse_set_poses(a, n, R, t);                      // FP64-composed, as pm_fuse
    a.row_trig = s->row_trig;
    a.col_trig = s->col_trig;
    a.thr = thr;
    a.alive = s->alive;
    a.target = s->target;
    a.cls = s->cls;
    a.first = s->first;  // reset to all-ones before every view by launch_fuse
    a.pruned = pruned;
    a.block_counts = s->block_counts;
    a.bgr = bgr;
    a.xyz = xyz;
    a.bgr_out = bgr ? bgr_out : nullptr;
    a.ij_out = ij;
    a.count = count;
    // every scratch entry a launch reads is written earlier in the same call
    // (alive/pruned by the init kernel, cls/target by classify, first by the
    // memset, block_counts by the count kernel), so nothing from the previous
    // call leaks in
    return pm::launch_fuse(st, a) == cudaSuccess ? PM_OK : PM_ECUDA;
}
