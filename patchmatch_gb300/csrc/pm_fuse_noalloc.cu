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
constexpr size_t kBlocks = (kMaxPix + 1023) / 1024 + 1;

// All working memory of one fusion, shared by every call on a device.
struct FuseScratch {
    uint8_t alive[kMaxPix];
    int8_t cls[kMaxPix];
    int target[kMaxPix];
    unsigned first[kMaxPix];
    unsigned block_counts[kBlocks];
    unsigned count;
    float *depths[pm::kMaxFilterViews];
    float2 row_trig[kMaxH];
    float2 col_trig[kMaxW];
};

static __device__ __align__(256) FuseScratch g_fuse_scratch;

constexpr int kMaxDevices = 64;
std::mutex g_mu;
FuseScratch *g_scratch_dev[kMaxDevices] = {};  // device address per device, from cudaGetSymbolAddress
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

    // bearing tables and the depth-map pointer table (same FP64 rounding as pm_fuse)
    for (int i = 0; i < H; ++i) {
        const double lat = -M_PI * ((double)i / H - 0.5);
        g_row_host[i] = make_float2((float)std::cos(lat), (float)std::sin(lat));
    }
    for (int j = 0; j < W; ++j) {
        const double lon = 2.0 * M_PI * ((double)j / W - 0.5);
        g_col_host[j] = make_float2((float)std::sin(lon), (float)std::cos(lon));
    }
    if (cudaMemcpyAsync(s->row_trig, g_row_host, sizeof(float2) * H, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(s->col_trig, g_col_host, sizeof(float2) * W, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(s->depths, depths, sizeof(float *) * n, cudaMemcpyHostToDevice, st) != cudaSuccess) {
        cudaGetLastError();
        return PM_ECUDA;
    }
    pm::FuseArgs a{};
    a.depths = s->depths;
    a.n = n;
    a.W = W;
    a.H = H;
    for (int k = 1; k < n; ++k) {
        // head camera -> view k, composed in FP64 (as pm_fuse)
        double Md[9];
        for (int r0 = 0; r0 < 3; ++r0)
            for (int c0 = 0; c0 < 3; ++c0)
                Md[3 * r0 + c0] = R[9 * k + 3 * r0] * R[3 * c0] + R[9 * k + 3 * r0 + 1] * R[3 * c0 + 1] +
                                  R[9 * k + 3 * r0 + 2] * R[3 * c0 + 2];
        for (int q = 0; q < 9; ++q) a.M[k][q] = (float)Md[q];
        for (int r0 = 0; r0 < 3; ++r0)
            a.c[k][r0] = (float)(t[3 * k + r0] - (Md[3 * r0] * t[0] + Md[3 * r0 + 1] * t[1] + Md[3 * r0 + 2] * t[2]));
    }
    for (int r0 = 0; r0 < 3; ++r0) {
        for (int c0 = 0; c0 < 3; ++c0) a.Rinv[3 * r0 + c0] = (float)R[3 * c0 + r0];
        a.tw[r0] = (float)(-(R[r0] * t[0] + R[3 + r0] * t[1] + R[6 + r0] * t[2]));
    }
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
    pm::launch_fuse(st, a);
    if (cudaGetLastError() != cudaSuccess) return PM_ECUDA;
    return PM_OK;
}
