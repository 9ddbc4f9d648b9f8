// Harness that runs the reference's own CUDA kernels (PatchMatchCuda.cu,
// compiled unmodified into oracle/_ref/refpm_sm103a.fatbin) through the CUDA
// driver API.  TEST INFRASTRUCTURE ONLY: it exists to pin the oracle and to
// compare the product against the reference's GPU path.  It contains no code
// from the reference: it allocates the buffers, creates the three texture
// objects and fills the constant symbols the way the reference's host code
// intends (PatchMatchCuda.cu:697-797,885-912; depthmap.cc:557-725), and
// launches the reference kernels with the reference's launch shapes.
//
// Build (on any machine with nvcc): nvcc -shared -Xcompiler -fPIC -o libref_harness.so ref_harness.cu -lcuda
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

struct Harness {
    CUmodule mod = nullptr;
    CUfunction f_bear = nullptr, f_seed = nullptr, f_rdepth = nullptr, f_rplane = nullptr, f_score = nullptr,
               f_pass = nullptr;
    int W = 0, H = 0;
    float *d_bear = nullptr, *d_depth = nullptr, *d_plane = nullptr, *d_score = nullptr;
    float *d_img[3] = {};
    size_t pitch = 0;
    void *d_states = nullptr;
    cudaTextureObject_t tex[3] = {};
    cudaTextureObject_t *d_texs = nullptr;
    std::string err;
};
Harness g;

int set_err(const char *what, int code) {
    g.err = std::string(what) + " (" + std::to_string(code) + ")";
    return code ? code : -1;
}

#define CU(x)                                   \
    do {                                        \
        CUresult r_ = (x);                      \
        if (r_ != CUDA_SUCCESS) return set_err(#x, (int)r_); \
    } while (0)
#define RT(x)                                   \
    do {                                        \
        cudaError_t r_ = (x);                   \
        if (r_ != cudaSuccess) return set_err(#x, (int)r_); \
    } while (0)

// Find a kernel of the module whose name contains `needle`.
int find(const char *needle, CUfunction *out) {
    unsigned n = 0;
    CU(cuModuleGetFunctionCount(&n, g.mod));
    std::vector<CUfunction> fs(n);
    CU(cuModuleEnumerateFunctions(fs.data(), n, g.mod));
    for (CUfunction f : fs) {
        const char *name = nullptr;
        CU(cuFuncGetName(&name, f));
        if (name && std::strstr(name, needle)) {
            *out = f;
            return 0;
        }
    }
    return set_err(needle, 404);
}

int upload_const(const char *sym, const float *v, size_t n) {
    CUdeviceptr p;
    size_t bytes;
    CU(cuModuleGetGlobal(&p, &bytes, g.mod, sym));
    if (bytes != n * sizeof(float)) return set_err(sym, 500);
    CU(cuMemcpyHtoD(p, v, bytes));
    return 0;
}

void free_buffers() {
    for (int k = 0; k < 3; ++k) {
        if (g.tex[k]) cudaDestroyTextureObject(g.tex[k]);
        g.tex[k] = 0;
        if (g.d_img[k]) cudaFree(g.d_img[k]);
        g.d_img[k] = nullptr;
    }
    cudaFree(g.d_texs);
    cudaFree(g.d_bear);
    cudaFree(g.d_depth);
    cudaFree(g.d_plane);
    cudaFree(g.d_score);
    cudaFree(g.d_states);
    g.d_texs = nullptr;
    g.d_bear = g.d_depth = g.d_plane = g.d_score = nullptr;
    g.d_states = nullptr;
}

int launch(CUfunction f, int gx, int gy, int bx, int by, unsigned smem, void **args) {
    CU(cuLaunchKernel(f, gx, gy, 1, bx, by, 1, smem, nullptr, args, nullptr));
    RT(cudaDeviceSynchronize());
    return 0;
}

}  // namespace

extern "C" {

const char *rh_error() { return g.err.c_str(); }

int rh_load(const char *fatbin_path) {
    RT(cudaFree(nullptr));  // create the primary context
    CU(cuModuleLoad(&g.mod, fatbin_path));
    if (find("ComputeBearingsEquirect_", &g.f_bear)) return -1;
    if (find("ComputeRandomSeed_", &g.f_seed)) return -1;
    if (find("ComputeRandomDepthmap_", &g.f_rdepth)) return -1;
    if (find("ComputeRandomPlanemap_", &g.f_rplane)) return -1;
    if (find("ScorePlaneDepth_", &g.f_score)) return -1;
    if (find("PatchMatchRedBlackPass_", &g.f_pass)) return -1;
    return 0;
}

// images: three H*W float images (reference, source 1, source 2); poses as
// the reference host code builds them (depthmap.cc:577-665): R12/t12 and
// R13/t13 are the sources' world->camera poses, R1inv/t1inv the reference's
// camera->world pose.  W must be a multiple of 64 and H of 32 (launch shapes).
int rh_setup(int W, int H, const float *img0, const float *img1, const float *img2, const float *R12,
             const float *t12, const float *R13, const float *t13, const float *R1inv, const float *t1inv) {
    if (!g.mod) return set_err("not loaded", 1);
    if (W % 64 || H % 32) return set_err("W must be a multiple of 64 and H of 32", 2);
    free_buffers();
    g.W = W;
    g.H = H;
    const size_t N = (size_t)W * H;
    RT(cudaMalloc(&g.d_bear, N * 12));
    RT(cudaMalloc(&g.d_depth, N * 4));
    RT(cudaMalloc(&g.d_plane, N * 12));
    RT(cudaMalloc(&g.d_score, N * 4));
    RT(cudaMalloc(&g.d_states, N * 64));
    RT(cudaMemset(g.d_depth, 0, N * 4));
    RT(cudaMemset(g.d_plane, 0, N * 12));
    RT(cudaMemset(g.d_score, 0, N * 4));
    const float *imgs[3] = {img0, img1, img2};
    for (int k = 0; k < 3; ++k) {
        RT(cudaMallocPitch((void **)&g.d_img[k], &g.pitch, sizeof(float) * W, H));
        RT(cudaMemcpy2D(g.d_img[k], g.pitch, imgs[k], sizeof(float) * W, sizeof(float) * W, H,
                        cudaMemcpyHostToDevice));
        cudaResourceDesc rd;
        std::memset(&rd, 0, sizeof rd);
        rd.resType = cudaResourceTypePitch2D;
        rd.res.pitch2D.devPtr = g.d_img[k];
        rd.res.pitch2D.desc = cudaCreateChannelDesc<float>();
        rd.res.pitch2D.width = W;
        rd.res.pitch2D.height = H;
        rd.res.pitch2D.pitchInBytes = g.pitch;
        cudaTextureDesc td;
        std::memset(&td, 0, sizeof td);
        td.addressMode[0] = cudaAddressModeWrap;  // as the reference requests
        td.addressMode[1] = cudaAddressModeWrap;
        td.filterMode = k == 0 ? cudaFilterModePoint : cudaFilterModeLinear;
        td.readMode = cudaReadModeElementType;
        td.normalizedCoords = 0;
        RT(cudaCreateTextureObject(&g.tex[k], &rd, &td, nullptr));
    }
    RT(cudaMalloc(&g.d_texs, sizeof(cudaTextureObject_t) * 3));
    RT(cudaMemcpy(g.d_texs, g.tex, sizeof(cudaTextureObject_t) * 3, cudaMemcpyHostToDevice));
    int rc = 0;
    rc = rc ? rc : upload_const("R12_", R12, 9);
    rc = rc ? rc : upload_const("t12_", t12, 3);
    rc = rc ? rc : upload_const("R13_", R13, 9);
    rc = rc ? rc : upload_const("t13_", t13, 3);
    rc = rc ? rc : upload_const("R1_inv_", R1inv, 9);
    rc = rc ? rc : upload_const("t1_inv_", t1inv, 3);
    const float sc = 50.0f, sx = 5.0f;
    const float cf = 1.0f / (2 * sc * sc), xf = 1.0f / (2 * sx * sx);
    rc = rc ? rc : upload_const("dcolor_sigma", &sc, 1);
    rc = rc ? rc : upload_const("dx_sigma", &sx, 1);
    rc = rc ? rc : upload_const("dcolor_factor", &cf, 1);
    rc = rc ? rc : upload_const("dx_factor", &xf, 1);
    if (rc) return rc;
    // bearing table (16x16 blocks, PatchMatchCuda.cu:429-433)
    void *args[] = {&g.d_bear, &g.W, &g.H};
    return launch(g.f_bear, W / 16, H / 16, 16, 16, 0, args);
}

int rh_bearings(float *out) {
    RT(cudaMemcpy(out, g.d_bear, (size_t)g.W * g.H * 12, cudaMemcpyDeviceToHost));
    return 0;
}

// ScorePlaneDepth_ on caller planes (H*W*3): 32x32 blocks (PatchMatchCuda.cu:538-546).
int rh_score(const float *planes, float *scores, float fill) {
    const size_t N = (size_t)g.W * g.H;
    RT(cudaMemcpy(g.d_plane, planes, N * 12, cudaMemcpyHostToDevice));
    std::vector<float> f(N, fill);
    RT(cudaMemcpy(g.d_score, f.data(), N * 4, cudaMemcpyHostToDevice));
    int ph = 5;
    void *args[] = {&ph, &g.d_score, &g.d_plane, &g.d_depth, &g.d_bear, &g.W, &g.H, &g.d_texs};
    int rc = launch(g.f_score, g.W / 32, g.H / 32, 32, 32, 36 * 36 * 4, args);
    if (rc) return rc;
    RT(cudaMemcpy(scores, g.d_score, N * 4, cudaMemcpyDeviceToHost));
    return 0;
}

// The reference GPU pipeline of one keyframe: clock-seeded XORWOW states,
// random depth/plane maps, init scoring, then `iterations` red/black passes
// (PatchMatchCuda.cu:568-663; depthmap.cc:557-725, without the host seeding).
int rh_run(int iterations, float min_depth, float max_depth, float *depth, float *plane, float *score) {
    const size_t N = (size_t)g.W * g.H;
    int ph = 5;
    {
        void *a[] = {&g.d_states, &g.W, &g.H};
        if (launch(g.f_seed, g.W / 8, g.H / 8, 8, 8, 0, a)) return -1;
    }
    {
        void *a[] = {&g.d_depth, &g.W, &g.H, &min_depth, &max_depth, &g.d_states};
        if (launch(g.f_rdepth, g.W / 16, g.H / 16, 16, 16, 0, a)) return -1;
    }
    {
        void *a[] = {&g.d_plane, &g.d_depth, &g.d_bear, &g.W, &g.H, &g.d_states};
        if (launch(g.f_rplane, g.W / 16, g.H / 16, 16, 16, 0, a)) return -1;
    }
    {
        std::vector<float> f(N, -1.0f);
        RT(cudaMemcpy(g.d_score, f.data(), N * 4, cudaMemcpyHostToDevice));
        void *a[] = {&ph, &g.d_score, &g.d_plane, &g.d_depth, &g.d_bear, &g.W, &g.H, &g.d_texs};
        if (launch(g.f_score, g.W / 32, g.H / 32, 32, 32, 36 * 36 * 4, a)) return -1;
    }
    for (int it = 0; it < iterations; ++it) {
        for (int off = 0; off < 2; ++off) {
            void *a[] = {&ph, &g.d_score, &g.d_depth, &g.d_plane, &g.d_states, &g.d_bear, &g.d_texs, &g.W, &g.H, &off};
            if (launch(g.f_pass, (g.W / 32) / 2, g.H / 32, 32, 32, 36 * 36 * 4, a)) return -1;
        }
    }
    if (depth) RT(cudaMemcpy(depth, g.d_depth, N * 4, cudaMemcpyDeviceToHost));
    if (plane) RT(cudaMemcpy(plane, g.d_plane, N * 12, cudaMemcpyDeviceToHost));
    if (score) RT(cudaMemcpy(score, g.d_score, N * 4, cudaMemcpyDeviceToHost));
    return 0;
}

// Time the reference's red/black passes alone (ms per iteration), from the
// current state.
int rh_time_passes(int iterations, float *ms_per_iteration) {
    int ph = 5;
    cudaEvent_t e0, e1;
    RT(cudaEventCreate(&e0));
    RT(cudaEventCreate(&e1));
    RT(cudaEventRecord(e0, nullptr));
    for (int it = 0; it < iterations; ++it)
        for (int off = 0; off < 2; ++off) {
            void *a[] = {&ph, &g.d_score, &g.d_depth, &g.d_plane, &g.d_states, &g.d_bear, &g.d_texs, &g.W, &g.H, &off};
            CU(cuLaunchKernel(g.f_pass, (g.W / 32) / 2, g.H / 32, 1, 32, 32, 1, 36 * 36 * 4, nullptr, a, nullptr));
            RT(cudaDeviceSynchronize());  // the reference synchronises after every pass
        }
    RT(cudaEventRecord(e1, nullptr));
    RT(cudaEventSynchronize(e1));
    float ms = 0.f;
    RT(cudaEventElapsedTime(&ms, e0, e1));
    *ms_per_iteration = iterations ? ms / iterations : 0.f;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return 0;
}

void rh_release() {
    free_buffers();
    if (g.mod) cuModuleUnload(g.mod);
    g.mod = nullptr;
}

}  // extern "C"

// Texture border probe (our own kernel): samples a linear-filtered float
// texture created with the reference's descriptor at caller coordinates, to
// record what the hardware does past the image edge with unnormalised
// coordinates and the wrap address mode.
__global__ void probe_tex_kernel(cudaTextureObject_t t, const float *xy, int n, float *out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) out[k] = tex2D<float>(t, xy[2 * k], xy[2 * k + 1]);
}

extern "C" int rh_probe_texture(int source, const float *xy, int n, float *out) {
    if (source < 0 || source > 2 || !g.tex[source] || n <= 0) return set_err("bad probe", 3);
    float *dxy = nullptr, *dout = nullptr;
    RT(cudaMalloc(&dxy, (size_t)n * 8));
    RT(cudaMalloc(&dout, (size_t)n * 4));
    RT(cudaMemcpy(dxy, xy, (size_t)n * 8, cudaMemcpyHostToDevice));
    probe_tex_kernel<<<(n + 255) / 256, 256>>>(g.tex[source], dxy, n, dout);
    RT(cudaGetLastError());
    RT(cudaMemcpy(out, dout, (size_t)n * 4, cudaMemcpyDeviceToHost));
    cudaFree(dxy);
    cudaFree(dout);
    return 0;
}
