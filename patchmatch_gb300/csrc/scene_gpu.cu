// Device renderer of the synthetic scenes (include/pm_scene.h): the same ray
// casting and 4-octave solid value-noise texture as scene.cpp, in FP32, for
// generating large benchmark workloads quickly.
#include <cuda_runtime.h>
#include <stdint.h>

#include "pm_scene.h"

namespace {

struct DevScene {
    float rlo[3], rhi[3];
    int nb, nc;
    float blo[PM_SCENE_MAX_BOXES][3], bhi[PM_SCENE_MAX_BOXES][3];
    float cyl[PM_SCENE_MAX_CYLS][5];
    uint32_t seed;
    float base_freq;
    float Rt[9];  // R_cw^T (camera -> world)
    float C[3];   // camera centre
};

__device__ __forceinline__ uint32_t hash3(int x, int y, int z, uint32_t seed) {
    uint32_t h = seed * 0x27d4eb2du;
    h ^= (uint32_t)x * 0x85ebca6bu;
    h = (h << 13) | (h >> 19);
    h ^= (uint32_t)y * 0xc2b2ae35u;
    h = (h << 17) | (h >> 15);
    h ^= (uint32_t)z * 0x165667b1u;
    h ^= h >> 16; h *= 0x7feb352du; h ^= h >> 15; h *= 0x846ca68bu; h ^= h >> 16;
    return h;
}
__device__ __forceinline__ float lattice(int x, int y, int z, uint32_t s) { return (hash3(x, y, z, s) >> 8) * (1.0f / 16777216.0f); }
__device__ __forceinline__ float fade(float t) { return t * t * t * (t * (t * 6.f - 15.f) + 10.f); }

__device__ float value_noise(float x, float y, float z, uint32_t seed) {
    const float fx = floorf(x), fy = floorf(y), fz = floorf(z);
    const int ix = (int)fx, iy = (int)fy, iz = (int)fz;
    const float ux = fade(x - fx), uy = fade(y - fy), uz = fade(z - fz);
    float c[2][2][2];
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            for (int d = 0; d < 2; ++d) c[a][b][d] = lattice(ix + a, iy + b, iz + d, seed);
    const float x00 = c[0][0][0] + ux * (c[1][0][0] - c[0][0][0]);
    const float x10 = c[0][1][0] + ux * (c[1][1][0] - c[0][1][0]);
    const float x01 = c[0][0][1] + ux * (c[1][0][1] - c[0][0][1]);
    const float x11 = c[0][1][1] + ux * (c[1][1][1] - c[0][1][1]);
    const float y0 = x00 + uy * (x10 - x00), y1 = x01 + uy * (x11 - x01);
    return y0 + uz * (y1 - y0);
}

__device__ float texture(const DevScene &s, const float p[3], uint32_t channel) {
    float sum = 0, amp = 1, norm = 0, f = s.base_freq;
    for (int o = 0; o < 4; ++o) {
        sum += amp * value_noise(p[0] * f + 17.3f * o, p[1] * f - 5.1f * o, p[2] * f + 3.7f * o,
                                 s.seed * 977u + channel * 131u + (uint32_t)o);
        norm += amp;
        amp *= 0.5f;
        f *= 2.0f;
    }
    const float v = 0.5f + (sum / norm - 0.5f) * 2.6f;
    return fminf(1.0f, fmaxf(0.0f, v));
}

__device__ float intersect(const DevScene &s, const float o[3], const float d[3]) {
    float best = 1e30f;
    for (int a = 0; a < 3; ++a) {
        if (fabsf(d[a]) < 1e-12f) continue;
        const float tt = d[a] > 0 ? (s.rhi[a] - o[a]) / d[a] : (s.rlo[a] - o[a]) / d[a];
        if (tt > 0 && tt < best) best = tt;
    }
    for (int k = 0; k < s.nb; ++k) {
        float t0 = -1e30f, t1 = 1e30f;
        bool miss = false;
        for (int a = 0; a < 3; ++a) {
            if (fabsf(d[a]) < 1e-12f) {
                if (o[a] < s.blo[k][a] || o[a] > s.bhi[k][a]) { miss = true; break; }
                continue;
            }
            float ta = (s.blo[k][a] - o[a]) / d[a], tb = (s.bhi[k][a] - o[a]) / d[a];
            if (ta > tb) { const float tmp = ta; ta = tb; tb = tmp; }
            t0 = fmaxf(t0, ta);
            t1 = fminf(t1, tb);
        }
        if (!miss && t0 <= t1 && t0 > 0 && t0 < best) best = t0;
    }
    for (int k = 0; k < s.nc; ++k) {
        const float ox = o[0] - s.cyl[k][0], oz = o[2] - s.cyl[k][1];
        const float A = d[0] * d[0] + d[2] * d[2];
        if (A < 1e-12f) continue;
        const float B = 2 * (ox * d[0] + oz * d[2]), Cc = ox * ox + oz * oz - s.cyl[k][2] * s.cyl[k][2];
        const float disc = B * B - 4 * A * Cc;
        if (disc < 0) continue;
        const float tt = (-B - sqrtf(disc)) / (2 * A);
        if (tt <= 0 || tt >= best) continue;
        const float y = o[1] + tt * d[1];
        if (y < s.cyl[k][3] || y > s.cyl[k][4]) continue;
        best = tt;
    }
    return best;
}

__global__ void render_kernel(const DevScene s, int W, int H, int ss, float noise_sigma, uint32_t noise_seed,
                              uint8_t *gray, float *depth, uint8_t *bgr, float *grayf) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= H || j >= W) return;
    const float kPi = 3.14159265358979323846f;
    float acc = 0.f, accc[3] = {0.f, 0.f, 0.f};
    for (int si = 0; si < ss; ++si)
        for (int sj = 0; sj < ss; ++sj) {
            const float y = i + (ss > 1 ? (si + 0.5f) / ss - 0.5f : 0.0f);
            const float x = j + (ss > 1 ? (sj + 0.5f) / ss - 0.5f : 0.0f);
            const float lon = 2.0f * kPi * (x / W - 0.5f), lat = -kPi * (y / H - 0.5f);
            const float b[3] = {cosf(lat) * sinf(lon), -sinf(lat), cosf(lat) * cosf(lon)};
            float d[3];
            for (int a = 0; a < 3; ++a) d[a] = s.Rt[3 * a] * b[0] + s.Rt[3 * a + 1] * b[1] + s.Rt[3 * a + 2] * b[2];
            const float tt = intersect(s, s.C, d);
            const float p[3] = {s.C[0] + tt * d[0], s.C[1] + tt * d[1], s.C[2] + tt * d[2]};
            acc += texture(s, p, 0);
            if (bgr)
                for (int c = 0; c < 3; ++c) accc[c] += texture(s, p, 1 + c);
        }
    const size_t idx = (size_t)i * W + j;
    if (depth) {
        const float lon = 2.0f * kPi * ((float)j / W - 0.5f), lat = -kPi * ((float)i / H - 0.5f);
        const float b[3] = {cosf(lat) * sinf(lon), -sinf(lat), cosf(lat) * cosf(lon)};
        float d[3];
        for (int a = 0; a < 3; ++a) d[a] = s.Rt[3 * a] * b[0] + s.Rt[3 * a + 1] * b[1] + s.Rt[3 * a + 2] * b[2];
        depth[idx] = intersect(s, s.C, d);
    }
    float g = 255.0f * acc / (ss * ss);
    if (noise_sigma > 0.0f) {
        const uint32_t h1 = hash3(i, j, 1, noise_seed), h2 = hash3(i, j, 2, noise_seed);
        const float u1 = ((h1 >> 8) + 0.5f) * (1.0f / 16777216.0f), u2 = ((h2 >> 8) + 0.5f) * (1.0f / 16777216.0f);
        g += noise_sigma * sqrtf(-2.0f * logf(u1)) * cosf(2.0f * kPi * u2);
    }
    if (gray) gray[idx] = (uint8_t)fminf(255.f, fmaxf(0.f, floorf(g + 0.5f)));
    if (grayf) grayf[idx] = g;
    if (bgr)
        for (int c = 0; c < 3; ++c)
            bgr[3 * idx + c] = (uint8_t)fminf(255.f, floorf(255.0f * accc[2 - c] / (ss * ss) + 0.5f));
}

}  // namespace

namespace {
int render_device(const pm_scene *sc, const double R[9], const double t[3], int W, int H, int supersample,
                  float noise_sigma, uint32_t noise_seed, uint8_t *gray, float *depth, uint8_t *bgr, float *grayf,
                  void *stream) {
    pm_scene_desc d;
    if (!sc || W <= 0 || H <= 0 || supersample < 1 || pm_scene_describe(sc, &d)) return 1;
    DevScene s{};
    for (int a = 0; a < 3; ++a) {
        s.rlo[a] = (float)d.room_lo[a];
        s.rhi[a] = (float)d.room_hi[a];
    }
    s.nb = d.n_boxes;
    s.nc = d.n_cyls;
    for (int k = 0; k < d.n_boxes; ++k)
        for (int a = 0; a < 3; ++a) {
            s.blo[k][a] = (float)d.box_lo[k][a];
            s.bhi[k][a] = (float)d.box_hi[k][a];
        }
    for (int k = 0; k < d.n_cyls; ++k)
        for (int a = 0; a < 5; ++a) s.cyl[k][a] = (float)d.cyl[k][a];
    s.seed = d.seed;
    s.base_freq = (float)d.base_freq;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) s.Rt[3 * a + b] = (float)R[3 * b + a];
    for (int a = 0; a < 3; ++a) s.C[a] = (float)(-(R[a] * t[0] + R[3 + a] * t[1] + R[6 + a] * t[2]));
    dim3 blk(16, 16), grd((W + 15) / 16, (H + 15) / 16);
    render_kernel<<<grd, blk, 0, (cudaStream_t)stream>>>(s, W, H, supersample, noise_sigma, noise_seed, gray, depth,
                                                         bgr, grayf);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}
}  // namespace

extern "C" int pm_scene_render_device(const pm_scene *sc, const double R[9], const double t[3], int W, int H,
                                      int supersample, float noise_sigma, uint32_t noise_seed, uint8_t *gray,
                                      float *depth, uint8_t *bgr, void *stream) {
    return render_device(sc, R, t, W, H, supersample, noise_sigma, noise_seed, gray, depth, bgr, nullptr, stream);
}

extern "C" int pm_scene_render_device_f32(const pm_scene *sc, const double R[9], const double t[3], int W, int H,
                                          int supersample, float noise_sigma, uint32_t noise_seed, float *gray,
                                          void *stream) {
    return render_device(sc, R, t, W, H, supersample, noise_sigma, noise_seed, nullptr, nullptr, nullptr, gray,
                         stream);
}
