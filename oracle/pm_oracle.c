/*
 * pm_oracle.c -- CPU restatement of the reference's densification hot path.
 * TEST INFRASTRUCTURE ONLY (the parity checker and the timed CPU baseline);
 * the product never links it.  See pm_oracle.h for the list of reference
 * functions restated and the parity status.
 *
 * Build: gcc -O2 -fopenmp -fPIC -shared -ffp-contract=off pm_oracle.c -lm
 */
#include "pm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PI_D 3.14159265358979323846
/* CUDART_PI_F as used by PatchMatchCuda.cu:143-144,191-192 */
#define PI_F 3.141592654f

/* ------------------------------------------------------------------ */
/* Philox4x32-10 (Salmon et al., SC'11): two 32x32->64 multiplies per round,
 * Weyl key schedule, 10 rounds. */
void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        uint64_t p0 = (uint64_t)0xD2511F53u * (uint64_t)c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * (uint64_t)c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* 24-bit uniform in (0, 1): exactly representable in float. */
static inline float u24(uint32_t x) { return ((float)(x >> 8) + 0.5f) * (1.0f / 16777216.0f); }

static void philox_words(uint32_t seed, uint32_t kf, uint32_t pixel, uint32_t tag,
                         int nblocks, uint32_t *words)
{
    uint32_t key[2] = {seed, kf};
    for (int d = 0; d < nblocks; ++d) {
        uint32_t ctr[4] = {pixel, tag, (uint32_t)d, 0x504d4742u /* "PMGB" */};
        or_philox4x32_10(ctr, key, words + 4 * d);
    }
}

/* Box-Muller pairs: 20 words -> 10 pairs -> first 18 normals. */
void or_refine_normals(uint32_t seed, uint32_t keyframe, uint32_t pixel, uint32_t tag, float out[18])
{
    uint32_t w[20];
    philox_words(seed, keyframe, pixel, tag, 5, w);
    for (int k = 0; k < 9; ++k) {
        float u1 = u24(w[2 * k]), u2 = u24(w[2 * k + 1]);
        float r = sqrtf(-2.0f * logf(u1));
        float th = 6.28318530717958647692f * u2;
        out[2 * k] = r * cosf(th);
        out[2 * k + 1] = r * sinf(th);
    }
}

/* ------------------------------------------------------------------ */
/* Bearings. */

/* Exact bearing: lon = 2 pi (j/W - 1/2), lat = -pi (i/H - 1/2),
 * b = (cos lat sin lon, -sin lat, cos lat cos lon)  (PatchMatchCuda.cu:191-198). */
void or_bearing64(int W, int H, int i, int j, double b[3])
{
    double lon = 2.0 * PI_D * ((double)j / (double)W - 0.5);
    double lat = -PI_D * ((double)i / (double)H - 0.5);
    double cl = cos(lat);
    b[0] = cl * sin(lon);
    b[1] = -sin(lat);
    b[2] = cl * cos(lon);
}

/* The reference kernel's float bearing table entry (PatchMatchCuda.cu:183-208). */
static void bearing_ref_f32(int W, int H, int i, int j, float b[3])
{
    float x = (float)j, y = (float)i;
    float lon = 2 * PI_F * (x / (float)W - 0.5f);
    float lat = -PI_F * (y / (float)H - 0.5f);
    float cl = cosf(lat), cn = cosf(lon), sn = sinf(lon), sl = sinf(lat);
    float bx = cl * sn, by = -sl, bz = cl * cn;
    float nrm = 1.0f / sqrtf(bx * bx + by * by + bz * bz);
    b[0] = bx * nrm; b[1] = by * nrm; b[2] = bz * nrm;
}

void or_bearing_ref_f32(int W, int H, int i, int j, float b[3]) { bearing_ref_f32(W, H, i, j, b); }

/* The reference host's double bearing table (depthmap.cc:113-128,1213-1223):
 * float trig, promoted to double, normalised in double. */
static void bearing_ref_host(int W, int H, int i, int j, double b[3])
{
    const float lon = (float)(((double)j / W - 0.5) * (2 * PI_D));
    const float lat = (float)(-((double)i / H - 0.5) * PI_D);
    const float cl = cosf(lat), cn = cosf(lon), sn = sinf(lon), sl = sinf(lat);
    double bx = (double)(cl * sn), by = (double)(-sl), bz = (double)(cl * cn);
    double n = sqrt(bx * bx + by * by + bz * bz);
    b[0] = bx / n; b[1] = by / n; b[2] = bz / n;
}

/* ------------------------------------------------------------------ */
/* Bilinear sampling.  Texel k sits at coordinate k (the reference samples its
 * texture at u + 0.5, PatchMatchCuda.cu:146, and the CPU path samples at u,
 * depthmap.cc:34-50).  Coordinates are clamped to [0, W] x [0, H]; texel
 * indices clamp at the borders (the reference's texture with unnormalised
 * coordinates) or, with OR_SEAM_WRAP, wrap around in longitude. */
static inline int wrapx(long k, int W, int seam)
{
    if (seam == OR_SEAM_WRAP) { long m = k % W; return (int)(m < 0 ? m + W : m); }
    return (int)(k < 0 ? 0 : (k >= W ? W - 1 : k));
}
static inline int clampy(long k, int H) { return (int)(k < 0 ? 0 : (k >= H ? H - 1 : k)); }

static double quantize_coord(double u, int interp)
{
    if (interp == OR_INTERP_TEX8_RN) return floor(u * 256.0 + 0.5) / 256.0;
    if (interp == OR_INTERP_TEX8_RZ) return floor(u * 256.0) / 256.0;
    return u;
}

static double bilinear64(const float *img, int W, int H, double u, double v, int seam, int interp)
{
    if (!isfinite(u)) u = 0.0;
    if (!isfinite(v)) v = 0.0;
    if (seam == OR_SEAM_ZERO && (u < 0.0 || u >= W - 1 || v < 0.0 || v >= H - 1)) return 0.0;
    u = u < 0.0 ? 0.0 : (u > W ? (double)W : u);
    v = v < 0.0 ? 0.0 : (v > H ? (double)H : v);
    u = quantize_coord(u, interp);
    v = quantize_coord(v, interp);
    double fx = floor(u), fy = floor(v);
    double ax = u - fx, ay = v - fy;
    long x0 = (long)fx, y0 = (long)fy;
    int xa = wrapx(x0, W, seam), xb = wrapx(x0 + 1, W, seam);
    int ya = clampy(y0, H), yb = clampy(y0 + 1, H);
    double t00 = img[(size_t)ya * W + xa], t01 = img[(size_t)ya * W + xb];
    double t10 = img[(size_t)yb * W + xa], t11 = img[(size_t)yb * W + xb];
    return (1 - ay) * ((1 - ax) * t00 + ax * t01) + ay * ((1 - ax) * t10 + ax * t11);
}

static float bilinear32(const float *img, int W, int H, float u, float v, int seam, int interp)
{
    if (!isfinite(u)) u = 0.0f;
    if (!isfinite(v)) v = 0.0f;
    if (seam == OR_SEAM_ZERO && (u < 0.0f || u >= W - 1 || v < 0.0f || v >= H - 1)) return 0.0f;
    u = u < 0.0f ? 0.0f : (u > (float)W ? (float)W : u);
    v = v < 0.0f ? 0.0f : (v > (float)H ? (float)H : v);
    if (interp != OR_INTERP_EXACT) {
        u = (float)quantize_coord(u, interp);
        v = (float)quantize_coord(v, interp);
    }
    float fx = floorf(u), fy = floorf(v);
    float ax = u - fx, ay = v - fy;
    long x0 = (long)fx, y0 = (long)fy;
    int xa = wrapx(x0, W, seam), xb = wrapx(x0 + 1, W, seam);
    int ya = clampy(y0, H), yb = clampy(y0 + 1, H);
    float t00 = img[(size_t)ya * W + xa], t01 = img[(size_t)ya * W + xb];
    float t10 = img[(size_t)yb * W + xa], t11 = img[(size_t)yb * W + xb];
    return (1 - ay) * ((1 - ax) * t00 + ax * t01) + ay * ((1 - ax) * t10 + ax * t11);
}

/* ------------------------------------------------------------------ */
/* View combination. */
static double fold(const double *v, int n)
{
    /* PatchMatchCuda.cu:93,161-171: average when within 25 %, else max */
    double score = -1.0;
    for (int r = 0; r < n; ++r) {
        double s2 = v[r];
        score = (fabs((score - s2) / s2) < 0.25) ? 0.5 * (score + s2) : fmax(score, s2);
    }
    return score;
}

/* ncc: per-view NCCs; cum: NCCs of the moments accumulated over views 0..r */
static double combine_scores(const double *ncc, const double *cum, int n, int mode, int top_k, int *best)
{
    int b = 0;
    for (int r = 1; r < n; ++r) if (ncc[r] > ncc[b]) b = r;
    if (best) *best = b;
    if (mode == OR_COMBINE_MAX) return ncc[b];
    if (mode == OR_COMBINE_TOPK) {
        double s[OR_MAX_VIEWS];
        memcpy(s, ncc, sizeof(double) * n);
        for (int a = 1; a < n; ++a) {   /* insertion sort, descending */
            double x = s[a]; int c = a - 1;
            while (c >= 0 && s[c] < x) { s[c + 1] = s[c]; --c; }
            s[c + 1] = x;
        }
        int k = top_k < 1 ? 1 : (top_k > n ? n : top_k);
        double acc = 0.0;
        for (int a = 0; a < k; ++a) acc += s[a];
        return acc / k;
    }
    if (mode == OR_COMBINE_FOLD_SEPARATE) return fold(ncc, n);
    return fold(cum, n);
}

static float combine_scores_f32(const float *ncc, const float *cum, int n, int mode, int top_k, int *best)
{
    int b = 0;
    for (int r = 1; r < n; ++r) if (ncc[r] > ncc[b]) b = r;
    if (best) *best = b;
    if (mode == OR_COMBINE_MAX || mode == OR_COMBINE_TOPK) {
        double d[OR_MAX_VIEWS];
        for (int r = 0; r < n; ++r) d[r] = ncc[r];
        return (float)combine_scores(d, d, n, mode, top_k, NULL);
    }
    const float *v = mode == OR_COMBINE_FOLD_SEPARATE ? ncc : cum;
    float score = -1.0f;
    for (int r = 0; r < n; ++r) {
        float s2 = v[r];
        score = (fabsf((score - s2) / s2) < 0.25f) ? (float)(0.5 * (score + s2)) : fmaxf(score, s2);
    }
    return score;
}

/* ------------------------------------------------------------------ */
/* Cost, exact arithmetic.  For each source: X_c = b / (pi . b);
 * X_r = R_r (R_0^T (X_c - t_0)) + t_r; sample source r at the equirect
 * projection of X_r; bilateral-weighted NCC over the 6x6 taps at odd offsets
 * -5..5 (PatchMatchCuda.cu:100-170). */
static double cost_f64(const or_views *v, const or_cost_params *p, int i, int j,
                       const double pl[3], double *ncc_out, int *best)
{
    const int W = v->W, H = v->H, ph = p->patch_half;
    const double cf = 1.0 / (2.0 * (double)p->sigma_color * (double)p->sigma_color);
    const double df = 1.0 / (2.0 * (double)p->sigma_x * (double)p->sigma_x);
    const double *R0 = v->R[0], *t0 = v->t[0];
    double ncc[OR_MAX_VIEWS], cum[OR_MAX_VIEWS];
    double c_sw = 0, c_swx = 0, c_swy = 0, c_swxx = 0, c_swyy = 0, c_swxy = 0;
    const double xc = v->ref[(size_t)i * W + j];
    for (int r = 0; r < v->n_src; ++r) {
        const double *Rr = v->R[r + 1], *tr = v->t[r + 1];
        /* composed pose: X_r = M X_c + c, M = R_r R_0^T, c = t_r - M t_0 */
        double M[9], c[3];
        for (int a = 0; a < 3; ++a)
            for (int bb = 0; bb < 3; ++bb)
                M[3 * a + bb] = Rr[3 * a + 0] * R0[3 * bb + 0] + Rr[3 * a + 1] * R0[3 * bb + 1] +
                                Rr[3 * a + 2] * R0[3 * bb + 2];
        for (int a = 0; a < 3; ++a)
            c[a] = tr[a] - (M[3 * a] * t0[0] + M[3 * a + 1] * t0[1] + M[3 * a + 2] * t0[2]);
        double sw = 0, swx = 0, swy = 0, swxx = 0, swyy = 0, swxy = 0;
        for (int k1 = -ph; k1 <= ph; k1 += 2) {
            for (int k2 = -ph; k2 <= ph; k2 += 2) {
                const int qi = i + k1, qj = j + k2;
                const double x = v->ref[(size_t)qi * W + qj];
                double b[3];
                or_bearing64(W, H, qi, qj, b);
                const double s = pl[0] * b[0] + pl[1] * b[1] + pl[2] * b[2];
                const double Xc[3] = {b[0] / s, b[1] / s, b[2] / s};
                double X[3];
                for (int a = 0; a < 3; ++a)
                    X[a] = M[3 * a] * Xc[0] + M[3 * a + 1] * Xc[1] + M[3 * a + 2] * Xc[2] + c[a];
                double d = sqrt(X[0] * X[0] + X[1] * X[1] + X[2] * X[2]);
                if (p->seam == OR_SEAM_ZERO && d < 1e-4) continue;  /* too near: skipped (depthmap.cc:147-149) */
                double sc = 1.0 / fmax(1e-6, d);
                double bx = X[0] * sc, by = X[1] * sc, bz = X[2] * sc;
                if (by > 1.0) by = 1.0;
                if (by < -1.0) by = -1.0;
                double lat = -asin(by), lon = atan2(bx, bz);
                double u = W * (0.5 + lon / (2.0 * PI_D));
                double vv = H * (0.5 - lat / PI_D);
                double y = bilinear64(v->src[r], W, H, u, vv, p->seam, p->interp);
                double dd = x - xc;
                double w = exp(-dd * dd * cf - (double)(k1 * k1 + k2 * k2) * df);
                sw += w; swx += w * x; swy += w * y;
                swxx += w * x * x; swyy += w * y * y; swxy += w * x * y;
            }
        }
        double mx = swx / sw, my = swy / sw;
        double vx = swxx / sw - mx * mx, vy = swyy / sw - my * my;
        ncc[r] = (sw == 0.0 || vx < 0.1 || vy < 0.1) ? -1.0 : (swxy / sw - mx * my) / sqrt(vx * vy);
        c_sw += sw; c_swx += swx; c_swy += swy; c_swxx += swxx; c_swyy += swyy; c_swxy += swxy;
        mx = c_swx / c_sw; my = c_swy / c_sw;
        vx = c_swxx / c_sw - mx * mx; vy = c_swyy / c_sw - my * my;
        cum[r] = (vx < 0.1 || vy < 0.1) ? -1.0 : (c_swxy / c_sw - mx * my) / sqrt(vx * vy);
    }
    if (ncc_out) memcpy(ncc_out, ncc, sizeof(double) * v->n_src);
    return combine_scores(ncc, cum, v->n_src, p->combine, p->top_k, best);
}

/* Cost, the reference kernel's float arithmetic (PatchMatchCuda.cu:46-180):
 * normalised float bearing table, R1_inv/t1_inv then R_r/t_r in float,
 * unshifted float moments. */
static float cost_f32_ref(const or_views *v, const or_cost_params *p, int i, int j,
                          const float pl[3], float *ncc_out, int *best)
{
    const int W = v->W, H = v->H, ph = p->patch_half;
    const float dcolor_factor = 1.0f / (2 * p->sigma_color * p->sigma_color);
    const float dx_factor = 1.0f / (2 * p->sigma_x * p->sigma_x);
    float R1i[9], t1i[3];
    {   /* R1_inv = R_0^T, t1_inv = -R_0^T t_0 in double, then float (depthmap.cc:604-628) */
        const double *R0 = v->R[0], *t0 = v->t[0];
        for (int y = 0; y < 3; ++y) {
            for (int x = 0; x < 3; ++x) R1i[3 * y + x] = (float)R0[3 * x + y];
            t1i[y] = (float)(-(R0[0 * 3 + y] * t0[0] + R0[1 * 3 + y] * t0[1] + R0[2 * 3 + y] * t0[2]));
        }
    }
    float ncc[OR_MAX_VIEWS], cum[OR_MAX_VIEWS];
    const float I_center = v->ref[(size_t)i * W + j];
    /* the reference declares its sums once, outside the view loop (PatchMatchCuda.cu:57-62) */
    float sum_x = 0, sum_y = 0, sum_xx = 0, sum_yy = 0, sum_xy = 0, sum_w = 0;
    for (int r = 0; r < v->n_src; ++r) {
        float Rt[9], tt[3];
        for (int a = 0; a < 9; ++a) Rt[a] = (float)v->R[r + 1][a];
        for (int a = 0; a < 3; ++a) tt[a] = (float)v->t[r + 1][a];
        float px_ = 0, py_ = 0, pxx = 0, pyy = 0, pxy = 0, pw_ = 0;  /* this view alone */
        for (int k1 = -ph; k1 <= ph; k1 += 2) {
            for (int k2 = -ph; k2 <= ph; k2 += 2) {
                float I_src = v->ref[(size_t)(i + k1) * W + (j + k2)];
                float b[3];
                bearing_ref_f32(W, H, i + k1, j + k2, b);
                float scale = pl[0] * b[0] + pl[1] * b[1] + pl[2] * b[2];
                float denom = 1.0f / scale;
                float pxc = b[0] * denom, pyc = b[1] * denom, pzc = b[2] * denom;
                float px = R1i[0] * pxc + R1i[1] * pyc + R1i[2] * pzc + t1i[0];
                float py = R1i[3] * pxc + R1i[4] * pyc + R1i[5] * pzc + t1i[1];
                float pz = R1i[6] * pxc + R1i[7] * pyc + R1i[8] * pzc + t1i[2];
                float qx = Rt[0] * px + Rt[1] * py + Rt[2] * pz + tt[0];
                float qy = Rt[3] * px + Rt[4] * py + Rt[5] * pz + tt[1];
                float qz = Rt[6] * px + Rt[7] * py + Rt[8] * pz + tt[2];
                float depth = sqrtf(qx * qx + qy * qy + qz * qz);
                float sc = 1.0f / fmaxf(1e-6f, depth);
                float bx = qx * sc, by = qy * sc, bz = qz * sc;
                float latitude = -asinf(by);
                float longitude = atan2f(bx, bz);
                float u = W * (0.5f + longitude / (2.0f * PI_F));
                float vv = H * (0.5f - latitude / PI_F);
                float I_tgt = bilinear32(v->src[r], W, H, u, vv, p->seam, p->interp);
                float I_diff = I_src - I_center;
                float w = expf(-I_diff * I_diff * dcolor_factor - (float)(k2 * k2 + k1 * k1) * dx_factor);
                sum_x = sum_x + I_src * w; sum_y = sum_y + I_tgt * w;
                sum_xx = sum_xx + I_src * I_src * w; sum_yy = sum_yy + I_tgt * I_tgt * w;
                sum_xy = sum_xy + I_src * I_tgt * w; sum_w = sum_w + w;
                px_ += I_src * w; py_ += I_tgt * w; pxx += I_src * I_src * w;
                pyy += I_tgt * I_tgt * w; pxy += I_src * I_tgt * w; pw_ += w;
            }
        }
        float prob = 1 / sum_w;
        float mean_x = sum_x * prob, mean_y = sum_y * prob;
        float mean_xx = sum_xx * prob, mean_yy = sum_yy * prob, mean_xy = sum_xy * prob;
        float var_x = mean_xx - mean_x * mean_x, var_y = mean_yy - mean_y * mean_y;
        float score_ = (mean_xy - mean_x * mean_y) / sqrtf(var_x * var_y);
        cum[r] = (var_x < 0.1 || var_y < 0.1) ? -1.0f : score_;
        prob = 1 / pw_;
        mean_x = px_ * prob; mean_y = py_ * prob;
        var_x = pxx * prob - mean_x * mean_x; var_y = pyy * prob - mean_y * mean_y;
        score_ = (pxy * prob - mean_x * mean_y) / sqrtf(var_x * var_y);
        ncc[r] = (var_x < 0.1 || var_y < 0.1) ? -1.0f : score_;
    }
    if (ncc_out) memcpy(ncc_out, ncc, sizeof(float) * v->n_src);
    return combine_scores_f32(ncc, cum, v->n_src, p->combine, p->top_k, best);
}

double or_cost(const or_views *v, const or_cost_params *p, int i, int j,
               const double plane[3], double *ncc, int *best)
{
    if (p->arith == OR_ARITH_F32_REF) {
        float pl[3] = {(float)plane[0], (float)plane[1], (float)plane[2]};
        float n32[OR_MAX_VIEWS];
        float s = cost_f32_ref(v, p, i, j, pl, n32, best);
        if (ncc) for (int r = 0; r < v->n_src; ++r) ncc[r] = n32[r];
        return s;
    }
    return cost_f64(v, p, i, j, plane, ncc, best);
}

void or_cost_batch(const or_views *v, const or_cost_params *p, int n, const int32_t *ij,
                   const float *planes, double *scores, int32_t *best, double *ncc_all, int threads)
{
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 64)
#endif
    for (int h = 0; h < n; ++h) {
        double pl[3] = {planes[3 * h], planes[3 * h + 1], planes[3 * h + 2]};
        int b = 0;
        scores[h] = or_cost(v, p, ij[2 * h], ij[2 * h + 1], pl,
                            ncc_all ? ncc_all + (size_t)h * v->n_src : NULL, &b);
        if (best) best[h] = b;
    }
}

/* ------------------------------------------------------------------ */
/* Full run.  State maps are float (like the GPU). */

static float run_cost(const or_views *v, const or_cost_params *p, int i, int j, const float pl[3], int *best)
{
    if (p->arith == OR_ARITH_F32_REF) return cost_f32_ref(v, p, i, j, pl, NULL, best);
    double d[3] = {pl[0], pl[1], pl[2]};
    return (float)cost_f64(v, p, i, j, d, NULL, best);
}

static void run_bearing(const or_views *v, const or_cost_params *p, int i, int j, float b[3])
{
    if (p->arith == OR_ARITH_F32_REF) { bearing_ref_f32(v->W, v->H, i, j, b); return; }
    double d[3];
    or_bearing64(v->W, v->H, i, j, d);
    b[0] = (float)d[0]; b[1] = (float)d[1]; b[2] = (float)d[2];
}

static int interior(const or_views *v, int ph, int i, int j)
{
    /* PatchMatchCuda.cu:262,283 */
    return !(i < ph + 1 || i > v->H - ph - 1 || j < ph + 1 || j > v->W - ph - 1);
}

/* Random init of one pixel (Philox tag 0). */
static void init_pixel(const or_views *v, const or_run_params *rp, int i, int j, float *pl, float *depth)
{
    uint32_t w[4];
    philox_words(rp->seed, rp->keyframe, (uint32_t)(i * v->W + j), 0u, 1, w);
    float b[3];
    run_bearing(v, &rp->cp, i, j, b);
    float d, n[3];
    if (rp->init_mode == OR_INIT_REF_UNIFORM) {
        /* PatchMatchCuda.cu:210-244: uniform depth, normal components U[-1,1] */
        d = u24(w[0]) * (rp->max_depth - rp->min_depth) + rp->min_depth;
        n[0] = u24(w[1]) * 2.0f - 1.0f;
        n[1] = u24(w[2]) * 2.0f - 1.0f;
        n[2] = u24(w[3]) * 2.0f - 1.0f;
    } else {
        /* log-uniform depth (depthmap.cc:924) and a uniform unit normal on the
         * hemisphere facing the camera */
        float lmin = logf(rp->min_depth), lmax = logf(rp->max_depth);
        d = expf(lmin + u24(w[0]) * (lmax - lmin));
        float z = 1.0f - 2.0f * u24(w[1]);
        float rxy = sqrtf(fmaxf(0.0f, 1.0f - z * z));
        float ph = 6.28318530717958647692f * u24(w[2]);
        n[0] = rxy * cosf(ph); n[1] = rxy * sinf(ph); n[2] = z;
        if (n[0] * b[0] + n[1] * b[1] + n[2] * b[2] > 0.0f) { n[0] = -n[0]; n[1] = -n[1]; n[2] = -n[2]; }
    }
    /* PlaneFromDepthNormal (PatchMatchCuda.cu:31-43) */
    float px = d * b[0], py = d * b[1], pz = d * b[2];
    float nom = 1 / (n[0] * px + n[1] * py + n[2] * pz);
    pl[0] = n[0] * nom; pl[1] = n[1] * nom; pl[2] = n[2] * nom;
    *depth = d;
}

/* A propagation neighbour outside the image is not a candidate.  Active
 * pixels sit patch_half + 1 from every edge (PatchMatchCuda.cu:283), so this
 * only matters for patch_half = 1, where the reference would read outside its
 * buffers (it only ever runs patch_half = 5). */
static int nbr_inside(const or_views *v, int ni, int nj)
{
    return ni >= 0 && ni < v->H && nj >= 0 && nj < v->W;
}

/* One pixel update of the reference's host variant (PatchMatchUpdatePixel,
 * depthmap.cc:1003-1067; CheckPlaneCandidate :1069-1078): pixels and
 * neighbours of depth 0 are ignored, candidates are compared by score alone
 * and taken at once (plane, score, depth = DepthOfPlaneBackprojection :97-104);
 * refinement t draws one depth normal and three normal-vector normals from
 * Philox block t (tag sweep + 1), perturbs the current plane and depth, builds
 * the plane with the 1e-5 clamp (:130-141) and is skipped without shrinking
 * the ranges when the current plane's z is 0 (:1044-1046). */
static void update_pixel_plain(const or_views *v, const or_run_params *rp, int sweep, int i, int j,
                               float *plane, float *depthm, float *scorem, int32_t *bestm)
{
    const int W = v->W;
    const size_t idx = (size_t)i * W + j;
    static const int adjacent[8][2] = {{0, 1}, {1, 0}, {0, -1}, {-1, 0}, {0, 3}, {3, 0}, {0, -3}, {-3, 0}};
    if (depthm[idx] == 0.0f) return;
    float score = scorem[idx];
    int best = bestm ? bestm[idx] : 0;
    float cx = plane[3 * idx], cy = plane[3 * idx + 1], cz = plane[3 * idx + 2];
    float cur_depth = depthm[idx];
    float b[3];
    run_bearing(v, &rp->cp, i, j, b);
    for (int a = 0; a < 8; ++a) {
        if (!nbr_inside(v, i + adjacent[a][0], j + adjacent[a][1])) continue;
        size_t n = (size_t)(i + adjacent[a][0]) * W + (j + adjacent[a][1]);
        if (depthm[n] == 0.0f) continue;
        float pl[3] = {plane[3 * n], plane[3 * n + 1], plane[3 * n + 2]};
        int hb = 0;
        float sc = run_cost(v, &rp->cp, i, j, pl, &hb);
        if (sc > score) {
            cx = pl[0]; cy = pl[1]; cz = pl[2]; score = sc; best = hb;
            float dn = b[0] * cx + b[1] * cy + b[2] * cz;
            cur_depth = 1 / fmaxf(1e-6f, fabsf(dn));
        }
    }
    uint32_t w[24];
    philox_words(rp->seed, rp->keyframe, (uint32_t)idx, (uint32_t)(sweep + 1), 6, w);
    float depth_range = 0.02f, normal_range = 0.5f;
    for (int t = 0; t < 6; ++t) {
        if (cz == 0.0f) continue;
        float z[4];
        for (int q = 0; q < 2; ++q) {
            float u1 = u24(w[4 * t + 2 * q]), u2 = u24(w[4 * t + 2 * q + 1]);
            float r = sqrtf(-2.0f * logf(u1)), th = 6.28318530717958647692f * u2;
            z[2 * q] = r * cosf(th);
            z[2 * q + 1] = r * sinf(th);
        }
        float depth_hyp = cur_depth * expf(depth_range * z[0]);
        float nhx = cx + normal_range * z[1], nhy = cy + normal_range * z[2], nhz = cz + normal_range * z[3];
        float px = depth_hyp * b[0], py = depth_hyp * b[1], pz = depth_hyp * b[2];
        float den = nhx * px + nhy * py + nhz * pz;
        if (den < 1e-5f && den >= 0.0f) den = 1e-5f;
        else if (den > -1e-5f && den < 0.0f) den = -1e-5f;
        float pl[3] = {nhx / den, nhy / den, nhz / den};
        int hb = 0;
        float sc = run_cost(v, &rp->cp, i, j, pl, &hb);
        if (sc > score) {
            cx = pl[0]; cy = pl[1]; cz = pl[2]; score = sc; best = hb;
            float dn = b[0] * cx + b[1] * cy + b[2] * cz;
            cur_depth = 1 / fmaxf(1e-6f, fabsf(dn));
        }
        depth_range = (float)(depth_range * 0.3);
        normal_range = (float)(normal_range * 0.8);
    }
    scorem[idx] = score;
    plane[3 * idx] = cx; plane[3 * idx + 1] = cy; plane[3 * idx + 2] = cz;
    depthm[idx] = cur_depth;
    if (bestm) bestm[idx] = best;
}

/* One red/black pixel update (PatchMatchCuda.cu:287-404). */
static void update_pixel(const or_views *v, const or_run_params *rp, int sweep, int i, int j,
                         float *plane, float *depthm, float *scorem, int32_t *bestm)
{
    if (rp->propagation == OR_PROP_PLAIN) {
        update_pixel_plain(v, rp, sweep, i, j, plane, depthm, scorem, bestm);
        return;
    }
    const int W = v->W;
    const size_t idx = (size_t)i * W + j;
    static const int adjacent[8][2] = {{0, 1}, {1, 0}, {0, -1}, {-1, 0}, {0, 3}, {3, 0}, {0, -3}, {-3, 0}};
    float score = scorem[idx];
    int best = bestm ? bestm[idx] : 0;
    float hx = plane[3 * idx], hy = plane[3 * idx + 1], hz = plane[3 * idx + 2];
    float b[3];
    run_bearing(v, &rp->cp, i, j, b);
    const float curr_depth = depthm[idx];
    for (int a = 0; a < 8; ++a) {
        if (!nbr_inside(v, i + adjacent[a][0], j + adjacent[a][1])) continue;
        size_t n = (size_t)(i + adjacent[a][0]) * W + (j + adjacent[a][1]);
        float nx = plane[3 * n], ny = plane[3 * n + 1], nz = plane[3 * n + 2];
        float pl[3] = {nx, ny, nz};
        int hb = 0;
        float score_hyp = run_cost(v, &rp->cp, i, j, pl, &hb);
        float scale = nx * b[0] + ny * b[1] + nz * b[2];
        float denom = 1 / fmaxf(1e-6f, fabsf(scale));
        float dq = (curr_depth - denom) / curr_depth;
        float depth_smooth_f = expf(-(dq * dq) * 1250.0f);
        float prod = hx * nx + hy * ny + hz * nz;
        float ex = hx - nx, ey = hy - ny, ez = hz - nz;
        float norm = sqrtf(ex * ex + ey * ey + ez * ez);
        float ac = acosf(prod / norm);
        float plane_smooth_f = expf(-(ac * ac) * 8.0f);
        score_hyp *= (1.0f - depth_smooth_f) * (1.0f - plane_smooth_f);
        if (score_hyp > score) { hx = nx; hy = ny; hz = nz; score = score_hyp; best = hb; }
    }
    float dn = b[0] * hx + b[1] * hy + b[2] * hz;
    float current_depth = 1 / fmaxf(1e-6f, fabsf(dn));
    float cx = hx, cy = hy, cz = hz;
    float nrm[18];
    or_refine_normals(rp->seed, rp->keyframe, (uint32_t)idx, (uint32_t)(sweep + 1), nrm);
    float depth_range = 0.02f, normal_range = 0.5f;
    for (int t = 0; t < 6; ++t) {
        float ra = nrm[3 * t], rb = nrm[3 * t + 1], rc = nrm[3 * t + 2];
        float depth_hyp = current_depth * expf(depth_range * ra);
        float nhx = cx + normal_range * ra, nhy = cy + normal_range * rb, nhz = cz + normal_range * rc;
        float px = depth_hyp * b[0], py = depth_hyp * b[1], pz = depth_hyp * b[2];
        float den = nhx * px + nhy * py + nhz * pz;
        float pl[3] = {nhx / den, nhy / den, nhz / den};
        int hb = 0;
        float score_hyp = run_cost(v, &rp->cp, i, j, pl, &hb);
        if (score_hyp > score) {
            cx = pl[0]; cy = pl[1]; cz = pl[2];
            score = score_hyp; current_depth = depth_hyp; best = hb;
        }
        depth_range = (float)(depth_range * 0.3);
        normal_range = (float)(normal_range * 0.8);
    }
    scorem[idx] = score;
    plane[3 * idx] = cx; plane[3 * idx + 1] = cy; plane[3 * idx + 2] = cz;
    float den = b[0] * cx + b[1] * cy + b[2] * cz;
    depthm[idx] = 1 / fmaxf(1e-6f, fabsf(den));
    if (bestm) bestm[idx] = best;
}

double or_patchmatch(const or_views *v, const or_run_params *rp, float *plane, float *depth,
                     float *score, int32_t *best)
{
    const int W = v->W, H = v->H, ph = rp->cp.patch_half;
    const int lo = rp->row_lo < 0 ? 0 : rp->row_lo;
    const int hi = rp->row_hi < 0 ? H : rp->row_hi;
#ifdef _OPENMP
    if (rp->threads > 0) omp_set_num_threads(rp->threads);
#endif
    /* init: every pixel gets a random plane (PatchMatchCuda.cu:210-244) */
#ifdef _OPENMP
#pragma omp parallel for
#endif
    for (int i = 0; i < H; ++i)
        for (int j = 0; j < W; ++j) {
            size_t idx = (size_t)i * W + j;
            init_pixel(v, rp, i, j, plane + 3 * idx, depth + idx);
            score[idx] = -1.0f;
            if (best) best[idx] = 0;
        }
#ifdef _OPENMP
    double t0 = omp_get_wtime();
#pragma omp parallel for collapse(2) schedule(dynamic, 128)
#endif
    for (int i = lo; i < hi; ++i)
        for (int j = 0; j < W; ++j) {
            if (!interior(v, ph, i, j)) continue;
            size_t idx = (size_t)i * W + j;
            int hb = 0;
            score[idx] = run_cost(v, &rp->cp, i, j, plane + 3 * idx, &hb);
            if (best) best[idx] = hb;
        }
    for (int s = 0; s < rp->iterations; ++s) {
        for (int off = 0; off < 2; ++off) {
#ifdef _OPENMP
#pragma omp parallel for collapse(2) schedule(dynamic, 128)
#endif
            for (int i = lo; i < hi; ++i)
                for (int j = 0; j < W; ++j) {
                    if (((i + j + off) & 1) != 0 || !interior(v, ph, i, j)) continue;
                    update_pixel(v, rp, s, i, j, plane, depth, score, best);
                }
        }
    }
#ifdef _OPENMP
    return omp_get_wtime() - t0;
#else
    return 0.0;
#endif
}

void or_sweeps(const or_views *v, const or_run_params *rp, float *plane, float *depth, float *score,
               int32_t *best, int first_half, int n_half)
{
    const int W = v->W, H = v->H, ph = rp->cp.patch_half;
    const int lo = rp->row_lo < 0 ? 0 : rp->row_lo;
    const int hi = rp->row_hi < 0 ? H : rp->row_hi;
#ifdef _OPENMP
    if (rp->threads > 0) omp_set_num_threads(rp->threads);
#endif
    for (int hs = first_half; hs < first_half + n_half; ++hs) {
        const int off = hs & 1, s = hs >> 1;
#ifdef _OPENMP
#pragma omp parallel for collapse(2) schedule(dynamic, 128)
#endif
        for (int i = lo; i < hi; ++i)
            for (int j = 0; j < W; ++j) {
                if (((i + j + off) & 1) != 0 || !interior(v, ph, i, j)) continue;
                update_pixel(v, rp, s, i, j, plane, depth, score, best);
            }
    }
}

/* ------------------------------------------------------------------ */
/* Post-processing. */

static int cmp_float(const void *a, const void *b)
{
    float x = *(const float *)a, y = *(const float *)b;
    return (x > y) - (x < y);
}

void or_median3(int W, int H, const float *in, float *out)
{
    for (int i = 0; i < H; ++i)
        for (int j = 0; j < W; ++j) {
            float s[9];
            int c = 0;
            for (int di = -1; di <= 1; ++di)
                for (int dj = -1; dj <= 1; ++dj) {
                    int y = clampy(i + di, H), x = clampy(j + dj, W);
                    s[c++] = in[(size_t)y * W + x];
                }
            qsort(s, 9, sizeof(float), cmp_float);
            out[(size_t)i * W + j] = s[4];
        }
}

void or_postprocess(int W, int H, int patch_half, const float *ref, const uint8_t *mask,
                    float min_patch_sd, float min_depth, float max_depth, float min_score,
                    float *depth, float *score)
{
    const size_t N = (size_t)W * H;
    float *d = (float *)malloc(N * sizeof(float));
    float *sc = (float *)malloc(N * sizeof(float));
    float *m1 = (float *)malloc(N * sizeof(float));
    float *m2 = (float *)malloc(N * sizeof(float));
    const float min_var = min_patch_sd * min_patch_sd;
    /* host window (depthmap.cc:731-760): rows/cols [patch_size-2, N-patch_size-2)
     * with patch_size = patch_half + 2; outside stays at depth 0 / score -1. */
    const int lo = patch_half, hiy = H - patch_half - 4, hix = W - patch_half - 4;
    for (int i = 0; i < H; ++i)
        for (int j = 0; j < W; ++j) {
            size_t idx = (size_t)i * W + j;
            d[idx] = 0.0f; sc[idx] = -1.0f;
            if (i < lo || i >= hiy || j < lo || j >= hix) continue;
            if (mask && !mask[idx]) continue;
            /* low-variance mask over the 36 taps (PatchVariance, depthmap.cc:963-973,
             * averaging over the taps actually filled) */
            float patch[64];
            int c = 0;
            for (int u = -patch_half; u <= patch_half; u += 2)
                for (int vv = -patch_half; vv <= patch_half; vv += 2)
                    patch[c++] = ref[(size_t)(i + u) * W + (j + vv)];
            float sum = 0;
            for (int a = 0; a < c; ++a) sum += patch[a];
            float mean = sum / c, sum2 = 0;
            for (int a = 0; a < c; ++a) sum2 += (patch[a] - mean) * (patch[a] - mean);
            if (sum2 / c < min_var) { d[idx] = 0.0f; sc[idx] = 0.0f; continue; }
            d[idx] = depth[idx];
            sc[idx] = score[idx];
        }
    or_median3(W, H, d, m1);
    or_median3(W, H, m1, m2);
    /* PostProcess (depthmap.cc:1176-1197) */
    for (size_t idx = 0; idx < N; ++idx) {
        float dd = d[idx], m = m2[idx], s = sc[idx];
        if (dd == 0.0f || (double)(fabsf(dd - m) / dd) > 0.05 || dd < min_depth || dd > max_depth ||
            s <= min_score) {
            depth[idx] = 0.0f;
            score[idx] = -1.0f;
        } else {
            depth[idx] = m;
            score[idx] = s;
        }
    }
    free(d); free(sc); free(m1); free(m2);
}

/* ------------------------------------------------------------------ */
/* Seeding candidates from a prior result (PreInitResultWarp, depthmap.cc:434-516):
 * lift each valid prior pixel onto its plane (PosPatchPartOnPlane :163-177),
 * move it into the new camera, round to the nearest pixel; the nearest splat
 * (then the lowest prior index) wins a pixel.  The prior's unit normal is
 * rotated into the new camera (the reference reuses it unrotated).  cand:
 * H*W*4 (plane xyz, range; range 0 = none). */
void or_warp_prior(int Wp, int Hp, const float *prev_plane, const float *prev_depth, const double *Rp,
                   const double *tp, int W, int H, const double *Rn, const double *tn, float *cand)
{
    double M[9], c[3];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
            M[3 * a + b] = Rn[3 * a] * Rp[3 * b] + Rn[3 * a + 1] * Rp[3 * b + 1] + Rn[3 * a + 2] * Rp[3 * b + 2];
    for (int a = 0; a < 3; ++a) c[a] = tn[a] - (M[3 * a] * tp[0] + M[3 * a + 1] * tp[1] + M[3 * a + 2] * tp[2]);
    const size_t N = (size_t)W * H;
    double *best_r = (double *)malloc(N * sizeof(double));
    long *best_i = (long *)malloc(N * sizeof(long));
    for (size_t q = 0; q < N; ++q) { best_r[q] = INFINITY; best_i[q] = -1; cand[4 * q + 3] = 0.0f; }
    for (int i = 0; i < Hp; ++i)
        for (int j = 0; j < Wp; ++j) {
            size_t idx = (size_t)i * Wp + j;
            if (!(prev_depth[idx] >= 1e-4f)) continue;
            const float *pl = prev_plane + 3 * idx;
            double b[3];
            or_bearing64(Wp, Hp, i, j, b);
            double sc = pl[0] * b[0] + pl[1] * b[1] + pl[2] * b[2];
            if (sc < 1e-6 && sc >= 0) sc = 1e-6;
            else if (sc > -1e-6 && sc < 0) sc = -1e-6;
            double P[3] = {b[0] / sc, b[1] / sc, b[2] / sc}, X[3];
            for (int a = 0; a < 3; ++a) X[a] = M[3 * a] * P[0] + M[3 * a + 1] * P[1] + M[3 * a + 2] * P[2] + c[a];
            double r = sqrt(X[0] * X[0] + X[1] * X[1] + X[2] * X[2]);
            if (!(r >= 1e-4) || !isfinite(r)) continue;
            double lon = atan2(X[0], X[2]), lat = -asin(fmin(1.0, fmax(-1.0, X[1] / r)));
            double x = W * (0.5 + lon / (2 * PI_D)), y = H * (0.5 - lat / PI_D);
            int ti = (int)(y + 0.5), tj = (int)(x + 0.5);
            if (ti < 0 || tj < 0 || ti >= H || tj >= W) continue;
            size_t t = (size_t)ti * W + tj;
            float rf = (float)r;
            if (rf < best_r[t] || (rf == best_r[t] && (long)idx < best_i[t])) {
                best_r[t] = rf; best_i[t] = (long)idx;
                double nn = 1.0 / sqrt((double)pl[0] * pl[0] + (double)pl[1] * pl[1] + (double)pl[2] * pl[2]);
                double n[3];
                for (int a = 0; a < 3; ++a) n[a] = (M[3 * a] * pl[0] + M[3 * a + 1] * pl[1] + M[3 * a + 2] * pl[2]) * nn;
                double bn[3];
                or_bearing64(W, H, ti, tj, bn);
                double den = r * (n[0] * bn[0] + n[1] * bn[1] + n[2] * bn[2]);
                if (den < 1e-5 && den >= 0) den = 1e-5;
                else if (den > -1e-5 && den < 0) den = -1e-5;
                for (int a = 0; a < 3; ++a) cand[4 * t + a] = (float)(n[a] / den);
                cand[4 * t + 3] = rf;
            }
        }
    free(best_r);
    free(best_i);
}

/* ------------------------------------------------------------------ */
/* Reprojection helpers of the reference host code (depthmap.cc:143-161). */

static void mat_t_vec(const double *R, const double *x, double *y)
{   /* y = R^T x */
    for (int a = 0; a < 3; ++a) y[a] = R[a] * x[0] + R[3 + a] * x[1] + R[6 + a] * x[2];
}
static void mat_vec(const double *R, const double *x, double *y)
{
    for (int a = 0; a < 3; ++a) y[a] = R[3 * a] * x[0] + R[3 * a + 1] * x[1] + R[3 * a + 2] * x[2];
}

/* returns 1 when too near (x, y untouched) */
static int reproject_equirect(int W, int H, const double *R, const double *t, const double *pw,
                              float *x, float *y)
{
    double bt[3];
    mat_vec(R, pw, bt);
    bt[0] += t[0]; bt[1] += t[1]; bt[2] += t[2];
    double depth = sqrt(bt[0] * bt[0] + bt[1] * bt[1] + bt[2] * bt[2]);
    if (depth < 1e-4) return 1;
    double b[3] = {bt[0] / depth, bt[1] / depth, bt[2] / depth};
    const float latitude = -asinf((float)b[1]);
    const float longitude = atan2f((float)b[0], (float)b[2]);
    *x = (float)(W * (0.5 + longitude / (2.0 * PI_D)));
    *y = (float)(H * (0.5 - latitude / PI_D));
    return 0;
}

static void backproject(int W, int H, int i, int j, float depth, const double *R, const double *t, double *pw)
{
    double b[3], p[3];
    bearing_ref_host(W, H, i, j, b);
    for (int a = 0; a < 3; ++a) p[a] = (double)depth * b[a] - t[a];
    mat_t_vec(R, p, pw);
}

/* LinearInterpolation<float> (depthmap.cc:34-50) */
static float linear_interp(const float *img, int W, int H, float y, float x)
{
    if (x < 0.0f || x >= W - 1 || y < 0.0f || y >= H - 1) return 0.0f;
    int ix = (int)x, iy = (int)y;
    float dx = x - ix, dy = y - iy;
    float im00 = img[(size_t)iy * W + ix], im01 = img[(size_t)iy * W + ix + 1];
    float im10 = img[(size_t)(iy + 1) * W + ix], im11 = img[(size_t)(iy + 1) * W + ix + 1];
    float im0 = (1 - dx) * im00 + dx * im01;
    float im1 = (1 - dx) * im10 + dx * im11;
    return (1 - dy) * im0 + dy * im1;
}

static int inside(int W, int H, int i, int j) { return i >= 0 && i < H && j >= 0 && j < W; }

void or_clean(int W, int H, int n, const float *const *depths, const double *R, const double *t,
              int center, float thr, int min_consistent_views, float reproj_px, float *out)
{
    const float *D0 = depths[center];
    const double *R0 = R + 9 * center, *t0 = t + 3 * center;
#ifdef _OPENMP
#pragma omp parallel for
#endif
    for (int i = 0; i < H; ++i)
        for (int j = 0; j < W; ++j) {
            size_t idx = (size_t)i * W + j;
            out[idx] = 0.0f;
            float depth = D0[idx];
            if (depth < 1e-6) continue;
            double pw[3];
            backproject(W, H, i, j, depth, R0, t0, pw);
            int consistent = 1;
            for (int k = 0; k < n; ++k) {
                if (k == center) continue;
                const double *Rk = R + 9 * k, *tk = t + 3 * k;
                float x, y;
                if (reproject_equirect(W, H, Rk, tk, pw, &x, &y)) continue;
                if (!inside(W, H, (int)y, (int)x)) continue;
                double pk[3];
                mat_vec(Rk, pw, pk);
                pk[0] += tk[0]; pk[1] += tk[1]; pk[2] += tk[2];
                float dop = (float)sqrt(pk[0] * pk[0] + pk[1] * pk[1] + pk[2] * pk[2]);
                float dat = linear_interp(depths[k], W, H, y, x);
                if (!(fabsf(dat - dop) < dop * thr)) continue;
                if (reproj_px > 0.0f) {
                    /* round trip: back-project view k's depth at (x, y) and
                     * reproject into the centre view */
                    double lon = 2.0 * PI_D * ((double)x / W - 0.5), lat = -PI_D * ((double)y / H - 0.5);
                    double bk[3] = {cos(lat) * sin(lon), -sin(lat), cos(lat) * cos(lon)}, q[3], qw[3];
                    for (int a = 0; a < 3; ++a) q[a] = (double)dat * bk[a] - tk[a];
                    mat_t_vec(Rk, q, qw);
                    float x0, y0;
                    if (reproject_equirect(W, H, R0, t0, qw, &x0, &y0)) continue;
                    float ex = fabsf(x0 - (float)j), ey = fabsf(y0 - (float)i);
                    if (ex > 0.5f * W) ex = W - ex;
                    if (ex > reproj_px || ey > reproj_px) continue;
                }
                consistent++;
            }
            if (consistent >= min_consistent_views) out[idx] = depth;
        }
}

int or_prune(int W, int H, int n, float *const *depths, const double *R, const double *t,
             const uint8_t *rgb, float thr, float *pruned, double *points, uint8_t *colors,
             int32_t *keypts)
{
    const float *D0 = depths[0];
    const double *R0 = R, *t0 = t;
    int count = 0;
    for (int i = 0; i < H; ++i)
        for (int j = 0; j < W; ++j) {
            size_t idx = (size_t)i * W + j;
            int filter_sparse = 0;
            float depth = D0[idx];
            if (depth == 0.0f) filter_sparse = 1;
            /* neighbour rule as written (depthmap.cc:1565-1576) */
            if (i - 1 > 0 && i - 1 < H) filter_sparse = filter_sparse || D0[idx - W] == 0.0f;
            if (j - 1 > 0 && j - 1 < W) filter_sparse = filter_sparse || D0[idx - 1] == 0.0f;
            if (i + 1 > 0 && i + 1 < H) filter_sparse = filter_sparse || D0[idx + W] == 0.0f;
            if (j + 1 > 0 && j + 1 < W) filter_sparse = filter_sparse || D0[idx + 1] == 0.0f;
            if (filter_sparse) { pruned[idx] = 0.0f; continue; }
            double pw[3];
            backproject(W, H, i, j, depth, R0, t0, pw);
            pruned[idx] = depth;
            int keep = 1;
            for (int k = 1; k < n; ++k) {
                const double *Rk = R + 9 * k, *tk = t + 3 * k;
                float x, y;
                /* a point nearer than 0.1 mm to camera k is skipped for k */
                if (reproject_equirect(W, H, Rk, tk, pw, &x, &y)) continue;
                int iu = (int)x, iv = (int)y;
                double pk[3];
                mat_vec(Rk, pw, pk);
                pk[0] += tk[0]; pk[1] += tk[1]; pk[2] += tk[2];
                float dop = (float)sqrt(pk[0] * pk[0] + pk[1] * pk[1] + pk[2] * pk[2]);
                if (!inside(W, H, iv, iu) || dop < 1e-5) continue;
                float *Dk = depths[k];
                float dat = Dk[(size_t)iv * W + iu];
                if (dat == 0.0f || fabsf(dat - dop) > thr * dop) continue;
                if (depth < dat) {
                    Dk[(size_t)iv * W + iu] = 0.0f;
                } else {
                    pruned[idx] = 0.0f;
                    keep = 0;
                    break;
                }
            }
            if (keep) {
                if (points) { points[3 * count] = pw[0]; points[3 * count + 1] = pw[1]; points[3 * count + 2] = pw[2]; }
                if (colors && rgb) memcpy(colors + 3 * count, rgb + 3 * idx, 3);
                if (keypts) { keypts[2 * count] = i; keypts[2 * count + 1] = j; }
                count++;
            }
        }
    return count;
}
