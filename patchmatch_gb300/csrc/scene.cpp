// Synthetic equirectangular scenes with analytic depth (see include/pm_scene.h).
// Host C++ with OpenMP; used to generate test and benchmark workloads.
#include "pm_scene.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

constexpr double kPi = 3.14159265358979323846;

struct Rng {  // splitmix64
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed * 0x9E3779B97F4A7C15ull + 0x1234567ull) {}
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uni() { return (next() >> 11) * (1.0 / 9007199254740992.0); }
    double uni(double a, double b) { return a + (b - a) * uni(); }
    double normal() {
        double u1 = uni(), u2 = uni();
        if (u1 < 1e-300) u1 = 1e-300;
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * kPi * u2);
    }
};

struct Box { double lo[3], hi[3]; };
struct Cyl { double cx, cz, r, y0, y1; };

inline uint32_t hash3(int x, int y, int z, uint32_t seed) {
    uint32_t h = seed * 0x27d4eb2du;
    h ^= (uint32_t)x * 0x85ebca6bu;
    h = (h << 13) | (h >> 19);
    h ^= (uint32_t)y * 0xc2b2ae35u;
    h = (h << 17) | (h >> 15);
    h ^= (uint32_t)z * 0x165667b1u;
    h ^= h >> 16; h *= 0x7feb352du; h ^= h >> 15; h *= 0x846ca68bu; h ^= h >> 16;
    return h;
}
inline double lattice(int x, int y, int z, uint32_t seed) { return (hash3(x, y, z, seed) >> 8) * (1.0 / 16777216.0); }
inline double fade(double t) { return t * t * t * (t * (t * 6 - 15) + 10); }

// Trilinear value noise with quintic fade, in [0, 1).
double value_noise(double x, double y, double z, uint32_t seed) {
    double fx = std::floor(x), fy = std::floor(y), fz = std::floor(z);
    int ix = (int)fx, iy = (int)fy, iz = (int)fz;
    double ux = fade(x - fx), uy = fade(y - fy), uz = fade(z - fz);
    double c[2][2][2];
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            for (int d = 0; d < 2; ++d) c[a][b][d] = lattice(ix + a, iy + b, iz + d, seed);
    double x00 = c[0][0][0] + ux * (c[1][0][0] - c[0][0][0]);
    double x10 = c[0][1][0] + ux * (c[1][1][0] - c[0][1][0]);
    double x01 = c[0][0][1] + ux * (c[1][0][1] - c[0][0][1]);
    double x11 = c[0][1][1] + ux * (c[1][1][1] - c[0][1][1]);
    double y0 = x00 + uy * (x10 - x00), y1 = x01 + uy * (x11 - x01);
    return y0 + uz * (y1 - y0);
}

}  // namespace

struct pm_scene {
    int kind;
    uint32_t seed;
    Box room;
    std::vector<Box> boxes;
    std::vector<Cyl> cyls;
    double base_freq;

    // 4-octave solid texture mapped to 0..1 with a contrast stretch.
    double texture(const double p[3], uint32_t channel) const {
        double sum = 0, amp = 1, norm = 0, f = base_freq;
        for (int o = 0; o < 4; ++o) {
            sum += amp * value_noise(p[0] * f + 17.3 * o, p[1] * f - 5.1 * o, p[2] * f + 3.7 * o,
                                     seed * 977u + channel * 131u + (uint32_t)o);
            norm += amp;
            amp *= 0.5;
            f *= 2.0;
        }
        double v = 0.5 + (sum / norm - 0.5) * 2.6;
        return std::min(1.0, std::max(0.0, v));
    }

    bool free_space(const double p[3], double clearance) const {
        for (int a = 0; a < 3; ++a)
            if (p[a] < room.lo[a] + clearance || p[a] > room.hi[a] - clearance) return false;
        for (const Box &b : boxes) {
            bool in = true;
            for (int a = 0; a < 3; ++a)
                if (p[a] < b.lo[a] - clearance || p[a] > b.hi[a] + clearance) in = false;
            if (in) return false;
        }
        for (const Cyl &c : cyls) {
            double dx = p[0] - c.cx, dz = p[2] - c.cz;
            if (std::sqrt(dx * dx + dz * dz) < c.r + clearance && p[1] > c.y0 - clearance &&
                p[1] < c.y1 + clearance)
                return false;
        }
        return true;
    }

    // Nearest hit along o + t d (|d| = 1); returns t and the world normal.
    double intersect(const double o[3], const double d[3], double n[3]) const {
        double best = 1e30;
        // room interior: exit distance
        for (int a = 0; a < 3; ++a) {
            if (std::fabs(d[a]) < 1e-15) continue;
            double tt = d[a] > 0 ? (room.hi[a] - o[a]) / d[a] : (room.lo[a] - o[a]) / d[a];
            if (tt > 0 && tt < best) {
                best = tt;
                n[0] = n[1] = n[2] = 0;
                n[a] = d[a] > 0 ? -1.0 : 1.0;
            }
        }
        for (const Box &b : boxes) {
            double t0 = -1e30, t1 = 1e30;
            int ax = -1;
            double sgn = 0;
            bool miss = false;
            for (int a = 0; a < 3; ++a) {
                if (std::fabs(d[a]) < 1e-15) {
                    if (o[a] < b.lo[a] || o[a] > b.hi[a]) { miss = true; break; }
                    continue;
                }
                double ta = (b.lo[a] - o[a]) / d[a], tb = (b.hi[a] - o[a]) / d[a];
                double s = -1.0;
                if (ta > tb) { std::swap(ta, tb); s = 1.0; }
                if (ta > t0) { t0 = ta; ax = a; sgn = s; }
                t1 = std::min(t1, tb);
            }
            if (miss || t0 > t1 || t0 <= 0 || ax < 0) continue;
            if (t0 < best) {
                best = t0;
                n[0] = n[1] = n[2] = 0;
                n[ax] = sgn;
            }
        }
        for (const Cyl &c : cyls) {
            double ox = o[0] - c.cx, oz = o[2] - c.cz;
            double A = d[0] * d[0] + d[2] * d[2];
            if (A < 1e-15) continue;
            double B = 2 * (ox * d[0] + oz * d[2]), C = ox * ox + oz * oz - c.r * c.r;
            double disc = B * B - 4 * A * C;
            if (disc < 0) continue;
            double tt = (-B - std::sqrt(disc)) / (2 * A);
            if (tt <= 0 || tt >= best) continue;
            double y = o[1] + tt * d[1];
            if (y < c.y0 || y > c.y1) continue;
            best = tt;
            double hx = ox + tt * d[0], hz = oz + tt * d[2];
            n[0] = hx / c.r; n[1] = 0; n[2] = hz / c.r;
        }
        return best;
    }
};

namespace {

void yaw_rotation_cw(double yaw, double R[9]) {
    // R_wc = rotation about the (down-pointing) y axis; R_cw = R_wc^T
    double c = std::cos(yaw), s = std::sin(yaw);
    double Rwc[9] = {c, 0, s, 0, 1, 0, -s, 0, c};
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) R[3 * a + b] = Rwc[3 * b + a];
}

void pose_from_center(const double R[9], const double C[3], double t[3]) {
    for (int a = 0; a < 3; ++a) t[a] = -(R[3 * a] * C[0] + R[3 * a + 1] * C[1] + R[3 * a + 2] * C[2]);
}

}  // namespace

extern "C" {

pm_scene *pm_scene_create(int kind, uint32_t seed) {
    pm_scene *s = new pm_scene();
    s->kind = kind;
    s->seed = seed;
    s->base_freq = 2.0;
    Rng rng(seed * 7919ull + 11);
    if (kind == PM_SCENE_HALL) {
        s->room = {{-15, -2, -5}, {15, 2, 5}};
        for (int k = 0; k < 24; ++k) {
            double sx = rng.uni(0.5, 2.0), sy = rng.uni(0.5, 3.0), sz = rng.uni(0.5, 2.0);
            double cx = rng.uni(-14, 14), cz = rng.uni(-4.5, 4.5);
            // keep a central corridor (|z| < 1.2) free for the trajectory
            if (std::fabs(cz) < 1.2 + sz / 2) cz = (cz < 0 ? -1 : 1) * (1.2 + sz / 2 + rng.uni(0, 1.5));
            Box b{{cx - sx / 2, 2 - sy, cz - sz / 2}, {cx + sx / 2, 2, cz + sz / 2}};
            s->boxes.push_back(b);
        }
        s->base_freq = 1.5;
    } else {
        s->room = {{-5, -1.5, -3}, {5, 1.5, 3}};
        if (kind == PM_SCENE_ROOM_OBJECTS) {
            int placed = 0, guard = 0;
            while (placed < 5 && guard++ < 1000) {
                double sx = rng.uni(0.3, 1.5), sy = rng.uni(0.3, 1.5), sz = rng.uni(0.3, 1.5);
                double cx = rng.uni(-4.5 + sx / 2, 4.5 - sx / 2), cz = rng.uni(-2.5 + sz / 2, 2.5 - sz / 2);
                // objects stand on the floor (y = +1.5 is down) and keep 1.2 m from the origin
                if (std::fabs(cx) < 1.2 + sx / 2 && std::fabs(cz) < 1.2 + sz / 2) continue;
                Box b{{cx - sx / 2, 1.5 - sy, cz - sz / 2}, {cx + sx / 2, 1.5, cz + sz / 2}};
                s->boxes.push_back(b);
                ++placed;
            }
            for (int guard2 = 0; guard2 < 1000; ++guard2) {
                double cx = rng.uni(-4.0, 4.0), cz = rng.uni(-2.0, 2.0);
                if (std::sqrt(cx * cx + cz * cz) < 1.8) continue;
                bool clash = false;
                for (const Box &b : s->boxes)
                    if (cx > b.lo[0] - 0.6 && cx < b.hi[0] + 0.6 && cz > b.lo[2] - 0.6 && cz < b.hi[2] + 0.6)
                        clash = true;
                if (clash) continue;
                s->cyls.push_back({cx, cz, 0.5, -1.5, 1.5});
                break;
            }
        }
    }
    return s;
}

void pm_scene_destroy(pm_scene *s) { delete s; }

int pm_scene_describe(const pm_scene *s, pm_scene_desc *out) {
    if (!s || !out) return 1;
    std::memset(out, 0, sizeof *out);
    for (int a = 0; a < 3; ++a) {
        out->room_lo[a] = s->room.lo[a];
        out->room_hi[a] = s->room.hi[a];
    }
    out->n_boxes = std::min((int)s->boxes.size(), PM_SCENE_MAX_BOXES);
    for (int k = 0; k < out->n_boxes; ++k)
        for (int a = 0; a < 3; ++a) {
            out->box_lo[k][a] = s->boxes[k].lo[a];
            out->box_hi[k][a] = s->boxes[k].hi[a];
        }
    out->n_cyls = std::min((int)s->cyls.size(), PM_SCENE_MAX_CYLS);
    for (int k = 0; k < out->n_cyls; ++k) {
        const Cyl &c = s->cyls[k];
        out->cyl[k][0] = c.cx; out->cyl[k][1] = c.cz; out->cyl[k][2] = c.r; out->cyl[k][3] = c.y0; out->cyl[k][4] = c.y1;
    }
    out->seed = s->seed;
    out->base_freq = s->base_freq;
    return 0;
}

int pm_scene_poses(const pm_scene *s, int n_views, uint32_t seed, float bmin, float bmax, float yaw_deg,
                   double *R, double *t) {
    if (!s || n_views < 1 || !R || !t) return 1;
    Rng rng(seed * 104729ull + 3);
    double C0[3] = {0, 0, 0};
    for (int guard = 0; guard < 10000; ++guard) {
        if (s->kind == PM_SCENE_HALL) {
            C0[0] = rng.uni(-12, 12); C0[1] = rng.uni(-0.5, 0.5); C0[2] = rng.uni(-0.6, 0.6);
        } else {
            C0[0] = rng.uni(-0.5, 0.5); C0[1] = rng.uni(-0.3, 0.3); C0[2] = rng.uni(-0.5, 0.5);
        }
        if (s->free_space(C0, 0.3 + bmax)) break;
    }
    double yaw0 = rng.uni(-kPi, kPi);
    yaw_rotation_cw(yaw0, R);
    pose_from_center(R, C0, t);
    for (int v = 1; v < n_views; ++v) {
        double C[3];
        for (int guard = 0; guard < 1000; ++guard) {
            double d[3] = {rng.normal(), rng.normal(), rng.normal()};
            double n = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            double b = rng.uni(bmin, bmax);
            for (int a = 0; a < 3; ++a) C[a] = C0[a] + b * d[a] / n;
            if (s->free_space(C, 0.3)) break;
        }
        double yaw = yaw0 + rng.uni(-yaw_deg, yaw_deg) * kPi / 180.0;
        yaw_rotation_cw(yaw, R + 9 * v);
        pose_from_center(R + 9 * v, C, t + 3 * v);
    }
    return 0;
}

int pm_scene_trajectory_pose(const pm_scene *s, uint32_t seed, int n_waypoints, double duration_s, double t_s,
                             double R[9], double t[3]) {
    if (!s || n_waypoints < 4) return 1;
    Rng rng(seed * 15485863ull + 5);
    std::vector<double> P(3 * n_waypoints), Y(n_waypoints);
    for (int k = 0; k < n_waypoints; ++k) {
        double p[3];
        for (int guard = 0; guard < 10000; ++guard) {
            if (s->kind == PM_SCENE_HALL) {
                p[0] = -13.0 + 26.0 * k / (n_waypoints - 1) + rng.uni(-0.4, 0.4);
                p[1] = rng.uni(-0.4, 0.4);
                p[2] = rng.uni(-0.6, 0.6);
            } else {
                p[0] = rng.uni(-3.5, 3.5); p[1] = rng.uni(-0.5, 0.5); p[2] = rng.uni(-1.8, 1.8);
            }
            if (s->free_space(p, 0.4)) break;
        }
        for (int a = 0; a < 3; ++a) P[3 * k + a] = p[a];
        Y[k] = rng.uni(-0.6, 0.6);
    }
    double u = std::min(std::max(t_s / duration_s, 0.0), 1.0) * (n_waypoints - 1);
    int seg = std::min((int)u, n_waypoints - 2);
    double f = u - seg;
    auto at = [&](int k) { return std::min(std::max(k, 0), n_waypoints - 1); };
    int k0 = at(seg - 1), k1 = at(seg), k2 = at(seg + 1), k3 = at(seg + 2);
    double f2 = f * f, f3 = f2 * f;
    double w0 = -0.5 * f3 + f2 - 0.5 * f, w1 = 1.5 * f3 - 2.5 * f2 + 1.0, w2 = -1.5 * f3 + 2.0 * f2 + 0.5 * f,
           w3 = 0.5 * f3 - 0.5 * f2;
    double C[3];
    for (int a = 0; a < 3; ++a)
        C[a] = w0 * P[3 * k0 + a] + w1 * P[3 * k1 + a] + w2 * P[3 * k2 + a] + w3 * P[3 * k3 + a];
    double yaw = w0 * Y[k0] + w1 * Y[k1] + w2 * Y[k2] + w3 * Y[k3];
    yaw_rotation_cw(yaw, R);
    pose_from_center(R, C, t);
    return 0;
}

int pm_scene_render(const pm_scene *s, const double R[9], const double t[3], int W, int H, int supersample,
                    float noise_sigma, uint32_t noise_seed, float *gray, uint8_t *gray_u8, uint8_t *rgb,
                    float *depth, float *normal) {
    if (!s || W <= 0 || H <= 0 || supersample < 1) return 1;
    double C[3];
    for (int a = 0; a < 3; ++a) C[a] = -(R[a] * t[0] + R[3 + a] * t[1] + R[6 + a] * t[2]);
    const int ss = supersample;
#pragma omp parallel for schedule(dynamic, 4)
    for (int i = 0; i < H; ++i) {
        Rng nrng((uint64_t)noise_seed * 1000003ull + (uint64_t)i);
        for (int j = 0; j < W; ++j) {
            double acc = 0, accc[3] = {0, 0, 0};
            for (int si = 0; si < ss; ++si)
                for (int sj = 0; sj < ss; ++sj) {
                    double y = i + (ss > 1 ? (si + 0.5) / ss - 0.5 : 0.0);
                    double x = j + (ss > 1 ? (sj + 0.5) / ss - 0.5 : 0.0);
                    double lon = 2.0 * kPi * (x / W - 0.5), lat = -kPi * (y / H - 0.5);
                    double b[3] = {std::cos(lat) * std::sin(lon), -std::sin(lat), std::cos(lat) * std::cos(lon)};
                    double d[3];
                    for (int a = 0; a < 3; ++a) d[a] = R[a] * b[0] + R[3 + a] * b[1] + R[6 + a] * b[2];
                    double n[3];
                    double tt = s->intersect(C, d, n);
                    double p[3] = {C[0] + tt * d[0], C[1] + tt * d[1], C[2] + tt * d[2]};
                    acc += s->texture(p, 0);
                    if (rgb)
                        for (int c = 0; c < 3; ++c) accc[c] += s->texture(p, 1 + c);
                }
            size_t idx = (size_t)i * W + j;
            // analytic depth and normal along the pixel's own bearing
            double lon = 2.0 * kPi * ((double)j / W - 0.5), lat = -kPi * ((double)i / H - 0.5);
            double b[3] = {std::cos(lat) * std::sin(lon), -std::sin(lat), std::cos(lat) * std::cos(lon)};
            double d[3];
            for (int a = 0; a < 3; ++a) d[a] = R[a] * b[0] + R[3 + a] * b[1] + R[6 + a] * b[2];
            double n[3];
            double tt = s->intersect(C, d, n);
            if (depth) depth[idx] = (float)tt;
            if (normal) {
                double nc[3];
                for (int a = 0; a < 3; ++a) nc[a] = R[3 * a] * n[0] + R[3 * a + 1] * n[1] + R[3 * a + 2] * n[2];
                double dot = nc[0] * b[0] + nc[1] * b[1] + nc[2] * b[2];
                if (dot > 0) for (int a = 0; a < 3; ++a) nc[a] = -nc[a];
                for (int a = 0; a < 3; ++a) normal[3 * idx + a] = (float)nc[a];
            }
            double g = 255.0 * acc / (ss * ss);
            double gq = std::floor(g + 0.5);
            double gv = gq;
            if (noise_sigma > 0.0f) gv = std::min(255.0, std::max(0.0, g + noise_sigma * nrng.normal()));
            if (gray) gray[idx] = (float)gv;
            if (gray_u8) gray_u8[idx] = (uint8_t)std::min(255.0, std::max(0.0, std::floor(gv + 0.5)));
            if (rgb)
                for (int c = 0; c < 3; ++c)
                    rgb[3 * idx + c] = (uint8_t)std::min(255.0, std::floor(255.0 * accc[2 - c] / (ss * ss) + 0.5));
        }
    }
    return 0;
}

}  // extern "C"
