// Dense map output: the fused point cloud as an ASCII PLY file and as the
// dense map message (MessagePack), the two formats the reference writes after
// densification.  Host code; points come from pm_fuse / pm_fuse_noalloc.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "pm_gb300.h"

namespace {

// A minimal MessagePack writer for the value kinds the dense map uses: maps,
// arrays, UTF-8 strings, unsigned integers and float64 (the encodings a JSON
// document of those kinds maps to: smallest integer width, float64 for reals).
struct Pack {
    std::vector<uint8_t> b;
    void be(uint64_t v, int bytes) {
        for (int k = bytes - 1; k >= 0; --k) b.push_back((uint8_t)(v >> (8 * k)));
    }
    void map(uint32_t n) {
        if (n < 16) b.push_back((uint8_t)(0x80 | n));
        else if (n < 65536) { b.push_back(0xde); be(n, 2); }
        else { b.push_back(0xdf); be(n, 4); }
    }
    void arr(uint32_t n) {
        if (n < 16) b.push_back((uint8_t)(0x90 | n));
        else if (n < 65536) { b.push_back(0xdc); be(n, 2); }
        else { b.push_back(0xdd); be(n, 4); }
    }
    void str(const std::string &s) {
        const size_t n = s.size();
        if (n < 32) b.push_back((uint8_t)(0xa0 | n));
        else if (n < 256) { b.push_back(0xd9); be(n, 1); }
        else if (n < 65536) { b.push_back(0xda); be(n, 2); }
        else { b.push_back(0xdb); be(n, 4); }
        b.insert(b.end(), s.begin(), s.end());
    }
    void uint(uint64_t v) {
        if (v < 128) b.push_back((uint8_t)v);
        else if (v < 256) { b.push_back(0xcc); be(v, 1); }
        else if (v < 65536) { b.push_back(0xcd); be(v, 2); }
        else if (v < 4294967296ull) { b.push_back(0xce); be(v, 4); }
        else { b.push_back(0xcf); be(v, 8); }
    }
    void f64(double d) {
        uint64_t u;
        std::memcpy(&u, &d, 8);
        b.push_back(0xcb);
        be(u, 8);
    }
};

bool points_ok(const pm_points *p) {
    return p && p->count >= 0 && p->count <= p->capacity && (p->count == 0 || p->xyz);
}

}  // namespace

extern "C" {

// map_database_io::save_point_cloud_dense (io/map_database_io.cc:45-80): ASCII
// PLY with float x y z and uchar red green blue properties; coordinates in
// fixed notation with 6 decimals, colours written in the stored order (the
// reference stores BGR from its colour thumbnails under these names).  Points
// without colours are written white.
int pm_write_ply(const char *path, const pm_points *pts) {
    if (!path || !points_ok(pts)) return PM_EINVAL;
    FILE *f = std::fopen(path, "w");
    if (!f) return PM_EINVAL;
    std::fprintf(f,
                 "ply\nformat ascii 1.0\nelement vertex %d\nproperty float x\nproperty float y\nproperty float z\n"
                 "property uchar red\nproperty uchar green\nproperty uchar blue\nend_header\n",
                 pts->count);
    for (int k = 0; k < pts->count; ++k) {
        const double *p = pts->xyz + 3 * (size_t)k;
        const unsigned c0 = pts->bgr ? pts->bgr[3 * (size_t)k] : 255u;
        const unsigned c1 = pts->bgr ? pts->bgr[3 * (size_t)k + 1] : 255u;
        const unsigned c2 = pts->bgr ? pts->bgr[3 * (size_t)k + 2] : 255u;
        std::fprintf(f, "%f %f %f %u %u %u\n", p[0], p[1], p[2], c0, c1, c2);
    }
    const int bad = std::ferror(f);
    std::fclose(f);
    return bad ? PM_EINVAL : PM_OK;
}

// map_database_io::save_message_pack_dense (io/map_database_io.cc:22-43) with
// the landmark records of landmark::to_json (data/landmark.cc:370-377):
// {"cameras": {}, "keyframes": {}, "landmarks": {"<id>": {"1st_keyfrm": kf,
// "pos_w": [x, y, z], "ref_keyfrm": kf, "n_vis": 1, "n_fnd": 1,
// "color": [c0, c1, c2]}}}, ids first_id, first_id + 1, ... in point order.
// Keys are written in sorted order (as a JSON object serialises); the camera
// and keyframe tables belong to the SLAM map and are left empty.
int pm_write_dense_msgpack(const char *path, const pm_points *pts, uint64_t first_id, uint32_t keyframe_id) {
    if (!path || !points_ok(pts)) return PM_EINVAL;
    Pack m;
    m.map(3);
    m.str("cameras");
    m.map(0);
    m.str("keyframes");
    m.map(0);
    m.str("landmarks");
    // the record keys sort as strings ("10" < "9"), like a JSON object's keys
    std::vector<std::string> keys(pts->count);
    std::vector<int> order(pts->count);
    for (int k = 0; k < pts->count; ++k) {
        keys[k] = std::to_string(first_id + (uint64_t)k);
        order[k] = k;
    }
    std::sort(order.begin(), order.end(), [&](int a, int b) { return keys[a] < keys[b]; });
    m.map((uint32_t)pts->count);
    for (int q = 0; q < pts->count; ++q) {
        const int k = order[q];
        m.str(keys[k]);
        m.map(6);
        m.str("1st_keyfrm");
        m.uint(keyframe_id);
        m.str("color");
        m.arr(3);
        for (int a = 0; a < 3; ++a) m.f64(pts->bgr ? (double)pts->bgr[3 * (size_t)k + a] : 255.0);
        m.str("n_fnd");
        m.uint(1);
        m.str("n_vis");
        m.uint(1);
        m.str("pos_w");
        m.arr(3);
        for (int a = 0; a < 3; ++a) m.f64(pts->xyz[3 * (size_t)k + a]);
        m.str("ref_keyfrm");
        m.uint(keyframe_id);
    }
    FILE *f = std::fopen(path, "wb");
    if (!f) return PM_EINVAL;
    const size_t w = std::fwrite(m.b.data(), 1, m.b.size(), f);
    std::fclose(f);
    return w == m.b.size() ? PM_OK : PM_EINVAL;
}

}  // extern "C"
