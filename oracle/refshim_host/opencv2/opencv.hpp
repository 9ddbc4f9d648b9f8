// A minimal stand-in for the parts of OpenCV that the reference's host
// densification code (src/openvslam/depthmap.{h,cc}) uses, so that file can
// be compiled unmodified as a parity checker for the restated host stages
// (post-filter, consistency filter, fusion).  TEST INFRASTRUCTURE ONLY: it is
// never linked into the product.  Semantics follow OpenCV's documentation:
// a Mat shares its buffer on copy (clone() makes a deep copy), element access
// by at<T>(row, col), row-major storage, Vec/Matx small fixed-size algebra,
// medianBlur with a 3x3 window and replicated borders.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <iostream>
#include <memory>
#include <vector>

typedef unsigned char uchar;

#define CV_8U 0
#define CV_32S 4
#define CV_32F 5
#define CV_64F 6
#define CV_MAKETYPE(d, c) ((d) + (((c) - 1) << 3))
#define CV_8UC3 CV_MAKETYPE(CV_8U, 3)
#define CV_32FC3 CV_MAKETYPE(CV_32F, 3)
#define CV_64FC3 CV_MAKETYPE(CV_64F, 3)

namespace cv {

template <typename T, int n>
struct Vec {
    T val[n];
    Vec() { for (int k = 0; k < n; ++k) val[k] = T(0); }
    Vec(T a, T b) { static_assert(n == 2, ""); val[0] = a; val[1] = b; }
    Vec(T a, T b, T c) { static_assert(n == 3, ""); val[0] = a; val[1] = b; val[2] = c; }
    T &operator[](int k) { return val[k]; }
    const T &operator[](int k) const { return val[k]; }
    T &operator()(int k) { return val[k]; }
    const T &operator()(int k) const { return val[k]; }
    T dot(const Vec &o) const { T s = T(0); for (int k = 0; k < n; ++k) s += val[k] * o.val[k]; return s; }
    Vec operator-() const { Vec r; for (int k = 0; k < n; ++k) r.val[k] = -val[k]; return r; }
    Vec &operator+=(const Vec &o) { for (int k = 0; k < n; ++k) val[k] += o.val[k]; return *this; }
    Vec &operator-=(const Vec &o) { for (int k = 0; k < n; ++k) val[k] -= o.val[k]; return *this; }
    Vec &operator*=(double s) { for (int k = 0; k < n; ++k) val[k] = T(val[k] * s); return *this; }
};
template <typename T, int n> Vec<T, n> operator+(Vec<T, n> a, const Vec<T, n> &b) { return a += b; }
template <typename T, int n> Vec<T, n> operator-(Vec<T, n> a, const Vec<T, n> &b) { return a -= b; }
template <typename T, int n> Vec<T, n> operator*(Vec<T, n> a, double s) {
    for (int k = 0; k < n; ++k) a.val[k] = T(a.val[k] * s);
    return a;
}
template <typename T, int n> Vec<T, n> operator*(double s, Vec<T, n> a) { return a * s; }
template <typename T, int n> Vec<T, n> operator/(Vec<T, n> a, double s) {
    for (int k = 0; k < n; ++k) a.val[k] = T(a.val[k] / s);
    return a;
}
typedef Vec<double, 3> Vec3d;
typedef Vec<float, 3> Vec3f;
typedef Vec<uchar, 3> Vec3b;
typedef Vec<int, 2> Vec2i;

template <typename T, int n> double norm(const Vec<T, n> &v) {
    double s = 0;
    for (int k = 0; k < n; ++k) s += (double)v.val[k] * (double)v.val[k];
    return std::sqrt(s);
}
template <typename T, int n> Vec<T, n> normalize(const Vec<T, n> &v) {
    const double l = norm(v);
    return l > 0 ? v / l : v;
}

template <typename T, int m, int n>
struct Matx {
    T val[m * n];
    Matx() { for (int k = 0; k < m * n; ++k) val[k] = T(0); }
    explicit Matx(const T *p) { for (int k = 0; k < m * n; ++k) val[k] = p[k]; }
    Matx(T a0, T a1, T a2, T a3, T a4, T a5, T a6, T a7, T a8) {
        static_assert(m * n == 9, "");
        T a[9] = {a0, a1, a2, a3, a4, a5, a6, a7, a8};
        for (int k = 0; k < 9; ++k) val[k] = a[k];
    }
    template <typename U>
    Matx(const Matx<U, m, n> &o) { for (int k = 0; k < m * n; ++k) val[k] = T(o.val[k]); }
    T &operator()(int i, int j) { return val[i * n + j]; }
    const T &operator()(int i, int j) const { return val[i * n + j]; }
    Matx<T, n, m> t() const {
        Matx<T, n, m> r;
        for (int i = 0; i < m; ++i)
            for (int j = 0; j < n; ++j) r(j, i) = (*this)(i, j);
        return r;
    }
    Matx operator-() const { Matx r; for (int k = 0; k < m * n; ++k) r.val[k] = -val[k]; return r; }
    static Matx eye() { Matx r; for (int k = 0; k < std::min(m, n); ++k) r(k, k) = T(1); return r; }
};
template <typename T, int m, int n, int p>
Matx<T, m, p> operator*(const Matx<T, m, n> &a, const Matx<T, n, p> &b) {
    Matx<T, m, p> r;
    for (int i = 0; i < m; ++i)
        for (int j = 0; j < p; ++j) {
            T s = T(0);
            for (int k = 0; k < n; ++k) s += a(i, k) * b(k, j);
            r(i, j) = s;
        }
    return r;
}
template <typename T, int m, int n>
Vec<T, m> operator*(const Matx<T, m, n> &a, const Vec<T, n> &v) {
    Vec<T, m> r;
    for (int i = 0; i < m; ++i) {
        T s = T(0);
        for (int k = 0; k < n; ++k) s += a(i, k) * v.val[k];
        r.val[i] = s;
    }
    return r;
}
typedef Matx<double, 3, 3> Matx33d;
typedef Matx<float, 3, 3> Matx33f;

struct Scalar {
    double v[4];
    Scalar(double a = 0, double b = 0, double c = 0, double d = 0) : v{a, b, c, d} {}
};

inline int elem_size(int type) {
    const int depth = type & 7, cn = (type >> 3) + 1;
    const int b = depth == CV_8U ? 1 : (depth == CV_32S || depth == CV_32F) ? 4 : 8;
    return b * cn;
}

class Mat {
  public:
    int rows = 0, cols = 0;
    uchar *data = nullptr;
    size_t step[2] = {0, 0};
    Mat() = default;
    Mat(int r, int c, int type) { create(r, c, type); }
    Mat(int r, int c, int type, const Scalar &s) { create(r, c, type); fill(s); }
    void create(int r, int c, int type) {
        rows = r;
        cols = c;
        type_ = type;
        step[1] = (size_t)elem_size(type);
        step[0] = step[1] * (size_t)c;
        buf_ = std::make_shared<std::vector<uchar>>(step[0] * (size_t)r, 0);
        data = buf_->data();
    }
    int type() const { return type_; }
    bool empty() const { return data == nullptr || rows * cols == 0; }
    template <typename T> T &at(int i, int j) { return *reinterpret_cast<T *>(data + step[0] * i + step[1] * j); }
    template <typename T> const T &at(int i, int j) const {
        return *reinterpret_cast<const T *>(data + step[0] * i + step[1] * j);
    }
    uchar *ptr(int i = 0) { return data + step[0] * i; }
    const uchar *ptr(int i = 0) const { return data + step[0] * i; }
    template <typename T> T *ptr(int i = 0) { return reinterpret_cast<T *>(ptr(i)); }
    Mat clone() const {
        Mat m;
        if (!data) return m;
        m.create(rows, cols, type_);
        std::memcpy(m.data, data, step[0] * rows);
        return m;
    }
    void convertTo(Mat &dst, int type, double alpha = 1.0, double beta = 0.0) const;
    static Mat eye(int r, int c, int type) {
        Mat m(r, c, type, Scalar(0));
        for (int k = 0; k < std::min(r, c); ++k) m.set_scalar(k, k, 1.0);
        return m;
    }
    double get_scalar(int i, int j, int ch = 0) const {
        const uchar *p = data + step[0] * i + step[1] * j;
        switch (type_ & 7) {
            case CV_8U: return p[ch];
            case CV_32S: return reinterpret_cast<const int32_t *>(p)[ch];
            case CV_32F: return reinterpret_cast<const float *>(p)[ch];
            default: return reinterpret_cast<const double *>(p)[ch];
        }
    }
    void set_scalar(int i, int j, double v, int ch = 0) {
        uchar *p = data + step[0] * i + step[1] * j;
        switch (type_ & 7) {
            case CV_8U: p[ch] = (uchar)v; break;
            case CV_32S: reinterpret_cast<int32_t *>(p)[ch] = (int32_t)v; break;
            case CV_32F: reinterpret_cast<float *>(p)[ch] = (float)v; break;
            default: reinterpret_cast<double *>(p)[ch] = v; break;
        }
    }

  private:
    void fill(const Scalar &s) {
        const int cn = (type_ >> 3) + 1;
        for (int i = 0; i < rows; ++i)
            for (int j = 0; j < cols; ++j)
                for (int ch = 0; ch < cn; ++ch) set_scalar(i, j, s.v[ch < 4 ? ch : 3], ch);
    }
    int type_ = 0;
    std::shared_ptr<std::vector<uchar>> buf_;
};

inline void Mat::convertTo(Mat &dst, int type, double alpha, double beta) const {
    const int cn = (type_ >> 3) + 1;
    Mat out(rows, cols, (type & 7) | ((cn - 1) << 3));
    for (int i = 0; i < rows; ++i)
        for (int j = 0; j < cols; ++j)
            for (int ch = 0; ch < cn; ++ch) out.set_scalar(i, j, get_scalar(i, j, ch) * alpha + beta, ch);
    dst = out;
}

inline Mat operator*(const Mat &a, const Mat &b) {
    Mat r(a.rows, b.cols, CV_64F, Scalar(0));
    for (int i = 0; i < a.rows; ++i)
        for (int j = 0; j < b.cols; ++j) {
            double s = 0;
            for (int k = 0; k < a.cols; ++k) s += a.get_scalar(i, k) * b.get_scalar(k, j);
            r.set_scalar(i, j, s);
        }
    return r;
}

inline Mat operator/(const Mat &a, double s) {
    Mat r = a.clone();
    const int cn = (r.type() >> 3) + 1;
    for (int i = 0; i < r.rows; ++i)
        for (int j = 0; j < r.cols; ++j)
            for (int ch = 0; ch < cn; ++ch) r.set_scalar(i, j, r.get_scalar(i, j, ch) / s, ch);
    return r;
}

// 3x3 median of a single-channel float image, replicated borders
// (OpenCV's medianBlur for CV_32F with ksize 3).
inline void medianBlur(const Mat &src, Mat &dst, int ksize) {
    Mat out(src.rows, src.cols, src.type());
    const int h = ksize / 2;
    std::vector<float> w;
    for (int i = 0; i < src.rows; ++i)
        for (int j = 0; j < src.cols; ++j) {
            w.clear();
            for (int di = -h; di <= h; ++di)
                for (int dj = -h; dj <= h; ++dj) {
                    const int y = std::min(std::max(i + di, 0), src.rows - 1);
                    const int x = std::min(std::max(j + dj, 0), src.cols - 1);
                    w.push_back(src.at<float>(y, x));
                }
            std::nth_element(w.begin(), w.begin() + w.size() / 2, w.end());
            out.at<float>(i, j) = w[w.size() / 2];
        }
    dst = out;
}

}  // namespace cv
