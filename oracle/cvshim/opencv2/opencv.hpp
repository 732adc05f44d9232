// Test infrastructure (oracle only): a minimal, project-written stand-in for the
// small part of OpenCV's core API that the reference's scene/physics headers
// use, so that those headers compile unmodified without OpenCV. It is written
// from OpenCV's documented semantics (cv::Vec, cv::Matx, cv::normalize,
// cv::Mat, cv::Scalar), not from OpenCV's sources, and implements only what
// the geodesic render path needs:
//   - cv::Vec<T,n>: element access, dot, cross, + - with vectors, * / with
//     scalars, +=, -=, *=, /=.
//   - cv::Matx<T,3,3>: 9-element constructor, inv() (adjugate / determinant,
//     a zero matrix when singular), Matx * Vec.
//   - cv::normalize(Vec): v * (1/|v|), and a zero vector for |v| == 0.
//   - cv::Mat: rows x cols of 8-bit, 3-channel (CV_8UC3) pixels with shared,
//     reference-counted storage; data, rows, cols, empty().
//   - cv::Scalar, CV_8UC3, IMREAD_COLOR.
// The rounding of OpenCV's own Matx::inv and normalize is not pinned by any
// reference test; on the orthonormal bases the render builds, inv() equals the
// transpose to about 1e-16.
#ifndef BH_ORACLE_CVSHIM_OPENCV_HPP_
#define BH_ORACLE_CVSHIM_OPENCV_HPP_

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <functional>
#include <initializer_list>
#include <iostream>
#include <map>
#include <memory>
#include <string>
#include <type_traits>
#include <vector>

namespace cv {

typedef unsigned char uchar;

enum { CV_8U = 0 };
#define CV_8UC3 16
enum ImreadModes { IMREAD_COLOR = 1 };

template <typename T, int n>
class Vec {
 public:
  typedef T value_type;
  T val[n];

  Vec() { for (int i = 0; i < n; ++i) val[i] = T(0); }
  Vec(T v0, T v1) { static_assert(n == 2, "Vec(2)"); val[0] = v0; val[1] = v1; }
  Vec(T v0, T v1, T v2) {
    static_assert(n == 3, "Vec(3)");
    val[0] = v0; val[1] = v1; val[2] = v2;
  }
  Vec(T v0, T v1, T v2, T v3) {
    static_assert(n == 4, "Vec(4)");
    val[0] = v0; val[1] = v1; val[2] = v2; val[3] = v3;
  }

  T& operator[](int i) { return val[i]; }
  const T& operator[](int i) const { return val[i]; }
  T& operator()(int i) { return val[i]; }
  const T& operator()(int i) const { return val[i]; }

  T dot(const Vec& o) const {
    T s = T(0);
    for (int i = 0; i < n; ++i) s += val[i] * o.val[i];
    return s;
  }

  Vec cross(const Vec& o) const {
    static_assert(n == 3, "cross needs 3 components");
    return Vec(val[1] * o.val[2] - val[2] * o.val[1],
               val[2] * o.val[0] - val[0] * o.val[2],
               val[0] * o.val[1] - val[1] * o.val[0]);
  }

  Vec& operator+=(const Vec& o) { for (int i = 0; i < n; ++i) val[i] += o.val[i]; return *this; }
  Vec& operator-=(const Vec& o) { for (int i = 0; i < n; ++i) val[i] -= o.val[i]; return *this; }
  template <typename S, std::enable_if_t<std::is_arithmetic_v<S>, int> = 0>
  Vec& operator*=(S s) { for (int i = 0; i < n; ++i) val[i] = T(val[i] * s); return *this; }
  template <typename S, std::enable_if_t<std::is_arithmetic_v<S>, int> = 0>
  Vec& operator/=(S s) { for (int i = 0; i < n; ++i) val[i] = T(val[i] / s); return *this; }
};

typedef Vec<uchar, 3> Vec3b;
typedef Vec<double, 3> Vec3d;
typedef Vec<float, 3> Vec3f;

template <typename T, int n>
inline Vec<T, n> operator+(Vec<T, n> a, const Vec<T, n>& b) { a += b; return a; }
template <typename T, int n>
inline Vec<T, n> operator-(Vec<T, n> a, const Vec<T, n>& b) { a -= b; return a; }
template <typename T, int n>
inline Vec<T, n> operator-(const Vec<T, n>& a) {
  Vec<T, n> r;
  for (int i = 0; i < n; ++i) r[i] = -a[i];
  return r;
}
template <typename T, int n, typename S, std::enable_if_t<std::is_arithmetic_v<S>, int> = 0>
inline Vec<T, n> operator*(Vec<T, n> a, S s) { a *= s; return a; }
template <typename T, int n, typename S, std::enable_if_t<std::is_arithmetic_v<S>, int> = 0>
inline Vec<T, n> operator*(S s, Vec<T, n> a) { a *= s; return a; }
template <typename T, int n, typename S, std::enable_if_t<std::is_arithmetic_v<S>, int> = 0>
inline Vec<T, n> operator/(Vec<T, n> a, S s) { a /= s; return a; }
template <typename T, int n>
inline bool operator==(const Vec<T, n>& a, const Vec<T, n>& b) {
  for (int i = 0; i < n; ++i) if (!(a[i] == b[i])) return false;
  return true;
}

template <typename T, int n>
inline std::ostream& operator<<(std::ostream& os, const Vec<T, n>& v) {
  os << '[';
  for (int i = 0; i < n; ++i) os << (i ? ", " : "") << +v[i];
  return os << ']';
}

template <typename T, int n>
inline Vec<T, n> normalize(const Vec<T, n>& v) {
  const double len = std::sqrt(double(v.dot(v)));
  const double k = len != 0.0 ? 1.0 / len : 0.0;
  Vec<T, n> r;
  for (int i = 0; i < n; ++i) r[i] = T(v[i] * k);
  return r;
}

template <typename T, int m, int n>
class Matx {
 public:
  T val[m * n];

  Matx() { for (int i = 0; i < m * n; ++i) val[i] = T(0); }
  Matx(T v0, T v1, T v2, T v3, T v4, T v5, T v6, T v7, T v8) {
    static_assert(m * n == 9, "9-element Matx");
    const T v[9] = {v0, v1, v2, v3, v4, v5, v6, v7, v8};
    for (int i = 0; i < 9; ++i) val[i] = v[i];
  }

  T& operator()(int i, int j) { return val[i * n + j]; }
  const T& operator()(int i, int j) const { return val[i * n + j]; }

  // Inverse of a 3x3 matrix as adjugate / determinant; zero matrix if singular.
  Matx<T, n, m> inv() const {
    static_assert(m == 3 && n == 3, "inv() implemented for 3x3 only");
    const Matx& a = *this;
    const T c00 = a(1, 1) * a(2, 2) - a(1, 2) * a(2, 1);
    const T c01 = a(1, 2) * a(2, 0) - a(1, 0) * a(2, 2);
    const T c02 = a(1, 0) * a(2, 1) - a(1, 1) * a(2, 0);
    const T det = a(0, 0) * c00 + a(0, 1) * c01 + a(0, 2) * c02;
    Matx<T, n, m> r;
    if (det == T(0)) return r;
    const T k = T(1) / det;
    r(0, 0) = c00 * k;
    r(1, 0) = c01 * k;
    r(2, 0) = c02 * k;
    r(0, 1) = (a(0, 2) * a(2, 1) - a(0, 1) * a(2, 2)) * k;
    r(1, 1) = (a(0, 0) * a(2, 2) - a(0, 2) * a(2, 0)) * k;
    r(2, 1) = (a(0, 1) * a(2, 0) - a(0, 0) * a(2, 1)) * k;
    r(0, 2) = (a(0, 1) * a(1, 2) - a(0, 2) * a(1, 1)) * k;
    r(1, 2) = (a(0, 2) * a(1, 0) - a(0, 0) * a(1, 2)) * k;
    r(2, 2) = (a(0, 0) * a(1, 1) - a(0, 1) * a(1, 0)) * k;
    return r;
  }
};

template <typename T, int m, int n>
inline Vec<T, m> operator*(const Matx<T, m, n>& a, const Vec<T, n>& v) {
  Vec<T, m> r;
  for (int i = 0; i < m; ++i) {
    T s = T(0);
    for (int j = 0; j < n; ++j) s += a(i, j) * v[j];
    r[i] = s;
  }
  return r;
}

class Scalar {
 public:
  double val[4] = {0, 0, 0, 0};
  Scalar() = default;
  Scalar(double v0, double v1 = 0, double v2 = 0, double v3 = 0) {
    val[0] = v0; val[1] = v1; val[2] = v2; val[3] = v3;
  }
  template <typename T, int n>
  Scalar(const Vec<T, n>& v) {
    for (int i = 0; i < n && i < 4; ++i) val[i] = double(v[i]);
  }
  double operator[](int i) const { return val[i]; }
};

// Row-major 8-bit, 3-channel image with shared storage (copies share pixels).
class Mat {
 public:
  int rows = 0;
  int cols = 0;
  uchar* data = nullptr;

  Mat() = default;
  Mat(int r, int c, int type) { create(r, c, type); }
  Mat(int r, int c, int type, const Scalar& s) {
    create(r, c, type);
    for (long i = 0; i < long(r) * c; ++i)
      for (int ch = 0; ch < 3; ++ch) data[i * 3 + ch] = uchar(s[ch]);
  }

  bool empty() const { return data == nullptr || rows == 0 || cols == 0; }
  int channels() const { return 3; }
  size_t total() const { return size_t(rows) * size_t(cols); }

 private:
  void create(int r, int c, int type) {
    if (type != CV_8UC3) {
      std::cerr << "cvshim: only CV_8UC3 is supported\n";
      std::abort();
    }
    rows = r;
    cols = c;
    storage_ = std::make_shared<std::vector<uchar>>(size_t(r) * size_t(c) * 3, uchar(0));
    data = storage_->data();
  }
  std::shared_ptr<std::vector<uchar>> storage_;
};

}  // namespace cv

#endif  // BH_ORACLE_CVSHIM_OPENCV_HPP_
