// blackhole_gb300.hpp -- header-only C++ face of the GB300 geodesic ray tracer.
//
// Drop-in for the reference's scene types and its render loop. The reference
// builds a scene from
//   Camera<T>(width, height, fov)                      camera.h:30-41
//   StaticBlackhole<T>(position, mass)                  blackhole_solution.h:24
//   Annulus<T>(p1, p2, p3, p4, r_outer, r_inner)        object/vector_object.h:320-325
//   Material::SetTexture(texture)                       object/material.h:29-35
//   Object pose methods RotateX/Y/Z, MoveTo, Move*      object/object.h:58-93
// and renders it inline in blackhole_solution_test.cc:161-298. The same class
// names, constructors, pose methods and accessors are kept here (same
// semantics: rotations about the object's own axes by Rodrigues' formula,
// matrix.h:342-356; the Annulus normal fixed at construction; the camera's
// fov clamp and focus length), and the loop becomes one call:
//
//   blackhole::Camera<double> cam(640, 360, fov);  cam.RotateY(...);  cam.MoveTo(...);
//   blackhole::StaticBlackhole<double> bh({0, 0, 0}, 1.0);
//   blackhole::Annulus<double> disc(p1, p2, p3, p4, 20.0, 6.0);
//   disc.SetTexture(blackhole::Texture::FromPixels(w, h, BH_TEXEL_BGR8, bytes));
//   blackhole::Image screen = blackhole::Render(cam, bh, &disc, nullptr);   // BGR24, CV_8UC3 layout
//
// Rectangle<T>, Triangle<T>, InfinitePlane<T> and ChessPattern2D<T> are kept
// as well: a Scene<T> lists them in `objects`.
//
// Additions the reference does not have: Annulus::r_inner()/r_outer()
// (private there, vector_object.h:353-355), a Background (equirectangular
// sky; the reference leaves missed rays black), Options (integrator,
// precision, schedule ...), batched renders, scenes with several holes
// (Scene<T>::extra_holes with BH_INTEGRATOR_MULTI) and the differentiable
// render's adjoint. Everything goes through the C ABI of bh_gb300.h; failures throw
// blackhole::Error (where the reference calls std::terminate on an empty
// texture, material.h:30-33, SetTexture throws).
//
// Vector type: blackhole::Vec3<T> (cv::Vec<T, 3> semantics for the
// operations used). Define BH_GB300_WITH_OPENCV before including to use
// cv::Vec<T, 3> instead and to get cv::Mat overloads of SetTexture, the
// Background constructor and Render (CV_8UC3 / CV_8UC4 textures, a CV_8UC3
// screen).
#ifndef BLACKHOLE_GB300_HPP_
#define BLACKHOLE_GB300_HPP_

#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <initializer_list>
#include <limits>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "bh_gb300.h"

#ifdef BH_GB300_WITH_OPENCV
#include <opencv2/core.hpp>
#endif

namespace blackhole {

// ---------------------------------------------------------------------------
// errors
class Error : public std::runtime_error {
 public:
  Error(int code, const std::string& what) : std::runtime_error(what), code_(code) {}
  int code() const { return code_; }

 private:
  int code_;
};

// ---------------------------------------------------------------------------
// vectors
#ifdef BH_GB300_WITH_OPENCV
template <typename T>
using Vec3 = cv::Vec<T, 3>;
template <typename T>
inline Vec3<T> normalize(const Vec3<T>& v) { return cv::normalize(v); }
#else
template <typename T>
struct Vec3 {
  T val[3] = {T(0), T(0), T(0)};
  Vec3() = default;
  Vec3(T x, T y, T z) : val{x, y, z} {}
  T& operator[](int i) { return val[i]; }
  const T& operator[](int i) const { return val[i]; }
  T dot(const Vec3& o) const { return val[0] * o[0] + val[1] * o[1] + val[2] * o[2]; }
  Vec3 cross(const Vec3& o) const {
    return {val[1] * o[2] - val[2] * o[1], val[2] * o[0] - val[0] * o[2], val[0] * o[1] - val[1] * o[0]};
  }
  Vec3& operator+=(const Vec3& o) { for (int i = 0; i < 3; ++i) val[i] += o[i]; return *this; }
  Vec3& operator-=(const Vec3& o) { for (int i = 0; i < 3; ++i) val[i] -= o[i]; return *this; }
  friend Vec3 operator+(Vec3 a, const Vec3& b) { return a += b; }
  friend Vec3 operator-(Vec3 a, const Vec3& b) { return a -= b; }
  friend Vec3 operator*(Vec3 a, T s) { for (int i = 0; i < 3; ++i) a[i] *= s; return a; }
  friend Vec3 operator*(T s, Vec3 a) { return a * s; }
  friend Vec3 operator/(Vec3 a, T s) { for (int i = 0; i < 3; ++i) a[i] /= s; return a; }
  friend bool operator==(const Vec3& a, const Vec3& b) { return a[0] == b[0] && a[1] == b[1] && a[2] == b[2]; }
};
// cv::normalize: v * (1 / |v|); a zero vector stays zero.
template <typename T>
inline Vec3<T> normalize(const Vec3<T>& v) {
  const T n = std::sqrt(v.dot(v));
  return v * (n != T(0) ? T(1) / n : T(0));
}
#endif

template <typename T>
using Mat3 = std::array<std::array<T, 3>, 3>;

// Rotation about the axis v by theta (Rodrigues; matrix.h:342-356).
template <typename T>
inline Mat3<T> RotationMatrixForAxis(const Vec3<T>& v, T theta) {
  const Vec3<T> u = normalize(v);
  const T c = std::cos(theta), c2 = T(1) - c, s = std::sin(theta);
  const T x = u[0], y = u[1], z = u[2];
  return {{{c + x * x * c2, x * y * c2 - z * s, x * z * c2 + y * s},
           {y * x * c2 + z * s, c + y * y * c2, y * z * c2 - x * s},
           {z * x * c2 - y * s, z * y * c2 + x * s, c + z * z * c2}}};
}

template <typename T>
inline Vec3<T> operator*(const Mat3<T>& m, const Vec3<T>& v) {
  return Vec3<T>(m[0][0] * v[0] + m[0][1] * v[1] + m[0][2] * v[2], m[1][0] * v[0] + m[1][1] * v[1] + m[1][2] * v[2],
                 m[2][0] * v[0] + m[2][1] * v[1] + m[2][2] * v[2]);
}

// ---------------------------------------------------------------------------
// Object<T> (object/object.h:23-118): vertices (vertex()[0] is the position)
// and three axes; rotations turn the axes and the vertices about the position.
template <typename T>
class Object {
 public:
  using value_type = T;
  using point_type = Vec3<T>;
  using vector_type = Vec3<T>;

  Object() = default;
  explicit Object(const point_type& p) : vertex_({p}) {}
  // appended to the default (0,0,0) vertex, as in the reference
  Object(std::initializer_list<point_type> il) { vertex_.insert(vertex_.end(), il); }
  Object(const vector_type& vx, const vector_type& vy, const vector_type& vz)
      : vx_(normalize(vx)), vy_(normalize(vy)), vz_(normalize(vz)) {}
  Object(const point_type& p, const vector_type& vx, const vector_type& vy, const vector_type& vz)
      : vertex_({p}), vx_(normalize(vx)), vy_(normalize(vy)), vz_(normalize(vz)) {}
  Object(const point_type& p, const vector_type& vx, const vector_type& vy, const vector_type& vz,
         std::initializer_list<point_type> il)
      : vertex_({p}), vx_(normalize(vx)), vy_(normalize(vy)), vz_(normalize(vz)) {
    vertex_.insert(vertex_.end(), il.begin(), il.end());
  }
  virtual ~Object() = default;

  void RotateZ(value_type rad) { Turn(vz_, rad, &vx_, &vy_); }
  void RotateY(value_type rad) { Turn(vy_, rad, &vx_, &vz_); }
  void RotateX(value_type rad) { Turn(vx_, rad, &vy_, &vz_); }

  void MoveTo(const point_type& p) { vertex_[0] = p; }
  void MoveTo(value_type x, value_type y, value_type z) { vertex_[0] = point_type(x, y, z); }
  void Move(value_type dx, value_type dy, value_type dz) { MoveX(dx); MoveY(dy); MoveZ(dz); }
  void MoveX(value_type d) { for (auto& v : vertex_) v += vx_ * d; }
  void MoveY(value_type d) { for (auto& v : vertex_) v += vy_ * d; }
  void MoveZ(value_type d) { for (auto& v : vertex_) v += vz_ * d; }

  const point_type& position() const { return vertex_[0]; }
  const vector_type& vector_x() const { return vx_; }
  const vector_type& vector_y() const { return vy_; }
  const vector_type& vector_z() const { return vz_; }
  const std::vector<point_type>& vertex() const { return vertex_; }

  void name(std::string n) { name_ = std::move(n); }
  const std::string& name() const { return name_; }

 private:
  void Turn(const vector_type& axis, value_type rad, vector_type* a, vector_type* b) {
    const Mat3<T> r = RotationMatrixForAxis(axis, rad);
    *a = normalize(r * *a);
    *b = normalize(r * *b);
    const point_type pos = vertex_[0];
    for (auto& v : vertex_) v = r * (v - pos) + pos;
  }

  std::vector<point_type> vertex_ = {point_type(0, 0, 0)};
  vector_type vx_ = vector_type(1, 0, 0), vy_ = vector_type(0, 1, 0), vz_ = vector_type(0, 0, 1);
  std::string name_ = "Unnamed";
};

// Camera<T> (camera.h:21-71): axes (1,0,0), (0,-1,0), (0,0,-1); the fov is
// clamped to [0, pi) and sets focus_len = width / (2 tan(fov / 2)).
template <typename T>
class Camera : public Object<T> {
 public:
  using typename Object<T>::value_type;
  using typename Object<T>::vector_type;

  Camera(int width, int height, value_type fov_x)
      : Object<T>(vector_type(0, 0, 0), vector_type(1, 0, 0), vector_type(0, -1, 0), vector_type(0, 0, -1)),
        width_(width),
        height_(height) {
    fov(fov_x);
  }
  void fov(value_type fov_x) {
    const value_type hi = std::nextafter(value_type(3.14159265358979323846), value_type(0));
    fov_x = std::min(std::max(value_type(0), fov_x), hi);
    fov_ = fov_x;
    focus_len_ = width() / (2 * std::tan(fov_x / 2.0));
  }
  value_type fov() const { return fov_; }
  int width() const { return width_; }
  int height() const { return height_; }
  const vector_type& focus() const { return this->position(); }
  value_type focus_len() const { return focus_len_; }
  vector_type focus_vector() const { return this->vector_x() * focus_len_; }
  vector_type PixelVector(int x, int y) const { return PixelVector(x, y, focus_vector()); }
  vector_type PixelVector(int x, int y, const vector_type& focus_v) const {
    return focus_v - this->vector_y() * static_cast<value_type>(width() / 2.0 - x) -
           this->vector_z() * static_cast<value_type>(height() / 2.0 - y);
  }

 private:
  int width_, height_;
  value_type fov_ = value_type(1.5707963267948966);
  value_type focus_len_ = 1;
};

// StaticBlackhole<T> (blackhole_solution.h:16-96).
template <typename T>
class StaticBlackhole : public Object<T> {
 public:
  using typename Object<T>::value_type;
  using typename Object<T>::vector_type;
  using typename Object<T>::point_type;

  StaticBlackhole(const vector_type& position, value_type mass)
      : Object<T>(position), mass_(mass), b_c_(3 * std::sqrt(value_type(3)) * mass) {}
  value_type mass() const { return mass_; }
  value_type b_c() const { return b_c_; }
  value_type radius() const { return 2 * mass(); }
  const point_type& center() const { return this->position(); }
  value_type G(value_type u, value_type b) const { return u * u * (2 * mass_ * u - 1) + 1 / (b * b); }
  value_type InvSqrtG(value_type u, value_type b) const { return 1 / std::sqrt(G(u, b)); }

 private:
  value_type mass_, b_c_;
};

// A host texture, copied to the device once per Renderer (the cv::Mat of
// Material::SetTexture). layout is BH_TEXEL_*; row_stride in bytes.
class Texture {
 public:
  Texture() = default;
  static Texture FromPixels(int width, int height, int32_t layout, const uint8_t* data, int64_t row_stride = 0) {
    Texture t;
    if (width <= 0 || height <= 0 || !data) return t;
    const int cpp = (layout == BH_TEXEL_BGRA8 || layout == BH_TEXEL_RGBA8) ? 4 : 3;
    const int64_t stride = row_stride ? row_stride : int64_t(width) * cpp;
    auto buf = std::make_shared<std::vector<uint8_t>>(size_t(width) * height * cpp);
    for (int y = 0; y < height; ++y) std::memcpy(buf->data() + size_t(y) * width * cpp, data + y * stride, size_t(width) * cpp);
    t.pixels_ = std::move(buf);
    t.width_ = width;
    t.height_ = height;
    t.layout_ = layout;
    return t;
  }
#ifdef BH_GB300_WITH_OPENCV
  // CV_8UC3 (BGR, as cv::imread gives) or CV_8UC4 (BGRA).
  static Texture FromMat(const cv::Mat& m) {
    if (m.empty()) return Texture();
    if (m.type() != CV_8UC3 && m.type() != CV_8UC4) throw Error(BH_ERR_BAD_TEXTURE, "texture must be CV_8UC3 or CV_8UC4");
    return FromPixels(m.cols, m.rows, m.type() == CV_8UC3 ? BH_TEXEL_BGR8 : BH_TEXEL_BGRA8, m.data, int64_t(m.step));
  }
#endif
  bool empty() const { return !pixels_ || pixels_->empty(); }
  int width() const { return width_; }
  int height() const { return height_; }
  int32_t layout() const { return layout_; }
  const uint8_t* data() const { return pixels_ ? pixels_->data() : nullptr; }
  // identity of the pixel storage (copies of a Texture share it)
  const void* key() const { return pixels_.get(); }

 private:
  std::shared_ptr<std::vector<uint8_t>> pixels_;
  int width_ = 0, height_ = 0;
  int32_t layout_ = BH_TEXEL_BGR8;
};

// Annulus<T> (vector_object.h:306-356): a disc given by its bounding quad
// p1..p4 (vertex()[0] stays the default (0,0,0) object position, the disc
// centre), r_outer, r_inner; the normal (p3 - p1) x (p2 - p1), normalised, is
// fixed at construction. Material::SetTexture throws on an empty texture.
template <typename T>
class Annulus : public Object<T> {
 public:
  using typename Object<T>::value_type;
  using typename Object<T>::vector_type;
  using typename Object<T>::point_type;

  Annulus(const point_type& p1, const point_type& p2, const point_type& p3, const point_type& p4,
          value_type r_outer, value_type r_inner)
      : Object<T>({p1, p2, p3, p4}),
        norm_(normalize((p3 - p1).cross(p2 - p1))),
        r_outer_(r_outer),
        r_inner_(r_inner) {}
  const vector_type& norm() const { return norm_; }
  value_type r_inner() const { return r_inner_; }
  value_type r_outer() const { return r_outer_; }
  void SetTexture(Texture texture) {
    if (texture.empty()) throw Error(BH_ERR_EMPTY_TEXTURE, "empty texture");
    texture_ = std::move(texture);
  }
#ifdef BH_GB300_WITH_OPENCV
  void SetTexture(const cv::Mat& m) { SetTexture(Texture::FromMat(m)); }
#endif
  const Texture& texture() const { return texture_; }
  // BH_DISC_MAP_REF_PLANAR (the reference's Rectangle::color) or POLAR
  void mapping(int32_t m) { mapping_ = m; }
  int32_t mapping() const { return mapping_; }

 private:
  vector_type norm_;
  value_type r_outer_, r_inner_;
  Texture texture_;
  int32_t mapping_ = BH_DISC_MAP_REF_PLANAR;
};

// ChessPattern2D<T> (pattern.h:14-50): black and white cells of
// pattern_size (the reference takes an int).
template <typename T>
class ChessPattern2D {
 public:
  ChessPattern2D() = default;
  explicit ChessPattern2D(int pattern_size) : pattern_size_(T(pattern_size)) {}
  T pattern_size() const { return pattern_size_; }

 private:
  T pattern_size_ = 1;
};

// Rectangle<T> (vector_object.h:80-183): corners p1..p4 after the default
// (0,0,0) vertex; drawn by Rectangle::color from its texture (black without).
template <typename T>
class Rectangle : public Object<T> {
 public:
  using typename Object<T>::value_type;
  using typename Object<T>::point_type;
  Rectangle() : Object<T>({point_type(1, 0, 1), point_type(-1, 0, 1), point_type(-1, 0, -1), point_type(1, 0, -1)}) {}
  Rectangle(const point_type& p1, const point_type& p2, const point_type& p3, const point_type& p4)
      : Object<T>({p1, p2, p3, p4}) {}
  Rectangle(value_type v11, value_type v12, value_type v13, value_type v21, value_type v22, value_type v23,
            value_type v31, value_type v32, value_type v33, value_type v41, value_type v42, value_type v43)
      : Rectangle(point_type(v11, v12, v13), point_type(v21, v22, v23), point_type(v31, v32, v33),
                  point_type(v41, v42, v43)) {}
  void SetTexture(Texture texture) {
    if (texture.empty()) throw Error(BH_ERR_EMPTY_TEXTURE, "empty texture");
    texture_ = std::move(texture);
  }
#ifdef BH_GB300_WITH_OPENCV
  void SetTexture(const cv::Mat& m) { SetTexture(Texture::FromMat(m)); }
#endif
  const Texture& texture() const { return texture_; }

 private:
  Texture texture_;
};

// Triangle<T> (vector_object.h:18-77): vertices after the default (0,0,0)
// vertex; drawn black (it has no colour of its own). The reference's own
// constructors do not compile when instantiated; these take the same
// arguments.
template <typename T>
class Triangle : public Object<T> {
 public:
  using typename Object<T>::value_type;
  using typename Object<T>::point_type;
  Triangle() : Object<T>({point_type(1, 0, 0), point_type(-1, 0, 0), point_type(0, 0, 1.73)}) {}
  Triangle(const point_type& a, const point_type& b, const point_type& c) : Object<T>({a, b, c}) {}
  Triangle(value_type v11, value_type v12, value_type v13, value_type v21, value_type v22, value_type v23,
           value_type v31, value_type v32, value_type v33)
      : Triangle(point_type(v11, v12, v13), point_type(v21, v22, v23), point_type(v31, v32, v33)) {}
};

// InfinitePlane<T> (vector_object.h:187-238): the plane through position()
// normal to vector_z(), coloured by a ChessPattern2D (black without one).
template <typename T>
class InfinitePlane : public Object<T> {
 public:
  using typename Object<T>::point_type;
  explicit InfinitePlane(const point_type& p) : Object<T>(p) {}
  InfinitePlane(const point_type& p, const ChessPattern2D<T>& pattern) : Object<T>(p), pattern_size_(pattern.pattern_size()) {}
  T pattern_size() const { return pattern_size_; }

 private:
  T pattern_size_ = 0;
};

// Equirectangular sky for escaped rays (not in the reference).
class Background {
 public:
  explicit Background(Texture t) : texture_(std::move(t)) {
    if (texture_.empty()) throw Error(BH_ERR_EMPTY_TEXTURE, "empty background texture");
  }
#ifdef BH_GB300_WITH_OPENCV
  explicit Background(const cv::Mat& m) : Background(Texture::FromMat(m)) {}
#endif
  const Texture& texture() const { return texture_; }

 private:
  Texture texture_;
};

// One rendered frame: row-major, BH_FORMAT_BGR8 (the reference's CV_8UC3
// screen) by default.
struct Image {
  int width = 0, height = 0;
  int32_t format = BH_FORMAT_BGR8;
  std::vector<uint8_t> pixels;
  std::vector<uint8_t> hit_class;  // filled when Options::want_classes
  int bytes_per_pixel() const { return format == BH_FORMAT_BGR8 ? 3 : 4; }
  const uint8_t* at(int x, int y) const { return pixels.data() + (size_t(y) * width + x) * bytes_per_pixel(); }
};

// Render options: bh_render_options with its defaults (RK4, FP32, REF ray
// generation, step 0.01, 4000 steps, escape at 100 M) and BGR8 output.
struct Options : bh_render_options {
  bool want_classes = false;
  Options() {
    bh_default_options(this);
    format = BH_FORMAT_BGR8;
  }
};

// One ordinary object of a scene (exactly one pointer set).
template <typename T>
struct SceneObject {
  const Rectangle<T>* rectangle = nullptr;
  const Triangle<T>* triangle = nullptr;
  const InfinitePlane<T>* plane = nullptr;
  SceneObject(const Rectangle<T>* r) : rectangle(r) {}
  SceneObject(const Triangle<T>* t) : triangle(t) {}
  SceneObject(const InfinitePlane<T>* p) : plane(p) {}
};

// One scene of a batch. The objects' order decides exact distance ties (the
// later one wins, as in the reference's ObjectManager).
template <typename T>
struct Scene {
  const Camera<T>* camera = nullptr;
  const StaticBlackhole<T>* hole = nullptr;  // may be null with the FLAT integrator
  const Annulus<T>* disc = nullptr;          // may be null
  const Background* background = nullptr;    // may be null
  std::vector<SceneObject<T>> objects;
  std::vector<const StaticBlackhole<T>*> extra_holes;  // BH_INTEGRATOR_MULTI: holes besides `hole`
};

template <typename T>
inline void copy3(double* dst, const Vec3<T>& v) {
  for (int i = 0; i < 3; ++i) dst[i] = double(v[i]);
}

// The bh_scene of a scene, given texture ids for its disc and background.
template <typename T>
inline bh_scene ToPod(const Camera<T>& cam, const StaticBlackhole<T>& bh, const Annulus<T>* disc, int32_t disc_tex,
                      int32_t bg_tex) {
  bh_scene s;
  std::memset(&s, 0, sizeof(s));
  copy3(s.camera.position, cam.position());
  copy3(s.camera.axis_x, cam.vector_x());
  copy3(s.camera.axis_y, cam.vector_y());
  copy3(s.camera.axis_z, cam.vector_z());
  s.camera.focus_len = double(cam.focus_len());
  s.camera.width = cam.width();
  s.camera.height = cam.height();
  copy3(s.hole.position, bh.position());
  s.hole.mass = double(bh.mass());
  if (disc) {
    const auto& v = disc->vertex();
    copy3(s.disc.center, v[0]);
    copy3(s.disc.normal, disc->norm());
    copy3(s.disc.corner, v[1]);
    copy3(s.disc.edge_s1, v[2] - v[1]);
    copy3(s.disc.edge_s2, v[4] - v[1]);
    s.disc.r_inner = double(disc->r_inner());
    s.disc.r_outer = double(disc->r_outer());
    s.disc.texture = disc_tex;
    s.disc.mapping = disc->mapping();
    s.disc.enabled = 1;
  } else {
    s.disc.texture = -1;
  }
  s.background = bg_tex;
  return s;
}

// The bh_object of an object, given the texture id of a rectangle's texture.
template <typename T>
inline bh_object ToPod(const SceneObject<T>& so, int32_t tex) {
  bh_object o;
  std::memset(&o, 0, sizeof(o));
  o.texture = -1;
  if (so.rectangle) {
    o.type = BH_OBJECT_RECTANGLE;
    o.texture = tex;
    const auto& v = so.rectangle->vertex();
    for (int k = 0; k < 4; ++k) copy3(o.v[k], v[k + 1]);
  } else if (so.triangle) {
    o.type = BH_OBJECT_TRIANGLE;
    const auto& v = so.triangle->vertex();
    for (int k = 0; k < 3; ++k) copy3(o.v[k], v[k + 1]);
  } else if (so.plane) {
    o.type = BH_OBJECT_PLANE;
    copy3(o.v[0], so.plane->position());
    copy3(o.axis_x, so.plane->vector_x());
    copy3(o.axis_y, so.plane->vector_y());
    copy3(o.axis_z, so.plane->vector_z());
    o.pattern_size = double(so.plane->pattern_size());
  } else {
    throw Error(BH_ERR_INVALID_ARGUMENT, "scene object without an object");
  }
  return o;
}

// Loss and gradient of the differentiable render (bh_render_adjoint).
struct AdjointResult {
  double loss = 0;
  std::array<double, BH_GRAD_COUNT> grad{};
  uint64_t steps = 0, band_rays = 0;
  double kernel_ms = 0;
};

// A CUDA device and stream (a bh_ctx) with its uploaded textures. Not
// re-entrant: one per host thread.
class Renderer {
 public:
  explicit Renderer(int device = 0) {
    Check(bh_create(&ctx_, device), "bh_create");
  }
  ~Renderer() {
    if (ctx_) bh_destroy(ctx_);
  }
  Renderer(const Renderer&) = delete;
  Renderer& operator=(const Renderer&) = delete;
  Renderer(Renderer&& o) noexcept : ctx_(o.ctx_), textures_(std::move(o.textures_)) { o.ctx_ = nullptr; }

  bh_ctx* context() const { return ctx_; }

  // The reference's frame body (blackhole_solution_test.cc:161-298): renders
  // the scene into `out` (resized; format from the options).
  template <typename T>
  void Render(const Camera<T>& cam, const StaticBlackhole<T>& bh, const Annulus<T>* disc, const Background* bg,
              Image& out, const Options& opts = Options()) {
    std::vector<Scene<T>> one{Scene<T>{&cam, &bh, disc, bg, {}, {}}};
    std::vector<Image> imgs(1);
    Render(one, imgs, opts);
    out = std::move(imgs[0]);
  }

  // Batched: every scene in one call (one launch over all of them on the
  // GRID, HYBRID and PERSISTENT schedules).
  template <typename T>
  void Render(const std::vector<Scene<T>>& scenes, std::vector<Image>& out, const Options& opts = Options()) {
    PodTables tables;
    std::vector<bh_scene> pods = Pods(scenes, &tables);
    out.resize(scenes.size());
    std::vector<bh_frame> frames(scenes.size());
    for (size_t i = 0; i < scenes.size(); ++i) {
      Image& im = out[i];
      im.width = scenes[i].camera->width();
      im.height = scenes[i].camera->height();
      im.format = opts.format;
      im.pixels.assign(size_t(im.width) * im.height * im.bytes_per_pixel(), 0);
      im.hit_class.assign(opts.want_classes ? size_t(im.width) * im.height : 0, 0);
      frames[i].pixels = im.pixels.data();
      frames[i].hit_class = opts.want_classes ? im.hit_class.data() : nullptr;
      frames[i].aux = nullptr;
    }
    Check(bh_render(ctx_, pods.data(), int32_t(pods.size()), frames.data(), &opts), "bh_render");
  }

  // Differentiable render at theta (BH_GRAD_COUNT values about the scene;
  // see bh_gb300.h) against a device target; device image / per-pixel
  // gradient buffers are optional.
  template <typename T>
  AdjointResult Adjoint(const Scene<T>& scene, const double* theta, const float* d_target, float* d_image = nullptr,
                        float* d_pixel_grad = nullptr, const bh_adjoint_options* opts = nullptr) {
    PodTables tables;
    std::vector<bh_scene> pods = Pods(std::vector<Scene<T>>{scene}, &tables);
    bh_adjoint_frame fr{d_target, d_image, d_pixel_grad};
    bh_adjoint_result r;
    Check(bh_render_adjoint(ctx_, pods.data(), 1, theta, &fr, opts, &r), "bh_render_adjoint");
    AdjointResult a;
    a.loss = r.loss;
    for (int i = 0; i < BH_GRAD_COUNT; ++i) a.grad[i] = r.grad[i];
    a.steps = r.steps;
    a.band_rays = r.band_rays;
    a.kernel_ms = r.kernel_ms;
    return a;
  }

  bh_render_stats Stats() {
    bh_render_stats s;
    Check(bh_get_stats(ctx_, &s), "bh_get_stats");
    return s;
  }

 private:
  void Check(int rc, const char* what) const {
    if (rc != BH_OK) throw Error(rc, std::string(what) + ": " + (ctx_ ? bh_last_error(ctx_) : "no context"));
  }

  int32_t TextureId(const Texture& t) {
    auto it = textures_.find(t.key());
    if (it != textures_.end()) return it->second.second;
    int32_t id = -1;
    Check(bh_texture_create(ctx_, t.data(), t.width(), t.height(), t.layout(), 0, &id), "bh_texture_create");
    textures_[t.key()] = {t, id};  // keeps the storage alive so the key stays unique
    return id;
  }

  // The object and extra-hole tables the PODs point at, kept during a call.
  struct PodTables {
    std::vector<std::vector<bh_object>> objects;
    std::vector<std::vector<bh_hole>> holes;
  };

  // The scenes' PODs; `tables` holds their object and hole tables.
  template <typename T>
  std::vector<bh_scene> Pods(const std::vector<Scene<T>>& scenes, PodTables* tables) {
    std::vector<bh_scene> pods;
    pods.reserve(scenes.size());
    tables->objects.assign(scenes.size(), {});
    tables->holes.assign(scenes.size(), {});
    const StaticBlackhole<T> no_hole(typename Object<T>::point_type(0, 0, 0), T(1));  // FLAT ignores the hole
    for (size_t i = 0; i < scenes.size(); ++i) {
      const Scene<T>& s = scenes[i];
      if (!s.camera) throw Error(BH_ERR_INVALID_ARGUMENT, "scene needs a camera");
      int32_t dt = -1, bt = -1;
      if (s.disc) {
        if (s.disc->texture().empty()) throw Error(BH_ERR_EMPTY_TEXTURE, "disc has no texture");
        dt = TextureId(s.disc->texture());
      }
      if (s.background) bt = TextureId(s.background->texture());
      bh_scene pod = ToPod(*s.camera, s.hole ? *s.hole : no_hole, s.disc, dt, bt);
      auto& tab = tables->objects[i];
      for (const SceneObject<T>& so : s.objects) {
        int32_t tex = -1;
        if (so.rectangle && !so.rectangle->texture().empty()) tex = TextureId(so.rectangle->texture());
        tab.push_back(ToPod(so, tex));
      }
      pod.n_objects = int32_t(tab.size());
      pod.objects = tab.empty() ? nullptr : tab.data();
      auto& holes = tables->holes[i];
      for (const StaticBlackhole<T>* h : s.extra_holes) {
        if (!h) throw Error(BH_ERR_INVALID_ARGUMENT, "null extra hole");
        bh_hole b;
        copy3(b.position, h->position());
        b.mass = double(h->mass());
        holes.push_back(b);
      }
      pod.n_extra_holes = int32_t(holes.size());
      pod.extra_holes = holes.empty() ? nullptr : holes.data();
      pods.push_back(pod);
    }
    return pods;
  }

  bh_ctx* ctx_ = nullptr;
  std::map<const void*, std::pair<Texture, int32_t>> textures_;
};

// Free-standing render on device 0 with a per-thread Renderer.
inline Renderer& DefaultRenderer() {
  thread_local Renderer r(0);
  return r;
}

template <typename T>
inline Image Render(const Camera<T>& cam, const StaticBlackhole<T>& bh, const Annulus<T>* disc, const Background* bg,
                    const Options& opts = Options()) {
  Image out;
  DefaultRenderer().Render(cam, bh, disc, bg, out, opts);
  return out;
}

template <typename T>
inline void Render(const Camera<T>& cam, const StaticBlackhole<T>& bh, const Annulus<T>* disc, const Background* bg,
                   Image& out, const Options& opts = Options()) {
  DefaultRenderer().Render(cam, bh, disc, bg, out, opts);
}

#ifdef BH_GB300_WITH_OPENCV
// Into the reference's CV_8UC3 screen (blackhole_solution_test.cc:117).
template <typename T>
inline void Render(const Camera<T>& cam, const StaticBlackhole<T>& bh, const Annulus<T>* disc, const Background* bg,
                   cv::Mat& screen, Options opts = Options()) {
  opts.format = BH_FORMAT_BGR8;
  Image out;
  DefaultRenderer().Render(cam, bh, disc, bg, out, opts);
  screen.create(out.height, out.width, CV_8UC3);
  for (int y = 0; y < out.height; ++y)
    std::memcpy(screen.ptr(y), out.pixels.data() + size_t(y) * out.width * 3, size_t(out.width) * 3);
}
#endif

}  // namespace blackhole

#endif  // BLACKHOLE_GB300_HPP_
