// Test infrastructure: FP64 oracle of the differentiable render and of its
// gradient. Used only by the tests (never by the product).
//
// The differentiable render is the RK4 render of bh_oracle.c with smooth
// shading, so that an image loss has gradients:
//   - disc: cubic B-spline texture in (radius, azimuth) and an opacity that falls
//     off smoothly at both edges, alpha = s((R - r_in)/w) s((r_out - R)/w),
//     s the logistic function, w = softness * M; crossings are composited
//     front to back (C += T alpha C_disc, T *= 1 - alpha; the ray stops once
//     T < 1e-4);
//   - sky: cubic B-spline equirectangular texture at the escape direction
//     (the filter is C2, so the loss is smooth across texel edges);
//   - horizon and step cap: black.
// Parameters theta (10): M; camera position offset (x, y, z); camera yaw,
// pitch and roll -- rotations of the camera axes about its own vz, vy and vx
// (base axes), applied as R(vz,yaw) R(vy,pitch) R(vx,roll); disc tilt -- a
// rotation of the disc about its in-plane axis e1 = s1/|s1|; r_inner;
// r_outer. The same code runs with T = double (loss, finite differences) and
// T = Dual (forward mode, 10 tangents: the exact gradient of the FP64 loss).
#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "bh_gb300.h"

namespace {

constexpr int kN = 10;
constexpr double kPi = 3.14159265358979323846;

struct Dual {
  double v;
  double d[kN];
  Dual() : v(0) { std::memset(d, 0, sizeof(d)); }
  Dual(double x) : v(x) { std::memset(d, 0, sizeof(d)); }
};
inline Dual operator+(const Dual& a, const Dual& b) { Dual r(a.v + b.v); for (int i = 0; i < kN; ++i) r.d[i] = a.d[i] + b.d[i]; return r; }
inline Dual operator-(const Dual& a, const Dual& b) { Dual r(a.v - b.v); for (int i = 0; i < kN; ++i) r.d[i] = a.d[i] - b.d[i]; return r; }
inline Dual operator-(const Dual& a) { Dual r(-a.v); for (int i = 0; i < kN; ++i) r.d[i] = -a.d[i]; return r; }
inline Dual operator*(const Dual& a, const Dual& b) { Dual r(a.v * b.v); for (int i = 0; i < kN; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i]; return r; }
inline Dual operator/(const Dual& a, const Dual& b) {
  Dual r(a.v / b.v);
  for (int i = 0; i < kN; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) / b.v;
  return r;
}
inline Dual scale(const Dual& a, double k) { Dual r(a.v * k); for (int i = 0; i < kN; ++i) r.d[i] = a.d[i] * k; return r; }
inline Dual chain(const Dual& a, double f, double df) { Dual r(f); for (int i = 0; i < kN; ++i) r.d[i] = df * a.d[i]; return r; }
inline Dual sqrt(const Dual& a) { const double s = std::sqrt(a.v); return chain(a, s, 0.5 / s); }
inline Dual sin(const Dual& a) { return chain(a, std::sin(a.v), std::cos(a.v)); }
inline Dual cos(const Dual& a) { return chain(a, std::cos(a.v), -std::sin(a.v)); }
inline Dual exp(const Dual& a) { const double e = std::exp(a.v); return chain(a, e, e); }
inline Dual asin(const Dual& a) { return chain(a, std::asin(a.v), 1.0 / std::sqrt(1.0 - a.v * a.v)); }
inline Dual atan2(const Dual& y, const Dual& x) {
  Dual r(std::atan2(y.v, x.v));
  const double q = x.v * x.v + y.v * y.v;
  for (int i = 0; i < kN; ++i) r.d[i] = (x.v * y.d[i] - y.v * x.d[i]) / q;
  return r;
}
inline double val(const Dual& a) { return a.v; }
inline double val(double a) { return a; }
inline double sqrt_(double a) { return std::sqrt(a); }
using std::asin;
using std::atan2;
using std::cos;
using std::exp;
using std::sin;
using std::sqrt;

template <class T>
struct V3 { T x, y, z; };
template <class T> V3<T> add(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> V3<T> sub(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> V3<T> mul(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> V3<T> cross(V3<T> a, V3<T> b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class T> V3<T> unit(V3<T> a) { const T l = sqrt(dot(a, a)); return mul(a, T(1.0) / l); }
template <class T> V3<T> lift(const double* v) { return {T(v[0]), T(v[1]), T(v[2])}; }

// Rodrigues rotation of v about the unit axis a (double) by angle th (T).
template <class T>
V3<T> rotate(V3<T> v, const double* a, T th) {
  const V3<T> ax = lift<T>(a);
  const T c = cos(th), s = sin(th);
  const T k = dot(ax, v) * (T(1.0) - c);
  return add(add(mul(v, c), mul(cross(ax, v), s)), mul(ax, k));
}

struct Tex {
  const uint8_t* bgra;
  int w, h;
};

// Uniform cubic B-spline weights of the four texels around a sample whose
// fractional texel offset is f.
template <class T>
void bspline_weights(T f, T w[4]) {
  const T g = T(1.0) - f, f2 = f * f, f3 = f2 * f;
  w[0] = g * g * g * T(1.0 / 6.0);
  w[1] = (T(3.0) * f3 - T(6.0) * f2 + T(4.0)) * T(1.0 / 6.0);
  w[2] = (T(-3.0) * f3 + T(3.0) * f2 + T(3.0) * f + T(1.0)) * T(1.0 / 6.0);
  w[3] = f3 * T(1.0 / 6.0);
}

// Cubic B-spline filter (C2 in s and u), texel centres at integers, s along
// x (columns), u along y (rows); a non-wrapping axis repeats its edge texel.
template <class T>
void bspline(const Tex& t, T s, T u, bool wrap_s, bool wrap_u, T out[3]) {
  const double fs0 = std::floor(val(s)), fu0 = std::floor(val(u));
  T ws[4], wu[4];
  bspline_weights(s - T(fs0), ws);
  bspline_weights(u - T(fu0), wu);
  auto index = [](long long i, int n, bool wrap) {
    if (wrap) { i %= n; return int(i < 0 ? i + n : i); }
    return int(i < 0 ? 0 : (i >= n ? n - 1 : i));
  };
  int is[4], iu[4];
  for (int k = 0; k < 4; ++k) {
    is[k] = index((long long)fs0 - 1 + k, t.w, wrap_s);
    iu[k] = index((long long)fu0 - 1 + k, t.h, wrap_u);
  }
  for (int c = 0; c < 3; ++c) {
    // BGRA -> RGB channel c
    const int ch = 2 - c;
    T acc = T(0.0);
    for (int j = 0; j < 4; ++j) {
      T row = T(0.0);
      for (int k = 0; k < 4; ++k) row = row + ws[k] * T(t.bgra[(size_t(iu[j]) * t.w + is[k]) * 4 + ch] / 255.0);
      acc = acc + wu[j] * row;
    }
    out[c] = acc;
  }
}

// logistic function, evaluated without overflow for large |z|
inline double logistic_v(double z) {
  if (z >= 0) return 1.0 / (1.0 + std::exp(-z));
  const double e = std::exp(z);
  return e / (1.0 + e);
}
inline double logistic(double z) { return logistic_v(z); }
inline Dual logistic(const Dual& z) {
  const double s = logistic_v(z.v);
  return chain(z, s, s * (1.0 - s));
}

struct SmoothOpts {
  double step;
  int max_steps;
  double r_escape;
  double softness;
};

template <class T>
void rk4(T& u, T& w, T h) {
  T k1w = T(3.0) * u * u - u;
  T u2 = u + T(0.5) * h * w, w2 = w + T(0.5) * h * k1w;
  T k2w = T(3.0) * u2 * u2 - u2;
  T u3 = u + T(0.5) * h * w2, w3 = w + T(0.5) * h * k2w;
  T k3w = T(3.0) * u3 * u3 - u3;
  T u4 = u + h * w3, w4 = w + h * k3w;
  T k4w = T(3.0) * u4 * u4 - u4;
  T nu = u + h / T(6.0) * (w + T(2.0) * w2 + T(2.0) * w3 + w4);
  T nw = w + h / T(6.0) * (k1w + T(2.0) * k2w + T(2.0) * k3w + k4w);
  u = nu;
  w = nw;
}

template <class T>
void hermite(T ua, T ha, T ub, T hb, T t, T* p, T* dp) {
  T t2 = t * t, t3 = t2 * t;
  *p = (T(2.0) * t3 - T(3.0) * t2 + T(1.0)) * ua + (t3 - T(2.0) * t2 + t) * ha + (T(3.0) * t2 - T(2.0) * t3) * ub +
       (t3 - t2) * hb;
  *dp = (T(6.0) * t2 - T(6.0) * t) * ua + (T(3.0) * t2 - T(4.0) * t + T(1.0)) * ha +
        (T(6.0) * t - T(6.0) * t2) * ub + (T(3.0) * t2 - T(2.0) * t) * hb;
}

// One pixel; returns its colour and a signature of the ray's structure
// (class, crossings taken, step count) that changes where the loss jumps.
template <class T>
uint32_t smooth_pixel(const bh_scene& sc, const T* th, int px, int py, const Tex& dtex, const Tex* btex,
                      const SmoothOpts& o, T rgb[3]) {
  const bh_camera& cam = sc.camera;
  const T M = th[0];
  // camera pose
  const V3<T> off = {th[1], th[2], th[3]};
  auto rot_cam = [&](const double* v) {
    V3<T> r = rotate(lift<T>(v), cam.axis_x, th[6]);
    r = rotate(r, cam.axis_y, th[5]);
    return rotate(r, cam.axis_z, th[4]);
  };
  const V3<T> vx = rot_cam(cam.axis_x), vy = rot_cam(cam.axis_y), vz = rot_cam(cam.axis_z);
  const V3<T> cpos = add(lift<T>(cam.position), off);
  const V3<T> F = sub(cpos, lift<T>(sc.hole.position));
  const V3<T> fv = mul(vx, T(cam.focus_len));
  const V3<T> E0 = sub(cpos, fv);  // REF ray generation: e = F - pv
  const T a = T(cam.width / 2.0 - px), c = T(cam.height / 2.0 - py);
  const V3<T> e = add(add(E0, mul(vy, a)), mul(vz, c));
  // disc pose
  double e1d[3];
  const double s1l = std::sqrt(sc.disc.edge_s1[0] * sc.disc.edge_s1[0] + sc.disc.edge_s1[1] * sc.disc.edge_s1[1] +
                               sc.disc.edge_s1[2] * sc.disc.edge_s1[2]);
  for (int i = 0; i < 3; ++i) e1d[i] = sc.disc.edge_s1[i] / s1l;
  const V3<T> n = rotate(lift<T>(sc.disc.normal), e1d, th[7]);
  const V3<T> e1 = lift<T>(e1d);
  const V3<T> e2 = unit(cross(n, e1));
  const T r_in = th[8], r_out = th[9];
  const T wsoft = T(o.softness) * M;
  // plane reduction
  const V3<T> yv = unit(e);
  const V3<T> cz = cross(F, yv);
  const T b = sqrt(dot(cz, cz));
  const V3<T> zv = mul(cz, T(1.0) / b);
  const V3<T> xv = cross(yv, zv);
  const T F1 = dot(yv, F);
  const T r0 = sqrt(dot(F, F));
  T u = M / r0;
  const T bm = b / M;
  const T phi0 = atan2(b, F1);
  T w = sqrt(T(1.0) / (bm * bm) - u * u * (T(1.0) - T(2.0) * u));
  if (val(F1) < 0) w = -w;
  const T A = dot(n, yv), B = dot(n, xv);
  T d = atan2(B, A) + T(kPi / 2) - phi0;
  d = d - T(kPi * std::floor(val(d) / kPi));  // into [0, pi)
  if (val(d) <= 0) d = d + T(kPi);
  const T h = T(o.step);
  const double u_esc = 1.0 / o.r_escape;
  T acc[3] = {T(0.0), T(0.0), T(0.0)};
  T trans = T(1.0);
  uint32_t sig = 0, crossings = 0;
  long long kc = (long long)std::floor(val(d) / o.step);
  int k = 0;
  int cls = BH_CLASS_MAXSTEPS;
  for (; k < o.max_steps; ++k) {
    if (k == kc) {
      T uc = u, wc = w;
      rk4(uc, wc, d - T(double(kc) * o.step));
      if (val(uc) < 0.5) {
        const T R = M / uc;
        const T alpha = logistic((R - r_in) / wsoft) * logistic((r_out - R) / wsoft);
        {
          const T phic = phi0 + d;
          const V3<T> ph = add(mul(yv, cos(phic)), mul(xv, sin(phic)));
          const T az = atan2(dot(e2, ph), dot(e1, ph));
          const T s = (R - r_in) / (r_out - r_in) * T(double(dtex.w)) - T(0.5);
          const T t = az * T(dtex.h / (2 * kPi)) - T(0.5);
          T col[3];
          bspline(dtex, s, t, false, true, col);
          for (int i = 0; i < 3; ++i) acc[i] = acc[i] + trans * alpha * col[i];
          trans = trans * (T(1.0) - alpha);
          ++crossings;
          sig = sig * 2654435761u + uint32_t(kc);
          if (val(trans) < 1e-4) {
            cls = BH_CLASS_DISC;
            break;
          }
        }
      }
      d = d + T(kPi);
      kc = (long long)std::floor(val(d) / o.step);
    }
    const T ua = u, wa = w;
    rk4(u, w, h);
    if (!(val(u) < 0.5)) {
      cls = BH_CLASS_HORIZON;
      ++k;
      break;
    }
    if (val(u) <= u_esc) {
      T tt = T((val(ua) - u_esc) / (val(ua) - val(u))), p, dp;
      for (int i = 0; i < 8; ++i) {
        hermite(ua, h * wa, u, h * w, tt, &p, &dp);
        tt = tt - (p - T(u_esc)) / dp;
      }
      hermite(ua, h * wa, u, h * w, tt, &p, &dp);
      const T we = dp / h;
      const T phie = phi0 + (T(double(k)) + tt) * h;
      const T psi = phie + atan2(T(u_esc), -we);
      cls = BH_CLASS_MISS;
      if (btex) {
        const V3<T> dir = add(mul(yv, cos(psi)), mul(xv, sin(psi)));
        const T lon = atan2(dir.y, dir.x);
        const T zc = val(dir.z) > 1 ? T(1.0) : (val(dir.z) < -1 ? T(-1.0) : dir.z);
        const T lat = asin(zc);
        const T s = (lon + T(kPi)) * T(btex->w / (2 * kPi)) - T(0.5);
        const T t = (T(kPi / 2) - lat) * T(btex->h / kPi) - T(0.5);
        T col[3];
        bspline(*btex, s, t, true, false, col);
        for (int i = 0; i < 3; ++i) acc[i] = acc[i] + trans * col[i];
      }
      ++k;
      break;
    }
  }
  for (int i = 0; i < 3; ++i) rgb[i] = acc[i];
  return (sig * 31u + uint32_t(k)) * 8u + uint32_t(cls) + (crossings << 28);
}

}  // namespace

extern "C" {

typedef struct {
  double step;
  int32_t max_steps;
  double r_escape;
  double softness;
} orc_smooth_opts;

// Image (W*H*3 RGB), per-pixel loss (vs target when not NULL) and signature
// at theta, FP64.
int orc_smooth_render(const bh_scene* sc, const double* theta, const uint8_t* disc_bgra, int dw, int dh,
                      const uint8_t* bg_bgra, int bw, int bh, const orc_smooth_opts* o, const float* target,
                      double* image, double* pixel_loss, uint32_t* signature, int nthreads) {
  const Tex dt{disc_bgra, dw, dh};
  const Tex bt{bg_bgra, bw, bh};
  const SmoothOpts so{o->step, o->max_steps, o->r_escape, o->softness};
  const int W = sc->camera.width, H = sc->camera.height;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(dynamic, 4)
  for (int y = 0; y < H; ++y) {
    for (int x = 0; x < W; ++x) {
      double rgb[3];
      const uint32_t sig = smooth_pixel<double>(*sc, theta, x, y, dt, bg_bgra ? &bt : nullptr, so, rgb);
      const size_t p = size_t(y) * W + x;
      if (image)
        for (int c = 0; c < 3; ++c) image[p * 3 + c] = rgb[c];
      if (pixel_loss) {
        double l = 0;
        for (int c = 0; c < 3; ++c) {
          const double dd = rgb[c] - (target ? target[p * 3 + c] : 0.0);
          l += dd * dd;
        }
        pixel_loss[p] = l;
      }
      if (signature) signature[p] = sig;
    }
  }
  return 0;
}

// Forward-mode (dual number) gradient of every pixel's loss term
// sum_c (C_c - target_c)^2 at theta: pixel_grad is W*H*10.
int orc_smooth_grad(const bh_scene* sc, const double* theta, const uint8_t* disc_bgra, int dw, int dh,
                    const uint8_t* bg_bgra, int bw, int bh, const orc_smooth_opts* o, const float* target,
                    double* pixel_grad, int nthreads) {
  const Tex dt{disc_bgra, dw, dh};
  const Tex bt{bg_bgra, bw, bh};
  const SmoothOpts so{o->step, o->max_steps, o->r_escape, o->softness};
  const int W = sc->camera.width, H = sc->camera.height;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(dynamic, 2)
  for (int y = 0; y < H; ++y) {
    Dual th[kN];
    for (int i = 0; i < kN; ++i) {
      th[i] = Dual(theta[i]);
      th[i].d[i] = 1.0;
    }
    for (int x = 0; x < W; ++x) {
      Dual rgb[3];
      smooth_pixel<Dual>(*sc, th, x, y, dt, bg_bgra ? &bt : nullptr, so, rgb);
      const size_t p = size_t(y) * W + x;
      Dual l(0.0);
      for (int c = 0; c < 3; ++c) {
        const Dual dd = rgb[c] - Dual(target[p * 3 + c]);
        l = l + dd * dd;
      }
      for (int i = 0; i < kN; ++i) pixel_grad[p * kN + i] = l.d[i];
    }
  }
  return 0;
}

}  // extern "C"
