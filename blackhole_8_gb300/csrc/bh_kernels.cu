// sm_103a kernels of the geodesic ray tracer.
//
// Per pixel the tracer (1) generates the reference's ray (camera.h:55-59 as
// used at blackhole_solution_test.cc:167-170), (2) reduces it to its orbital
// plane through the hole (:170-193; the basis is orthonormal, so the
// reference's 3x3 inverse is a transpose here), (3) integrates the photon
// orbit with either the reference's 20+20-step trapezoid rule in u with chord
// collisions (:202-296) or fixed fourth-order steps in phi on
// u'' = -u + 3 u^2 (u = M/r; classical RK4 in FP64, Nystrom's three-stage
// method in FP32) with horizon, escape and disc-plane events, (4) samples the disc or
// background texture and (5) stores the pixel.
//
// RK4 details. The state is x = u - 1/3, w = du/dphi: the orbit equation
// becomes x'' = x + 3 x^2 (no constant term), so FP32 keeps relative
// precision near the unstable photon orbit x = 0. The change of variables is
// affine, so the trajectory is the same as in u. Because the right-hand
// side does not depend on w, the FP32 tracers take Nystrom's three-stage
// fourth-order method for y'' = f(y) (15 FP32 instructions, 26 flops) and
// the FP64 tracer classical RK4 in its Runge-Kutta-Nystrom form (18
// instructions), the oracle's scheme (rk4_step). Horizon and escape are
// tested once per block of 4 steps; a block that ends outside takes the
// event from its kept states.
//
// Mixed precision. FP32 rays keep the first integral
// eps = w^2 - x^2 - 2 x^3 (= 1/b^2 - 1/27, the G of blackhole_solution.h:
// 27-29) only to FP32 rounding, and near x = 0 (the saddle of the photon
// orbit) that drift is amplified by 1/|b - b_c|. The mixed tracer therefore
// (a) takes eps exactly (double-float, from the per-scene quadratic forms of
// |e|^2 and |F x e|^2) for rays with |b - b_c| < setup_band, (b) projects
// (x, w) back onto eps = const after every 4-step block spent near the saddle
// (|x| < 0.1) by rays with |b - b_c| < 0.3 M, (c) traces rays with
// |b - b_c| < band fully in FP64 with the band step, and (d) refines
// disc-plane crossings near the disc edges in double-float. Double-float
// (bh_df.cuh) runs on the FP32 pipe, where an FP64 instruction costs a warp
// ~64-80 issue cycles.
//
// The path has no dense contraction, so there is no tensor-core work; it is
// bound by FP32 issue. Textures (a few MB) stay in L2 and are read once per
// ray through the read-only path.
#include <math_constants.h>
#include <stdint.h>

#include <algorithm>
#include <type_traits>

#include "bh_df.cuh"
#include "bh_internal.h"

namespace bhgb {
namespace {

constexpr unsigned kFull = 0xffffffffu;

// ---------------------------------------------------------------------------
// small vector algebra
template <typename R>
struct V3 {
  R x, y, z;
};
template <typename R>
__device__ __forceinline__ V3<R> operator+(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <typename R>
__device__ __forceinline__ V3<R> operator-(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <typename R>
__device__ __forceinline__ V3<R> operator*(V3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <typename R>
__device__ __forceinline__ R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename R>
__device__ __forceinline__ V3<R> cross(V3<R> a, V3<R> b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <typename R>
__device__ __forceinline__ R length(V3<R> a) { return sqrt(dot(a, a)); }
// 1/sqrt: the hardware approximation in FP32, exact division in FP64.
__device__ __forceinline__ float rnorm(float l2) { return rsqrtf(l2); }
__device__ __forceinline__ double rnorm(double l2) { return 1.0 / sqrt(l2); }
// cv::normalize semantics: v * (1/|v|), zero vector stays zero.
template <typename R>
__device__ __forceinline__ V3<R> normalize(V3<R> a) {
  const R l2 = dot(a, a);
  const R k = l2 != R(0) ? rnorm(l2) : R(0);
  return a * k;
}
template <typename R, typename S>
__device__ __forceinline__ V3<R> cast3(V3<S> a) { return {R(a.x), R(a.y), R(a.z)}; }
__device__ __forceinline__ V3<float> xyz(float4 v) { return {v.x, v.y, v.z}; }

// Per-precision scene terms of the RK4 tracers: FP32 from the scene's 16-byte
// hot groups (one load each), FP64 from the exact fields.
template <typename R>
struct DiscRadii {
  R M, r_in, r_out;
};
template <typename R>
__device__ __forceinline__ DiscRadii<R> disc_radii(const DevScene& s) {
  if constexpr (sizeof(R) == 4) {
    const float4 m = s.hot[kHotMass];
    return {m.x, m.z, m.w};
  } else {
    return {s.mass, s.r_in, s.r_out};
  }
}
template <typename R>
__device__ __forceinline__ V3<R> fhat_of(const DevScene& s) {
  if constexpr (sizeof(R) == 4) {
    return xyz(s.hot[kHotFhat]);
  } else {
    return {s.Fhat[0], s.Fhat[1], s.Fhat[2]};
  }
}

// Precision-dependent view of a DevScene field.
template <typename R>
struct Pick;
template <>
struct Pick<float> {
  static __device__ __forceinline__ V3<float> v(const double*, const float* f) { return {f[0], f[1], f[2]}; }
  static __device__ __forceinline__ float s(double, float f) { return f; }
};
template <>
struct Pick<double> {
  static __device__ __forceinline__ V3<double> v(const double* d, const float*) { return {d[0], d[1], d[2]}; }
  static __device__ __forceinline__ double s(double d, float) { return d; }
};
#define BH_V(R, obj, name) Pick<R>::v((obj).name, (obj).name##_f)
#define BH_S(R, obj, name) Pick<R>::s((obj).name, (obj).name##_f)

template <typename R>
__device__ __forceinline__ R kPi() { return R(CUDART_PI); }

// Division, sine/cosine and atan2 of the setup and the shading: fast forms
// in FP32 (a quotient within 2 ulp; sin/cos within ~1e-6 rad over the angles
// a ray sweeps; atan2 within ~2e-7 rad), against ~3e-3 rad per sky texel and
// the FP32 integration's own ~1e-5 rad; the exact ones in FP64.
template <typename R>
__device__ __forceinline__ R shade_div(R a, R b) { return a / b; }
template <>
__device__ __forceinline__ float shade_div<float>(float a, float b) { return __fdividef(a, b); }
template <typename R>
__device__ __forceinline__ void shade_sincos(R x, R* s, R* c) { sincos(x, s, c); }
template <>
__device__ __forceinline__ void shade_sincos<float>(float x, float* s, float* c) { __sincosf(x, s, c); }

// atan2 in FP32: reduction to t = min(|x|, |y|) / max(|x|, |y|) in [0, 1],
// atan(t) = t P(t^2) with P the degree-7 minimax polynomial of atan(t) / t
// on [0, 1] (Remez exchange on the absolute error of t P(t^2), fitted by
// csrc/atan_poly_fit.py: |error| <= 3.8e-8 in exact arithmetic), then the
// octant: pi/2 - r above the diagonal, pi - r for x < 0, the sign of y.
// atan2(0, 0) = 0.
__device__ __forceinline__ float atan2_poly(float y, float x) {
  const float ax = fabsf(x), ay = fabsf(y);
  const float mx = fmaxf(ax, ay), mn = fminf(ax, ay);
  const float t = mx > 0.f ? __fdividef(mn, mx) : 0.f;
  const float z = t * t;
  float p = -4.0545672e-3f;
  p = fmaf(p, z, 2.1862958e-2f);
  p = fmaf(p, z, -5.5912327e-2f);
  p = fmaf(p, z, 9.6421973e-2f);
  p = fmaf(p, z, -1.3908630e-1f);
  p = fmaf(p, z, 1.9946566e-1f);
  p = fmaf(p, z, -3.3329861e-1f);
  p = fmaf(p, z, 9.9999934e-1f);
  float r = p * t;
  if (ay > ax) r = 1.57079633f - r;
  if (x < 0.f) r = 3.14159265f - r;
  return copysignf(r, y);
}
template <typename R>
__device__ __forceinline__ R shade_atan2(R y, R x) { return atan2(y, x); }
template <>
__device__ __forceinline__ float shade_atan2<float>(float y, float x) { return atan2_poly(y, x); }

// ---------------------------------------------------------------------------
// textures and pixels
__device__ __forceinline__ uchar4 texel(const DevTexture& t, long long idx) {
  const long long last = (long long)t.width * t.height - 1;
  idx = idx < 0 ? 0 : (idx > last ? last : idx);
  return __ldg(t.texels + idx);
}

// Texel (tx, ty) of coordinates already clamped to the texture.
__device__ __forceinline__ uchar4 texel_at(const DevTexture& t, int tx, int ty) {
  return __ldg(t.texels + ((long long)ty * t.width + tx));
}

__device__ __forceinline__ int trunc_to_int(double v) {
  // (int) cast of the reference with out-of-range and NaN values pinned down.
  if (!(v == v)) return 0;
  v = fmin(fmax(v, -1073741824.0), 1073741824.0);
  return (int)v;
}

// Rectangle::color (vector_object.h:159-179): nearest texel on the quad basis,
// truncating casts, linear index px_h * cols + px_w (clamped to the texture
// where the reference reads out of bounds).
template <typename R>
__device__ uchar4 quad_texel(const DevTexture& t, V3<R> v1, V3<R> s1, R s1l, R s2l, V3<R> hit) {
  const V3<R> v = hit - v1;
  const R r = length(v);
  R th = acos(dot(s1, v) / (s1l * r));
  th = (th == th) ? th : R(0);
  const int px_w = trunc_to_int(double(r * cos(th) / s1l) * t.width);
  const int px_h = trunc_to_int(double(r * sin(th) / s2l) * t.height);
  return texel(t, (long long)px_h * t.width + px_w);
}

template <typename R>
__device__ uchar4 disc_color_planar(const DevScene& s, V3<R> hit) {
  return quad_texel<R>(s.disc_tex, BH_V(R, s, dv1), BH_V(R, s, ds1), BH_S(R, s, s1_len), BH_S(R, s, s2_len), hit);
}

// Polar disc mapping: x over [r_in, r_out], y over the azimuth about e1.
template <typename R>
__device__ uchar4 disc_color_polar(const DevScene& s, V3<R> hit) {
  const V3<R> q = hit - BH_V(R, s, dc);
  const R rr = length(q);
  const R rin = BH_S(R, s, r_in), rout = BH_S(R, s, r_out);
  int tx = (int)floor(shade_div(rr - rin, rout - rin) * R(s.disc_tex.width));
  tx = min(max(tx, 0), s.disc_tex.width - 1);
  R a = shade_atan2(dot(BH_V(R, s, de2), q), dot(BH_V(R, s, de1), q)) * (R(0.5) / kPi<R>());
  a -= floor(a);
  int ty = (int)floor(a * R(s.disc_tex.height));
  ty = min(max(ty, 0), s.disc_tex.height - 1);
  return texel_at(s.disc_tex, tx, ty);
}

// disc_color_polar in FP32 for a disc centred on the hole (the RK4 tracer's
// crossings lie in its plane): the hit is rw (cos phi F^ + sin phi xv) from
// the centre, so its radius is rw itself and its azimuth about e1 is
// atan2(e2 . dir, e1 . dir) of the unit direction, with e1 . F^ and e2 . F^
// per-scene constants; the texel column scale W / (r_out - r_in) is one too.
__device__ __forceinline__ uchar4 disc_color_polar_centred(const DevScene& s, float rw, float cp, float sp,
                                                           V3<float> xv) {
  const int W = s.disc_tex.width, H = s.disc_tex.height;
  const float4 e1 = s.hot[kHotDe1], e2 = s.hot[kHotDe2];
  int tx = (int)floorf((rw - s.hot[kHotMass].z) * s.hot[kHotDisc].x);
  tx = min(max(tx, 0), W - 1);
  const float y = fmaf(cp, e2.w, sp * dot(xyz(e2), xv));
  const float x = fmaf(cp, e1.w, sp * dot(xyz(e1), xv));
  float a = atan2_poly(y, x) * 0.159154943f;  // 1 / (2 pi)
  a -= floorf(a);
  int ty = (int)floorf(a * float(H));
  ty = min(max(ty, 0), H - 1);
  return texel_at(s.disc_tex, tx, ty);
}

template <typename R>
__device__ __forceinline__ uchar4 disc_color(const DevScene& s, V3<R> hit) {
  return s.disc_map == BH_DISC_MAP_POLAR ? disc_color_polar(s, hit) : disc_color_planar(s, hit);
}

// Equirectangular background by world direction (unit vector).
template <typename R>
__device__ uchar4 background_color(const DevScene& s, V3<R> d) {
  const int W = s.bg_tex.width, H = s.bg_tex.height;
  const R lon = shade_atan2(d.y, d.x);
  // angle from the +z pole: pi/2 - asin(z), in FP32 as atan2(|(x, y)|, z)
  R colat;
  if constexpr (sizeof(R) == 4) {
    const float q2 = d.x * d.x + d.y * d.y;
    colat = atan2_poly(q2 > 1e-30f ? q2 * rsqrtf(q2) : 0.f, d.z);
  } else {
    colat = kPi<R>() * R(0.5) - asin(fmin(fmax(d.z, R(-1)), R(1)));
  }
  int tx = (int)floor((lon + kPi<R>()) * (R(W) * R(0.5) / kPi<R>()));
  tx = tx >= W ? tx - W : (tx < 0 ? 0 : tx);
  int ty = (int)floor(colat * (R(H) / kPi<R>()));
  ty = min(max(ty, 0), H - 1);
  return texel_at(s.bg_tex, tx, ty);
}

struct Hit {
  uchar4 bgra;
  int cls;
  float aux;
};

__device__ __forceinline__ Hit miss_hit() { return {make_uchar4(0, 0, 0, 255), BH_CLASS_MISS, 0.f}; }

// Class and aux outputs of pixel (x, y), where the frame asks for them.
__device__ __forceinline__ void store_extras(const DevScene& s, int x, int y, const Hit& h) {
  const int4 fl = s.hot_i;
  const long long pix = (long long)y * fl.y + x;
  if (fl.x & kSceneCls) s.cls[pix] = (uint8_t)h.cls;
  if (fl.x & kSceneAux) s.aux[pix] = h.aux;
}

__device__ __forceinline__ void store_hit(const DevScene& s, int format, int x, int y, const Hit& h) {
  const int4 fl = s.hot_i;
  const long long pix = (long long)y * fl.y + x;
  uchar4 c = h.bgra;
  c.w = 255;
  if (format == BH_FORMAT_BGRA8) {
    reinterpret_cast<uchar4*>(s.pixels)[pix] = c;
  } else if (format == BH_FORMAT_RGBA8) {
    reinterpret_cast<uchar4*>(s.pixels)[pix] = make_uchar4(c.z, c.y, c.x, c.w);
  } else {
    uint8_t* p = s.pixels + pix * 3;
    p[0] = c.x;
    p[1] = c.y;
    p[2] = c.z;
  }
  if (fl.x & kSceneCls) s.cls[pix] = (uint8_t)h.cls;
  if (fl.x & kSceneAux) s.aux[pix] = h.aux;
}

// ---------------------------------------------------------------------------
// ray generation and orbital-plane reduction
template <typename R>
struct PlaneRay {
  V3<R> yv, xv;   // in-plane basis: position = r (cos phi yv + sin phi xv)
  R F0, F1, b;    // F' = (zv.F, yv.F, xv.F); b = xv.F >= 0
};

template <typename R>
__device__ __forceinline__ PlaneRay<R> make_ray(const DevScene& s, int x, int y) {
  const V3<R> F = BH_V(R, s, F);
  const R a = BH_S(R, s, half_w) - R(x);
  const R c = BH_S(R, s, half_h) - R(y);
  const V3<R> e = BH_V(R, s, E0) + BH_V(R, s, vy) * a + BH_V(R, s, vz) * c;
  PlaneRay<R> r;
  r.yv = normalize(e);
  // zv = normalize(pv x yv) == normalize(F x yv): pv = F - |e| yv.
  const V3<R> zv = normalize(cross(F, r.yv));
  r.xv = normalize(cross(r.yv, zv));
  r.F0 = dot(zv, F);
  r.F1 = dot(r.yv, F);
  r.b = dot(r.xv, F);
  return r;
}

// The RK4 ray of pixel (x, y): F1 = F . e^ and b = |F x e^| (e^ the unit ray
// direction), and X0, the second axis of the ray's orbital basis rotated to
// the camera (the first is the scene's F / |F|): F = F1 e^ + b x^ with x^ the
// in-plane normal of e^, so X0 = (x^ F1 - e^ b) / |F| = (F^ F1 - e^ |F|) / b
// = F x (F x e^) / (|F| b). Both come from the cross product, which keeps
// them accurate to rounding where |F| - F1 would cancel (near-critical rays
// seen from afar).
template <typename R>
struct RkRay {
  V3<R> X0;
  R F1, b;
};

// The scene terms of the RK4 ray setup: in FP32 four 16-byte loads of the
// scene's hot groups, in FP64 the exact fields.
template <typename R>
struct RaySetupScene {
  V3<R> E0, vy, vz, F;
  R half_w, half_h, Flen, inv_mass;
};
template <typename R>
__device__ __forceinline__ RaySetupScene<R> ray_setup_scene(const DevScene& s) {
  if constexpr (sizeof(R) == 4) {
    const float4 e0 = s.hot[kHotE0], vy = s.hot[kHotVy], vz = s.hot[kHotVz], f = s.hot[kHotF];
    return {xyz(e0), xyz(vy), xyz(vz), xyz(f), e0.w, vy.w, vz.w, f.w};
  } else {
    return {BH_V(R, s, E0), BH_V(R, s, vy), BH_V(R, s, vz), BH_V(R, s, F), s.half_w, s.half_h, s.Flen, 1.0 / s.mass};
  }
}

template <typename R>
__device__ __forceinline__ RkRay<R> make_ray_rk4(const DevScene& s, int x, int y) {
  const RaySetupScene<R> q = ray_setup_scene<R>(s);
  const R a = q.half_w - R(x);
  const R c = q.half_h - R(y);
  const V3<R> yv = normalize(q.E0 + q.vy * a + q.vz * c);
  const R L = q.Flen;
  const V3<R> F = q.F;
  const V3<R> fx = cross(F, yv);
  RkRay<R> r;
  r.F1 = dot(yv, F);
  R ilb;
  if constexpr (sizeof(R) == 4) {
    // b and 1 / (|F| b) from one reciprocal square root (the correctly
    // rounded square root is a longer dependent sequence on this path;
    // b errs by ~2 ulp instead of 0.5)
    const float fx2 = dot(fx, fx);
    const float rb = fx2 > 1e-30f ? rsqrtf(fx2) : 0.f;
    r.b = fx2 * rb;
    ilb = __fdividef(rb, L);
  } else {
    r.b = length(fx);
    ilb = r.b > R(0) ? R(1) / (L * r.b) : R(0);
  }
  r.X0 = cross(F, fx) * ilb;
  return r;
}

// ---------------------------------------------------------------------------
// REF_TRAPEZOID: blackhole_solution_test.cc:185-296 with
// StaticBlackhole::G / InvSqrtG / SolveG (blackhole_solution.h:27-53),
// StaticBlackhole::Collide (:65-88), Annulus::Collide (vector_object.h:
// 328-347) and ObjectManager::FindCollision (object_manager.h:69-85).
template <typename R>
__device__ __forceinline__ R inv_sqrt_g(R u, R b, R M) {
  return R(1) / sqrt((u * u * (R(2) * M * u - R(1))) + (R(1) / (b * b)));
}

template <typename R>
__device__ R solve_g(R b, R M) {
  // epsilon<double>() = cbrt(DBL_EPSILON) (utility.h:17-21)
  R l = R(6.0554544523933395e-06);
  R r = R(1) / (R(3) * M);
  for (int i = 0; i < 20; ++i) {
    const R mid = (l + r) / R(2);
    const R g = (mid * mid * (R(2) * M * mid - R(1))) + (R(1) / (b * b));
    if (g > R(0)) l = mid;
    else r = mid;
  }
  return l;
}

// Nearest collision on the chord p1 -> p2; the hole is tested first (the
// iteration order of the reference's two-object map), ties keep it.
// ---------------------------------------------------------------------------
// ordinary objects (bh_object) on a chord p1 -> p2, in precision R

template <typename R>
__device__ __forceinline__ V3<R> div3(V3<R> a, R d) { return {a.x / d, a.y / d, a.z / d}; }

// ChessPattern2D<T>{size} (pattern.h:23-46): white or black by the parity of
// the cells containing (x, y), mirrored across the axes. The (int) casts are
// pinned for non-finite and huge values.
template <typename R>
__device__ uchar4 chess(R size, R x, R y) {
  const R two = size * R(2);
  const int m = trunc_to_int(double(two));
  if (m == 0) return make_uchar4(0, 0, 0, 255);
  const R bx = fabs(x), by = fabs(y);
  const R x2 = bx - R(trunc_to_int(double(bx)) / m) * two;
  const R y2 = by - R(trunc_to_int(double(by)) / m) * two;
  const bool in = (x2 <= size && y2 <= size) || (size <= x2 && size <= y2);
  const bool white = (x * y > R(0)) ? in : !in;
  return white ? make_uchar4(255, 255, 255, 255) : make_uchar4(0, 0, 0, 255);
}

// Colour of a hit on an object (hit relative to the hole).
template <typename R>
__device__ uchar4 object_color(const DevObject& o, V3<R> hit) {
  if (o.type == BH_OBJECT_RECTANGLE) {
    if (!o.tex.texels) return make_uchar4(0, 0, 0, 255);
    // Rectangle::color (vector_object.h:163-180)
    return quad_texel<R>(o.tex, BH_V(R, o, p0), BH_V(R, o, e1), BH_S(R, o, e1_len), BH_S(R, o, e2_len), hit);
  }
  if (o.type == BH_OBJECT_PLANE) {
    const R size = BH_S(R, o, pattern);
    if (!(size > R(0))) return make_uchar4(0, 0, 0, 255);
    // InfinitePlane::color (vector_object.h:227-232): plane coordinates
    // from the world x and y of the hit
    const V3<R> w = hit + BH_V(R, o, hw);
    const V3<R> ax = BH_V(R, o, ax), ay = BH_V(R, o, ay);
    const R b = (ax.x * w.y - ax.y * w.x) / (ax.x * ay.y - ax.y * ay.x);
    const R a = (w.x - b * ay.x) / ax.x;
    return chess<R>(size, a, b);
  }
  return make_uchar4(0, 0, 0, 255);  // Triangle: Material::color (material.h:54)
}

// Object::Collide of each type (points relative to the hole).
template <typename R>
__device__ bool object_collide(const DevObject& o, V3<R> a, V3<R> b, V3<R>* hit) {
  const V3<R> p0 = BH_V(R, o, p0);
  if (o.type == BH_OBJECT_RECTANGLE) {
    // Rectangle::Collide (vector_object.h:107-127): the chord crosses the
    // quad's plane inside the parallelogram on v1, v2 - v1, v4 - v1
    const V3<R> e1 = BH_V(R, o, e1), e2 = BH_V(R, o, e2), n = BH_V(R, o, n);
    const V3<R> Q1 = a - p0, Q2 = b - p0;
    const R q1 = dot(n, Q1), q2 = dot(n, Q2);
    if (!(q1 * q2 < R(0))) return false;
    const R a1 = fabs(q1), a2 = fabs(q2);
    const V3<R> Q = div3(Q1 * a2 + Q2 * a1, a1 + a2);
    const R d1 = dot(e1, Q), d2 = dot(e2, Q);
    if (d1 > R(0) && dot(e1, e1) > d1 && d2 > R(0) && dot(e2, e2) > d2) {
      *hit = Q + p0;
      return true;
    }
    return false;
  }
  if (o.type == BH_OBJECT_TRIANGLE) {
    // Triangle::Collide (vector_object.h:39-71), Moller-Trumbore; as in the
    // reference, t has no upper bound: a hit may lie past the chord's end
    const R ep = R(sizeof(R) == 8 ? 2.220446049250313e-15 : 1.1920928955078125e-06);
    const V3<R> rv = b - a;
    const V3<R> e1 = BH_V(R, o, e1), e2 = BH_V(R, o, e2);
    const V3<R> h = cross(rv, e2);
    const R det = dot(e1, h);
    if (-ep < det && det < ep) return false;
    const R f = R(1) / det;
    const V3<R> sv = a - p0;
    const R u = f * dot(sv, h);
    if (u < R(0) || u > R(1)) return false;
    const V3<R> q = cross(sv, e1);
    const R v = f * dot(rv, q);
    if (v < R(0) || u + v > R(1)) return false;
    const R t = f * dot(e2, q);
    if (t <= ep) return false;
    *hit = a + rv * t;
    return true;
  }
  // InfinitePlane::Collide (vector_object.h:210-225)
  const V3<R> n = BH_V(R, o, n);
  const R t1 = dot(n, a - p0), t2 = dot(n, b - p0);
  if (t1 * t2 > R(0)) return false;
  const R d1 = fabs(t1), d2 = fabs(t2);
  *hit = div3(a * d2 + b * d1, d1 + d2);
  return true;
}

// The object hit nearest a on the chord a -> b, visiting the objects from
// last to first and keeping the first on ties; -1 when none.
template <typename R>
__device__ int nearest_object(const DevScene& s, V3<R> a, V3<R> b, R* dd_out, V3<R>* hit) {
  int obj = -1;
  R best = R(0);
  for (int i = s.n_objects - 1; i >= 0; --i) {
    V3<R> h;
    if (object_collide<R>(s.objects[i], a, b, &h)) {
      const V3<R> d = a - h;
      const R dd = dot(d, d);
      if (obj < 0 || dd < best) {
        best = dd;
        *hit = h;
        obj = i;
      }
    }
  }
  *dd_out = best;
  return obj;
}

// ObjectManager::FindCollision (object_manager.h:69-85): the hit nearest p1
// over the scene's objects (kObjects), the hole (kHole) and the disc. Ties
// keep the first one visited, in the order the reference's object map
// visits them: the objects from last to first, then the hole, then the disc.
template <typename R, bool kHole = true, bool kObjects = false>
__device__ bool find_collision(const DevScene& s, V3<R> p1, V3<R> p2, Hit* out) {
  bool any = false;
  R best = R(0);
  V3<R> hp{};
  int which = BH_CLASS_MISS;
  int obj = -1;
  if (kObjects && s.n_objects > 0) {
    obj = nearest_object<R>(s, p1, p2, &best, &hp);
    if (obj >= 0) {
      any = true;
      which = BH_CLASS_OBJECT;
    }
  }
  if (kHole) {
    const R rad = BH_S(R, s, r_h);
    const R d1 = length(p1), d2 = length(p2);
    if (!(d1 < rad && d2 < rad)) {
      const V3<R> Q = p2 - p1;
      const R qp = dot(Q, p1), qq = dot(Q, Q);
      const R c = qp * qp - qq * (dot(p1, p1) - rad * rad);
      if (c > R(0)) {
        const R t = (R(1) / qq) * (-qp - sqrt(c));
        if (t > R(0) && t < R(1)) {
          const V3<R> h = p1 + Q * t;
          const V3<R> d = p1 - h;
          const R dd = dot(d, d);
          if (!any || dd < best) {
            best = dd;
            hp = h;
            any = true;
            which = BH_CLASS_HORIZON;
          }
        }
      }
    }
  }
  if (s.disc_on) {
    const V3<R> dc = BH_V(R, s, dc), n = BH_V(R, s, dn);
    const V3<R> q1 = p1 - dc, q2 = p2 - dc;
    const R t1 = dot(n, q1), t2 = dot(n, q2);
    if (!(t1 * t2 >= R(0))) {
      const R a1 = fabs(t1), a2 = fabs(t2);
      const V3<R> c = (q1 * a2 + q2 * a1) * (R(1) / (a1 + a2));
      const R lc = sqrt(dot(c, c));
      if (!(lc > BH_S(R, s, r_out)) && !(lc < BH_S(R, s, r_in))) {
        const V3<R> h = c + dc;
        const V3<R> d = p1 - h;
        const R dd = dot(d, d);
        if (!any || dd < best) {
          best = dd;
          hp = h;
          any = true;
          which = BH_CLASS_DISC;
        }
      }
    }
  }
  if (!any) return false;
  out->cls = which;
  out->aux = which == BH_CLASS_OBJECT ? float(obj) : 0.f;
  out->bgra = which == BH_CLASS_DISC     ? disc_color(s, hp)
              : which == BH_CLASS_OBJECT ? object_color<R>(s.objects[obj], hp)
                                         : make_uchar4(0, 0, 0, 255);
  return true;
}

// FLAT: the reference's flat-space RayTracer (ray_tracer.h:52-96) with
// BasicLinearRayRecurrence (:17-33) as ray_tracer_test.cc:140-155 drives it:
// from the focus toward the PixelVector point (REF raygen; PINHOLE: along
// it), ten chords, the step scaled by 100 / |step|^2 when |step|^2 < 100.
// e = focus - PixelVector point, so the first chord ends at F - e.
template <typename R>
__device__ Hit trace_flat(const DevScene& s, int x, int y) {
  const R a = BH_S(R, s, half_w) - R(x), c = BH_S(R, s, half_h) - R(y);
  const V3<R> e = BH_V(R, s, E0) + BH_V(R, s, vy) * a + BH_V(R, s, vz) * c;
  V3<R> old = BH_V(R, s, F);
  V3<R> pres = old - e;
  V3<R> vec = pres - old;
  const R d2 = dot(vec, vec);
  if (d2 < R(100)) vec = vec * (R(100) / d2);
  Hit hit = miss_hit();
  for (int i = 0; i < 10; ++i) {
    if (find_collision<R, false, true>(s, old, pres, &hit)) return hit;
    const V3<R> next = pres + vec;
    old = pres;
    pres = next;
  }
  return hit;
}

template <typename R, bool kObjects = false>
__device__ Hit trace_ref(const DevScene& s, int x, int y) {
  const PlaneRay<R> ray = make_ray<R>(s, x, y);
  const R M = BH_S(R, s, mass);
  const R b = ray.b;
  R sol = R(-1);
  if (b >= BH_S(R, s, b_c)) sol = solve_g<R>(b, M);
  const R periapsis = b < BH_S(R, s, b_c) ? R(1) / (R(3) * M) : sol;
  const R r0 = sqrt(ray.F0 * ray.F0 + ray.F1 * ray.F1 + b * b);
  R phi = atan(b / ray.F1);
  R dphi = R(0), dphi_prev = R(0);
  R u = R(1) / r0;
  const R du = (periapsis - u) * (R(1) / R(20));
  const R du_h = du / R(2);
  V3<R> prev = BH_V(R, s, F);
  Hit hit = miss_hit();
  for (int i = 0; i < 19; ++i) {
    u += du;
    dphi = inv_sqrt_g(u, b, M);
    phi += (dphi_prev + dphi) * du_h;
    const R r = R(1) / u;
    const V3<R> cur = ray.yv * (r * cos(phi)) + ray.xv * (r * sin(phi));
    dphi_prev = dphi;
    if (find_collision<R, true, kObjects>(s, prev, cur, &hit)) return hit;
    prev = cur;
  }
  {
    u += du * R(0.9);
    dphi = inv_sqrt_g(u, b, M);
    phi += (dphi_prev + dphi) * du_h;
    const R r = R(1) / u;
    const V3<R> cur = ray.yv * (r * cos(phi)) + ray.xv * (r * sin(phi));
    dphi_prev = dphi;
    if (find_collision<R, true, kObjects>(s, prev, cur, &hit)) return hit;
    prev = cur;
  }
  if (sol < R(0)) {
    find_collision<R, true, kObjects>(s, prev, V3<R>{R(0), R(0), R(0)}, &hit);
    return hit;
  }
  for (int i = 0; i < 19; ++i) {
    u -= du;
    dphi = inv_sqrt_g(u, b, M);
    phi += (dphi_prev + dphi) * du_h;
    const R r = R(1) / u;
    const V3<R> cur = ray.yv * (r * cos(phi)) + ray.xv * (r * sin(phi));
    if (find_collision<R, true, kObjects>(s, prev, cur, &hit)) return hit;
    dphi_prev = dphi;
    prev = cur;
  }
  return hit;
}

// ---------------------------------------------------------------------------
// RK4 in phi on x'' = x + 3 x^2, x = M/r - 1/3 (constants: Rk4Consts,
// precomputed on the host so that the FP32 paths issue no FP64 instruction).
template <typename R>
__device__ __forceinline__ const Rk4Consts<R>& bulk_consts(const LaunchParams& p);
template <>
__device__ __forceinline__ const Rk4Consts<float>& bulk_consts<float>(const LaunchParams& p) { return p.c32; }
template <>
__device__ __forceinline__ const Rk4Consts<double>& bulk_consts<double>(const LaunchParams& p) { return p.c64; }

template <typename R>
__device__ __forceinline__ R fx(R x) { return x * fma(R(3), x, R(1)); }

// One fourth-order step in phi of x'' = f(x). FP32: Nystrom's three-stage
// method for y'' = f(y) (no y' term; order 4 with stages at 0, h/2, h:
//   k1 = f(x), k2 = f(x + h/2 w + h^2/8 k1), k3 = f(x + h w + h^2/2 k2),
//   x' = x + h w + h^2/6 (k1 + 2 k2), w' = w + h/6 (k1 + 4 k2 + k3)),
// 15 FP32 instructions, 26 flops (FMA = 2); on this orbit equation its
// error constant is the smaller: on every escaped pixel of four frames of
// the 1080p fly-through at step 0.15 the deflection stays within 2.7e-5 rad
// of FP64 RK4 at step 0.01, where classical RK4 errs up to 4.1e-5. FP64:
// classical RK4 in Runge-Kutta-Nystrom form (18 instructions), the
// oracle's scheme, so that the FP64 tracer agrees with the oracle to
// rounding.
template <typename R>
__device__ __forceinline__ void rk4_step(R& x, R& w, const Rk4Consts<R>& c) {
  if constexpr (sizeof(R) == 4) {
    const float k1 = fx(x);
    const float k2 = fx(fmaf(c.h8, k1, fmaf(c.hh, w, x)));
    const float s3a = fmaf(c.h, w, x);
    const float k3 = fx(fmaf(c.q2, k2, s3a));
    x = fmaf(c.h26, fmaf(2.f, k2, k1), s3a);
    w = fmaf(c.h6, fmaf(4.f, k2, k1 + k3), w);
    return;
  }
  const R k1 = fx(x);
  const R s1 = fma(c.hh, w, x);
  const R k2 = fx(s1);
  const R s2 = fma(c.q, k1, s1);
  const R k3 = fx(s2);
  const R s3a = fma(c.h, w, x);
  const R s3 = fma(c.q2, k2, s3a);
  const R k4 = fx(s3);
  const R A = k2 + k3;
  const R S = A + k1;
  x = fma(c.h26, S, s3a);
  w = fma(c.h6, (S + A) + k4, w);
}

template <typename R>
__device__ __forceinline__ void rk4_partial(R& x, R& w, R h) {
  Rk4Consts<R> c;
  c.h = h;
  c.hh = h * R(0.5);
  c.q = h * h * R(0.25);
  c.q2 = h * h * R(0.5);
  c.h26 = h * h * R(1.0 / 6.0);
  c.h6 = h * R(1.0 / 6.0);
  c.h8 = h * h * R(0.125);
  rk4_step<R>(x, w, c);
}

// Moves (x, w) back onto w^2 - x^2 - 2 x^3 = eps along the gradient.
__device__ __forceinline__ void project_energy(float& x, float& w, float eps) {
  const float g = x * x * fmaf(2.f, x, 1.f);
  const float r = fmaf(w, w, -g) - eps;
  const float gx = -2.f * x * fmaf(3.f, x, 1.f);
  const float gw = 2.f * w;
  const float g2 = fmaf(gx, gx, gw * gw);
  if (g2 > 1e-30f) {
    const float k = __fdividef(r, g2);
    x = fmaf(-k, gx, x);
    w = fmaf(-k, gw, w);
  }
}
__device__ __forceinline__ void project_energy(double&, double&, double) {}

enum : int { kRunning = 0, kHorizon = 1, kEscape = 2, kDisc = 3, kMaxSteps = 4, kDone = 5 };

template <typename R>
struct RayState {
  R x, w;       // current state
  R xa, wa;     // state before the last step (escape refinement)
  R eps;        // first integral w^2 - x^2 - 2x^3 = 1/b^2 - 1/27 (units of M)
  R phi0;       // in-plane angle of the camera from the ray direction (aux only)
  R dcr;        // angle of the next disc-plane crossing from the camera, phi - phi0
  R ev;         // event payload: u at the disc crossing
  int k, kc;    // steps taken, step index holding the next crossing
  int status;
  bool near;    // mixed FP32 pass: |b - b_c| < kProjectBand M, (x, w) kept on eps
  V3<R> xv;     // with the scene's F / |F|, the ray's orbital basis rotated to the
                // camera: position = r (cos(phi - phi0) F^ + sin(phi - phi0) xv)
};

// Sets up the RK4 state of a ray; everything in precision R. The camera sits
// at angle phi0 = atan2(b, F1) from the ray direction; the basis rotated by
// phi0 (F^, X0) measures every later angle from the camera, so phi0 itself is
// only needed for the aux output.
template <typename R>
__device__ __forceinline__ void init_rk4(const DevScene& s, const RkRay<R>& ray, R h, RayState<R>& st) {
  R M, inv_m, x0, g0;
  if constexpr (sizeof(R) == 4) {
    const float4 m = s.hot[kHotMass];
    M = m.x;
    g0 = m.y;
    inv_m = s.hot[kHotF].w;
    x0 = s.hot[kHotFhat].w;
  } else {
    M = s.mass;
    g0 = s.g0;
    inv_m = 1.0 / s.mass;
    x0 = s.x0;
  }
  st.k = 0;
  st.kc = 0x7fffffff;
  st.near = false;
  st.dcr = R(0);
  st.ev = R(0);
  const R bm = ray.b * inv_m;
  st.xv = ray.X0;
  const int flags = s.hot_i.x;
  st.phi0 = (flags & kSceneAux) ? atan2(ray.b, ray.F1) : R(0);
  st.x = x0;
  if (!(bm > R(1e-6))) {  // heads into the centre
    st.status = kHorizon;
    st.w = R(0);
    st.eps = R(0);
    return;
  }
  const R mb = shade_div(M, ray.b);
  const R eps = mb * mb - R(1.0 / 27.0);
  st.eps = eps;
  const R P0 = fmax(eps + g0, R(0));  // w^2 at the camera; g0 = x0^2 (1 + 2 x0)
  if constexpr (sizeof(R) == 4) {
    st.w = copysignf(P0 > 1e-30f ? P0 * rsqrtf(P0) : 0.f, ray.F1);
  } else {
    st.w = copysign(sqrt(P0), ray.F1);
  }
  st.status = kRunning;
  if (flags & kSceneDisc) {
    R A, B;
    if constexpr (sizeof(R) == 4) {
      const float4 n = s.hot[kHotDn];
      A = n.w;
      B = dot(xyz(n), st.xv);
    } else {
      A = s.dnF;
      B = dot(BH_V(R, s, dn), st.xv);
    }
    if (A * A + B * B > R(1e-24)) {
      // the line of nodes: crossings at d + j pi, d in (0, pi]
      R d = shade_atan2(B, A) + kPi<R>() * R(0.5);
      if (d > kPi<R>()) d -= kPi<R>();
      if (d <= R(0)) d += kPi<R>();
      st.dcr = d;
      st.kc = (int)floor(shade_div(d, h));
    }
  }
}

// u at a disc-plane crossing: a partial RK4 step of length dcr - kc*h from
// the state at the start of step kc, in precision RC.
template <typename RC, typename R>
__device__ __forceinline__ RC crossing_u(const RayState<R>& st, R h) {
  const RC sc = RC(st.dcr) - RC(st.kc) * RC(h);
  RC x = RC(st.x), w = RC(st.w);
  rk4_partial<RC>(x, w, sc);
  return x + RC(1.0 / 3.0);
}

template <typename RC>
__device__ __forceinline__ bool on_disc(const DevScene& s, RC u) {
  if (!(u < RC(0.5))) return false;
  const RC rc = shade_div(BH_S(RC, s, mass), u);
  return rc >= BH_S(RC, s, r_in) && rc <= BH_S(RC, s, r_out);
}

// Root refinement of an FP32 crossing whose radius lies within 2e-3 M of a
// disc edge, in double-float (out of line): the partial step of length
// dcr - kc h from the step's FP32 start state, and the in/out decision
// r_in <= M / u <= r_out taken as r_in u <= M <= r_out u (u > 0), without a
// division. The state comes by value: a reference would pin the caller's ray
// state to its stack frame for the whole step loop.
struct CrossU {
  float u;
  int hit;
};
__device__ __noinline__ CrossU crossing_u_df(float dcr, int kc, float x, float w, float h, const DevScene& s) {
  const float kh = __fmul_rn(float(kc), h);  // kc h exactly, as kh + its rounding error
  const DF sc = df_sub(df_two_sum(dcr, -kh), DF{fmaf(float(kc), h, -kh), 0.f});
  DF k[6];
  df_rk4_consts(sc, k);
  DF xd{x, 0.f}, wd{w, 0.f};
  df_rk4_step(xd, wd, k);
  const DF u = df_add(xd, DF{0x1.555556p-2f, -0x1.555556p-27f});  // + 1/3
  const DF M{s.mass_df[0], s.mass_df[1]};
  const bool hit = u.hi > 0.f && u.hi < 0.5f && df_le(df_mul(DF{s.r_in_df[0], s.r_in_df[1]}, u), M) &&
                   df_le(M, df_mul(DF{s.r_out_df[0], s.r_out_df[1]}, u));
  return CrossU{u.hi, hit ? 1 : 0};
}

// Disc-plane crossing inside step kc. kRefine64: FP32 crossing with FP64
// refinement near the disc edges (mixed tracer).
template <typename R, bool kRefine64>
__device__ __forceinline__ bool cross_disc(const DevScene& s, RayState<R>& st, R h) {
  R u = crossing_u<R>(st, h);
  // on_disc, with the crossing radius kept for the refinement test
  const DiscRadii<R> d = disc_radii<R>(s);
  const R rc = shade_div(d.M, u);
  bool hit = u < R(0.5) && rc >= d.r_in && rc <= d.r_out;
  if (kRefine64) {
    const R tol = R(2e-3) * d.M;
    if (fabs(rc - d.r_in) < tol || fabs(rc - d.r_out) < tol) {
      const CrossU r64 = crossing_u_df(float(st.dcr), st.kc, float(st.x), float(st.w), float(h), s);
      u = R(r64.u);
      hit = r64.hit != 0;
    }
  }
  if (hit) {
    st.ev = u;
    return true;
  }
  st.dcr += kPi<R>();
  st.kc = (int)floor(shade_div(st.dcr, h));
  return false;
}

template <typename R>
__device__ __forceinline__ bool inside(R x, const Rk4Consts<R>& c) { return x > c.x_esc && x < c.x_hor; }

// Advances up to `budget` steps; returns the steps taken. kMixed (FP32 mixed
// tracer): energy projection near the saddle and FP64 refinement of
// crossings near the disc edges. kSliced: the persistent kernels' slices of
// `budget` steps; a trace to the end (false) skips the budget's tests.
template <typename R, bool kMixed, bool kSliced = true>
__device__ __forceinline__ int advance_rk4(const DevScene& s, RayState<R>& st, const Rk4Consts<R>& c,
                                           int budget) {
  constexpr bool kProject = kMixed;
  int taken = 0;
  while (st.status == kRunning) {
    if (st.k >= c.kmax) {
      st.status = kMaxSteps;
      break;
    }
    if (st.k == st.kc) {
      if (cross_disc<R, kMixed>(s, st, c.h)) {
        st.status = kDisc;
        break;
      }
    }
    if (kSliced && taken >= budget) break;
    const int kstop = kSliced ? min(min(st.kc, c.kmax), st.k + (budget - taken)) : min(st.kc, c.kmax);
    R x = st.x, w = st.w;
    int k = st.k;
    R xa = x, wa = w;
    int ev = kRunning;
    // blocks of 4 steps, event test once per block; a block that ends outside
    // takes the event from its kept states: the first step whose end lies
    // outside, as single steps would find it (same steps, same order)
    while (k + 4 <= kstop) {
      const R x0 = x, w0 = w;
      rk4_step<R>(x, w, c);
      const R x1 = x, w1 = w;
      rk4_step<R>(x, w, c);
      const R x2 = x, w2 = w;
      rk4_step<R>(x, w, c);
      const R x3 = x, w3 = w;
      rk4_step<R>(x, w, c);
      if (!inside(x, c)) {
        if (!inside(x1, c)) {
          xa = x0, wa = w0, x = x1, w = w1, k += 1;
        } else if (!inside(x2, c)) {
          xa = x1, wa = w1, x = x2, w = w2, k += 2;
        } else if (!inside(x3, c)) {
          xa = x2, wa = w2, x = x3, w = w3, k += 3;
        } else {
          xa = x3, wa = w3, k += 4;
        }
        ev = x <= c.x_esc ? kEscape : kHorizon;
        break;
      }
      k += 4;
      if (kProject) {
        if (st.near && fabs(x) < R(0.1)) project_energy(x, w, st.eps);
      }
    }
    // single steps up to kstop or the event
    while (ev == kRunning && k < kstop) {
      xa = x;
      wa = w;
      rk4_step<R>(x, w, c);
      ++k;
      if (!inside(x, c)) {
        ev = x <= c.x_esc ? kEscape : kHorizon;
        break;
      }
    }
    taken += k - st.k;
    st.k = k;
    st.x = x;
    st.w = w;
    st.xa = xa;
    st.wa = wa;
    st.status = ev;
  }
  return taken;
}

// Escape point of an FP32 ray that leaves outward through the whole last
// step: on the orbit, w^2 = P(x) = eps + x^2 (1 + 2x), so the angle from the
// step's start (x_a) to x_esc is the orbit integral
//   dphi = integral over [x_esc, x_a] of dx / sqrt(P(x)),
// taken by two-point Gauss-Legendre, and w there is -sqrt(P(x_esc)). Against
// the exact integral from the same x_a at step 0.15 this errs <= 1e-6 rad for
// cameras within 50 M (the Hermite interpolation below: up to 1e-5 rad). It
// is used where P varies by less than 30 % over the interval (P decreases
// with x there, so P(x_a) > 0.7 P(x_esc) bounds every node); otherwise (the
// ray turned within the step, or a camera close to the escape radius) the
// caller interpolates. FP64 rays always interpolate.
template <typename R>
__device__ __forceinline__ bool escape_by_integral(const RayState<R>& st, const Rk4Consts<R>& c, R* phie, R* we) {
  if constexpr (sizeof(R) != 4) {
    return false;
  } else {
    const float xa = st.xa, xe = c.x_esc, eps = st.eps;
    const float Pa = fmaf(xa * xa, fmaf(2.f, xa, 1.f), eps);
    const float Pe = fmaf(xe * xe, fmaf(2.f, xe, 1.f), eps);
    if (!(st.wa < 0.f && Pa > 0.f && Pa > 0.7f * Pe)) return false;
    const float m = 0.5f * (xa + xe), r = 0.5f * (xa - xe);
    const float x1 = fmaf(-0.57735027f, r, m), x2 = fmaf(0.57735027f, r, m);
    const float P1 = fmaf(x1 * x1, fmaf(2.f, x1, 1.f), eps);
    const float P2 = fmaf(x2 * x2, fmaf(2.f, x2, 1.f), eps);
    *phie = fmaf(r, rsqrtf(P1) + rsqrtf(P2), float(st.k - 1) * c.h);
    *we = -Pe * rsqrtf(Pe);
    return true;
  }
}

// Escape point by interpolation: cubic Hermite through (xa, wa) and (xb, wb)
// over the last step (step k, length h), Newton for the parameter t where
// x(t) = x_esc; returns the angle from the camera and w there.
template <typename R>
struct EscapePoint {
  R phie, we;
};
template <typename R>
__device__ __forceinline__ EscapePoint<R> escape_hermite(R xa, R wa, R xb, R wb, int k, R h, R xe) {
  const R ha = h * wa, hb = h * wb;
  R t = shade_div(xa - xe, xa - xb);
  t = fmin(fmax(t, R(0)), R(1));
  for (int i = 0; i < (sizeof(R) == 4 ? 2 : 3); ++i) {
    const R t2 = t * t, t3 = t2 * t;
    const R p = (R(2) * t3 - R(3) * t2 + R(1)) * xa + (t3 - R(2) * t2 + t) * ha + (R(3) * t2 - R(2) * t3) * xb +
                (t3 - t2) * hb;
    const R dp = (R(6) * t2 - R(6) * t) * xa + (R(3) * t2 - R(4) * t + R(1)) * ha + (R(6) * t - R(6) * t2) * xb +
                 (R(3) * t2 - R(2) * t) * hb;
    t = fmin(fmax(t - shade_div(p - xe, dp), R(0)), R(1));
  }
  const R t2 = t * t;
  const R dp = (R(6) * t2 - R(6) * t) * xa + (R(3) * t2 - R(4) * t + R(1)) * ha + (R(6) * t - R(6) * t2) * xb +
               (R(3) * t2 - R(2) * t) * hb;
  return EscapePoint<R>{(R(k - 1) + t) * h, shade_div(dp, h)};
}
// The same and the general disc colour as calls: finish_rk4's rare paths out
// of line (the plain tracers measured faster so: the FP32 grid kernel at
// step 0.01 29.0 ms against 32.4 ms with them inline on the 120-frame
// fly-through, where the mixed tracer's FP32 pass measured 0.06 ms slower).
template <typename R>
__device__ __noinline__ EscapePoint<R> escape_hermite_outlined(R xa, R wa, R xb, R wb, int k, R h, R xe) {
  return escape_hermite<R>(xa, wa, xb, wb, k, h, xe);
}
template <typename R>
__device__ __noinline__ uchar4 disc_color_outlined(const DevScene& s, V3<R> hit) {
  return disc_color(s, hit);
}

// Shades a finished RK4 ray. kRareInline: the interpolated escape and the
// general disc colour inline (the mixed tracer's FP32 pass) or as calls.
template <typename R, bool kRareInline = false>
__device__ Hit finish_rk4(const DevScene& s, const RayState<R>& st, const Rk4Consts<R>& c) {
  Hit hit = {make_uchar4(0, 0, 0, 255), BH_CLASS_HORIZON, 0.f};
  if (st.status == kMaxSteps) {
    hit.cls = BH_CLASS_MAXSTEPS;
  } else if (st.status == kDisc) {
    const int flags = s.hot_i.x;
    const R phic = st.dcr;
    const R rw = shade_div(disc_radii<R>(s).M, st.ev);
    R sp, cp;
    shade_sincos(phic, &sp, &cp);
    hit.cls = BH_CLASS_DISC;
    if (flags & kSceneAux) hit.aux = float(R(1) / st.ev);
    if (sizeof(R) == 4 && (flags & kSceneDiscPolarCentred)) {
      hit.bgra = disc_color_polar_centred(s, float(rw), float(cp), float(sp), cast3<float>(st.xv));
    } else {
      const V3<R> p = fhat_of<R>(s) * (rw * cp) + st.xv * (rw * sp);
      hit.bgra = kRareInline ? disc_color(s, p) : disc_color_outlined<R>(s, p);
    }
  } else if (st.status == kEscape) {
    R phie, we;  // angle from the camera and w = du/dphi at the escape radius
    if (!escape_by_integral(st, c, &phie, &we)) {
      const EscapePoint<R> e = kRareInline ? escape_hermite<R>(st.xa, st.wa, st.x, st.w, st.k, c.h, c.x_esc)
                                           : escape_hermite_outlined<R>(st.xa, st.wa, st.x, st.w, st.k, c.h, c.x_esc);
      phie = e.phie;
      we = e.we;
    }
    // direction angle psi = phie + atan2(u, -w) (from the radial direction,
    // measured from yv toward xv); its cosine and sine without atan2
    hit.cls = BH_CLASS_MISS;
    const int flags = s.hot_i.x;
    if (flags & kSceneAux) hit.aux = float(st.phi0 + phie + atan2(c.u_esc, -we) - kPi<R>());
    if (flags & kSceneBg) {
      R sp, cp;
      shade_sincos(phie, &sp, &cp);
      const R k = rnorm(we * we + c.u_esc * c.u_esc);
      const R cd = -we * k, sd = c.u_esc * k;
      const V3<R> d = fhat_of<R>(s) * (cp * cd - sp * sd) + st.xv * (sp * cd + cp * sd);
      hit.bgra = background_color(s, d);
    }
  }
  return hit;
}

// ---------------------------------------------------------------------------
// per-ray drivers
constexpr double kBC = 5.196152422706632;  // 3 sqrt(3)
// The mixed FP32 pass keeps (x, w) on the first integral near the photon
// sphere only for rays with |b - b_c| < kProjectBand M: elsewhere the FP32
// drift of eps moves the deflection by < 3e-6 M / |b - b_c| < 1e-5 rad.
constexpr float kProjectBand = 0.3f;

// Full trace in one precision R.
template <typename R, bool kMixed>
__device__ Hit trace_rk4(const DevScene& s, int x, int y, const Rk4Consts<R>& c, int* steps) {
  RayState<R> st;
  init_rk4<R>(s, make_ray_rk4<R>(s, x, y), c.h, st);
  *steps = advance_rk4<R, kMixed, false>(s, st, c, 0x7fffffff);
  return finish_rk4<R>(s, st, c);
}

// Full trace in one precision R of a scene with objects: single RK4 steps,
// each one's chord between the 3-D positions at its ends tested against the
// objects (as the reference tests every chord of its integration). Within a
// step the earlier event wins: a disc crossing at the fraction of the step's
// angle where it lies, an object hit at its fraction of the chord. Horizon
// and escape end the ray after the step's chord was tested.
template <typename R>
__device__ Hit trace_rk4_obj(const DevScene& s, int x, int y, const Rk4Consts<R>& c, int* steps) {
  RayState<R> st;
  init_rk4<R>(s, make_ray_rk4<R>(s, x, y), c.h, st);
  const R M = BH_S(R, s, mass);
  V3<R> prev = BH_V(R, s, F);
  int k = 0;
  while (st.status == kRunning) {
    if (k >= c.kmax) {
      st.status = kMaxSteps;
      break;
    }
    // the step's disc crossing (if any) decided first, from the step's start
    R f_disc = R(2);
    if (k == st.kc) {
      const R fr = (st.dcr - R(k) * c.h) / c.h;
      if (cross_disc<R, false>(s, st, c.h)) f_disc = fmax(fr, R(0));
    }
    R xn = st.x, wn = st.w;
    rk4_step<R>(xn, wn, c);
    const R un = xn + R(1.0 / 3.0);
    R f_obj = R(2);
    Hit ho;
    if (un > R(0)) {
      const R rn = shade_div(M, un);
      R sp, cp;
      shade_sincos(R(k + 1) * c.h, &sp, &cp);
      const V3<R> next = BH_V(R, s, Fhat) * (rn * cp) + st.xv * (rn * sp);
      V3<R> hp;
      R bd = R(0);
      const int best = nearest_object<R>(s, prev, next, &bd, &hp);
      if (best >= 0) {
        const V3<R> ch = next - prev;
        f_obj = sqrt(bd / dot(ch, ch));
        ho.cls = BH_CLASS_OBJECT;
        ho.aux = float(best);
        ho.bgra = object_color<R>(s.objects[best], hp);
      }
      prev = next;
    }
    if (f_disc <= R(1) && f_disc <= f_obj) {
      st.status = kDisc;
      break;
    }
    if (f_obj <= R(1)) {
      *steps = k + 1;
      return ho;
    }
    st.xa = st.x;
    st.wa = st.w;
    st.x = xn;
    st.w = wn;
    st.k = ++k;
    if (!inside(xn, c)) st.status = xn <= c.x_esc ? kEscape : kHorizon;
  }
  *steps = k;
  return finish_rk4<R>(s, st, c);
}

// ---------------------------------------------------------------------------
// MULTI: several holes. Null rays of the static metric
//   ds^2 = -a^2 dt^2 + p^4 |dx|^2,  p = 1 + S,  a = (1 - S) / (1 + S),
//   S = sum_i m_i / (2 |x - x_i|)
// in isotropic coordinates (one hole: Schwarzschild). Their spatial paths are
// the rays of the index n = p^2 / a = (1 + S)^3 / (1 - S) (Fermat): with s
// the Euclidean arc length and T the unit tangent,
//   dx/ds = T,  dT/ds = g - T (T . g),  g = grad ln n = (3 / (1 + S) + 1 / (1 - S)) grad S.
// One evaluation: the bending g - T (T . g) at (x, T), S at x and the
// squared distance to the nearest hole centre.
template <typename R>
struct MultiEval {
  V3<R> a;
  R S, d2;
};

template <typename R>
__device__ __forceinline__ void load_hole(const DevHole& h, V3<R>* p, R* hm);
template <>
__device__ __forceinline__ void load_hole<float>(const DevHole& h, V3<float>* p, float* hm) {
  const float4 q = *reinterpret_cast<const float4*>(h.p_f);
  *p = {q.x, q.y, q.z};
  *hm = q.w;
}
template <>
__device__ __forceinline__ void load_hole<double>(const DevHole& h, V3<double>* p, double* hm) {
  *p = {h.p[0], h.p[1], h.p[2]};
  *hm = h.hm;
}

// Reciprocal square root and reciprocal of the MULTI integrator: in FP32 the
// PTX approximations (rsqrt.approx / rcp.approx, relative error below 2^-22,
// flush-to-zero: squared distances are at least (m/2)^2 and 1 +- S lies in
// [0.1, 2] away from the capture), the exact forms in FP64.
__device__ __forceinline__ float multi_rsqrt(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ double multi_rsqrt(double x) { return 1.0 / sqrt(x); }
__device__ __forceinline__ float multi_rcp(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float multi_sqrt(float x) { return x * multi_rsqrt(x); }
__device__ __forceinline__ double multi_sqrt(double x) { return sqrt(x); }
template <typename R>
__device__ __forceinline__ V3<R> multi_normalize(V3<R> a) { return a * multi_rsqrt(dot(a, a)); }

// kN: the number of holes when known at compile time (1 or 2), 0 for any.
template <typename R, int kN>
__device__ __forceinline__ MultiEval<R> multi_eval(const DevScene& s, V3<R> x, V3<R> T) {
  R S = R(0), d2 = R(3e38);
  V3<R> gS = {R(0), R(0), R(0)};
  const int n = kN > 0 ? kN : s.n_holes;
#pragma unroll
  for (int i = 0; i < (kN > 0 ? kN : BH_MAX_HOLES); ++i) {
    if (kN == 0 && i >= n) break;
    V3<R> p;
    R hm;
    load_hole<R>(s.holes[i], &p, &hm);
    const V3<R> d = x - p;
    const R r2 = dot(d, d);
    const R ir = multi_rsqrt(r2);
    const R k = hm * ir;
    S += k;
    gS = gS - d * (k * ir * ir);
    d2 = fmin(d2, r2);
  }
  R f;
  if constexpr (sizeof(R) == 4) {
    f = R(3) * multi_rcp(R(1) + S) + multi_rcp(R(1) - S);
  } else {
    f = R(3) / (R(1) + S) + R(1) / (R(1) - S);
  }
  const V3<R> g = gS * f;
  return {g - T * dot(T, g), S, d2};
}

// Cubic Hermite through (x0, h T0) and (x1, h T1) at t: position and d/dt.
template <typename R>
__device__ __forceinline__ void hermite3(V3<R> x0, V3<R> m0, V3<R> x1, V3<R> m1, R t, V3<R>* p, V3<R>* dp) {
  const R t2 = t * t, t3 = t2 * t;
  *p = x0 * (R(2) * t3 - R(3) * t2 + R(1)) + m0 * (t3 - R(2) * t2 + t) + x1 * (R(3) * t2 - R(2) * t3) +
       m1 * (t3 - t2);
  *dp = x0 * (R(6) * t2 - R(6) * t) + m0 * (R(3) * t2 - R(4) * t + R(1)) + x1 * (R(6) * t - R(6) * t2) +
        m1 * (R(3) * t2 - R(2) * t);
}

// One ray of the MULTI integrator, all in precision R, positions relative to
// the scene's hole. Each step: RK4 in s with h = step * (distance to the
// nearest hole); the disc is found on the step's Hermite curve (the sign of
// n . (x - c) changes; three Newton steps for the crossing from the chord's
// estimate), the objects on the step's chord. Within a step the earlier
// event wins (the disc on ties), as in the RK4 render with objects; a ray
// whose S reaches 0.9 is captured; one that leaves the escape sphere moving
// outward escapes in the direction of the Hermite tangent where the curve
// meets the sphere (three Newton steps).
template <typename R, int kN>
__device__ Hit trace_multi_n(const DevScene& s, int px, int py, const Rk4Consts<R>& c, int* steps) {
  const R a_ = BH_S(R, s, half_w) - R(px);
  const R c_ = BH_S(R, s, half_h) - R(py);
  const V3<R> T0 = normalize(BH_V(R, s, E0) + BH_V(R, s, vy) * a_ + BH_V(R, s, vz) * c_) * R(-1);
  const V3<R> cen = BH_V(R, s, mcen);
  const R resc = BH_S(R, s, r_esc), resc2 = resc * resc;
  const bool disc_on = s.disc_on != 0;
  const V3<R> dn = BH_V(R, s, dn), dc = BH_V(R, s, dc);
  const R r_in = BH_S(R, s, r_in), r_out = BH_S(R, s, r_out);
  V3<R> X = BH_V(R, s, F), T = T0;
  MultiEval<R> e = multi_eval<R, kN>(s, X, T);
  Hit hit = {make_uchar4(0, 0, 0, 255), BH_CLASS_MAXSTEPS, 0.f};
  int k = 0;
  for (;; ++k) {
    if (e.S >= R(0.9)) {
      hit.cls = BH_CLASS_HORIZON;
      break;
    }
    if (k >= c.kmax) break;
    const R h = c.h * multi_sqrt(e.d2), hh = h * R(0.5);
    const V3<R> t2 = T + e.a * hh;
    const MultiEval<R> e2 = multi_eval<R, kN>(s, X + T * hh, t2);
    const V3<R> t3 = T + e2.a * hh;
    const MultiEval<R> e3 = multi_eval<R, kN>(s, X + t2 * hh, t3);
    const V3<R> t4 = T + e3.a * h;
    const MultiEval<R> e4 = multi_eval<R, kN>(s, X + t3 * h, t4);
    const R h6 = h * R(1.0 / 6.0);
    const V3<R> Xn = X + (T + (t2 + t3) * R(2) + t4) * h6;
    const V3<R> Tn = multi_normalize(T + (e.a + (e2.a + e3.a) * R(2) + e4.a) * h6);
    // disc crossing on the step's curve
    R f_disc = R(2);
    V3<R> dhit;
    if (disc_on) {
      const R g0 = dot(dn, X - dc), g1 = dot(dn, Xn - dc);
      if ((g0 > R(0)) != (g1 > R(0))) {
        R t = g0 != g1 ? shade_div(g0, g0 - g1) : R(0.5);
        V3<R> p, dp;
        for (int i = 0; i < 3; ++i) {
          hermite3<R>(X, T * h, Xn, Tn * h, t, &p, &dp);
          const R dd = dot(dn, dp);
          if (dd != R(0)) t = fmin(fmax(t - shade_div(dot(dn, p - dc), dd), R(0)), R(1));
        }
        hermite3<R>(X, T * h, Xn, Tn * h, t, &p, &dp);
        const R rr = length(p - dc);
        if (rr >= r_in && rr <= r_out) {
          f_disc = t;
          dhit = p;
        }
      }
    }
    // objects on the step's chord
    R f_obj = R(2);
    Hit ho;
    if (s.n_objects > 0) {
      V3<R> hp;
      R bd = R(0);
      const int best = nearest_object<R>(s, X, Xn, &bd, &hp);
      if (best >= 0) {
        const V3<R> ch = Xn - X;
        f_obj = sqrt(shade_div(bd, dot(ch, ch)));
        ho.cls = BH_CLASS_OBJECT;
        ho.aux = float(best);
        ho.bgra = object_color<R>(s.objects[best], hp);
      }
    }
    if (f_disc <= R(1) && f_disc <= f_obj) {
      hit.cls = BH_CLASS_DISC;
      hit.aux = float(length(dhit - dc) / BH_S(R, s, mass));
      hit.bgra = disc_color(s, dhit);
      ++k;
      break;
    }
    if (f_obj <= R(1)) {
      hit = ho;
      ++k;
      break;
    }
    const V3<R> q = Xn - cen;
    if (dot(q, q) >= resc2 && dot(Tn, q) > R(0)) {
      // the curve meets the escape sphere: |p(t) - cen|^2 = resc^2
      const V3<R> q0 = X - cen;
      const R r0 = length(q0), r1 = length(q);
      R t = r1 != r0 ? fmin(fmax(shade_div(resc - r0, r1 - r0), R(0)), R(1)) : R(1);
      V3<R> p, dp;
      for (int i = 0; i < 3; ++i) {
        hermite3<R>(X, T * h, Xn, Tn * h, t, &p, &dp);
        const V3<R> w = p - cen;
        const R dd = R(2) * dot(w, dp);
        if (dd != R(0)) t = fmin(fmax(t - shade_div(dot(w, w) - resc2, dd), R(0)), R(1));
      }
      hermite3<R>(X, T * h, Xn, Tn * h, t, &p, &dp);
      const V3<R> Te = normalize(dp);
      hit.cls = BH_CLASS_MISS;
      hit.aux = float(atan2(length(cross(T0, Te)), dot(T0, Te)));
      if (s.has_bg) hit.bgra = background_color(s, Te);
      ++k;
      break;
    }
    X = Xn;
    T = Tn;
    e = multi_eval<R, kN>(s, X, T);
  }
  *steps = k;
  return hit;
}

// The hole count is the same for every ray of a scene: one and two holes
// get their own unrolled copy.
template <typename R>
__device__ Hit trace_multi(const DevScene& s, int px, int py, const Rk4Consts<R>& c, int* steps) {
  if (s.n_holes == 2) return trace_multi_n<R, 2>(s, px, py, c, steps);
  if (s.n_holes == 1) return trace_multi_n<R, 1>(s, px, py, c, steps);
  return trace_multi_n<R, 0>(s, px, py, c, steps);
}

// The FP64 band pass's integration, in double-float on the FP32 pipe: the
// loop of advance_rk4 (blocks of 4 steps with one event test, then single
// steps to the event or the next crossing's step) over a state of two floats
// each, with the band step's constants split on the host. Setup, crossings
// and the escape stay in FP64 (once per ray or event), on the state converted
// exactly to double. Double-float rounding (~2^-48) is amplified like FP64's
// (2^-53) near the photon orbit: against the FP64 integration of the same
// step it errs ~1e-7 rad at |b - b_c| = 1e-6 M and ~1e-6 rad at 1e-8 M, so
// rays with |b - b_c| below ~1e-7 M stay in FP64 (band_needs_fp64). The state
// is not projected onto the first integral: RK4's own truncation moves that
// integral, and a projected trajectory leaves the FP64 one by ~2e-11 / |b - b_c|
// rad at the band step 0.01.
__device__ __forceinline__ int advance_band_df(const DevScene& s, RayState<double>& st, const Rk4Consts<double>& c,
                                               const LaunchParams& p, int budget) {
  DF k[6];
  for (int i = 0; i < 6; ++i) k[i] = DF{p.band_df[i][0], p.band_df[i][1]};
  const DF x_esc{p.band_df[6][0], p.band_df[6][1]}, x_hor{p.band_df[7][0], p.band_df[7][1]};
  int taken = 0;
  while (st.status == kRunning) {
    if (st.k >= c.kmax) {
      st.status = kMaxSteps;
      break;
    }
    if (st.k == st.kc) {
      if (cross_disc<double, false>(s, st, c.h)) {
        st.status = kDisc;
        break;
      }
    }
    if (taken >= budget) break;
    const int kstop = min(min(st.kc, c.kmax), st.k + (budget - taken));
    DF x = df_from(st.x), w = df_from(st.w);
    int kk = st.k;
    while (kk + 4 <= kstop) {
      const DF x0 = x, w0 = w;
      df_rk4_step(x, w, k);
      df_rk4_step(x, w, k);
      df_rk4_step(x, w, k);
      df_rk4_step(x, w, k);
      if (!(df_lt(x_esc, x) && df_lt(x, x_hor))) {
        x = x0;
        w = w0;
        break;
      }
      kk += 4;
    }
    DF xa = x, wa = w;
    int ev = kRunning;
    while (kk < kstop) {
      xa = x;
      wa = w;
      df_rk4_step(x, w, k);
      ++kk;
      if (!(df_lt(x_esc, x) && df_lt(x, x_hor))) {  // also NaN
        ev = df_le(x, x_esc) ? kEscape : kHorizon;
        break;
      }
    }
    taken += kk - st.k;
    st.k = kk;
    st.x = df_to(x);
    st.w = df_to(w);
    st.xa = df_to(xa);
    st.wa = df_to(wa);
    st.status = ev;
  }
  return taken;
}

// Band rays whose first integral lies within ~1.5e-9 of the photon orbit's
// (|b - b_c| < ~1e-7 M) integrate in FP64, the rest in double-float.
__device__ __forceinline__ bool band_needs_fp64(const RayState<double>& st) { return fabs(st.eps) < 1.5e-9; }

// One band slice: up to `budget` steps in the precision the ray needs.
__device__ __forceinline__ int advance_band(const DevScene& s, RayState<double>& st, const Rk4Consts<double>& c,
                                            const LaunchParams& p, int budget) {
  if (band_needs_fp64(st)) return advance_rk4<double, false>(s, st, c, budget);
  return advance_band_df(s, st, c, p, budget);
}

// Trace of a band ray: FP64 setup and events, the integration of
// advance_band (out of line: keeps its register pressure away from the FP32
// callers).
__device__ __noinline__ Hit trace_band(const DevScene& s, int x, int y, const LaunchParams& p, int* steps) {
  RayState<double> st;
  init_rk4<double>(s, make_ray_rk4<double>(s, x, y), p.cband.h, st);
  *steps = advance_band(s, st, p.cband, p, 0x7fffffff);
  return finish_rk4<double>(s, st, p.cband);
}

// First integral eps = 1/(b/M)^2 - 1/27 of pixel (x, y), exact to double-float
// (~1e-13 relative): b = |F x e| / |e|, so (b/M)^-2 = M^2 |e|^2 / |F x e|^2,
// both squares evaluated from their per-scene quadratic forms in the pixel
// offsets (resolve_derived). About 200 FP32 instructions, where the same in
// FP64 took ~25 FP64 instructions of ~64 issue cycles each. Every operation is
// an explicitly rounded double-float step (no contraction the compiler could
// choose differently), so each kernel that inlines this and decides the FP64
// band with it takes the same decision for every ray.
__device__ __forceinline__ DF eps_df(const DevScene& s, int x, int y) {
  const float a = s.half_w_f - float(x), c = s.half_h_f - float(y);  // exact: half sizes are k / 2
  return df_first_integral(df_quad_form(s.eq_e, a, c), df_quad_form(s.eq_g, a, c), DF{s.m2_df[0], s.m2_df[1]});
}

// The FP64 band test of the mixed tracer: an FP32 prefilter on b, then the
// exact first integral of the candidates. setup_mixed and the classification
// pass make the same decision (same code, same ray).
__device__ __forceinline__ bool band_candidate(const DevScene& s, const RkRay<float>& r, const LaunchParams& p) {
  return fabsf(r.b * s.hot[kHotF].w - float(kBC)) < p.setup_band;
}
__device__ __forceinline__ bool in_band_eps(DF eps, const LaunchParams& p) {
  return df_lt(DF{p.eps_band_df[0], p.eps_band_df[1]}, eps) && df_lt(eps, DF{p.eps_band_df[2], p.eps_band_df[3]});
}

// Sets up one ray of the mixed tracer. Returns false when the ray belongs to
// the FP64 band: the lane is left idle (status kDone) and the FP64 pass alone
// traces and writes the ray. Rays within setup_band of b_c take their first
// integral from FP64; everything else of the setup is FP32.
__device__ __forceinline__ bool setup_mixed(const DevScene& s, int x, int y, const LaunchParams& p,
                                            RayState<float>& st) {
  const RkRay<float> r = make_ray_rk4<float>(s, x, y);
  init_rk4<float>(s, r, p.c32.h, st);
  st.near = fabsf(r.b * s.hot[kHotF].w - float(kBC)) < kProjectBand;
  if (band_candidate(s, r, p)) {
    const DF eps = eps_df(s, x, y);
    if (in_band_eps(eps, p)) {
      st.status = kDone;
      return false;
    }
    if (st.status == kRunning) {
      st.eps = eps.hi;
      st.w = copysignf(sqrtf(fmaxf(st.eps + s.hot[kHotMass].y, 0.f)), st.w);
    }
  }
  return true;
}

// ---------------------------------------------------------------------------
// warp-aggregated counter update
// The thread's lane in its warp (2-D blocks narrower than 32 threads put
// several rows of the block in one warp, so threadIdx.x is not the lane).
__device__ __forceinline__ unsigned lane_id() {
  unsigned l;
  asm volatile("mov.u32 %0, %%laneid;" : "=r"(l));
  return l;
}

// Sums v over the active lanes into *dst: two 32-bit warp reductions, of the
// low 27 bits and of the rest, exact for every v below 2^54 (a thread's step
// count stays below 8 * 1e8 < 2^30).
__device__ __forceinline__ void warp_add(unsigned long long* dst, unsigned long long v) {
  const unsigned m = __activemask();
  const unsigned lo = __reduce_add_sync(m, unsigned(v & 0x7ffffffull));
  const unsigned hi = __reduce_add_sync(m, unsigned(v >> 27));
  const unsigned long long t = (unsigned long long)lo + ((unsigned long long)hi << 27);
  if (lane_id() == unsigned(__ffs(m) - 1) && t) atomicAdd(dst, t);
}

// BGR8 (CV_8UC3) frames. In a warp whose lanes hold rows of pixels in
// order (rows of 4, 8, 16 or 32 pixels starting at a multiple of 4 in x:
// lane l + 1 holds the right neighbour of lane l unless x % 4 == 3), the
// lanes with k = x % 4 < 3 write the 32-bit word that starts k bytes into
// their own pixel (byte 3 x + k; four pixels make three words): bytes k .. 2
// of their pixel and the first k + 1 of the next lane's, one shuffle and 24
// word stores per 32 pixels where byte stores would take 96. `bgr` is the
// lane's pixel as B | G << 8 | R << 16. Rows must start on 4-byte
// boundaries (frame base 4-aligned, width a multiple of 4). Called by all 32
// lanes.
__device__ __forceinline__ void store_bgr8_words(uint8_t* frame, int width, int x, int y, uint32_t bgr) {
  const uint32_t next = __shfl_down_sync(kFull, bgr, 1);
  const int k = x & 3;
  if (k < 3)
    *reinterpret_cast<uint32_t*>(frame + 3 * ((long long)y * width + x) + k) = (bgr >> (8 * k)) | (next << (24 - 8 * k));
}

__device__ __forceinline__ uint32_t bgr_word(const Hit& h) {
  return uint32_t(h.bgra.x) | (uint32_t(h.bgra.y) << 8) | (uint32_t(h.bgra.z) << 16);
}

// True when store_bgr8_words can write the warp's pixels: the GRID kernels'
// warps cover whole rows of bw pixels (lane l at (x0 + l % bw, y0 + l / bw),
// x0 a multiple of bw, so of 4), and then it takes every lane's pixel in the
// frame (`valid`: the next lane's pixel is part of the word) and frame rows
// that start on 4-byte boundaries. Called by all 32 lanes; the result is the
// same on every lane.
__device__ __forceinline__ bool bgr8_block_ok(const DevScene& s, bool valid) {
  return __all_sync(kFull, valid) && (s.hot_i.y & 3) == 0 && (reinterpret_cast<uintptr_t>(s.pixels) & 3) == 0;
}

// The frame of this GRID block and the block's column and row of block tiles
// in it: blocks enumerate the frames' blocks back to back (block_begin), so
// a binary search over the frames' first blocks finds it (once per block).
__device__ __forceinline__ int grid_block_frame(const LaunchParams& p, long long b, int* bxi, int* byi) {
  int lo = 0, hi = p.n_scenes - 1;
  if (p.frame_blocks > 0) {
    // frames of one size: a division instead of a chain of dependent loads
    lo = int(b / p.frame_blocks);
  } else {
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (p.scenes[mid].block_begin <= b) lo = mid;
      else hi = mid - 1;
    }
  }
  const int local = int(b - p.scenes[lo].block_begin);
  const int bx_count = p.scenes[lo].blocks_x;
  *byi = local / bx_count;
  *bxi = local - *byi * bx_count;
  return lo;
}

// GRID store of pixel (x, y) (`valid`: it lies in the frame). In BGR8 frames
// a warp of a block whose rows are whole warps or hold a whole number of
// warp rows writes packed words. Called by all 32 lanes of the warp.
__device__ __forceinline__ void grid_store(const DevScene& s, int format, int x, int y, bool valid, const Hit& h) {
  if (format == BH_FORMAT_BGR8) {
    // warps cover whole rows of bw pixels: block rows of a multiple of 32
    // pixels, or of 4, 8 or 16 (powers of two dividing 32)
    const int bx = int(blockDim.x);
    const bool rows = (bx & 31) == 0 || (bx >= 4 && bx < 32 && (bx & (bx - 1)) == 0);
    if (rows && bgr8_block_ok(s, valid)) {
      store_bgr8_words(s.pixels, s.hot_i.y, x, y, bgr_word(h));
      store_extras(s, x, y, h);
      return;
    }
  }
  if (valid) store_hit(s, format, x, y, h);
}

// GRID schedule: one thread per pixel of each of rays_per_thread block tiles
// (consecutive down the image, traced one after the other), gridDim.z =
// scene; one kernel per precision and integrator, each with the registers
// (and the occupancy) of its own variant. kDefer (MIXED on the HYBRID
// schedule): FP64 band rays are left to the persistent FP64 pass, which
// traces and writes them; a drain_only launch (the host's, after the FP64
// pass) traces only when the FP64 pass could not launch this kernel itself.
template <int kPrecision, int kIntegrator, bool kDefer>
__device__ __forceinline__ void grid_block(const LaunchParams& p, long long vb) {
  int bxi, byi;
  const DevScene& s = p.scenes[grid_block_frame(p, vb, &bxi, &byi)];
  const int x = bxi * blockDim.x + threadIdx.x;
  // every lane stays to the end: BGR8 stores are whole-warp operations
  unsigned long long steps_all = 0, rays = 0, band_rays = 0, band_steps = 0;
  for (int k = 0; k < p.rays_per_thread; ++k) {
    const int4 fl = s.hot_i;  // flags, width, height
    const int row0 = (byi * p.rays_per_thread + k) * blockDim.y;
    if (row0 >= fl.z) break;  // the same for the whole block
    const int y = row0 + threadIdx.y;
    const bool valid = x < fl.y && y < fl.z;
    Hit h = miss_hit();
    int steps = 0;
    int band_ray = 0;
    bool deferred = false;
    if (!valid) {
    } else if (kIntegrator == BH_INTEGRATOR_REF_TRAPEZOID) {
      h = kPrecision == BH_PRECISION_FP64 ? trace_ref<double>(s, x, y) : trace_ref<float>(s, x, y);
    } else if (kPrecision == BH_PRECISION_FP64) {
      h = trace_rk4<double, false>(s, x, y, p.c64, &steps);
    } else if (kPrecision == BH_PRECISION_MIXED) {
      RayState<float> st;
      if (setup_mixed(s, x, y, p, st)) {
        steps = advance_rk4<float, true, false>(s, st, p.c32, 0x7fffffff);
        h = finish_rk4<float, true>(s, st, p.c32);
      } else if (kDefer) {
        deferred = true;
      } else {
        band_ray = 1;
        h = trace_band(s, x, y, p, &steps);
      }
    } else {
      h = trace_rk4<float, false>(s, x, y, p.c32, &steps);
    }
    grid_store(s, p.format, x, y, valid && !deferred, h);
    steps_all += steps;
    rays += valid && !deferred ? 1 : 0;
    band_rays += band_ray;
    band_steps += band_ray ? steps : 0;
  }
  if (p.counters) {
    warp_add(&p.counters->steps, steps_all);
    warp_add(&p.counters->rays, rays);
    if (__any_sync(__activemask(), band_rays != 0)) {
      warp_add(&p.counters->band_rays, band_rays);
      warp_add(&p.counters->band_steps, band_steps);
    }
  }
}

template <int kPrecision, int kIntegrator, bool kDefer = false>
__global__ void __launch_bounds__(256) grid_kernel(LaunchParams p) {
  if (kDefer && p.drain_only) {
    // the host's launch after the FP64 pass: about one wave of blocks, which
    // trace every frame block only when the FP64 pass did not launch this
    // kernel (band_serial 2, or its device-side launch failed); a launch of
    // the full grid spent ~0.13 ms on the 120-frame fly-through scheduling
    // blocks that return at once
    if (p.mixed_blocks && !(p.counters->flags & kFlagBandLaunchFailed)) return;
    for (long long vb = blockIdx.x; vb < p.grid_dim[0]; vb += gridDim.x) grid_block<kPrecision, kIntegrator, kDefer>(p, vb);
    return;
  }
  grid_block<kPrecision, kIntegrator, kDefer>(p, blockIdx.x);
}


// GRID schedule for the FLAT and MULTI integrators and for scenes with objects: one
// kernel per precision and integrator, so that the object code does not
// raise the register count of grid_kernel and each variant gets the
// occupancy of its own registers (FP32 RK4 with objects: 64, where one
// kernel over all six variants took 128).
template <typename R, int kIntegrator>
__global__ void __launch_bounds__(256) grid_objects_kernel(LaunchParams p) {
  int bxi, byi;
  const DevScene& s = p.scenes[grid_block_frame(p, blockIdx.x, &bxi, &byi)];
  const int x = bxi * blockDim.x + threadIdx.x;
  // every lane stays to the end: BGR8 stores are whole-warp operations
  unsigned long long steps_all = 0, rays = 0;
  for (int k = 0; k < p.rays_per_thread; ++k) {
    const int row0 = (byi * p.rays_per_thread + k) * blockDim.y;
    if (row0 >= s.height) break;  // the same for the whole block
    const int y = row0 + threadIdx.y;
    const bool valid = x < s.width && y < s.height;
    Hit h = miss_hit();
    int steps = 0;
    if (!valid) {
    } else if (kIntegrator == BH_INTEGRATOR_FLAT) {
      h = trace_flat<R>(s, x, y);
    } else if (kIntegrator == BH_INTEGRATOR_MULTI) {
      h = trace_multi<R>(s, x, y, bulk_consts<R>(p), &steps);
    } else if (kIntegrator == BH_INTEGRATOR_REF_TRAPEZOID) {
      h = trace_ref<R, true>(s, x, y);
    } else if (s.n_objects > 0) {
      h = trace_rk4_obj<R>(s, x, y, bulk_consts<R>(p), &steps);
    } else {
      h = trace_rk4<R, false>(s, x, y, bulk_consts<R>(p), &steps);
    }
    grid_store(s, p.format, x, y, valid, h);
    steps_all += steps;
    rays += valid ? 1 : 0;
  }
  if (p.counters) {
    warp_add(&p.counters->steps, steps_all);
    warp_add(&p.counters->rays, rays);
  }
}

// ---------------------------------------------------------------------------
// PERSISTENT schedule.
//
// Work is a queue of 32-ray items: 8x4-pixel tiles over all scenes of the call
// (scenes back to back, each padded to whole tiles), or 32 entries of the
// band list in the FP64 pass. Each warp keeps one pending item: a 32-bit mask
// of its rays not yet handed to a lane. After each slice of integration steps
// the warp counts its idle lanes (ballot); once at least `refill_threshold`
// are idle it hands them the pending item's next rays in lane order
// (re-packing the warp), and takes the next item from the queue (one
// atomicAdd per 32 rays) when the pending one runs dry. A tile's scene is
// looked up once per tile. With MIXED precision, rays of the FP64 band are
// not traced in the FP32 pass: their indices go to the band list, which a
// second persistent pass traces in FP64.

__device__ __forceinline__ int find_scene(const LaunchParams& p, long long ray) {
  int lo = 0, hi = p.n_scenes - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (p.scenes[mid].ray_begin <= ray) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Pixel of ray `local` (index within its scene). The tile index stays below
// 2^25, so the division by tiles_x is a multiply and a shift (DivMagic).
__device__ __forceinline__ bool ray_pixel(const DevScene& s, long long local, int* x, int* y) {
  const unsigned tile = (unsigned)(local >> 5);
  const int l = (int)(local & 31);
  const int ty = (int)(((unsigned long long)tile * s.tiles_x_magic) >> s.tiles_x_shift);
  const int tx = (int)tile - ty * s.tiles_x;
  *x = tx * 8 + (l & 7);
  *y = ty * 4 + (l >> 3);
  return *x < s.width && *y < s.height;
}

// Sets up the FP32-pass ray `item` (global ray index) on this lane; returns
// false when the lane stays idle (padding pixel or deferred band ray).
template <bool kMixed>
__device__ __forceinline__ bool take_fp32_ray(const LaunchParams& p, int scene, long long item,
                                              RayState<float>& st, int* px, int* py, unsigned long long* steps) {
  const DevScene& s = p.scenes[scene];
  if (!ray_pixel(s, item - s.ray_begin, px, py)) return false;
  if (!kMixed) {
    init_rk4<float>(s, make_ray_rk4<float>(s, *px, *py), p.c32.h, st);
    return true;
  }
  // a band ray is traced by the FP64 pass (listed by classify_band_kernel)
  return setup_mixed(s, *px, *py, p, st);
}

// Global ray index of pixel (x, y): the inverse of ray_pixel.
__device__ __forceinline__ long long pixel_ray(const DevScene& s, int x, int y) {
  const long long tile = (long long)(y >> 2) * s.tiles_x + (x >> 3);
  return s.ray_begin + tile * 32 + ((y & 3) << 3) + (x & 7);
}

// Sort key of a band ray: a near-critical ray winds about -ln|eps| / (2 pi)
// times before it leaves, so its length grows with -log2 |eps|. Four keys per
// octave of |eps| below the band's edge; the last key takes the rest.
__device__ __forceinline__ int band_key(float eps, const LaunchParams& p) {
  const float ae = fmaxf(fabsf(eps) * p.band_key_scale, 1e-30f);
  return (int)fminf(float(kBandKeys - 1), fmaxf(0.f, -__log2f(ae) * 4.f));
}

// MIXED: lists the FP64-band rays (global ray indices) before the two passes.
// Each lane tests one 32-pixel row segment: b / M at the segment's centre
// (between pixels x0 + 15 and x0 + 16) is within 15.5 b_lip of every pixel's,
// so only segments whose centre lies within the pixels' prefilter + 15.5 b_lip
// (+ a rounding margin for the two FP32 evaluations) of b_c / M can hold a
// band ray. The warp then takes the pixels of each such segment together, one
// per lane: an FP32 b within the prefilter (class_band_for), then the exact
// band test the FP32 pass's setup also takes, so the listed rays are exactly
// the ones the FP32 pass leaves out. The band is a ring a few pixels wide:
// the rest of the frame costs one b per 32 pixels. The list has one slot per
// ray of the call.
__global__ void __launch_bounds__(256) classify_band_kernel(LaunchParams p) {
  const int lane = threadIdx.x & 31;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long warps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (int scene = blockIdx.y; scene < p.n_scenes; scene += gridDim.y) {
    const DevScene& s = p.scenes[scene];
    const int segs_x = (s.width + 31) >> 5;
    const long long n_segs = (long long)segs_x * s.height;
    const V3<float> F = BH_V(float, s, F), E0 = BH_V(float, s, E0);
    const V3<float> vy = BH_V(float, s, vy), vz = BH_V(float, s, vz);
    // the pixels' prefilter: class_band plus the scene's FP32 rounding term
    const float cband = p.class_band > 0.f ? p.class_band + 1e-6f * length(F) * s.inv_mass_f : 0.f;
    const float reach = cband + 15.5f * s.b_lip + 1e-5f * length(F) * s.inv_mass_f;
    for (long long base = warp * 32; base < n_segs; base += warps * 32) {
      const long long seg = base + lane;
      bool hit = false;
      if (seg < n_segs) {
        // 32-bit: a scene has at most 1024 x 32768 segments
        const unsigned y = unsigned(seg) / unsigned(segs_x);
        const int x0 = int(unsigned(seg) - y * unsigned(segs_x)) << 5;
        const V3<float> e = E0 + vy * (s.half_w_f - (float(x0) + 15.5f)) + vz * (s.half_h_f - float(y));
        const V3<float> fe = cross(F, e);
        const float bm = sqrtf(__fdividef(dot(fe, fe), dot(e, e))) * s.inv_mass_f;  // within ~3e-7 b
        hit = !(fabsf(bm - float(kBC)) > reach);  // NaN counts as a hit
      }
      for (unsigned hits = __ballot_sync(kFull, hit); hits; hits &= hits - 1u) {
        const unsigned hseg = unsigned(base) + unsigned(__ffs(hits) - 1);
        const int y = int(hseg / unsigned(segs_x));
        const int x = (int(hseg - unsigned(y) * unsigned(segs_x)) << 5) + lane;
        if (x >= s.width) continue;
        // b = |F x e| / |e| in FP32 (within ~1e-5 M of make_ray's, far inside
        // the 1e-3 M between this prefilter's edge and the FP32 pass's)
        const V3<float> e = E0 + vy * (s.half_w_f - float(x)) + vz * (s.half_h_f - float(y));
        const V3<float> fe = cross(F, e);
        const float bm = sqrtf(__fdividef(dot(fe, fe), dot(e, e))) * s.inv_mass_f;
        if (!(fabsf(bm - float(kBC)) < cband)) continue;
        const DF eps = eps_df(s, x, y);
        if (!in_band_eps(eps, p)) continue;
        const unsigned long long slot = atomicAdd(&p.counters->band_count, 1ull);
        if (slot < p.band_capacity) {
          const int key = band_key(eps.hi, p);
          p.band_tmp[slot] = (uint32_t)pixel_ray(s, x, y);
          p.band_key[slot] = (uint8_t)key;
          atomicAdd(&p.counters->band_hist[key], 1u);
        } else {
          atomicOr(&p.counters->flags, kFlagBandQueueFull);
        }
      }
    }
  }
}

// MIXED: writes the band list in key order, the longest rays (largest keys)
// first, so that each warp of the FP64 pass takes rays of about the same
// length (an FP64 warp instruction costs the same with 1 or 32 lanes active)
// and the longest chains start first. A counting sort: every block scans the
// histogram, then each entry takes the next slot of its key.
__global__ void __launch_bounds__(256) sort_band_kernel(LaunchParams p) {
  __shared__ unsigned base[kBandKeys];
  if (threadIdx.x == 0) {
    unsigned run = 0;
    for (int k = kBandKeys - 1; k >= 0; --k) {
      base[k] = run;
      run += p.counters->band_hist[k];
    }
  }
  __syncthreads();
  const unsigned long long n = min(p.counters->band_count, (unsigned long long)p.band_capacity);
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    const int k = p.band_key[i];
    p.band_list[base[k] + atomicAdd(&p.counters->band_cursor[k], 1u)] = p.band_tmp[i];
  }
}

// kPass: 0 = FP32 plain, 1 = FP32 mixed (band rays deferred), 2 = FP64 band.
template <int kPass>
__device__ __forceinline__ void persistent_body(const LaunchParams& p) {
  using R = typename std::conditional<kPass == 2, double, float>::type;
  const int lane = threadIdx.x & 31;
  const unsigned lt_mask = (1u << lane) - 1;
  Rk4Consts<R> c;
  if constexpr (kPass == 2) c = p.cband;
  else c = p.c32;
  const R h = c.h;
  const long long n_items =
      kPass == 2 ? (long long)min(*(volatile unsigned long long*)&p.counters->band_count,
                                  (unsigned long long)p.band_capacity)
                 : p.total_rays;
  unsigned long long* queue = kPass == 2 ? &p.counters->band_next : &p.counters->next_ray;
  RayState<R> st;
  st.status = kDone;
  int scene = 0, px = 0, py = 0;
  unsigned long long steps = 0, rays = 0;
  // The FP64 pass can leave lanes unused: FP64 issue is the bottleneck there,
  // and fewer band rays per warp spread them over more warps and SMs.
  const int chunk = kPass == 2 ? max(1, min(32, p.band_lanes)) : 32;
  const unsigned usable = chunk == 32 ? kFull : ((1u << chunk) - 1u);
  const int thr = max(1, min(chunk, p.refill_threshold));
  long long pend_base = 0;  // first item index of the pending chunk
  unsigned pend_mask = 0;   // its items not yet handed out
  int pend_scene = 0;
  long long scene_end = 0;  // first ray after pend_scene (FP32 pass)
  bool exhausted = false;

  for (;;) {
    unsigned idle = __ballot_sync(kFull, st.status == kDone) & usable;
    if (idle == usable && exhausted && pend_mask == 0) break;
    if (__popc(idle) >= thr || idle == usable) {
      // Hand out pending items until every lane is busy or work runs out. A
      // lane takes at most one item per refill: a lane whose item is deferred
      // (band ray, padding pixel) sits out the round. Handing it the next
      // item instead would leave the warp holding 31 items of one 8x4 tile
      // and one of a tile fetched anywhere, and every later refill of the
      // warp would mix two tiles (+27 % on the FP32 pass at 30 k band rays).
      unsigned given = 0;
      while (idle) {
        if (pend_mask == 0) {
          if (exhausted) break;
          unsigned long long t = 0;
          if (lane == 0) t = atomicAdd(queue, (unsigned long long)chunk);
          t = __shfl_sync(kFull, t, 0);
          if ((long long)t >= n_items) {
            exhausted = true;
            break;
          }
          pend_base = (long long)t;
          const long long left = n_items - pend_base;
          pend_mask = left >= chunk ? usable : ((1u << left) - 1u);
          if constexpr (kPass != 2) {
            // a warp's chunks come in increasing order: its scene stays or
            // moves forward, so step from the last one while the next scene
            // has begun (a search only after a long jump)
            if (pend_base >= scene_end) {
              int sc = pend_scene;
              if (lane == 0) {
                int hops = 0;
                while (sc + 1 < p.n_scenes && p.scenes[sc + 1].ray_begin <= pend_base && ++hops < 4) ++sc;
                if (sc + 1 < p.n_scenes && p.scenes[sc + 1].ray_begin <= pend_base) sc = find_scene(p, pend_base);
              }
              pend_scene = __shfl_sync(kFull, sc, 0);
              long long end = p.total_rays;
              if (lane == 0 && pend_scene + 1 < p.n_scenes) end = p.scenes[pend_scene + 1].ray_begin;
              scene_end = __shfl_sync(kFull, end, 0);
            }
          }
        }
        const int n = min(__popc(idle), __popc(pend_mask));
        const int rank = __popc(idle & lt_mask);
        if (((idle >> lane) & 1u) && rank < n) {
          const long long item = pend_base + (long long)__fns(pend_mask, 0, rank + 1);
          if constexpr (kPass == 2) {
            const long long ray = (long long)p.band_list[item];
            scene = find_scene(p, ray);
            const DevScene& s = p.scenes[scene];
            if (ray_pixel(s, ray - s.ray_begin, &px, &py)) {
              ++rays;
              init_rk4<R>(s, make_ray_rk4<R>(s, px, py), h, st);
            }
          } else {
            scene = pend_scene;
            if (take_fp32_ray<kPass == 1>(p, scene, item, st, &px, &py, &steps)) ++rays;
          }
        }
        // drop the n lowest items: keep the bits from the (n+1)-th set one up
        if (n > 0) {
          const unsigned next = __fns(pend_mask, 0, n + 1);  // 0xffffffff when fewer are set
          pend_mask = next > 31u ? 0u : pend_mask & ~((1u << next) - 1u);
        }
        given |= __ballot_sync(kFull, ((idle >> lane) & 1u) && rank < n);
        idle = __ballot_sync(kFull, st.status == kDone) & usable & ~given;
      }
    }
    // one store per finished ray: packing BGR8 tiles into words here (as the
    // GRID schedule does) measured 3.5 % slower on the 120-frame fly-through
    if (st.status != kDone) {
      const DevScene& s = p.scenes[scene];
      if constexpr (kPass == 2) steps += advance_band(s, st, c, p, p.slice_steps);
      else steps += advance_rk4<R, kPass == 1>(s, st, c, p.slice_steps);
      if (st.status != kRunning) {
        store_hit(s, p.format, px, py, finish_rk4<R, kPass == 1>(s, st, c));
        st.status = kDone;
      }
    }
  }
  // per-warp totals
  unsigned long long wsteps = steps, wrays = rays;
  for (int o = 16; o > 0; o >>= 1) {
    wsteps += __shfl_xor_sync(kFull, wsteps, o);
    wrays += __shfl_xor_sync(kFull, wrays, o);
  }
  if (lane == 0) {
    if (kPass == 2) {
      atomicAdd(&p.counters->band_steps, wsteps);
      atomicAdd(&p.counters->band_rays, wrays);
    }
    atomicAdd(&p.counters->steps, wsteps);
    atomicAdd(&p.counters->rays, wrays);
  }
}

__global__ void __launch_bounds__(256) persistent_plain_kernel(LaunchParams p) { persistent_body<0>(p); }

__global__ void __launch_bounds__(256, 4) persistent_mixed_kernel(LaunchParams p) { persistent_body<1>(p); }

// The FP64 band pass of the mixed tracer, on one block per SM. It is
// latency-bound: a few long near-critical rays set its length, which is about
// a third of the tracer's time when it runs after the FP32 pass. Run beside
// the FP32 pass from its start, the chains hide under the FP32 throughput
// work, at the cost of the issue slots its FP64 warps take. The block that
// begins last launches the FP32 pass: every band block is then resident, so
// the FP32 blocks fill the rest of each SM (and the ones that do not fit
// start as band blocks exit). The parent completes after its child, so
// stream order holds.
__global__ void __launch_bounds__(512) persistent_band_kernel(LaunchParams p) {
  if (p.mixed_blocks > 0 && threadIdx.x == 0 &&
      atomicAdd(&p.counters->blocks_started, 1ull) == (unsigned long long)gridDim.x - 1ull) {
    if (p.hybrid) {
      grid_kernel<BH_PRECISION_MIXED, BH_INTEGRATOR_RK4, true>
          <<<dim3(p.grid_dim[0], p.grid_dim[1], p.grid_dim[2]), dim3(p.block_dim[0], p.block_dim[1], 1), 0,
             cudaStreamFireAndForget>>>(p);
    } else {
      persistent_mixed_kernel<<<p.mixed_blocks, blockDim.x, 0, cudaStreamFireAndForget>>>(p);
    }
    if (cudaGetLastError() != cudaSuccess) atomicOr(&p.counters->flags, kFlagBandLaunchFailed);
  }
  persistent_body<2>(p);
}

// Grid of the band classification: scenes along y; along x, blocks of 256
// threads for about 8 of an average scene's 32-pixel row segments per thread
// (a grid-stride loop covers larger scenes). One thread per segment took ~30
// waves of short blocks on the 120-frame 1080p fly-through, ~0.1 ms of block
// scheduling before the FP32 pass could start.
dim3 classify_grid(const LaunchParams& q, int sms) {
  const long long per_scene = q.total_rays / 32 / std::max(1, q.n_scenes);
  const long long gx = (per_scene + 256 * 8 - 1) / (256 * 8);
  return dim3(unsigned(std::max(1ll, std::min<long long>(gx, 2ll * sms))), unsigned(std::min(q.n_scenes, 65535)));
}

// ---------------------------------------------------------------------------
// throughput probes (roofline denominators)
__global__ void fp32_probe_kernel(float* sink, int iters) {
  float a0 = threadIdx.x * 1e-7f, a1 = a0 + 1e-7f, a2 = a0 + 2e-7f, a3 = a0 + 3e-7f;
  float a4 = a0 + 4e-7f, a5 = a0 + 5e-7f, a6 = a0 + 6e-7f, a7 = a0 + 7e-7f;
  const float m = 0.999999f, k = 1e-7f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      a0 = fmaf(a0, m, k); a1 = fmaf(a1, m, k); a2 = fmaf(a2, m, k); a3 = fmaf(a3, m, k);
      a4 = fmaf(a4, m, k); a5 = fmaf(a5, m, k); a6 = fmaf(a6, m, k); a7 = fmaf(a7, m, k);
    }
  }
  const float r = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (r == 12345.f) sink[blockIdx.x] = r;
}

__global__ void fp64_probe_kernel(double* sink, int iters) {
  double a0 = threadIdx.x * 1e-7, a1 = a0 + 1e-7, a2 = a0 + 2e-7, a3 = a0 + 3e-7;
  const double m = 0.999999, k = 1e-7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      a0 = fma(a0, m, k); a1 = fma(a1, m, k); a2 = fma(a2, m, k); a3 = fma(a3, m, k);
    }
  }
  const double r = a0 + a1 + a2 + a3;
  if (r == 12345.0) sink[blockIdx.x] = r;
}

}  // namespace

// ---------------------------------------------------------------------------
// launchers
// The GRID / HYBRID launch's block count (the frames' blocks back to back, as
// assign_grid_blocks numbers them) and, when every frame has as many blocks,
// that number in q.frame_blocks.
static int64_t frame_block_layout(LaunchParams& q, const int32_t* scene_w, const int32_t* scene_h, int block_x,
                           int block_y) {
  int64_t blocks = 0, first = -1;
  bool uniform = true;
  for (int i = 0; i < q.n_scenes; ++i) {
    const int64_t b = grid_blocks(scene_w[i], scene_h[i], block_x, block_y, q.rays_per_thread);
    if (first < 0) first = b;
    uniform = uniform && b == first;
    blocks += b;
  }
  q.frame_blocks = uniform && first > 0 && first <= 0x7fffffff ? int32_t(first) : 0;
  return blocks;
}

cudaError_t launch_grid(const LaunchParams& p, const int32_t* scene_w, const int32_t* scene_h,
                        int block_x, int block_y, cudaStream_t stream, bool objects) {
  // the frames' blocks back to back (the records' block_begin, assign_grid_blocks)
  LaunchParams q = p;
  const int64_t blocks = frame_block_layout(q, scene_w, scene_h, block_x, block_y);
  if (blocks < 1 || blocks > 0x7fffffff) return cudaErrorInvalidConfiguration;
  const dim3 block(block_x, block_y, 1);
  const dim3 grid(unsigned(blocks), 1, 1);
  void (*kernel)(LaunchParams);
  const bool fp64 = p.precision == BH_PRECISION_FP64;
  if (!objects) {
    if (p.integrator == BH_INTEGRATOR_REF_TRAPEZOID) {
      kernel = fp64 ? grid_kernel<BH_PRECISION_FP64, BH_INTEGRATOR_REF_TRAPEZOID>
                    : grid_kernel<BH_PRECISION_FP32, BH_INTEGRATOR_REF_TRAPEZOID>;
    } else if (p.precision == BH_PRECISION_MIXED) {
      kernel = grid_kernel<BH_PRECISION_MIXED, BH_INTEGRATOR_RK4>;
    } else {
      kernel = fp64 ? grid_kernel<BH_PRECISION_FP64, BH_INTEGRATOR_RK4> : grid_kernel<BH_PRECISION_FP32, BH_INTEGRATOR_RK4>;
    }
    kernel<<<grid, block, 0, stream>>>(q);
    return cudaGetLastError();
  }
  switch (p.integrator) {
    case BH_INTEGRATOR_FLAT:
      kernel = fp64 ? grid_objects_kernel<double, BH_INTEGRATOR_FLAT> : grid_objects_kernel<float, BH_INTEGRATOR_FLAT>;
      break;
    case BH_INTEGRATOR_REF_TRAPEZOID:
      kernel = fp64 ? grid_objects_kernel<double, BH_INTEGRATOR_REF_TRAPEZOID>
                    : grid_objects_kernel<float, BH_INTEGRATOR_REF_TRAPEZOID>;
      break;
    case BH_INTEGRATOR_MULTI:
      kernel = fp64 ? grid_objects_kernel<double, BH_INTEGRATOR_MULTI> : grid_objects_kernel<float, BH_INTEGRATOR_MULTI>;
      break;
    default:
      kernel = fp64 ? grid_objects_kernel<double, BH_INTEGRATOR_RK4> : grid_objects_kernel<float, BH_INTEGRATOR_RK4>;
      break;
  }
  kernel<<<grid, block, 0, stream>>>(q);
  return cudaGetLastError();
}

cudaError_t launch_persistent(const LaunchParams& p, int threads, int blocks, cudaStream_t stream) {
  if (p.precision == BH_PRECISION_MIXED) {
    // Classification, the FP64 band pass (which launches the FP32 pass
    // itself, see persistent_band_kernel), then the FP32 pass once more from
    // the host: it finds the ray queue drained unless the device-side launch
    // failed.
    cudaError_t e;
    int dev = 0, sms = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    LaunchParams q = p;
    q.mixed_blocks = p.band_serial ? 0 : blocks;
    const int band_blocks = std::max(1, std::min(blocks, sms));
    classify_band_kernel<<<classify_grid(q, sms), 256, 0, stream>>>(q);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    sort_band_kernel<<<sms, 256, 0, stream>>>(q);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (p.band_serial == 1) {
      persistent_mixed_kernel<<<blocks, threads, 0, stream>>>(q);
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
      persistent_band_kernel<<<band_blocks, threads, 0, stream>>>(q);
      return cudaGetLastError();
    }
    persistent_band_kernel<<<band_blocks, threads, 0, stream>>>(q);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    persistent_mixed_kernel<<<blocks, threads, 0, stream>>>(q);
    return cudaGetLastError();
  }
  persistent_plain_kernel<<<blocks, threads, 0, stream>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_hybrid(const LaunchParams& p, const int32_t* scene_w, const int32_t* scene_h, int block_x,
                          int block_y, int band_threads, cudaStream_t stream) {
  if (p.precision != BH_PRECISION_MIXED) return launch_grid(p, scene_w, scene_h, block_x, block_y, stream);
  cudaError_t e;
  int dev = 0, sms = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  LaunchParams q = p;
  const int64_t blocks = frame_block_layout(q, scene_w, scene_h, block_x, block_y);
  if (blocks < 1 || blocks > 0x7fffffff) return cudaErrorInvalidConfiguration;
  q.hybrid = 1;
  q.grid_dim[0] = int32_t(blocks);
  q.grid_dim[1] = 1;
  q.grid_dim[2] = 1;
  q.block_dim[0] = block_x;
  q.block_dim[1] = block_y;
  q.mixed_blocks = p.band_serial ? 0 : 1;  // nonzero: the FP64 pass launches the FP32 pass
  q.drain_only = 0;
  const dim3 grid(q.grid_dim[0], q.grid_dim[1], q.grid_dim[2]), block(block_x, block_y, 1);
  classify_band_kernel<<<classify_grid(q, sms), 256, 0, stream>>>(q);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  sort_band_kernel<<<sms, 256, 0, stream>>>(q);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (p.band_serial == 1) {
    grid_kernel<BH_PRECISION_MIXED, BH_INTEGRATOR_RK4, true><<<grid, block, 0, stream>>>(q);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    persistent_band_kernel<<<sms, band_threads, 0, stream>>>(q);
    return cudaGetLastError();
  }
  persistent_band_kernel<<<sms, band_threads, 0, stream>>>(q);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  LaunchParams d = q;
  d.drain_only = 1;
  const dim3 drain(unsigned(std::min<int64_t>(blocks, int64_t(sms) * 8)));
  grid_kernel<BH_PRECISION_MIXED, BH_INTEGRATOR_RK4, true><<<drain, block, 0, stream>>>(d);
  return cudaGetLastError();
}

cudaError_t persistent_occupancy(const LaunchParams& p, int threads, int* blocks_per_sm) {
  if (p.precision == BH_PRECISION_MIXED)
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, persistent_mixed_kernel, threads, 0);
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, persistent_plain_kernel, threads, 0);
}

cudaError_t launch_fp32_probe(float* sink, int blocks, int threads, int iters, cudaStream_t stream) {
  fp32_probe_kernel<<<blocks, threads, 0, stream>>>(sink, iters);
  return cudaGetLastError();
}

cudaError_t launch_fp64_probe(double* sink, int blocks, int threads, int iters, cudaStream_t stream) {
  fp64_probe_kernel<<<blocks, threads, 0, stream>>>(sink, iters);
  return cudaGetLastError();
}

}  // namespace bhgb
