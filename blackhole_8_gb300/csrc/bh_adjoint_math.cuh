// Per-ray math of the differentiable render and its adjoint (reverse mode
// through the fixed-step RK4 integrator). Host + device: the kernels in
// bh_adjoint.cu instantiate it on the GPU; the host side only builds the
// per-scene records (build_adj_scene).
//
// The render (no counterpart in the reference, which has no gradients): the
// RK4 ray of the tracer -- REF ray generation (camera.h:55-59 as used at
// blackhole_solution_test.cc:167-170), plane reduction, u'' = -u + 3 u^2 in
// phi (u = M/r) -- with smooth shading so that an image loss has gradients:
// disc crossings composite front to back with a logistic edge opacity and a
// (radius, azimuth) texture; escaped rays read an equirectangular sky at the
// escape direction; both textures through a cubic B-spline filter.
//
// Adjoint. The parameters theta enter a ray only through its constants
//   K = (yv, xv, x0, w0, phi0, d0)  (plane basis, initial state, initial
//        phase, phase of the first disc-plane crossing)
// and through M, r_in, r_out and the disc's polar axis e2 at events. The ODE
// itself has no parameter. The backward pass propagates the adjoint of the
// state (x, w) from the last event to step 0 by the transposed Jacobian of
// each RK4 step, adding the adjoint of every crossing and of the escape, and
// collects dL/dK; the gradient is then sum_K dL/dK . dK/dtheta_i with dK/dtheta
// from forward-mode tangents of the ray setup (one dual number per
// parameter), seeded with per-scene tangents computed on the host.
//
// Checkpointing. The forward pass stores the trajectory state every
// kSeg = 64 steps (global memory, one slot per ray). Backwards, each 64-step
// segment is re-run from its checkpoint storing 8 sub-checkpoints (shared
// memory), and each 8-step piece is re-run into registers and reversed.
// Memory per ray: ceil(steps / 64) checkpoints of 24 (FP32) or 48 (FP64)
// bytes; work: about 3 forward passes plus one reverse pass.
//
// Precision. FP64: everything double. FP32: everything float. MIXED: ray
// setup and every phase (first-crossing phase d0 + j pi, escape phase) in
// double; the integration in float with compensated (2Sum) state updates
// started from the FP64 initial state (its low parts seed the compensation)
// and RK4 constants whose first-order coefficients are exact floats; rays
// near the critical impact parameter go to the FP64 path.
#pragma once

#include <math.h>
#include <stdint.h>

#include <cmath>

#include "bh_df.cuh"
#include "bh_internal.h"

#if defined(__CUDACC__)
#define BHA_HD __host__ __device__ __forceinline__
#define BHA_NOINLINE __host__ __device__ __noinline__
#else
#define BHA_HD inline
#define BHA_NOINLINE
#endif

namespace bhgb {
namespace adj {

// the scalar overloads stay visible beside the dual-number ones below
using ::asin;
using ::atan2;
using ::cos;
using ::exp;
using ::floor;
using ::fma;
using ::sin;
using ::sqrt;

constexpr int kParams = BH_GRAD_COUNT;
constexpr int kSeg = 64;  // steps per checkpoint
constexpr int kSub = 8;   // steps per sub-checkpoint
constexpr double kPiD = 3.14159265358979323846;
constexpr double kTwoPiD = 6.28318530717958647692;

// ---------------------------------------------------------------------------
// per-scene record (host-built)
struct AdjScene {
  // primal, about the hole: E0 = camera position - focus * vx (REF ray
  // generation), F = camera position - hole, n the disc normal, e1, e2 its
  // polar basis (e2 = unit(n x e1))
  double E0[3], vy[3], vz[3], F[3], n[3], e1[3], e2[3];
  double mass, r_in, r_out, half_w, half_h, wsoft;
  // d/dtheta_i of the vectors above (e1 does not depend on theta)
  double dE0[kParams][3], dvy[kParams][3], dvz[kParams][3], dF[kParams][3], dn[kParams][3], de2[kParams][3];
  // float copies
  float E0_f[3], vy_f[3], vz_f[3], F_f[3], n_f[3], e1_f[3], e2_f[3];
  float mass_f, r_in_f, r_out_f, half_w_f, half_h_f, wsoft_f;
  float dE0_f[kParams][3], dvy_f[kParams][3], dvz_f[kParams][3], dF_f[kParams][3], dn_f[kParams][3],
      de2_f[kParams][3];
  DevTexture disc_tex, bg_tex;
  int32_t width, height, tiles_x, disc_on, has_bg, scene;
  int32_t tex32;        // MIXED: FP64 colours take the texture filter in FP32 (tex_sample_at)
  int32_t pad_;
  int64_t block_begin;  // first block of this scene in the grid
  int64_t ray_begin;    // first ray of this scene (row-major pixels, scenes back to back)
  const float* target;
  float* image;
  float* pixel_grad;
};

struct AdjParams {
  Rk4Consts<float> c32;
  Rk4Consts<double> c64;
  double inv_h32;    // 1 / step as the FP32 and FP64 integrations take it
  double inv_h64;
  double hstep32;    // the step the FP32 / FP64 trajectories take (phases)
  double hstep64;
  float df_c[2 * 8]; // double-float split (hi, lo) of c64: h, hh, q, q2, h26, h6, x_esc, x_hor
  double softness;
  double band;       // MIXED: |b/M - 3 sqrt 3| < band goes to FP64
  int32_t kmax;
  int32_t want_grad;
};

// ---------------------------------------------------------------------------
// small algebra
template <typename R>
struct V3 {
  R x, y, z;
};
template <typename R>
BHA_HD V3<R> operator+(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <typename R>
BHA_HD V3<R> operator-(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <typename R, typename S>
BHA_HD V3<R> operator*(V3<R> a, S s) { return {a.x * s, a.y * s, a.z * s}; }
template <typename R>
BHA_HD R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename R>
BHA_HD V3<R> cross(V3<R> a, V3<R> b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <typename R, typename S>
BHA_HD V3<R> cast3(V3<S> a) { return {R(a.x), R(a.y), R(a.z)}; }
template <typename R>
BHA_HD V3<R> load3(const double* d) { return {R(d[0]), R(d[1]), R(d[2])}; }
BHA_HD V3<float> load3f(const float* f) { return {f[0], f[1], f[2]}; }

// value with one tangent (forward mode)
template <typename R>
struct D1 {
  R v, d;
  BHA_HD D1() : v(0), d(0) {}
  BHA_HD D1(R x) : v(x), d(0) {}
  BHA_HD D1(R x, R dx) : v(x), d(dx) {}
};
template <typename R>
BHA_HD D1<R> operator+(D1<R> a, D1<R> b) { return {a.v + b.v, a.d + b.d}; }
template <typename R>
BHA_HD D1<R> operator-(D1<R> a, D1<R> b) { return {a.v - b.v, a.d - b.d}; }
template <typename R>
BHA_HD D1<R> operator-(D1<R> a) { return {-a.v, -a.d}; }
template <typename R>
BHA_HD D1<R> operator*(D1<R> a, D1<R> b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
template <typename R>
BHA_HD D1<R> operator/(D1<R> a, D1<R> b) {
  const R q = a.v / b.v;
  return {q, (a.d - q * b.d) / b.v};
}
template <typename R>
BHA_HD D1<R> sqrt(D1<R> a) {
  const R s = sqrt(a.v);
  return {s, a.d * (R(0.5) / s)};
}
template <typename R>
BHA_HD D1<R> atan2(D1<R> y, D1<R> x) {
  return {R(atan2(y.v, x.v)), (x.v * y.d - y.v * x.d) / (x.v * x.v + y.v * y.v)};
}
template <typename R>
BHA_HD R val(D1<R> a) { return a.v; }
BHA_HD float val(float a) { return a; }
BHA_HD double val(double a) { return a; }

// ---------------------------------------------------------------------------
// ray setup: the reference's ray reduced to its orbital plane.
//   e = E0 + a vy + c vz (a = W/2 - x, c = H/2 - y); yv = e/|e|
//   zv = (F x yv)/b, b = |F x yv|; xv = yv x zv; position = r (cos phi yv + sin phi xv)
//   u0 = M/|F|, phi0 = atan2(b, yv.F), w0 = du/dphi = sign(yv.F) sqrt(1/(b/M)^2 - u0^2 (1 - 2 u0))
//   d0: phase after phi0 of the first disc-plane crossing, in (0, pi]
template <typename T>
struct RayInit {
  V3<T> yv, xv;
  T x0, w0, phi0, d0, bm;
};

template <typename T>
BHA_HD RayInit<T> ray_init(V3<T> E0, V3<T> vy, V3<T> vz, V3<T> F, V3<T> n, T M, T a, T c) {
  const V3<T> e = E0 + vy * a + vz * c;
  const V3<T> yv = e * (T(1.0) / sqrt(dot(e, e)));
  const V3<T> cz = cross(F, yv);
  const T b = sqrt(dot(cz, cz));
  const V3<T> zv = cz * (T(1.0) / b);
  RayInit<T> r;
  r.yv = yv;
  r.xv = cross(yv, zv);
  const T F1 = dot(yv, F);
  const T u0 = M / sqrt(dot(F, F));
  r.bm = b / M;
  r.phi0 = atan2(b, F1);
  T w = sqrt(T(1.0) / (r.bm * r.bm) - u0 * u0 * (T(1.0) - T(2.0) * u0));
  if (val(F1) < 0) w = -w;
  r.w0 = w;
  r.x0 = u0 - T(1.0 / 3.0);
  const T A = dot(n, yv), B = dot(n, r.xv);
  T d = atan2(B, A) + T(kPiD / 2) - r.phi0;
  d = d - T(kPiD * floor(double(val(d)) / kPiD));
  if (val(d) <= 0) d = d + T(kPiD);
  r.d0 = d;
  return r;
}

// ---------------------------------------------------------------------------
// RK4 on x = u - 1/3 (x'' = x + 3 x^2), Runge-Kutta-Nystrom form of the
// classical method (the same trajectory as the render kernels).
template <typename R>
BHA_HD R fx(R x) { return x * fma(R(3), x, R(1)); }
template <typename R>
BHA_HD R dfx(R x) { return fma(R(6), x, R(1)); }

template <typename R>
struct Traj {
  R x, w;    // state
  R cx, cw;  // compensation (low parts lost by the state updates), MIXED
};

// 2Sum (Knuth): s + e == a + b exactly.
#if !defined(__CUDA_ARCH__)
template <typename R>
inline R rn_round(volatile R v) { return v; }
template <typename R>
BHA_HD R rn_add(R a, R b) { return rn_round<R>(a + b); }
template <typename R>
BHA_HD R rn_sub(R a, R b) { return rn_round<R>(a - b); }
#else
template <typename R>
BHA_HD R rn_add(R a, R b) { return a + b; }
template <typename R>
BHA_HD R rn_sub(R a, R b) { return a - b; }
#endif
#if defined(__CUDA_ARCH__)
template <>
BHA_HD float rn_add<float>(float a, float b) { return __fadd_rn(a, b); }
template <>
BHA_HD float rn_sub<float>(float a, float b) { return __fsub_rn(a, b); }
template <>
BHA_HD double rn_add<double>(double a, double b) { return __dadd_rn(a, b); }
template <>
BHA_HD double rn_sub<double>(double a, double b) { return __dsub_rn(a, b); }
#endif
// (rounded separately: a product fused into these sums would break them)
template <typename R>
BHA_HD void two_sum_acc(R& a, R b, R& e) {
  const R y = rn_add(b, e);
  const R s = rn_add(a, y);
  const R bb = rn_sub(s, a);
  e = rn_add(rn_sub(a, rn_sub(s, bb)), rn_sub(y, bb));
  a = s;
}

template <typename R, bool kComp>
BHA_HD void step(Traj<R>& s, const Rk4Consts<R>& c) {
  const R k1 = fx(s.x);
  const R s1 = fma(c.hh, s.w, s.x);
  const R k2 = fx(s1);
  const R s2 = fma(c.q, k1, s1);
  const R k3 = fx(s2);
  const R s3a = fma(c.h, s.w, s.x);
  const R s3 = fma(c.q2, k2, s3a);
  const R k4 = fx(s3);
  const R A = k2 + k3;
  const R S = A + k1;
  if (kComp) {
    const R dx = fma(c.h26, S, c.h * s.w);
    const R dw = c.h6 * ((S + A) + k4);
    two_sum_acc(s.x, dx, s.cx);
    two_sum_acc(s.w, dw, s.cw);
  } else {
    s.x = fma(c.h26, S, s3a);
    s.w = fma(c.h6, (S + A) + k4, s.w);
  }
}

// RK4 step of length h (the partial step to a disc-plane crossing).
template <typename R>
BHA_HD void step_h(R& x, R& w, R h) {
  const R hh = h * R(0.5), q = h * h * R(0.25), q2 = h * h * R(0.5), h26 = h * h * R(1.0 / 6.0),
          h6 = h * R(1.0 / 6.0);
  const R k1 = fx(x);
  const R s1 = fma(hh, w, x);
  const R k2 = fx(s1);
  const R s2 = fma(q, k1, s1);
  const R k3 = fx(s2);
  const R s3a = fma(h, w, x);
  const R s3 = fma(q2, k2, s3a);
  const R k4 = fx(s3);
  const R A = k2 + k3;
  const R S = A + k1;
  x = fma(h26, S, s3a);
  w = fma(h6, (S + A) + k4, w);
}

// Transposed Jacobian of one step: (lx, lw) = adjoint of the state after the
// step -> adjoint of the state (x, w) before it.
template <typename R>
BHA_HD void step_vjp(R x, R w, const Rk4Consts<R>& c, R& lx, R& lw) {
  const R a1 = fx(x);
  const R x2 = fma(c.hh, w, x);
  const R a2 = fx(x2);
  const R x3 = fma(c.q, a1, x2);
  const R s3a = fma(c.h, w, x);
  const R x4 = fma(c.q2, a2, s3a);
  const R S3b = c.h26 * lx;  // adjoint of a1 + a2 + a3
  const R S4b = c.h6 * lw;   // adjoint of a1 + 2 a2 + 2 a3 + a4
  const R a3b = fma(R(2), S4b, S3b);
  const R x4b = S4b * dfx(x4);
  const R a2b = fma(c.q2, x4b, a3b);
  const R x3b = a3b * dfx(x3);
  const R a1b = fma(c.q, x3b, S3b + S4b);
  const R x2b = fma(a2b, dfx(x2), x3b);
  const R s3ab = lx + x4b;
  const R nlx = fma(a1b, dfx(x), s3ab + x2b);
  const R nlw = fma(c.h, s3ab, fma(c.hh, x2b, lw));
  lx = nlx;
  lw = nlw;
}

// step_vjp with the update of the adjoint written as lambda + delta and
// accumulated with 2Sum (compensation terms clx, clw): the reverse pass of a
// near-critical ray crosses the same unstable saddle as the forward pass, so
// plain FP32 accumulation of lambda loses ~1e-3 there.
template <typename R>
BHA_HD void step_vjp_comp(R x, R w, const Rk4Consts<R>& c, R& lx, R& lw, R& clx, R& clw) {
  const R a1 = fx(x);
  const R x2 = fma(c.hh, w, x);
  const R a2 = fx(x2);
  const R x3 = fma(c.q, a1, x2);
  const R s3a = fma(c.h, w, x);
  const R x4 = fma(c.q2, a2, s3a);
  const R S3b = c.h26 * lx;
  const R S4b = c.h6 * lw;
  const R a3b = fma(R(2), S4b, S3b);
  const R x4b = S4b * dfx(x4);
  const R a2b = fma(c.q2, x4b, a3b);
  const R x3b = a3b * dfx(x3);
  const R a1b = fma(c.q, x3b, S3b + S4b);
  const R x2b = fma(a2b, dfx(x2), x3b);
  const R dlx = fma(a1b, dfx(x), x4b + x2b);
  const R dlw = fma(c.h, lx + x4b, c.hh * x2b);
  two_sum_acc(lx, dlx, clx);
  two_sum_acc(lw, dlw, clw);
}

// The same for a step of length h, with the adjoint of h.
template <typename R>
BHA_HD void step_h_vjp(R x, R w, R h, R lxo, R lwo, R& lx, R& lw, R& lh) {
  const R hh = h * R(0.5), q = h * h * R(0.25), q2 = h * h * R(0.5), h26 = h * h * R(1.0 / 6.0),
          h6 = h * R(1.0 / 6.0);
  const R a1 = fx(x);
  const R x2 = fma(hh, w, x);
  const R a2 = fx(x2);
  const R x3 = fma(q, a1, x2);
  const R a3 = fx(x3);
  const R x4 = fma(q2, a2, fma(h, w, x));
  const R a4 = fx(x4);
  const R S3 = a1 + a2 + a3;
  const R S4 = a1 + R(2) * (a2 + a3) + a4;
  R xb = lxo, wb = lwo;
  R hb = lxo * (w + h * R(1.0 / 3.0) * S3) + lwo * S4 * R(1.0 / 6.0);
  wb += h * lxo;
  const R S3b = h26 * lxo, S4b = h6 * lwo;
  R a1b = S3b + S4b;
  R a2b = S3b + R(2) * S4b;
  const R a3b = a2b;
  const R x4b = S4b * dfx(x4);
  xb += x4b;
  wb += h * x4b;
  hb += x4b * (w + h * a2);
  a2b += q2 * x4b;
  const R x3b = a3b * dfx(x3);
  a1b += q * x3b;
  hb += x3b * hh * a1;
  const R x2b = x3b + a2b * dfx(x2);
  xb += x2b;
  wb += hh * x2b;
  hb += x2b * w * R(0.5);
  xb += a1b * dfx(x);
  lx = xb;
  lw = wb;
  lh = hb;
}

// ---------------------------------------------------------------------------
// textures: uniform cubic B-spline filter (C2, so the loss is smooth across
// texel edges), texel centres at integers, RGB = BGRA8 / 255; a non-wrapping
// axis repeats its edge texel.
BHA_HD uchar4 fetch(const DevTexture& t, int i, int j) {
#if defined(__CUDA_ARCH__)
  return __ldg(t.texels + (size_t)j * t.width + i);
#else
  return t.texels[(size_t)j * t.width + i];
#endif
}

BHA_HD int tex_index(int i, int n, bool wrap) {
  if (wrap) {
    i %= n;
    return i < 0 ? i + n : i;
  }
  return i < 0 ? 0 : (i >= n ? n - 1 : i);
}

// weights of the texels at floor - 1 .. floor + 2 and their derivatives in f
template <typename R>
BHA_HD void bspline_weights(R f, R w[4], R dw[4]) {
  const R g = R(1) - f, f2 = f * f, f3 = f2 * f;
  w[0] = g * g * g * R(1.0 / 6.0);
  w[1] = (R(3) * f3 - R(6) * f2 + R(4)) * R(1.0 / 6.0);
  w[2] = (R(-3) * f3 + R(3) * f2 + R(3) * f + R(1)) * R(1.0 / 6.0);
  w[3] = f3 * R(1.0 / 6.0);
  dw[0] = -g * g * R(0.5);
  dw[1] = (R(3) * f2 - R(4) * f) * R(0.5);
  dw[2] = (R(-3) * f2 + R(2) * f + R(1)) * R(0.5);
  dw[3] = f2 * R(0.5);
}

// Colour and its derivatives in s (columns) and u (rows) at cell (cs, cu)
// with fractions (fs, fu) in [0, 1).
template <typename R>
BHA_HD void tex_sample_cell(const DevTexture& t, int cs, int cu, R fs, R fu, bool wrap_s, bool wrap_u, R col[3],
                            R dcs[3], R dcu[3]) {
  R ws[4], dws[4], wu[4], dwu[4];
  bspline_weights(fs, ws, dws);
  bspline_weights(fu, wu, dwu);
  const int bs = cs - 1, bu = cu - 1;
  int is[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) is[k] = tex_index(bs + k, t.width, wrap_s);
  const R kq = R(1.0 / 255.0);
#pragma unroll
  for (int ch = 0; ch < 3; ++ch) col[ch] = dcs[ch] = dcu[ch] = R(0);
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int ju = tex_index(bu + j, t.height, wrap_u);
    R row[3] = {R(0), R(0), R(0)}, rowd[3] = {R(0), R(0), R(0)};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const uchar4 q = fetch(t, is[k], ju);
      const R c3[3] = {R(q.z) * kq, R(q.y) * kq, R(q.x) * kq};
#pragma unroll
      for (int ch = 0; ch < 3; ++ch) {
        row[ch] = fma(ws[k], c3[ch], row[ch]);
        rowd[ch] = fma(dws[k], c3[ch], rowd[ch]);
      }
    }
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
      col[ch] = fma(wu[j], row[ch], col[ch]);
      dcs[ch] = fma(wu[j], rowd[ch], dcs[ch]);
      dcu[ch] = fma(dwu[j], row[ch], dcu[ch]);
    }
  }
}

// Colour and its derivatives in s (columns) and u (rows).
template <typename R>
BHA_HD void tex_sample(const DevTexture& t, R s, R u, bool wrap_s, bool wrap_u, R col[3], R dcs[3], R dcu[3]) {
  const R fs0 = floor(s), fu0 = floor(u);
  tex_sample_cell(t, int(fs0), int(fu0), s - fs0, u - fu0, wrap_s, wrap_u, col, dcs, dcu);
}

// The texture filter of a colour in precision R. With s.tex32 (MIXED) an
// FP64 colour takes the sample point in FP64 -- the cell and the fraction
// exactly, the fraction then rounded to FP32 (~6e-8 texel) -- and the
// B-spline weights and texel sums in FP32 (~1e-7 of the colour): an FP64
// filter costs ~250 FP64 operations per sample, the largest FP64 load of the
// band rays' crossings. The FP64 mode keeps it in FP64.
template <typename S, typename R>
BHA_HD void tex_sample_at(const S& s, const DevTexture& t, R a, R b, bool wrap_s, bool wrap_u, R col[3], R dcs[3],
                          R dcu[3]) {
  if (sizeof(R) == sizeof(double) && s.tex32) {
    const R fa = floor(a), fb = floor(b);
    float c[3], da[3], db[3];
    tex_sample_cell<float>(t, int(fa), int(fb), float(a - fa), float(b - fb), wrap_s, wrap_u, c, da, db);
    for (int ch = 0; ch < 3; ++ch) {
      col[ch] = R(c[ch]);
      dcs[ch] = R(da[ch]);
      dcu[ch] = R(db[ch]);
    }
    return;
  }
  tex_sample(t, a, b, wrap_s, wrap_u, col, dcs, dcu);
}

template <typename R>
BHA_HD R logistic(R z) { return R(1) / (R(1) + exp(-z)); }

// ---------------------------------------------------------------------------
// per-ray constants in the working precisions: R for the state and geometry,
// P for phases
template <typename R, typename P>
struct RayC {
  V3<R> yv, xv;
  R x0, w0;
  R x0lo, w0lo;  // MIXED: the FP64 initial state's parts below FP32 rounding
  P phi0, d0;
  R M, r_in, r_out, wsoft;
};

// Trajectory checkpoint: the state, the transmittance and the count m of
// disc-plane crossings passed (the next one is at phase d0 + m pi); the
// compensation terms only where the integration carries them.
template <typename R, bool kComp>
struct Ckpt {
  R x, w, trans, cx, cw;
  int32_t m;
  BHA_HD static Ckpt make(const Traj<R>& t, R tr, int mm) { return Ckpt{t.x, t.w, tr, t.cx, t.cw, mm}; }
  BHA_HD Traj<R> traj() const { return Traj<R>{x, w, cx, cw}; }
};
template <typename R>
struct Ckpt<R, false> {
  R x, w, trans;
  int32_t m;
  BHA_HD static Ckpt make(const Traj<R>& t, R tr, int mm) { return Ckpt{t.x, t.w, tr, mm}; }
  BHA_HD Traj<R> traj() const { return Traj<R>{x, w, R(0), R(0)}; }
};

// forward record of one ray
template <typename R>
struct Fwd {
  R rgb[3];
  R trans;   // transmittance at the end
  R xa, wa, xb, wb;  // MISS: the states around the escape
  int32_t cls, k_end;
  int32_t m_end;     // disc-plane crossing phases reached (DISC: index of the last)
};

// adjoints collected by the backward pass
template <typename R>
struct Acc {
  V3<R> yv, xv, e2;
  R phi0, d0, M, r_in, r_out;
};

// FP32 constants of the RK4 step whose first-order coefficients are exact:
// h/6 is kept to 21 significant bits so that h = 6 (h/6) and h/2 = 3 (h/6)
// are exact floats. Rounding h, h/2 and h/6 independently makes the x and w
// updates take slightly different steps (a relative 1e-8 first-order
// inconsistency), a systematic error that the unstable photon orbit
// amplifies. The step actually taken, 6 (h/6), differs from the requested
// one by a relative 1e-7; phases use it (see crossing_step).
inline Rk4Consts<float> exact_rk4_consts_f32(double h, double u_escape, int kmax) {
  Rk4Consts<float> c = make_rk4_consts<float>(h, u_escape, kmax);
  int ex = 0;
  const double m = std::frexp(double(float(h / 6.0)), &ex);
  const float h6 = float(std::ldexp(std::nearbyint(std::ldexp(m, 21)), ex - 21));
  c.h6 = h6;
  c.h = 6.0f * h6;
  c.hh = 3.0f * h6;
  c.h26 = c.h * h6;
  c.q = c.hh * c.hh;
  c.q2 = 2.0f * c.q;
  return c;
}

template <typename R>
BHA_HD const Rk4Consts<R>& consts(const AdjParams& p);
template <>
BHA_HD const Rk4Consts<float>& consts<float>(const AdjParams& p) { return p.c32; }
template <>
BHA_HD const Rk4Consts<double>& consts<double>(const AdjParams& p) { return p.c64; }

// Index of the step whose state starts the partial step to phase dm.
template <typename R, typename P>
BHA_HD int crossing_step(P dm, const AdjParams& p) {
  return int(floor(dm * P(sizeof(R) == sizeof(float) ? p.inv_h32 : p.inv_h64)));
}

template <typename R>
BHA_HD double phase_step(const AdjParams& p) { return sizeof(R) == sizeof(float) ? p.hstep32 : p.hstep64; }

template <typename P>
BHA_HD P reduce_2pi(P a) { return a - P(kTwoPiD) * floor(a * P(1.0 / kTwoPiD)); }

// Disc-plane crossing at phase dm (after phi0), from the state at step kc.
// Returns false for a crossing inside the horizon. Every other crossing is
// composited: far from the annulus the logistic opacity is already
// negligible, and a cut-off there would put a jump in the gradient of
// near-critical rays.
template <typename R, typename P>
struct Crossing {
  R x, w, delta;    // state at step kc, partial step
  R uc, Rr, z1, z2, s1, s2, alpha;
  R cs, sn;         // cos, sin of the crossing phase
  V3<R> ph;         // crossing direction
  R X1, Y1;         // ph . e1, ph . e2
  R tc_s, tc_u;     // texture coordinates
};

template <typename R, typename P>
BHA_HD bool crossing_eval(const AdjScene& s, const AdjParams& p, const RayC<R, P>& rc, R x, R w, P dm, int kc,
                          Crossing<R, P>& c) {
  c.x = x;
  c.w = w;
  c.delta = R(dm - P(kc) * P(phase_step<R>(p)));
  R xc = x, wc = w;
  step_h(xc, wc, c.delta);
  c.uc = xc + R(1.0 / 3.0);
  if (!(c.uc < R(0.5))) return false;
  c.Rr = rc.M / c.uc;
  c.z1 = (c.Rr - rc.r_in) / rc.wsoft;
  c.z2 = (rc.r_out - c.Rr) / rc.wsoft;
  c.s1 = logistic(c.z1);
  c.s2 = logistic(c.z2);
  c.alpha = c.s1 * c.s2;
  return true;
}

template <typename R, typename P, typename Pick>
BHA_HD void crossing_colour(const AdjScene& s, const RayC<R, P>& rc, P dm, Crossing<R, P>& c, R col[3], R dcs[3],
                            R dcu[3]) {
  const R phic = R(reduce_2pi(rc.phi0 + dm));
  c.cs = cos(phic);
  c.sn = sin(phic);
  c.ph = rc.yv * c.cs + rc.xv * c.sn;
  c.X1 = dot(Pick::v(s.e1, s.e1_f), c.ph);
  c.Y1 = dot(Pick::v(s.e2, s.e2_f), c.ph);
  const R az = atan2(c.Y1, c.X1);
  c.tc_s = (c.Rr - rc.r_in) / (rc.r_out - rc.r_in) * R(s.disc_tex.width) - R(0.5);
  c.tc_u = az * R(s.disc_tex.height / kTwoPiD) - R(0.5);
  tex_sample_at(s, s.disc_tex, c.tc_s, c.tc_u, false, true, col, dcs, dcu);
}

// Field access by precision.
template <typename R>
struct PickA;
template <>
struct PickA<float> {
  static BHA_HD V3<float> v(const double*, const float* f) { return {f[0], f[1], f[2]}; }
};
template <>
struct PickA<double> {
  static BHA_HD V3<double> v(const double* d, const float*) { return {d[0], d[1], d[2]}; }
};

// Cubic Hermite on [0, 1] between (pa, ma) and (pb, mb): value, first and
// second derivative in t, and the basis values.
template <typename R>
struct Herm {
  R p, dp, ddp;
  R h00, h10, h01, h11;      // basis
  R d00, d10, d01, d11;      // basis derivatives
};
template <typename R>
BHA_HD Herm<R> hermite(R pa, R ma, R pb, R mb, R t) {
  Herm<R> h;
  const R t2 = t * t, t3 = t2 * t;
  h.h00 = R(2) * t3 - R(3) * t2 + R(1);
  h.h10 = t3 - R(2) * t2 + t;
  h.h01 = R(3) * t2 - R(2) * t3;
  h.h11 = t3 - t2;
  h.d00 = R(6) * t2 - R(6) * t;
  h.d10 = R(3) * t2 - R(4) * t + R(1);
  h.d01 = R(6) * t - R(6) * t2;
  h.d11 = R(3) * t2 - R(2) * t;
  h.p = h.h00 * pa + h.h10 * ma + h.h01 * pb + h.h11 * mb;
  h.dp = h.d00 * pa + h.d10 * ma + h.d01 * pb + h.d11 * mb;
  h.ddp = (R(12) * t - R(6)) * pa + (R(6) * t - R(4)) * ma + (R(6) - R(12) * t) * pb + (R(6) * t - R(2)) * mb;
  return h;
}

// Escape between the states a (step k_end - 1) and b (step k_end): the
// crossing of u = u_esc by the Hermite interpolant (Newton, 8 iterations),
// the escape direction and the sky colour.
template <typename R, typename P>
struct Escape {
  R t, we, psi_c, psi_s;
  Herm<R> hm;
  V3<R> dir;
  R lon, lat, zc;
  R ts, tu;
};

template <typename R, typename P>
BHA_HD void escape_eval(const AdjScene& s, const AdjParams& p, const RayC<R, P>& rc, R xa, R wa, R xb, R wb, int ka,
                        Escape<R, P>& e, R col[3], R dcs[3], R dcu[3]) {
  const Rk4Consts<R>& c = consts<R>(p);
  const R xe = c.x_esc;
  R t = (xa - xe) / (xa - xb);
  for (int i = 0; i < 8; ++i) {
    const Herm<R> h = hermite(xa, c.h * wa, xb, c.h * wb, t);
    t = t - (h.p - xe) / h.dp;
  }
  e.t = t;
  e.hm = hermite(xa, c.h * wa, xb, c.h * wb, t);
  e.we = e.hm.dp / c.h;
  const R psi = R(reduce_2pi(rc.phi0 + P(ka) * P(phase_step<R>(p)))) + t * c.h + atan2(c.u_esc, -e.we);
  e.psi_c = cos(psi);
  e.psi_s = sin(psi);
  e.dir = rc.yv * e.psi_c + rc.xv * e.psi_s;
  e.lon = atan2(e.dir.y, e.dir.x);
  e.zc = e.dir.z > R(1) ? R(1) : (e.dir.z < R(-1) ? R(-1) : e.dir.z);
  e.lat = asin(e.zc);
  const int W = s.bg_tex.width, H = s.bg_tex.height;
  e.ts = (e.lon + R(kPiD)) * R(W / kTwoPiD) - R(0.5);
  e.tu = (R(kPiD / 2) - e.lat) * R(H / kPiD) - R(0.5);
  tex_sample_at(s, s.bg_tex, e.ts, e.tu, true, false, col, dcs, dcu);
}

// ---------------------------------------------------------------------------
// forward pass: colour, class and (want_grad) the checkpoints
// Stored trajectory state of the FP64 band pass.
template <typename R>
struct Vec2T;
template <>
struct Vec2T<float> {
  using type = float2;
};
template <>
struct Vec2T<double> {
  using type = double2;
};
template <typename R>
BHA_HD typename Vec2T<R>::type make_v2(double x, double w) {
  return typename Vec2T<R>::type{R(x), R(w)};
}

// forward pass: colour, class and (want_grad) the checkpoints. With kStore
// every state is also kept, rounded to float, in traj[k * stride] and the
// transmittance before crossing m in cross_t[m * stride] (the FP64 band pass,
// whose reverse pass runs in FP32 over the stored states).
template <typename R, typename P, bool kComp, bool kStore = false, typename TS = float>
BHA_HD void forward(const AdjScene& s, const AdjParams& p, const RayC<R, P>& rc, Ckpt<R, kComp>* ck,
                    int64_t ck_stride, Fwd<R>& f, typename Vec2T<TS>::type* traj = nullptr, float* cross_t = nullptr,
                    int64_t store_stride = 0, int max_cross = 0, double2* cross_xw = nullptr) {
  const Rk4Consts<R>& c = consts<R>(p);
  Traj<R> st{rc.x0, rc.w0, kComp ? rc.x0lo : R(0), kComp ? rc.w0lo : R(0)};
  R trans = R(1);
  R acc[3] = {R(0), R(0), R(0)};
  int m = 0;
  P dm = rc.d0;
  int kc = s.disc_on ? crossing_step<R, P>(dm, p) : -1;
  int k = 0;
  f.cls = BH_CLASS_MAXSTEPS;
  for (; k < p.kmax; ++k) {
    if (ck && (k & (kSeg - 1)) == 0) ck[(k / kSeg) * ck_stride] = Ckpt<R, kComp>::make(st, trans, m);
    if (kStore && traj) traj[(int64_t)k * store_stride] = make_v2<TS>(double(st.x), double(st.w));
    if (k == kc) {
      if (kStore && traj && m < max_cross) {
        cross_t[(int64_t)m * store_stride] = float(trans);
        if (cross_xw) cross_xw[(int64_t)m * store_stride] = make_double2(double(st.x), double(st.w));
      }
      Crossing<R, P> cr;
      if (crossing_eval(s, p, rc, st.x, st.w, dm, kc, cr)) {
        R col[3], dcs[3], dcu[3];
        crossing_colour<R, P, PickA<R>>(s, rc, dm, cr, col, dcs, dcu);
        for (int i = 0; i < 3; ++i) acc[i] = fma(trans * cr.alpha, col[i], acc[i]);
        trans = trans * (R(1) - cr.alpha);
        if (trans < R(1e-4)) {
          f.cls = BH_CLASS_DISC;
          break;
        }
      }
      ++m;
      dm = rc.d0 + P(m) * P(kPiD);
      kc = crossing_step<R, P>(dm, p);
    }
    const R xa = st.x, wa = st.w;
    step<R, kComp>(st, c);
    if (!(st.x < c.x_hor)) {
      f.cls = BH_CLASS_HORIZON;
      ++k;
      break;
    }
    if (st.x <= c.x_esc) {
      f.cls = BH_CLASS_MISS;
      f.xa = xa;
      f.wa = wa;
      f.xb = st.x;
      f.wb = st.w;
      if (s.has_bg) {
        Escape<R, P> e;
        R col[3], dcs[3], dcu[3];
        escape_eval(s, p, rc, xa, wa, st.x, st.w, k, e, col, dcs, dcu);
        for (int i = 0; i < 3; ++i) acc[i] = fma(trans, col[i], acc[i]);
      }
      ++k;
      break;
    }
  }
  if (kStore && traj) traj[(int64_t)k * store_stride] = make_v2<TS>(double(st.x), double(st.w));
  f.k_end = k;
  f.m_end = m;
  f.trans = trans;
  for (int i = 0; i < 3; ++i) f.rgb[i] = acc[i];
}

// ---------------------------------------------------------------------------
// backward pieces
template <typename R, typename P>
BHA_NOINLINE void crossing_adjoint(const AdjScene& s, const AdjParams& p, const RayC<R, P>& rc, R x, R w, P dm,
                                   int kc, R T, const R* ab, R& Tb, R& lx, R& lw, Acc<R>& A) {
  Crossing<R, P> c;
  if (!crossing_eval(s, p, rc, x, w, dm, kc, c)) return;
  R col[3], dcs[3], dcu[3];
  crossing_colour<R, P, PickA<R>>(s, rc, dm, c, col, dcs, dcu);
  const R acol = ab[0] * col[0] + ab[1] * col[1] + ab[2] * col[2];
  const R alpha_b = T * (acol - Tb);
  const R ca = T * c.alpha;  // colour adjoint = ca * ab
  const R sb = ca * (ab[0] * dcs[0] + ab[1] * dcs[1] + ab[2] * dcs[2]);
  const R ub = ca * (ab[0] * dcu[0] + ab[1] * dcu[1] + ab[2] * dcu[2]);
  Tb = c.alpha * acol + (R(1) - c.alpha) * Tb;
  // azimuth -> crossing direction -> plane basis, phase
  const R azb = ub * R(s.disc_tex.height / kTwoPiD);
  const R q = c.X1 * c.X1 + c.Y1 * c.Y1;
  const R Y1b = azb * c.X1 / q, X1b = -azb * c.Y1 / q;
  const V3<R> e1 = PickA<R>::v(s.e1, s.e1_f), e2 = PickA<R>::v(s.e2, s.e2_f);
  const V3<R> phb = e2 * Y1b + e1 * X1b;
  A.e2 = A.e2 + c.ph * Y1b;
  A.yv = A.yv + phb * c.cs;
  A.xv = A.xv + phb * c.sn;
  const R phicb = dot(phb, rc.xv * c.cs - rc.yv * c.sn);
  A.phi0 += phicb;
  R dmb = phicb;
  // opacity and radial texture coordinate -> R, r_in, r_out, M
  const R z1b = alpha_b * c.s1 * (R(1) - c.s1) * c.s2;
  const R z2b = alpha_b * c.s1 * c.s2 * (R(1) - c.s2);
  const R span = rc.r_out - rc.r_in;
  const R kw = R(s.disc_tex.width) / span;
  const R Rb = (z1b - z2b) / rc.wsoft + sb * kw;
  A.r_in += -z1b / rc.wsoft + sb * kw * (c.Rr - rc.r_out) / span;
  A.r_out += z2b / rc.wsoft - sb * kw * (c.Rr - rc.r_in) / span;
  const R wsb = -(z1b * c.z1 + z2b * c.z2) / rc.wsoft;
  A.M += wsb * R(p.softness) + Rb / c.uc;
  const R ucb = -Rb * c.Rr / c.uc;
  // partial step from the state at kc
  R gx, gw, gh;
  step_h_vjp(x, w, c.delta, ucb, R(0), gx, gw, gh);
  dmb += gh;
  A.d0 += dmb;
  lx += gx;
  lw += gw;
}

// Escape (MISS with a sky): adjoint of the colour trans * sky(dir(psi)) with
// respect to trans, the plane basis, phi0 and the two states around the
// escape (the escape parameter t by the implicit function theorem).
template <typename R, typename P>
BHA_NOINLINE void escape_adjoint(const AdjScene& s, const AdjParams& p, const RayC<R, P>& rc, const Fwd<R>& f,
                                 const R* ab, R& Tb, R& lxa, R& lwa, R& lxb, R& lwb, Acc<R>& A) {
  const Rk4Consts<R>& c = consts<R>(p);
  Escape<R, P> e;
  R col[3], dcs[3], dcu[3];
  escape_eval(s, p, rc, f.xa, f.wa, f.xb, f.wb, f.k_end - 1, e, col, dcs, dcu);
  Tb = ab[0] * col[0] + ab[1] * col[1] + ab[2] * col[2];
  const R sb = f.trans * (ab[0] * dcs[0] + ab[1] * dcs[1] + ab[2] * dcs[2]);
  const R ub = f.trans * (ab[0] * dcu[0] + ab[1] * dcu[1] + ab[2] * dcu[2]);
  const int W = s.bg_tex.width, H = s.bg_tex.height;
  const R lonb = sb * R(W / kTwoPiD);
  const R latb = -ub * R(H / kPiD);
  const R qq = e.dir.x * e.dir.x + e.dir.y * e.dir.y;
  V3<R> dirb;
  dirb.x = -lonb * e.dir.y / qq;
  dirb.y = lonb * e.dir.x / qq;
  dirb.z = (e.dir.z < R(1) && e.dir.z > R(-1)) ? latb / sqrt(R(1) - e.dir.z * e.dir.z) : R(0);
  A.yv = A.yv + dirb * e.psi_c;
  A.xv = A.xv + dirb * e.psi_s;
  const R psib = dot(dirb, rc.xv * e.psi_c - rc.yv * e.psi_s);
  A.phi0 += psib;
  // psi = phi0 + (k + t) h + atan2(u_esc, -we), we = p'(t) / h
  const R web = psib * c.u_esc / (e.we * e.we + c.u_esc * c.u_esc);
  const R tb = psib * c.h + web * e.hm.ddp / c.h;
  const R g = tb / e.hm.dp;
  lxa = web * e.hm.d00 / c.h - g * e.hm.h00;
  lwa = web * e.hm.d10 - g * c.h * e.hm.h10;
  lxb = web * e.hm.d01 / c.h - g * e.hm.h01;
  lwb = web * e.hm.d11 - g * c.h * e.hm.h11;
}

// Backward pass over the whole trajectory. sub: kSeg / kSub sub-checkpoints
// (stride sub_stride). Leaves the adjoint of (x0, w0) in (lx, lw).
template <typename R, typename P, bool kComp>
BHA_HD void backward(const AdjScene& s, const AdjParams& p, const RayC<R, P>& rc, const Fwd<R>& f, const R* ab,
                     const Ckpt<R, kComp>* ck, int64_t ck_stride, Ckpt<R, kComp>* sub, int sub_stride, Acc<R>& A,
                     R& lx, R& lw) {
  const Rk4Consts<R>& c = consts<R>(p);
  const int k_end = f.k_end;
  R Tb = R(0), lxa = R(0), lwa = R(0);
  lx = R(0);
  lw = R(0);
  if (f.cls == BH_CLASS_MISS && s.has_bg) escape_adjoint(s, p, rc, f, ab, Tb, lxa, lwa, lx, lw, A);
  // The last crossing is at k_end for a ray stopped by the disc; otherwise no
  // event sits at the state k_end (it may lie past the last checkpoint).
  const bool end_cross = f.cls == BH_CLASS_DISC;
  const int first_seg = end_cross ? k_end / kSeg : (k_end > 0 ? (k_end - 1) / kSeg : 0);
  for (int sg = first_seg; sg >= 0; --sg) {
    const int k0 = sg * kSeg;
    const int kstop = k0 + kSeg - 1 < k_end ? k0 + kSeg - 1 : k_end;
    const int nsub = (kstop - k0) / kSub + 1;
    {  // re-run the segment, storing the sub-checkpoints
      const Ckpt<R, kComp> cp = ck[sg * ck_stride];
      Traj<R> st = cp.traj();
      R trans = cp.trans;
      int m = cp.m;
      P dm = rc.d0 + P(m) * P(kPiD);
      int kc = s.disc_on ? crossing_step<R, P>(dm, p) : -1;
      for (int j = 0; j < nsub; ++j) {
        sub[j * sub_stride] = Ckpt<R, kComp>::make(st, trans, m);
        if (j == nsub - 1) break;
        for (int i = 0; i < kSub; ++i) {
          const int k = k0 + j * kSub + i;
          if (k == kc) {
            Crossing<R, P> cr;
            if (crossing_eval(s, p, rc, st.x, st.w, dm, kc, cr)) trans = trans * (R(1) - cr.alpha);
            ++m;
            dm = rc.d0 + P(m) * P(kPiD);
            kc = crossing_step<R, P>(dm, p);
          }
          step<R, kComp>(st, c);
        }
      }
    }
    for (int j = nsub - 1; j >= 0; --j) {
      const Ckpt<R, kComp> b = sub[j * sub_stride];
      const int kj = k0 + j * kSub;
      R X[kSub], Wv[kSub];
      Traj<R> st = b.traj();
#pragma unroll
      for (int i = 0; i < kSub; ++i) {
        X[i] = st.x;
        Wv[i] = st.w;
        if (i < kSub - 1) step<R, kComp>(st, c);
      }
      const P dm = rc.d0 + P(b.m) * P(kPiD);
      const int kc = s.disc_on ? crossing_step<R, P>(dm, p) : -1;
#pragma unroll
      for (int i = kSub - 1; i >= 0; --i) {
        const int k = kj + i;
        if (k <= kstop) {
          if (k < k_end) {
            step_vjp(X[i], Wv[i], c, lx, lw);
            if (k == k_end - 1) {
              lx += lxa;
              lw += lwa;
            }
          }
          if (k == kc && (k < k_end || end_cross)) crossing_adjoint(s, p, rc, X[i], Wv[i], dm, kc, b.trans, ab, Tb, lx, lw, A);
        }
      }
    }
  }
}

// Backward pass over states stored by forward<..., kStore>, in precision R.
// p must describe the stored trajectory: for R = float the FP64 step in c32
// (rounded), inv_h32 and hstep32 (band_view).
// double-float arithmetic: DF, df_add, df_mul, ... (bh_df.cuh)

// x (3x + 1): df_fx (bh_df.cuh)

// The RK4 step of step() in double-float.
BHA_HD void df_step(DF& x, DF& w, const float* k) {
  const DF h{k[0], k[1]}, hh{k[2], k[3]}, q{k[4], k[5]}, q2{k[6], k[7]}, h26{k[8], k[9]}, h6{k[10], k[11]};
  const DF k1 = df_fx(x);
  const DF s1 = df_fma(hh, w, x);
  const DF k2 = df_fx(s1);
  const DF s2 = df_fma(q, k1, s1);
  const DF k3 = df_fx(s2);
  const DF s3a = df_fma(h, w, x);
  const DF s3 = df_fma(q2, k2, s3a);
  const DF k4 = df_fx(s3);
  const DF A = df_add(k2, k3);
  const DF S = df_add(A, k1);
  x = df_fma(h26, S, s3a);
  w = df_fma(h6, df_add(df_add(S, A), k4), w);
}


inline void set_df_consts(AdjParams* p) {
  const double v[8] = {p->c64.h, p->c64.hh, p->c64.q, p->c64.q2, p->c64.h26, p->c64.h6, p->c64.x_esc, p->c64.x_hor};
  for (int i = 0; i < 8; ++i) {
    const float h = float(v[i]);
    p->df_c[2 * i] = h;
    p->df_c[2 * i + 1] = float(v[i] - double(h));
  }
}

// forward<double, double, false, true> with the integration in double-float:
// the same trajectory as the FP64 one to ~1e-14; crossings and the escape
// are evaluated in FP64 from the converted state.
BHA_HD void forward_df(const AdjScene& s, const AdjParams& p, const RayC<double, double>& rc, Fwd<double>& f,
                       float2* traj, float* cross_t, double2* cross_xw, int64_t stride, int max_cross) {
  DF x = df_from(rc.x0), w = df_from(rc.w0);
  const DF x_esc{p.df_c[12], p.df_c[13]}, x_hor{p.df_c[14], p.df_c[15]};
  double trans = 1;
  double acc[3] = {0, 0, 0};
  int m = 0;
  double dm = rc.d0;
  int kc = s.disc_on ? crossing_step<double, double>(dm, p) : -1;
  int k = 0;
  f.cls = BH_CLASS_MAXSTEPS;
  for (; k < p.kmax; ++k) {
    if (traj) traj[(int64_t)k * stride] = make_float2(x.hi, w.hi);
    if (k == kc) {
      const double xd = df_to(x), wd = df_to(w);
      if (traj && m < max_cross) {
        cross_t[(int64_t)m * stride] = float(trans);
        cross_xw[(int64_t)m * stride] = make_double2(xd, wd);
      }
      Crossing<double, double> cr;
      if (crossing_eval(s, p, rc, xd, wd, dm, kc, cr)) {
        double col[3], dcs[3], dcu[3];
        crossing_colour<double, double, PickA<double>>(s, rc, dm, cr, col, dcs, dcu);
        for (int i = 0; i < 3; ++i) acc[i] = fma(trans * cr.alpha, col[i], acc[i]);
        trans = trans * (1 - cr.alpha);
        if (trans < 1e-4) {
          f.cls = BH_CLASS_DISC;
          break;
        }
      }
      ++m;
      dm = rc.d0 + double(m) * kPiD;
      kc = crossing_step<double, double>(dm, p);
    }
    const DF xa = x, wa = w;
    df_step(x, w, p.df_c);
    if (!df_lt(x, x_hor)) {  // also NaN
      f.cls = BH_CLASS_HORIZON;
      ++k;
      break;
    }
    if (df_le(x, x_esc)) {
      f.cls = BH_CLASS_MISS;
      f.xa = df_to(xa);
      f.wa = df_to(wa);
      f.xb = df_to(x);
      f.wb = df_to(w);
      if (s.has_bg) {
        Escape<double, double> e;
        double col[3], dcs[3], dcu[3];
        escape_eval(s, p, rc, f.xa, f.wa, f.xb, f.wb, k, e, col, dcs, dcu);
        for (int i = 0; i < 3; ++i) acc[i] = fma(trans, col[i], acc[i]);
      }
      ++k;
      break;
    }
  }
  if (traj) traj[(int64_t)k * stride] = make_float2(x.hi, w.hi);
  f.k_end = k;
  f.m_end = m;
  f.trans = trans;
  for (int i = 0; i < 3; ++i) f.rgb[i] = acc[i];
}

// MIXED: whether the ray of pixel (px, py) belongs to the FP64 band,
// |b/M - 3 sqrt 3| < band. FP64, from b^2 = |F|^2 - (F.e)^2 / |e|^2 (about 20
// operations); every kernel that needs the decision calls this.
BHA_HD bool in_band(const AdjScene& s, int px, int py, double band) {
  const double a = s.half_w - double(px), c = s.half_h - double(py);
  double e[3], ee = 0, fe = 0, ff = 0;
  for (int i = 0; i < 3; ++i) {
    e[i] = fma(s.vz[i], c, fma(s.vy[i], a, s.E0[i]));
    ee = fma(e[i], e[i], ee);
    fe = fma(s.F[i], e[i], fe);
    ff = fma(s.F[i], s.F[i], ff);
  }
  const double b2 = fmax(ff - fe * fe / ee, 0.0);
  return fabs(sqrt(b2) / s.mass - 5.196152422706632) < band;
}

// Results of an escape adjoint computed elsewhere (in FP64 for the band).
template <typename R>
struct EscInit {
  R Tb, lxa, lwa, lxb, lwb;
};

// The adjoint of (x0, w0) is returned as lx + clx, lw + clw: for a
// near-critical ray it is large and nearly orthogonal to the tangents it is
// contracted with, so its low parts matter. esc (may be null) replaces the
// escape adjoint (whose contributions to A the caller has added).
// With x64 (the FP64 ray, parameters, stored crossing states and
// accumulators) the crossings' adjoints are taken in FP64.
struct Cross64 {
  const AdjParams* p;
  const RayC<double, double>* rc;
  const double2* xw;
  const double* ab;
  Acc<double>* A;
};

template <typename R, typename P>
BHA_HD void backward_stored(const AdjScene& s, const AdjParams& p, const RayC<R, P>& rc, const Fwd<R>& f,
                            const R* ab, const typename Vec2T<R>::type* traj, const float* cross_t, int64_t stride,
                            int max_cross, Acc<R>& A, R& lx, R& lw, R& clx, R& clw, const EscInit<R>* esc = nullptr,
                            const Cross64* x64 = nullptr) {
  const Rk4Consts<R>& c = consts<R>(p);
  const int k_end = f.k_end;
  R Tb = R(0), lxa = R(0), lwa = R(0);
  lx = R(0);
  lw = R(0);
  if (esc) {
    Tb = esc->Tb;
    lxa = esc->lxa;
    lwa = esc->lwa;
    lx = esc->lxb;
    lw = esc->lwb;
  } else if (f.cls == BH_CLASS_MISS && s.has_bg) {
    escape_adjoint(s, p, rc, f, ab, Tb, lxa, lwa, lx, lw, A);
  }
  // the last crossing taken: index m_end for a disc stop, m_end - 1 otherwise
  int j = s.disc_on ? (f.cls == BH_CLASS_DISC ? f.m_end : f.m_end - 1) : -1;
  P dm = rc.d0 + P(j) * P(kPiD);
  int kc = j >= 0 ? crossing_step<R, P>(dm, p) : -1;
  clx = R(0);
  clw = R(0);
  // the stored states are read 8 at a time ahead of the serial chain
  constexpr int kAhead = 8;
  typename Vec2T<R>::type buf[kAhead];
  for (int k = k_end; k >= 0; --k) {
    const int slot = (k_end - k) % kAhead;
    if (slot == 0) {
#pragma unroll
      for (int i = 0; i < kAhead; ++i) {
        const int kk = k - i;
        if (kk >= 0) buf[i] = traj[(int64_t)kk * stride];
      }
    }
    typename Vec2T<R>::type q = buf[0];
#pragma unroll
    for (int i = 1; i < kAhead; ++i)
      if (slot == i) q = buf[i];
    if (k < k_end) {
      step_vjp_comp(q.x, q.y, c, lx, lw, clx, clw);
      if (k == k_end - 1) {
        two_sum_acc(lx, lxa, clx);
        two_sum_acc(lw, lwa, clw);
      }
    }
    while (j >= 0 && kc == k) {
      const R T = j < max_cross ? R(cross_t[(int64_t)j * stride]) : R(0);
      R gx = R(0), gw = R(0);
      if (x64 && j < max_cross) {
        const double2 xw = x64->xw[(int64_t)j * stride];
        double Tb64 = double(Tb), gx64 = 0, gw64 = 0;
        crossing_adjoint(s, *x64->p, *x64->rc, xw.x, xw.y, double(dm), kc, double(T), x64->ab, Tb64, gx64, gw64,
                         *x64->A);
        Tb = R(Tb64);
        gx = R(gx64);
        gw = R(gw64);
      } else {
        crossing_adjoint(s, p, rc, q.x, q.y, dm, kc, T, ab, Tb, gx, gw, A);
      }
      two_sum_acc(lx, gx, clx);
      two_sum_acc(lw, gw, clw);
      --j;
      dm = rc.d0 + P(j) * P(kPiD);
      kc = j >= 0 ? crossing_step<R, P>(dm, p) : -1;
    }
  }
}

// Gradient of the pixel's loss: sum over the ray constants K of dL/dK dK/dtheta_i,
// dK/dtheta_i by forward-mode tangents of the ray setup.
template <typename R, typename P>
BHA_HD void assemble(const AdjScene& s, R a, R cc, const Acc<R>& A, R lx0, R lw0, float* g) {
  for (int i = 0; i < kParams; ++i) {
    V3<D1<R>> E0, vy, vz, F, n;
    const V3<R> pE0 = PickA<R>::v(s.E0, s.E0_f), pvy = PickA<R>::v(s.vy, s.vy_f), pvz = PickA<R>::v(s.vz, s.vz_f),
                pF = PickA<R>::v(s.F, s.F_f), pn = PickA<R>::v(s.n, s.n_f);
    const V3<R> tE0 = PickA<R>::v(s.dE0[i], s.dE0_f[i]), tvy = PickA<R>::v(s.dvy[i], s.dvy_f[i]),
                tvz = PickA<R>::v(s.dvz[i], s.dvz_f[i]), tF = PickA<R>::v(s.dF[i], s.dF_f[i]),
                tn = PickA<R>::v(s.dn[i], s.dn_f[i]), te2 = PickA<R>::v(s.de2[i], s.de2_f[i]);
    E0 = {{pE0.x, tE0.x}, {pE0.y, tE0.y}, {pE0.z, tE0.z}};
    vy = {{pvy.x, tvy.x}, {pvy.y, tvy.y}, {pvy.z, tvy.z}};
    vz = {{pvz.x, tvz.x}, {pvz.y, tvz.y}, {pvz.z, tvz.z}};
    F = {{pF.x, tF.x}, {pF.y, tF.y}, {pF.z, tF.z}};
    n = {{pn.x, tn.x}, {pn.y, tn.y}, {pn.z, tn.z}};
    const D1<R> M(R(s.mass), R(i == BH_GRAD_MASS ? 1 : 0));
    const RayInit<D1<R>> r = ray_init<D1<R>>(E0, vy, vz, F, n, M, D1<R>(a), D1<R>(cc));
    // a radial ray (b = 0) has no orbital plane; the set has measure zero
    if (!(r.bm.v > R(0))) return;
    R gi = A.yv.x * r.yv.x.d + A.yv.y * r.yv.y.d + A.yv.z * r.yv.z.d;
    gi += A.xv.x * r.xv.x.d + A.xv.y * r.xv.y.d + A.xv.z * r.xv.z.d;
    gi += lx0 * r.x0.d + lw0 * r.w0.d + A.phi0 * r.phi0.d + A.d0 * r.d0.d;
    gi += dot(A.e2, te2);
    if (i == BH_GRAD_MASS) gi += A.M;
    if (i == BH_GRAD_R_INNER) gi += A.r_in;
    if (i == BH_GRAD_R_OUTER) gi += A.r_out;
    g[i] = float(gi);
  }
}

// ---------------------------------------------------------------------------
// one ray end to end: forward, loss, backward, gradient
struct RayOut {
  float rgb[3];
  float loss;
  float grad[kParams];
  int32_t cls, steps;
};

template <typename R, typename P>
BHA_HD RayC<R, P> ray_constants(const AdjScene& s, int px, int py, R* bm_out) {
  const P a = P(s.half_w) - P(px), cc = P(s.half_h) - P(py);
  const RayInit<P> r = ray_init<P>(PickA<P>::v(s.E0, s.E0_f), PickA<P>::v(s.vy, s.vy_f), PickA<P>::v(s.vz, s.vz_f),
                                   PickA<P>::v(s.F, s.F_f), PickA<P>::v(s.n, s.n_f), P(s.mass), a, cc);
  RayC<R, P> rc;
  rc.yv = cast3<R>(r.yv);
  rc.xv = cast3<R>(r.xv);
  rc.x0 = R(r.x0);
  rc.w0 = R(r.w0);
  rc.x0lo = R(r.x0 - P(rc.x0));
  rc.w0lo = R(r.w0 - P(rc.w0));
  rc.phi0 = r.phi0;
  rc.d0 = r.d0;
  rc.M = R(s.mass);
  rc.r_in = R(s.r_in);
  rc.r_out = R(s.r_out);
  rc.wsoft = R(s.wsoft);
  if (bm_out) *bm_out = R(r.bm);
  return rc;
}

template <typename R, typename P, bool kComp>
BHA_HD void trace_adjoint(const AdjScene& s, const AdjParams& p, const RayC<R, P>& rc, int px, int py,
                          Ckpt<R, kComp>* ck, int64_t ck_stride, Ckpt<R, kComp>* sub, int sub_stride, RayOut& out) {
  const size_t pix = (size_t)py * s.width + px;
  const bool grad = p.want_grad && s.target;
  Fwd<R> f;
  forward<R, P, kComp>(s, p, rc, grad ? ck : nullptr, ck_stride, f);
  out.cls = f.cls;
  out.steps = f.k_end;
  for (int i = 0; i < 3; ++i) out.rgb[i] = float(f.rgb[i]);
  out.loss = 0.f;
  for (int i = 0; i < kParams; ++i) out.grad[i] = 0.f;
  if (!s.target) return;
  R ab[3];
  R loss = R(0);
  for (int i = 0; i < 3; ++i) {
    const R dlt = f.rgb[i] - R(s.target[pix * 3 + i]);
    loss += dlt * dlt;
    ab[i] = R(2) * dlt;
  }
  out.loss = float(loss);
  // A black ray (horizon or step cap) that composited no disc crossing has a
  // locally constant colour: its gradient is zero and needs no backward pass.
  if (!grad || ((f.cls == BH_CLASS_HORIZON || f.cls == BH_CLASS_MAXSTEPS) && f.trans == R(1))) return;
  Acc<R> A;
  A.yv = A.xv = A.e2 = V3<R>{R(0), R(0), R(0)};
  A.phi0 = A.d0 = A.M = A.r_in = A.r_out = R(0);
  R lx0, lw0;
  backward<R, P, kComp>(s, p, rc, f, ab, ck, ck_stride, sub, sub_stride, A, lx0, lw0);
  assemble<R, P>(s, R(s.half_w) - R(px), R(s.half_h) - R(py), A, lx0, lw0, out.grad);
}

// One ray of the FP64 band: forward in FP64 (double-float integration with
// FP64 events for RR = float) storing every state (in RR), the transmittance
// and the FP64 state at each crossing; reverse pass in RR over the stored
// states (pb: the RR view of the FP64 trajectory, see backward_stored) with
// the escape and crossing adjoints in FP64; tangents of the ray setup in FP64.
template <typename RR>
BHA_HD void trace_adjoint_band(const AdjScene& s, const AdjParams& p, const AdjParams& pb, int px, int py,
                               typename Vec2T<RR>::type* traj, float* cross_t, double2* cross_xw, int64_t stride,
                               int max_cross, RayOut& out) {
  const RayC<double, double> rd = ray_constants<double, double>(s, px, py, nullptr);
  const size_t pix = (size_t)py * s.width + px;
  const bool grad = p.want_grad && s.target;
  Fwd<double> f;
  if constexpr (sizeof(RR) == sizeof(float))
    forward_df(s, p, rd, f, grad ? traj : nullptr, cross_t, cross_xw, stride, max_cross);
  else
    forward<double, double, false, true, RR>(s, p, rd, nullptr, 0, f, grad ? traj : nullptr, cross_t, stride,
                                             max_cross, cross_xw);
  out.cls = f.cls;
  out.steps = f.k_end;
  for (int i = 0; i < 3; ++i) out.rgb[i] = float(f.rgb[i]);
  out.loss = 0.f;
  for (int i = 0; i < kParams; ++i) out.grad[i] = 0.f;
  if (!s.target) return;
  RR ab[3];
  double loss = 0;
  for (int i = 0; i < 3; ++i) {
    const double dlt = f.rgb[i] - double(s.target[pix * 3 + i]);
    loss += dlt * dlt;
    ab[i] = RR(2 * dlt);
  }
  out.loss = float(loss);
  if (!grad || ((f.cls == BH_CLASS_HORIZON || f.cls == BH_CLASS_MAXSTEPS) && f.trans == 1.0)) return;
  RayC<RR, double> rf;
  rf.yv = cast3<RR>(rd.yv);
  rf.xv = cast3<RR>(rd.xv);
  rf.x0 = RR(rd.x0);
  rf.w0 = RR(rd.w0);
  rf.x0lo = rf.w0lo = RR(0);
  rf.phi0 = rd.phi0;
  rf.d0 = rd.d0;
  rf.M = RR(rd.M);
  rf.r_in = RR(rd.r_in);
  rf.r_out = RR(rd.r_out);
  rf.wsoft = RR(rd.wsoft);
  Fwd<RR> ff;
  for (int i = 0; i < 3; ++i) ff.rgb[i] = RR(f.rgb[i]);
  ff.trans = RR(f.trans);
  ff.xa = RR(f.xa);
  ff.wa = RR(f.wa);
  ff.xb = RR(f.xb);
  ff.wb = RR(f.wb);
  ff.cls = f.cls;
  ff.k_end = f.k_end;
  ff.m_end = f.m_end;
  // the escape (the largest adjoint of a near-critical ray) in FP64: its sky
  // derivative at an FP32 escape direction is off by ~1e-3 there
  Acc<double> Ae;
  Ae.yv = Ae.xv = Ae.e2 = V3<double>{0, 0, 0};
  Ae.phi0 = Ae.d0 = Ae.M = Ae.r_in = Ae.r_out = 0;
  EscInit<RR> esc{RR(0), RR(0), RR(0), RR(0), RR(0)};
  const bool escaped = f.cls == BH_CLASS_MISS && s.has_bg;
  if (escaped) {
    const double abe[3] = {double(ab[0]), double(ab[1]), double(ab[2])};
    double Tb, lxa, lwa, lxb, lwb;
    escape_adjoint(s, p, rd, f, abe, Tb, lxa, lwa, lxb, lwb, Ae);
    esc = EscInit<RR>{RR(Tb), RR(lxa), RR(lwa), RR(lxb), RR(lwb)};
  }
  Acc<RR> A;
  A.yv = A.xv = A.e2 = V3<RR>{RR(0), RR(0), RR(0)};
  A.phi0 = A.d0 = A.M = A.r_in = A.r_out = RR(0);
  // the crossings in FP64 too: from float states their sample point moves by
  // ~1e-4 texel, which shifts the filtered texture's slope at steep edges
  const double abd[3] = {double(ab[0]), double(ab[1]), double(ab[2])};
  Cross64 x64{&p, &rd, cross_xw, abd, &Ae};
  RR lx0, lw0, clx0, clw0;
  backward_stored<RR, double>(s, pb, rf, ff, ab, traj, cross_t, stride, max_cross, A, lx0, lw0, clx0, clw0,
                              escaped ? &esc : nullptr, cross_xw ? &x64 : nullptr);
  Acc<double> Ad;
  Ad.yv = cast3<double>(A.yv) + Ae.yv;
  Ad.xv = cast3<double>(A.xv) + Ae.xv;
  Ad.e2 = cast3<double>(A.e2) + Ae.e2;
  Ad.phi0 = A.phi0 + Ae.phi0;
  Ad.d0 = A.d0 + Ae.d0;
  Ad.M = A.M + Ae.M;
  Ad.r_in = A.r_in + Ae.r_in;
  Ad.r_out = A.r_out + Ae.r_out;
  assemble<double, double>(s, s.half_w - double(px), s.half_h - double(py), Ad, double(lx0) + double(clx0),
                           double(lw0) + double(clw0), out.grad);
}

// Most disc-plane crossings a ray can reach in kmax steps of h.
inline int max_crossings(int kmax, double h) { return int(kmax * h / kPiD) + 3; }

// The FP32 view of the FP64 trajectory (reverse pass of the band).
inline AdjParams band_view(const AdjParams& p) {
  AdjParams b = p;
  b.c32 = exact_rk4_consts_f32(p.c64.h, p.c64.u_esc, p.kmax);
  b.inv_h32 = p.inv_h64;
  b.hstep32 = p.hstep64;
  return b;
}

// ---------------------------------------------------------------------------
// host: per-scene record at theta, with tangents (FP64 forward mode over the
// 10 parameters)
struct HD {
  double v;
  double d[kParams];
};
inline HD hd_const(double v) {
  HD r;
  r.v = v;
  for (int i = 0; i < kParams; ++i) r.d[i] = 0;
  return r;
}
inline HD hd_add(const HD& a, const HD& b) {
  HD r;
  r.v = a.v + b.v;
  for (int i = 0; i < kParams; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
inline HD hd_mul(const HD& a, const HD& b) {
  HD r;
  r.v = a.v * b.v;
  for (int i = 0; i < kParams; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
inline HD hd_scale(const HD& a, double k) {
  HD r;
  r.v = a.v * k;
  for (int i = 0; i < kParams; ++i) r.d[i] = a.d[i] * k;
  return r;
}
inline HD hd_chain(const HD& a, double f, double df) {
  HD r;
  r.v = f;
  for (int i = 0; i < kParams; ++i) r.d[i] = a.d[i] * df;
  return r;
}
struct HD3 {
  HD x, y, z;
};
inline HD3 hd3_const(const double* v) { return {hd_const(v[0]), hd_const(v[1]), hd_const(v[2])}; }
inline HD3 hd3_add(const HD3& a, const HD3& b) { return {hd_add(a.x, b.x), hd_add(a.y, b.y), hd_add(a.z, b.z)}; }
inline HD3 hd3_scale(const HD3& a, const HD& s) { return {hd_mul(a.x, s), hd_mul(a.y, s), hd_mul(a.z, s)}; }
inline HD hd3_dot(const HD3& a, const HD3& b) { return hd_add(hd_add(hd_mul(a.x, b.x), hd_mul(a.y, b.y)), hd_mul(a.z, b.z)); }
inline HD3 hd3_cross(const HD3& a, const HD3& b) {
  return {hd_add(hd_mul(a.y, b.z), hd_scale(hd_mul(a.z, b.y), -1)),
          hd_add(hd_mul(a.z, b.x), hd_scale(hd_mul(a.x, b.z), -1)),
          hd_add(hd_mul(a.x, b.y), hd_scale(hd_mul(a.y, b.x), -1))};
}
// Rodrigues: v rotated about the unit axis ax by th.
inline HD3 hd3_rotate(const HD3& v, const double* ax, const HD& th) {
  const HD3 a = hd3_const(ax);
  const HD c = hd_chain(th, std::cos(th.v), -std::sin(th.v));
  const HD s = hd_chain(th, std::sin(th.v), std::cos(th.v));
  const HD k = hd_mul(hd3_dot(a, v), hd_add(hd_const(1), hd_scale(c, -1)));
  return hd3_add(hd3_add(hd3_scale(v, c), hd3_scale(hd3_cross(a, v), s)), hd3_scale(a, k));
}
inline HD3 hd3_unit(const HD3& a) {
  const HD l2 = hd3_dot(a, a);
  const double l = std::sqrt(l2.v);
  const HD inv = hd_chain(l2, 1.0 / l, -0.5 / (l * l * l));
  return hd3_scale(a, inv);
}

// The scene's theta: M, zero offsets and rotations, its radii.
inline void base_theta(const bh_scene& sc, double* th) {
  th[BH_GRAD_MASS] = sc.hole.mass;
  for (int i = 1; i <= BH_GRAD_TILT; ++i) th[i] = 0;
  th[BH_GRAD_R_INNER] = sc.disc.r_inner;
  th[BH_GRAD_R_OUTER] = sc.disc.r_outer;
}

struct Posed {
  HD3 vx, vy, vz, cpos, n, e2;
  double e1[3];
  HD M, r_in, r_out;
};

inline Posed pose_at(const bh_scene& sc, const double* theta) {
  HD th[kParams];
  for (int i = 0; i < kParams; ++i) {
    th[i] = hd_const(theta[i]);
    th[i].d[i] = 1.0;
  }
  const bh_camera& cam = sc.camera;
  auto rot = [&](const double* v) {
    HD3 r = hd3_rotate(hd3_const(v), cam.axis_x, th[BH_GRAD_ROLL]);
    r = hd3_rotate(r, cam.axis_y, th[BH_GRAD_PITCH]);
    return hd3_rotate(r, cam.axis_z, th[BH_GRAD_YAW]);
  };
  Posed q;
  q.vx = rot(cam.axis_x);
  q.vy = rot(cam.axis_y);
  q.vz = rot(cam.axis_z);
  q.cpos = hd3_add(hd3_const(cam.position), HD3{th[BH_GRAD_CAM_X], th[BH_GRAD_CAM_Y], th[BH_GRAD_CAM_Z]});
  const double* s1 = sc.disc.edge_s1;
  const double l1 = std::sqrt(s1[0] * s1[0] + s1[1] * s1[1] + s1[2] * s1[2]);
  for (int i = 0; i < 3; ++i) q.e1[i] = l1 > 0 ? s1[i] / l1 : 0.0;
  q.n = hd3_rotate(hd3_const(sc.disc.normal), q.e1, th[BH_GRAD_TILT]);
  q.e2 = hd3_unit(hd3_cross(q.n, hd3_const(q.e1)));
  q.M = th[BH_GRAD_MASS];
  q.r_in = th[BH_GRAD_R_INNER];
  q.r_out = th[BH_GRAD_R_OUTER];
  return q;
}

inline void put3(const HD3& a, double* v, float* vf, double (*dv)[3], float (*dvf)[3]) {
  const HD* c[3] = {&a.x, &a.y, &a.z};
  for (int k = 0; k < 3; ++k) {
    v[k] = c[k]->v;
    vf[k] = float(c[k]->v);
    for (int i = 0; i < kParams; ++i) {
      if (dv) dv[i][k] = c[k]->d[i];
      if (dvf) dvf[i][k] = float(c[k]->d[i]);
    }
  }
}

inline void build_adj_scene(const bh_scene& sc, const double* theta, double softness, AdjScene* a) {
  const Posed q = pose_at(sc, theta);
  const HD3 hole = hd3_const(sc.hole.position);
  const HD3 F = hd3_add(q.cpos, hd3_scale(hole, hd_const(-1)));
  const HD3 E0 = hd3_add(q.cpos, hd3_scale(q.vx, hd_const(-sc.camera.focus_len)));
  put3(E0, a->E0, a->E0_f, a->dE0, a->dE0_f);
  put3(q.vy, a->vy, a->vy_f, a->dvy, a->dvy_f);
  put3(q.vz, a->vz, a->vz_f, a->dvz, a->dvz_f);
  put3(F, a->F, a->F_f, a->dF, a->dF_f);
  put3(q.n, a->n, a->n_f, a->dn, a->dn_f);
  put3(q.e2, a->e2, a->e2_f, a->de2, a->de2_f);
  for (int k = 0; k < 3; ++k) {
    a->e1[k] = q.e1[k];
    a->e1_f[k] = float(q.e1[k]);
  }
  a->mass = q.M.v;
  a->r_in = q.r_in.v;
  a->r_out = q.r_out.v;
  a->half_w = sc.camera.width / 2.0;
  a->half_h = sc.camera.height / 2.0;
  a->wsoft = softness * q.M.v;
  a->mass_f = float(a->mass);
  a->r_in_f = float(a->r_in);
  a->r_out_f = float(a->r_out);
  a->half_w_f = float(a->half_w);
  a->half_h_f = float(a->half_h);
  a->wsoft_f = float(a->wsoft);
  a->width = sc.camera.width;
  a->height = sc.camera.height;
  a->tiles_x = (sc.camera.width + 7) / 8;
  a->disc_on = sc.disc.enabled ? 1 : 0;
}

}  // namespace adj
}  // namespace bhgb
