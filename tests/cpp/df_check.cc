// Host checks of the double-float arithmetic the tracer's FP32 passes use for
// their rare exact paths and the band pass uses for its integration
// (blackhole_8_gb300/csrc/bh_df.cuh, compiled here for the CPU from the same
// source). Each mode prints one line of measured errors, which
// tests/test_df_cpu.py bounds:
//   arith  relative errors of df_add, df_mul, df_div against long double
//   eps    the first integral from the per-scene quadratic forms
//          (resolve_derived) against FP64 straight from the ray direction
//   rk4    the escape angle of double-float RK4 against FP64 RK4 (the same
//          Nystrom operations) for rays near the critical impact parameter
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>

#include "bh_df.cuh"
#include "bh_internal.h"

using bhgb::DF;

static long double to_ld(DF a) { return (long double)a.hi + (long double)a.lo; }

static int arith() {
  std::mt19937_64 rng(11);
  std::uniform_real_distribution<double> mant(1.0, 2.0), ex(-20.0, 20.0);
  auto draw = [&]() {
    const double v = mant(rng) * std::ldexp(1.0, int(ex(rng)));
    return (rng() & 1) ? v : -v;
  };
  double add = 0, mul = 0, div = 0;
  for (int i = 0; i < 200000; ++i) {
    const DF a = bhgb::df_from(draw()), b = bhgb::df_from(draw());
    const long double A = to_ld(a), B = to_ld(b);
    const long double s = A + B, p = A * B, q = A / B;
    // sums are measured against the larger operand (cancellation is exact)
    add = std::fmax(add, double(std::fabs(to_ld(bhgb::df_add(a, b)) - s) / std::fmax(std::fabs(A), std::fabs(B))));
    mul = std::fmax(mul, double(std::fabs(to_ld(bhgb::df_mul(a, b)) - p) / std::fabs(p)));
    div = std::fmax(div, double(std::fabs(to_ld(bhgb::df_div(a, b)) - q) / std::fabs(q)));
  }
  std::printf("add %.3e mul %.3e div %.3e\n", add, mul, div);
  return 0;
}

static void cross(const double* u, const double* v, double* o) {
  o[0] = u[1] * v[2] - u[2] * v[1];
  o[1] = u[2] * v[0] - u[0] * v[2];
  o[2] = u[0] * v[1] - u[1] * v[0];
}

// A camera at distance r from a hole of mass M, looking at the hole with
// an image of W x H pixels and focus length f (pixel units), turned by tilt.
static void camera(bhgb::DevScene* d, double r, double M, int W, int H, double f, double tilt) {
  std::memset(d, 0, sizeof(*d));
  const double az[3] = {std::cos(tilt), std::sin(tilt), 0.3};
  const double n = std::sqrt(az[0] * az[0] + az[1] * az[1] + az[2] * az[2]);
  double ax[3] = {az[0] / n, az[1] / n, az[2] / n};  // view axis (toward the camera's back)
  double ay[3], azz[3];
  const double up[3] = {0, 0, 1};
  cross(up, ax, ay);
  const double ly = std::sqrt(ay[0] * ay[0] + ay[1] * ay[1] + ay[2] * ay[2]);
  for (double& v : ay) v /= ly;
  cross(ax, ay, azz);
  for (int i = 0; i < 3; ++i) {
    d->F[i] = r * ax[i];
    d->E0[i] = d->F[i] - f * ax[i];  // the reference's raygen: position - focus vector
    d->vy[i] = ay[i];
    d->vz[i] = azz[i];
  }
  d->mass = M;
  d->half_w = W / 2.0;
  d->half_h = H / 2.0;
  d->half_w_f = float(d->half_w);
  d->half_h_f = float(d->half_h);
  d->width = W;
  d->height = H;
  d->r_in = 6 * M;
  d->r_out = 20 * M;
  bhgb::resolve_derived(d);
}

static int eps() {
  double worst = 0, worst_rel = 0;
  long near = 0;
  std::mt19937_64 rng(3);
  const double cases[][5] = {{20, 1, 1920, 1080, 1662}, {8, 1, 1920, 1080, 1662}, {30, 1, 640, 360, 554},
                             {50, 2, 1024, 1024, 800},  {20, 1, 4096, 4096, 469000}};
  for (const auto& cs : cases) {
    bhgb::DevScene d;
    camera(&d, cs[0], cs[1], int(cs[2]), int(cs[3]), cs[4], 0.4);
    std::uniform_int_distribution<int> px(0, d.width - 1), py(0, d.height - 1);
    for (int i = 0; i < 200000; ++i) {
      const int x = px(rng), y = py(rng);
      const float a = d.half_w_f - float(x), c = d.half_h_f - float(y);
      const DF e = bhgb::df_first_integral(bhgb::df_quad_form(d.eq_e, a, c), bhgb::df_quad_form(d.eq_g, a, c),
                                           DF{d.m2_df[0], d.m2_df[1]});
      long double ev[3], fe[3];
      for (int k = 0; k < 3; ++k) ev[k] = d.E0[k] + (long double)d.vy[k] * a + (long double)d.vz[k] * c;
      fe[0] = d.F[1] * ev[2] - d.F[2] * ev[1];
      fe[1] = d.F[2] * ev[0] - d.F[0] * ev[2];
      fe[2] = d.F[0] * ev[1] - d.F[1] * ev[0];
      const long double ee = ev[0] * ev[0] + ev[1] * ev[1] + ev[2] * ev[2];
      const long double gg = fe[0] * fe[0] + fe[1] * fe[1] + fe[2] * fe[2];
      const long double ref = ee * d.mass * d.mass / gg - 1.0L / 27.0L;
      const long double bm = std::sqrt(gg / ee) / d.mass;  // b / M
      if (bm < 1) continue;  // the hole's centre: never near the FP64 band
      worst_rel = std::fmax(worst_rel, double(std::fabs(to_ld(e) - ref) / (ref + 1.0L / 27.0L)));
      if (std::fabs(bm - 3.0L * std::sqrt(3.0L)) < 0.5L) {  // where the tracer takes it
        ++near;
        worst = std::fmax(worst, double(std::fabs(to_ld(e) - ref)));
      }
    }
  }
  std::printf("eps_abs %.3e eps_rel %.3e near %ld\n", worst, worst_rel, near);
  return 0;
}

static double fx(double x) { return x * std::fma(3.0, x, 1.0); }
static void step64(double& x, double& w, const double* c) {
  const double k1 = fx(x), s1 = std::fma(c[1], w, x), k2 = fx(s1), s2 = std::fma(c[2], k1, s1), k3 = fx(s2);
  const double s3a = std::fma(c[0], w, x), s3 = std::fma(c[3], k2, s3a), k4 = fx(s3);
  const double A = k2 + k3, S = A + k1;
  x = std::fma(c[4], S, s3a);
  w = std::fma(c[5], (S + A) + k4, w);
}

// Escape angle (linear in the last step) of a ray from r0 = 20 M, ingoing,
// with b = b_c + db, in FP64 or double-float; -1 when it is captured.
static double escape_angle(double db, bool df) {
  const double h = 0.01, xe = 0.01 - 1.0 / 3.0, xh = 0.5 - 1.0 / 3.0;
  const double c[6] = {h, h * 0.5, h * h * 0.25, h * h * 0.5, h * h / 6.0, h / 6.0};
  DF k[6];
  for (int i = 0; i < 6; ++i) k[i] = bhgb::df_from(c[i]);
  const double b = 3.0 * std::sqrt(3.0) + db, e = 1 / (b * b) - 1.0 / 27.0, x0 = 1.0 / 20.0 - 1.0 / 3.0;
  double x = x0, w = std::sqrt(e + x0 * x0 * (1 + 2 * x0));
  DF X = bhgb::df_from(x), W = bhgb::df_from(w);
  for (int s = 0; s < 20000; ++s) {
    double xa, xb;
    if (df) {
      xa = bhgb::df_to(X);
      bhgb::df_rk4_step(X, W, k);
      xb = bhgb::df_to(X);
    } else {
      xa = x;
      step64(x, w, c);
      xb = x;
    }
    if (xb <= xe) return (s + (xa - xe) / (xa - xb)) * h;
    if (xb >= xh) return -1;
  }
  return -1;
}

static int rk4() {
  double worst = 0, worst_near = 0;
  for (double db : {1e-2, 1e-3, 1e-4, 3e-5, 1e-5, 3e-6, 1e-6, 3e-7, 1e-7}) {
    for (double sgn : {1.0, -1.0}) {
      const double a = escape_angle(sgn * db, false), b = escape_angle(sgn * db, true);
      if ((a < 0) != (b < 0)) {
        std::printf("class differs at db %g\n", sgn * db);
        return 1;
      }
      if (a < 0) continue;
      (db >= 1e-6 ? worst : worst_near) = std::fmax(db >= 1e-6 ? worst : worst_near, std::fabs(a - b));
    }
  }
  std::printf("rk4_phi %.3e rk4_phi_near %.3e\n", worst, worst_near);
  return 0;
}

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  if (!std::strcmp(argv[1], "arith")) return arith();
  if (!std::strcmp(argv[1], "eps")) return eps();
  if (!std::strcmp(argv[1], "rk4")) return rk4();
  return 2;
}
