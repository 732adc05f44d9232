// Double-float arithmetic: a value is the unevaluated sum hi + lo of two
// floats (about 48 significant bits), built from the error-free
// transformations of Knuth (2Sum) and Dekker (Fast2Sum), with an FMA giving a
// product's exact rounding error. It runs on the FP32 pipe: on this part an
// FP64 warp instruction holds an SM sub-partition's FP64 unit for ~64-80
// cycles, so a double-float operation of 3-20 FP32 instructions is several
// times cheaper than the FP64 instruction it replaces, in throughput and in a
// serial chain alike.
//
// The transformations need every sum and product rounded on its own. On the
// device they use the intrinsics that the compiler never contracts into an
// FMA (it would otherwise fuse a product into the following sum across
// inlined calls, and the error terms would be wrong); the explicit fmaf calls
// are the only fused operations. The same source therefore gives bit-identical
// results in every kernel that inlines it.
#pragma once

#include <math.h>

#if defined(__CUDACC__)
#define BHDF_HD __host__ __device__ __forceinline__
#else
#define BHDF_HD inline
#endif

#if defined(__CUDA_ARCH__)
#define BHDF_ADD(a, b) __fadd_rn((a), (b))
#define BHDF_SUB(a, b) __fsub_rn((a), (b))
#define BHDF_MUL(a, b) __fmul_rn((a), (b))
#else
// host: a rounded store that no compiler fuses
inline float bhdf_round(volatile float v) { return v; }
#define BHDF_ADD(a, b) bhdf_round((a) + (b))
#define BHDF_SUB(a, b) bhdf_round((a) - (b))
#define BHDF_MUL(a, b) bhdf_round((a) * (b))
#endif

namespace bhgb {

struct DF {
  float hi, lo;
};

// a + b when |a| >= |b| (or a == 0), exactly, as hi + lo
BHDF_HD DF df_fast2sum(float a, float b) {
  const float s = BHDF_ADD(a, b);
  return DF{s, BHDF_SUB(b, BHDF_SUB(s, a))};
}
// a + b for any a, b, exactly, as hi + lo
BHDF_HD DF df_two_sum(float a, float b) {
  const float s = BHDF_ADD(a, b);
  const float bb = BHDF_SUB(s, a);
  return DF{s, BHDF_ADD(BHDF_SUB(a, BHDF_SUB(s, bb)), BHDF_SUB(b, bb))};
}
BHDF_HD DF df_add(DF a, DF b) {
  const DF s = df_two_sum(a.hi, b.hi);
  return df_fast2sum(s.hi, BHDF_ADD(s.lo, BHDF_ADD(a.lo, b.lo)));
}
BHDF_HD DF df_neg(DF a) { return DF{-a.hi, -a.lo}; }
BHDF_HD DF df_sub(DF a, DF b) { return df_add(a, df_neg(b)); }
BHDF_HD DF df_add_f(DF a, float b) {
  const DF s = df_two_sum(a.hi, b);
  return df_fast2sum(s.hi, BHDF_ADD(s.lo, a.lo));
}
BHDF_HD DF df_mul(DF a, DF b) {
  const float p = BHDF_MUL(a.hi, b.hi);
  const float e = fmaf(a.hi, b.hi, -p);
  return df_fast2sum(p, fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e)));
}
BHDF_HD DF df_fma(DF a, DF b, DF c) { return df_add(df_mul(a, b), c); }
BHDF_HD DF df_mul_f(DF a, float b) {
  const float p = BHDF_MUL(a.hi, b);
  const float e = fmaf(a.hi, b, -p);
  return df_fast2sum(p, fmaf(a.lo, b, e));
}
// a / b: one Newton correction of the float quotient (about 46 bits)
BHDF_HD DF df_div(DF a, DF b) {
  const float q1 = a.hi / b.hi;
  const DF r = df_sub(a, df_mul_f(b, q1));
  const float q2 = r.hi / b.hi;
  return df_fast2sum(q1, q2);
}
BHDF_HD DF df_from(double v) {
  const float h = float(v);
  return DF{h, float(v - double(h))};
}
BHDF_HD double df_to(DF a) { return double(a.hi) + double(a.lo); }
// a <= b and a < b, exactly
BHDF_HD bool df_le(DF a, DF b) { return a.hi < b.hi || (a.hi == b.hi && a.lo <= b.lo); }
BHDF_HD bool df_lt(DF a, DF b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }


// The classical RK4 step on x'' = x + 3 x^2 in its Runge-Kutta-Nystrom form
// (the operations of the FP32 and FP64 tracers' rk4_step) in double-float,
// with constants k = (h, h/2, h^2/4, h^2/2, h^2/6, h/6).
BHDF_HD DF df_fx(DF x) { return df_mul(x, df_add_f(df_mul_f(x, 3.f), 1.f)); }
BHDF_HD void df_rk4_step(DF& x, DF& w, const DF* k) {
  const DF k1 = df_fx(x);
  const DF s1 = df_fma(k[1], w, x);
  const DF k2 = df_fx(s1);
  const DF s2 = df_fma(k[2], k1, s1);
  const DF k3 = df_fx(s2);
  const DF s3a = df_fma(k[0], w, x);
  const DF s3 = df_fma(k[3], k2, s3a);
  const DF k4 = df_fx(s3);
  const DF A = df_add(k2, k3);
  const DF S = df_add(A, k1);
  x = df_fma(k[4], S, s3a);
  w = df_fma(k[5], df_add(df_add(S, A), k4), w);
}
// The step's constants for a step h given in double-float.
BHDF_HD void df_rk4_consts(DF h, DF* k) {
  const DF sixth{0x1.555556p-3f, -0x1.555556p-28f};  // 1/6
  const DF h2 = df_mul(h, h);
  k[0] = h;
  k[1] = df_mul_f(h, 0.5f);
  k[2] = df_mul_f(h2, 0.25f);
  k[3] = df_mul_f(h2, 0.5f);
  k[4] = df_mul(h2, sixth);
  k[5] = df_mul(h, sixth);
}

// Q(a, c) = k0 + a (k1 + a k3) + c (k2 + a k4 + c k5) for double-float
// coefficients k[i] = (hi, lo) and float a, c.
BHDF_HD DF df_quad_form(const float (*k)[2], float a, float c) {
  const DF k0{k[0][0], k[0][1]}, k1{k[1][0], k[1][1]}, k2{k[2][0], k[2][1]};
  const DF k3{k[3][0], k[3][1]}, k4{k[4][0], k[4][1]}, k5{k[5][0], k[5][1]};
  const DF ta = df_mul_f(df_add(k1, df_mul_f(k3, a)), a);
  const DF tc = df_mul_f(df_add(df_add(k2, df_mul_f(k4, a)), df_mul_f(k5, c)), c);
  return df_add(k0, df_add(ta, tc));
}

// (M/b)^2 - 1/27 of a ray whose |e|^2 and |F x e|^2 are ee and gg: the first
// integral of the photon orbit in double-float.
BHDF_HD DF df_first_integral(DF ee, DF gg, DF m2) {
  return df_add(df_mul(df_div(ee, gg), m2), DF{-0x1.2f684cp-5f, 0x1.2f684cp-32f});  // - 1/27
}

}  // namespace bhgb
