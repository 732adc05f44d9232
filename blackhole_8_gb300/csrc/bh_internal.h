// Internal types shared by the kernels (bh_kernels.cu) and the C ABI
// (bh_capi.cu). Nothing here is part of the public interface.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <cstdio>
#include <cstring>

#include "bh_gb300.h"

namespace bhgb {

// Texture resident in device memory, texels stored as BGRA8 (uchar4.x = B).
struct DevTexture {
  const uchar4* texels;
  int32_t width;
  int32_t height;
};

// An ordinary object (bh_object) resolved for the device: positions relative
// to the hole, in FP64 and rounded once to FP32.
struct DevObject {
  double p0[3];   // RECTANGLE, TRIANGLE: vertex()[1]; PLANE: position()
  double e1[3];   // RECTANGLE: vertex()[2] - vertex()[1]; TRIANGLE: vertex()[2] - vertex()[1]
  double e2[3];   // RECTANGLE: vertex()[4] - vertex()[1]; TRIANGLE: vertex()[3] - vertex()[1]
  double n[3];    // RECTANGLE: normalize(e1 x e2); PLANE: vector_z()
  double ax[3];   // PLANE: vector_x()
  double ay[3];   // PLANE: vector_y()
  double hw[3];   // PLANE: the hole's world position (the colour takes world x, y)
  double e1_len, e2_len;  // RECTANGLE: |e1|, |e2|
  double pattern;         // PLANE: ChessPattern2D size (<= 0: black)
  float p0_f[3], e1_f[3], e2_f[3], n_f[3], ax_f[3], ay_f[3], hw_f[3];
  float e1_len_f, e2_len_f, pattern_f;
  DevTexture tex;         // RECTANGLE: texels, or null (black)
  int32_t type;           // BH_OBJECT_*
  int32_t pad;
};

// A hole of the MULTI integrator, relative to the scene's hole: position and
// half its mass (the term m / (2 rho) of the conformal factor), in FP64 and
// rounded once to FP32 (one 16-byte load).
struct alignas(16) DevHole {
  double p[3];
  double hm;
  float p_f[3];
  float hm_f;
};

// One scene resolved for the device. Positions are relative to the hole.
// The FP64 block drives the FP64 paths; the FP32 block is the same data
// rounded once on the host.
//
// Ray generation (camera.h:55-59, blackhole_solution_test.cc:167-170): the
// reference's pv = focus_vector - vy*(W/2 - x) - vz*(H/2 - y) - hole and
// yv = normalize(F - pv). With E0 = F - pv(W/2, H/2) this is
// yv = normalize(E0 + vy*(W/2 - x) + vz*(H/2 - y)).
struct DevScene {
  double F[3];    // camera focus
  double E0[3];   // F - pv at the image centre (REF) or -focus_vector (PINHOLE)
  double vy[3];
  double vz[3];
  double dc[3];   // disc centre
  double dn[3];   // disc normal (fixed at construction, vector_object.h:325)
  double dv1[3];  // quad corner vertex()[1]
  double ds1[3];  // vertex()[2] - vertex()[1]
  double ds2[3];  // vertex()[4] - vertex()[1]
  double de1[3];  // polar basis e1 = s1 / |s1|
  double de2[3];  // polar basis e2 = n x e1
  double mass, b_c, r_h;      // M, 3 sqrt(3) M, 2 M
  double r_in, r_out;
  double s1_len, s2_len;
  double half_w, half_h;      // W / 2.0, H / 2.0
  double Fhat[3], Flen, x0;   // RK4: F / |F|, |F|, M / |F| - 1/3 (the same for every ray)
  double g0, dnF;             //   x0^2 (1 + 2 x0) (w0^2 = eps + g0), disc normal . F / |F|

  float F_f[3], E0_f[3], vy_f[3], vz_f[3];
  float dc_f[3], dn_f[3], dv1_f[3], ds1_f[3], ds2_f[3], de1_f[3], de2_f[3];
  float mass_f, b_c_f, r_h_f, r_in_f, r_out_f, s1_len_f, s2_len_f, half_w_f, half_h_f;
  float inv_mass_f;
  float Fhat_f[3], Flen_f, x0_f;
  float g0_f, dnF_f;
  float b_lip;                // bound on |b(x+1) - b(x)| / M along an image row (row_b_lipschitz)
  // MIXED, double-float (hi, lo) copies for the FP32 passes' rare exact paths:
  // |e|^2 and |F x e|^2 as quadratic forms in the pixel offsets (a, c), six
  // coefficients each (resolve_derived), M^2, and M, r_in, r_out for the
  // crossing refinement
  float eq_e[6][2], eq_g[6][2], m2_df[2];
  float mass_df[2], r_in_df[2], r_out_df[2];
  // FP32 terms every RK4 ray reads, grouped in 16-byte vectors so that a
  // group is one load (resolve_derived; kHot* indices)
  float4 hot[10];
  int4 hot_i;                 // kScene* flags, width, height, 0 (resolve_frame_flags)
  // FP32 polar disc lookup of a disc centred on the hole (resolve_derived)
  int32_t disc_centred;       // 1 when the disc centre is the hole's position
  float disc_tx_scale_f;      // disc texture width / (r_out - r_in)
  float de1F_f, de2F_f;       // e1 . F^, e2 . F^

  DevTexture disc_tex;
  DevTexture bg_tex;
  int32_t width, height;
  int32_t disc_on, disc_map, has_bg;
  int32_t tiles_x;            // ceil(W / 8): persistent schedule, 8x4 tiles
  int32_t tiles_x_shift;      // tile / tiles_x == (tile * tiles_x_magic) >> tiles_x_shift
  uint64_t tiles_x_magic;     //   for every tile index below 2^31 (DivMagic)
  int64_t ray_begin;          // first ray index of this scene (persistent)
  int64_t block_begin;        // GRID / HYBRID: index of this frame's first block (assign_grid_blocks)
  int32_t blocks_x;           //   blocks per block row of this frame
  int32_t pad_blocks;
  const DevObject* objects;   // this scene's objects (n_objects of them)
  int32_t n_objects;
  int32_t n_holes;            // MULTI: holes[0] is the scene's hole, then the extra holes
  double mcen[3];             // MULTI: the holes' centre of mass (escape sphere centre)
  double r_esc;               // MULTI: escape sphere radius, r_escape * total mass
  float mcen_f[3], r_esc_f;
  DevHole holes[BH_MAX_HOLES];
  uint8_t* pixels;
  uint8_t* cls;
  float* aux;
};

// The groups of DevScene::hot: (x, y, z, w) of each.
enum : int {
  kHotE0 = 0,    // E0, half_w
  kHotVy = 1,    // vy, half_h
  kHotVz = 2,    // vz, Flen
  kHotF = 3,     // F, 1 / M
  kHotDn = 4,    // disc normal, normal . F^
  kHotFhat = 5,  // F^, x0
  kHotMass = 6,  // M, g0, r_in, r_out
  kHotDe1 = 7,   // polar disc e1, e1 . F^
  kHotDe2 = 8,   // polar disc e2, e2 . F^
  kHotDisc = 9,  // disc texture width / (r_out - r_in), -, -, -
};

// DevScene::hot_i.x flags.
enum : int {
  kSceneDisc = 1,           // disc_on
  kSceneBg = 2,             // has_bg
  kSceneDiscPolarCentred = 4,  // POLAR mapping of a disc centred on the hole
  kSceneAux = 8,            // the frame takes aux output
  kSceneCls = 16,           // the frame takes hit classes
};

// The flags group of a resolved scene whose frame pointers are set.
inline void resolve_frame_flags(DevScene* d) {
  d->hot_i = int4{(d->disc_on ? kSceneDisc : 0) | (d->has_bg ? kSceneBg : 0) |
                      (d->disc_map == BH_DISC_MAP_POLAR && d->disc_centred ? kSceneDiscPolarCentred : 0) |
                      (d->aux ? kSceneAux : 0) | (d->cls ? kSceneCls : 0),
                  d->width, d->height, 0};
}

// Device-side counters of one render (reset before every render).
struct DevCounters {
  unsigned long long next_ray;      // persistent work queue head
  unsigned long long band_count;    // entries appended to the band list
  unsigned long long band_next;     // band work queue head
  unsigned long long steps;
  unsigned long long band_steps;
  unsigned long long band_rays;
  unsigned long long band_overflow;
  unsigned long long rays;
  unsigned long long flags;
  unsigned long long blocks_started;  // MIXED FP64 pass: blocks that have begun
  unsigned long long pad[6];
  // persistent MIXED: the band list's counting sort (kBandKeys buckets of log2 |eps|)
  unsigned int band_hist[64];
  unsigned int band_cursor[64];
};
constexpr int kBandKeys = 64;

enum : unsigned long long {
  kFlagBandQueueFull = 1ull << 0,
  kFlagBandLaunchFailed = 1ull << 1,  // device-side launch of the FP32 pass failed
};

// Constants of the RK4 integration in one precision, on x = u - 1/3.
template <typename R>
struct Rk4Consts {
  R h, hh, q, q2, h26, h6;  // h, h/2, h^2/4, h^2/2, h^2/6, h/6
  R h8;                     // h^2/8 (the FP32 three-stage step)
  R x_esc, x_hor;           // escape: x <= u_esc - 1/3; horizon: x >= 1/2 - 1/3
  R u_esc;                  // M / r_escape
  int32_t kmax;
};

template <typename R>
inline Rk4Consts<R> make_rk4_consts(double h, double u_escape, int kmax) {
  Rk4Consts<R> c;
  c.h = R(h);
  c.hh = R(h * 0.5);
  c.q = R(h * h * 0.25);
  c.q2 = R(h * h * 0.5);
  c.h26 = R(h * h / 6.0);
  c.h6 = R(h / 6.0);
  c.h8 = R(h * h * 0.125);
  c.x_esc = R(u_escape - 1.0 / 3.0);
  c.x_hor = R(0.5 - 1.0 / 3.0);
  c.u_esc = R(u_escape);
  c.kmax = kmax;
  return c;
}

struct LaunchParams {
  const DevScene* scenes;
  int32_t n_scenes;
  int32_t integrator;
  int32_t precision;
  int32_t format;
  int32_t raygen;
  int32_t max_steps;
  Rk4Consts<float> c32;       // bulk step, FP32
  Rk4Consts<double> c64;      // bulk step, FP64
  Rk4Consts<double> cband;    // band step, FP64 (MIXED)
  float band_df[8][2];        // cband's h, h/2, h^2/4, h^2/2, h^2/6, h/6, x_esc, x_hor in double-float
  float setup_band;           // |b - b_c| / M below which MIXED takes eps from FP64
  float class_band;           // persistent MIXED: |b - b_c| / M (FP32 b) below which the
                              //   classification takes the FP64 band test (class_band_for)
  double eps_band_lo;         // the FP64 band in terms of eps = 1/(b/M)^2 - 1/27:
  double eps_band_hi;         //   eps(b_c + band) < eps < eps(b_c - band)
  float eps_band_df[4];       //   the same bounds in double-float: lo (hi, lo), hi (hi, lo)
  int64_t total_rays;         // persistent: sum of padded scene ray counts
  DevCounters* counters;
  uint32_t* band_list;        // persistent MIXED: band rays, longest first (sorted by |eps|)
  uint32_t* band_tmp;         //   the classification's unsorted list
  uint8_t* band_key;          //   and its sort keys
  uint32_t band_capacity;
  float band_key_scale;       //   1 / |eps| at the band's edge
  int32_t refill_threshold;
  int32_t slice_steps;
  int32_t band_lanes;
  int32_t band_serial;        // MIXED: 1 = FP32 pass, then FP64 pass; 2 = FP64 pass, then FP32 pass (from the host)
  int32_t mixed_blocks;       // persistent MIXED: grid of the FP32 pass the FP64 pass launches (0: none)
  int32_t rays_per_thread;    // GRID: consecutive block tiles down the image per block (>= 1)
  int32_t hybrid;             // HYBRID MIXED: the FP32 pass is grid_kernel with band rays deferred
  int32_t grid_dim[3];        //   its grid and block (the FP64 pass launches it from the device)
  int32_t block_dim[2];
  int32_t drain_only;         //   host launch after the FP64 pass: traces only if the device launch failed
  int32_t frame_blocks;       // GRID / HYBRID: blocks per frame when every frame has as many (else 0)
};

// Bound on how much b / M changes between neighbouring pixels of a row. The
// ray direction is e = E0 + a vy + c vz (a, c: pixel offsets) and
// b = |F x e| / |e|, so |db/da| <= |F| |vy| / |e|, and |e| is at least the
// distance from the origin to the image plane E0 + span(vy, vz). Infinite
// when that plane passes through the origin (every segment is then tested).
inline float row_b_lipschitz(const double F[3], const double E0[3], const double vy[3], const double vz[3],
                             double mass) {
  const double n[3] = {vy[1] * vz[2] - vy[2] * vz[1], vy[2] * vz[0] - vy[0] * vz[2], vy[0] * vz[1] - vy[1] * vz[0]};
  const double nn = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
  const double dist = nn > 0 ? std::fabs(E0[0] * n[0] + E0[1] * n[1] + E0[2] * n[2]) / nn : 0.0;
  const double f = std::sqrt(F[0] * F[0] + F[1] * F[1] + F[2] * F[2]);
  const double v = std::sqrt(vy[0] * vy[0] + vy[1] * vy[1] + vy[2] * vy[2]);
  if (!(dist > 0) || !(mass > 0)) return INFINITY;
  return float(f * v / (dist * mass));
}

// The FP32 prefilters on b of the mixed tracer. A band ray has
// |b - b_c| < band exactly, and b in FP32 differs from it by at most
// ~1.2e-7 |F| (the rounding of the ray direction e = E0 + a vy + c vz) plus
// ~2e-7 b (the cross product and the norms): ~5e-6 M with the camera at 30 M.
// The classification tests the rays within band + 1e-4 M + 1e-6 |F| (its
// per-scene term added in the kernel), the FP32 pass's setup the rays within
// setup_band, raised to band + 2e-3 M when smaller. Both edges lie far
// outside the FP64 band by more than that rounding, so the two kernels (each
// with its own FP32 b) take the same decision for every ray: only the exact
// band test, the same code in both, decides. The classification then skips
// the exact test for all but a ring about two pixels wide around b_c.
inline float class_band_for(double band) { return band > 0 ? float(band + 1e-4) : 0.f; }
inline float setup_band_for(double band, double setup_band) {
  return float(band > 0 && band + 2e-3 > setup_band ? band + 2e-3 : setup_band);
}

// Resolves a bh_object for the device, relative to the hole at h (host).
// Edges are formed in world coordinates as the reference forms them;
// the rectangle's normal is cv::normalize(e1 x e2) = v * (1 / |v|).
// The RK4 ray's per-scene constants: every ray of a scene starts at F (the
// camera relative to the hole), so the unit vector F / |F|, which is also the
// first axis of each ray's orbital basis rotated to the camera, and the
// initial x = M / |F| - 1/3 are the scene's.
inline void resolve_rk4_constants(double* Fhat, float* Fhat_f, double* Flen, float* Flen_f, double* x0, float* x0_f,
                                  const double F[3], double mass) {
  const double L = std::sqrt(F[0] * F[0] + F[1] * F[1] + F[2] * F[2]);
  const double k = L > 0 ? 1.0 / L : 0.0;
  for (int i = 0; i < 3; ++i) {
    Fhat[i] = F[i] * k;
    Fhat_f[i] = float(Fhat[i]);
  }
  *Flen = L;
  *Flen_f = float(L);
  *x0 = L > 0 ? mass / L - 1.0 / 3.0 : 0.0;
  *x0_f = float(*x0);
}

// (hi, lo) float split of v: hi = v rounded to float, lo = the rest rounded
inline void split_df(double v, float* out) {
  out[0] = float(v);
  out[1] = float(v - double(out[0]));
}

// Per-scene values derived from a resolved scene (mass, radii, disc basis,
// textures, camera vectors and RK4 constants set): the double-float copies,
// the RK4 setup's per-scene terms and the FP32 polar disc lookup's constants. With the pixel offsets a = W/2 - x, c = H/2 - y, the ray direction is
// e = E0 + a vy + c vz, so |e|^2 and |F x e|^2 = |G0 + a G1 + c G2|^2 (Gi = F x
// E0, F x vy, F x vz) are quadratic forms in (a, c); their coefficients, in
// the order of Q = k0 + a (k1 + a k3) + c (k2 + a k4 + c k5), are formed here
// in FP64 and split. The mixed tracer's first integral of a near-critical ray
// is then M^2 |e|^2 / |F x e|^2 - 1/27 in double-float.
inline void resolve_derived(DevScene* d) {
  auto dot = [](const double* u, const double* v) { return u[0] * v[0] + u[1] * v[1] + u[2] * v[2]; };
  auto cross = [](const double* u, const double* v, double* o) {
    o[0] = u[1] * v[2] - u[2] * v[1];
    o[1] = u[2] * v[0] - u[0] * v[2];
    o[2] = u[0] * v[1] - u[1] * v[0];
  };
  auto form = [&](const double* v0, const double* v1, const double* v2, float (*k)[2]) {
    const double c[6] = {dot(v0, v0), 2 * dot(v0, v1), 2 * dot(v0, v2), dot(v1, v1), 2 * dot(v1, v2), dot(v2, v2)};
    for (int i = 0; i < 6; ++i) split_df(c[i], k[i]);
  };
  form(d->E0, d->vy, d->vz, d->eq_e);
  double g0[3], g1[3], g2[3];
  cross(d->F, d->E0, g0);
  cross(d->F, d->vy, g1);
  cross(d->F, d->vz, g2);
  form(g0, g1, g2, d->eq_g);
  split_df(d->mass * d->mass, d->m2_df);
  split_df(d->mass, d->mass_df);
  split_df(d->r_in, d->r_in_df);
  split_df(d->r_out, d->r_out_df);
  d->g0 = d->x0 * d->x0 * (1.0 + 2.0 * d->x0);
  d->g0_f = float(d->g0);
  d->dnF = dot(d->dn, d->Fhat);
  d->dnF_f = float(d->dnF);
  d->disc_centred = d->dc[0] == 0 && d->dc[1] == 0 && d->dc[2] == 0 ? 1 : 0;
  d->disc_tx_scale_f = d->r_out > d->r_in ? float(d->disc_tex.width / (d->r_out - d->r_in)) : 0.f;
  d->de1F_f = float(dot(d->de1, d->Fhat));
  d->de2F_f = float(dot(d->de2, d->Fhat));
  auto f4 = [](const float* v, float w) { return float4{v[0], v[1], v[2], w}; };
  d->hot[kHotE0] = f4(d->E0_f, d->half_w_f);
  d->hot[kHotVy] = f4(d->vy_f, d->half_h_f);
  d->hot[kHotVz] = f4(d->vz_f, d->Flen_f);
  d->hot[kHotF] = f4(d->F_f, d->inv_mass_f);
  d->hot[kHotDn] = f4(d->dn_f, d->dnF_f);
  d->hot[kHotFhat] = f4(d->Fhat_f, d->x0_f);
  d->hot[kHotMass] = float4{d->mass_f, d->g0_f, d->r_in_f, d->r_out_f};
  d->hot[kHotDe1] = f4(d->de1_f, d->de1F_f);
  d->hot[kHotDe2] = f4(d->de2_f, d->de2F_f);
  d->hot[kHotDisc] = float4{d->disc_tx_scale_f, 0.f, 0.f, 0.f};
}

// The band step's constants in double-float (the band pass integrates in
// double-float on the FP32 pipe).
inline void split_band_consts(const Rk4Consts<double>& c, float (*out)[2]) {
  const double v[8] = {c.h, c.hh, c.q, c.q2, c.h26, c.h6, c.x_esc, c.x_hor};
  for (int i = 0; i < 8; ++i) split_df(v[i], out[i]);
}

// The FP64 band of the mixed tracer in terms of eps (empty for band 0), with
// the sort-key scale and the double-float copies of the bounds.
inline void set_band_eps(double band, double* eps_lo, double* eps_hi, float* key_scale, float eps_df[4]) {
  const double bc = 3.0 * std::sqrt(3.0), lo = bc + band, hi = bc - band;
  *eps_lo = band == 0 ? 0.0 : 1.0 / (lo * lo) - 1.0 / 27.0;
  *eps_hi = band == 0 ? 0.0 : (hi > 0 ? 1.0 / (hi * hi) - 1.0 / 27.0 : 1e300);
  const double edge = std::fmax(std::fabs(*eps_lo), std::fabs(*eps_hi));
  *key_scale = edge > 0 ? float(1.0 / edge) : 0.f;
  split_df(*eps_lo, eps_df);
  split_df(std::fmin(*eps_hi, 1e30), eps_df + 2);  // beyond every eps when b_c - band <= 0
}

inline void resolve_object(const bh_object& b, const double h[3], DevTexture tex, DevObject* d) {
  std::memset(d, 0, sizeof(*d));
  d->type = b.type;
  auto put = [](double* dst, float* dstf, const double* v) {
    for (int k = 0; k < 3; ++k) {
      dst[k] = v[k];
      dstf[k] = float(v[k]);
    }
  };
  const double p0[3] = {b.v[0][0] - h[0], b.v[0][1] - h[1], b.v[0][2] - h[2]};
  put(d->p0, d->p0_f, p0);
  if (b.type == BH_OBJECT_PLANE) {
    put(d->n, d->n_f, b.axis_z);
    put(d->ax, d->ax_f, b.axis_x);
    put(d->ay, d->ay_f, b.axis_y);
    put(d->hw, d->hw_f, h);
    d->pattern = b.pattern_size;
    d->pattern_f = float(b.pattern_size);
    return;
  }
  const int third = b.type == BH_OBJECT_RECTANGLE ? 3 : 2;
  double e1[3], e2[3];
  for (int k = 0; k < 3; ++k) {
    e1[k] = b.v[1][k] - b.v[0][k];
    e2[k] = b.v[third][k] - b.v[0][k];
  }
  put(d->e1, d->e1_f, e1);
  put(d->e2, d->e2_f, e2);
  if (b.type == BH_OBJECT_RECTANGLE) {
    const double n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
    const double len = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    const double k = len > 0 ? 1.0 / len : 0.0;
    const double nn[3] = {n[0] * k, n[1] * k, n[2] * k};
    put(d->n, d->n_f, nn);
    d->e1_len = std::sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
    d->e2_len = std::sqrt(e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2]);
    d->e1_len_f = float(d->e1_len);
    d->e2_len_f = float(d->e2_len);
    d->tex = tex;
  }
}

// Exact division of 31-bit indices by a fixed divisor d >= 1 with a multiply
// and a shift (Granlund and Montgomery, "Division by invariant integers
// using multiplication", 1994): with l = ceil(log2 d), s = 31 + l and
// m = floor(2^s / d) + 1, floor(n m / 2^s) = floor(n / d) for 0 <= n < 2^31;
// m < 2^33, so n m fits 64 bits. Frames are at most 32768 x 32768, i.e.
// below 2^25 tiles.
struct DivMagic {
  uint64_t m;
  int32_t s;
};
inline DivMagic div_magic(uint32_t d) {
  int l = 0;
  while ((uint64_t(1) << l) < d) ++l;
  const int s = 31 + l;
  return {(uint64_t(1) << s) / d + 1, s};
}

// The band buffer of the persistent mixed tracer, in 32-bit words: the list,
// the unsorted list and one key byte per entry, `cap` entries each.
constexpr size_t band_words(uint32_t cap) { return 2 * size_t(cap) + (size_t(cap) + 3) / 4; }
inline void carve_band(uint32_t* base, uint32_t cap, uint32_t** list, uint32_t** tmp, uint8_t** key) {
  *list = base;
  *tmp = base + cap;
  *key = reinterpret_cast<uint8_t*>(base + 2 * size_t(cap));
}
inline float band_key_scale_for(double eps_lo, double eps_hi) {
  const double edge = std::fmax(std::fabs(eps_lo), std::fabs(eps_hi));
  return edge > 0 ? float(1.0 / edge) : 0.f;
}

// True when a render of these options lists the FP64 band rays and traces
// them in a persistent pass of their own (MIXED on the PERSISTENT or HYBRID
// schedule): it needs the band list.
inline bool uses_band_pass(const bh_render_options& o) {
  return o.precision == BH_PRECISION_MIXED &&
         (o.schedule == BH_SCHEDULE_PERSISTENT || o.schedule == BH_SCHEDULE_HYBRID);
}

// The checks of bh_render_options that need no context, shared by every
// render entry point (bh_render, bh_render_device, bh_sequence_create,
// bh_render_noalloc) so that they accept and refuse the same options.
// Returns BH_OK, or a status with a message of at most `len` bytes in `msg`.
inline int render_options_problem(const bh_render_options& o, char* msg, size_t len) {
  auto bad = [&](int code, const char* text) {
    std::snprintf(msg, len, "%s", text);
    return code;
  };
  if (o.integrator != BH_INTEGRATOR_REF_TRAPEZOID && o.integrator != BH_INTEGRATOR_RK4 &&
      o.integrator != BH_INTEGRATOR_FLAT && o.integrator != BH_INTEGRATOR_MULTI) {
    std::snprintf(msg, len, "unknown integrator %d", o.integrator);
    return BH_ERR_INVALID_ARGUMENT;
  }
  if (o.precision < BH_PRECISION_FP32 || o.precision > BH_PRECISION_MIXED) {
    std::snprintf(msg, len, "unknown precision %d", o.precision);
    return BH_ERR_INVALID_ARGUMENT;
  }
  if (o.integrator != BH_INTEGRATOR_RK4 && o.precision == BH_PRECISION_MIXED)
    return bad(BH_ERR_UNSUPPORTED, "MIXED precision applies to the RK4 integrator only");
  if ((o.integrator == BH_INTEGRATOR_FLAT || o.integrator == BH_INTEGRATOR_MULTI) && o.schedule != BH_SCHEDULE_GRID)
    return bad(BH_ERR_UNSUPPORTED, "the FLAT and MULTI integrators run on the GRID schedule");
  if (o.raygen != BH_RAYGEN_REF && o.raygen != BH_RAYGEN_PINHOLE) {
    std::snprintf(msg, len, "unknown raygen %d", o.raygen);
    return BH_ERR_INVALID_ARGUMENT;
  }
  if (o.format < BH_FORMAT_BGRA8 || o.format > BH_FORMAT_RGBA8) {
    std::snprintf(msg, len, "unknown format %d", o.format);
    return BH_ERR_INVALID_ARGUMENT;
  }
  if (o.schedule != BH_SCHEDULE_GRID && o.schedule != BH_SCHEDULE_PERSISTENT && o.schedule != BH_SCHEDULE_HYBRID) {
    std::snprintf(msg, len, "unknown schedule %d", o.schedule);
    return BH_ERR_INVALID_ARGUMENT;
  }
  if (o.schedule != BH_SCHEDULE_GRID && (o.integrator != BH_INTEGRATOR_RK4 || o.precision == BH_PRECISION_FP64))
    return bad(BH_ERR_UNSUPPORTED, "the persistent and hybrid schedules run RK4 in FP32 or MIXED precision");
  if (!(o.step > 0 && o.step <= 1.0)) return bad(BH_ERR_INVALID_ARGUMENT, "step must be in (0, 1]");
  if (o.max_steps < 1 || o.max_steps > 100000000)
    return bad(BH_ERR_INVALID_ARGUMENT, "max_steps must be in [1, 1e8]");
  if (!(o.r_escape > 2.0) || !std::isfinite(o.r_escape))
    return bad(BH_ERR_INVALID_ARGUMENT, "r_escape must exceed the horizon (2 M)");
  if (!(o.band >= 0) || !std::isfinite(o.band)) return bad(BH_ERR_INVALID_ARGUMENT, "band must be >= 0");
  if (!(o.band_step > 0 && o.band_step <= 1.0)) return bad(BH_ERR_INVALID_ARGUMENT, "band_step must be in (0, 1]");
  if (!(o.setup_band >= 0) || !std::isfinite(o.setup_band))
    return bad(BH_ERR_INVALID_ARGUMENT, "setup_band must be >= 0");
  if (o.slice_steps < 4 || o.slice_steps > 4096)
    return bad(BH_ERR_INVALID_ARGUMENT, "slice_steps must be in [4, 4096]");
  if (o.band_lanes < 1 || o.band_lanes > 32) return bad(BH_ERR_INVALID_ARGUMENT, "band_lanes must be in [1, 32]");
  if (o.band_serial < 0 || o.band_serial > 2) return bad(BH_ERR_INVALID_ARGUMENT, "band_serial must be 0, 1 or 2");
  if (o.block_x < 1 || o.block_y < 1 || o.block_x * o.block_y > 256 || (o.block_x * o.block_y) % 32 != 0)
    return bad(BH_ERR_INVALID_ARGUMENT, "grid block must hold a multiple of 32 threads, at most 256");
  // the HYBRID band pass's blocks may hold 512 threads (persistent_band_kernel's bound)
  const int max_threads = o.schedule == BH_SCHEDULE_HYBRID ? 512 : 256;
  if (o.threads_per_block < 32 || o.threads_per_block > max_threads || o.threads_per_block % 32 != 0)
    return bad(BH_ERR_INVALID_ARGUMENT, o.schedule == BH_SCHEDULE_HYBRID
                                            ? "threads_per_block must be a multiple of 32 in [32, 512] (HYBRID)"
                                            : "threads_per_block must be a multiple of 32 in [32, 256]");
  if (o.blocks_per_sm < 0 || o.blocks_per_sm > 64) return bad(BH_ERR_INVALID_ARGUMENT, "blocks_per_sm must be in [0, 64]");
  if (o.refill_threshold < 1 || o.refill_threshold > 32)
    return bad(BH_ERR_INVALID_ARGUMENT, "refill_threshold must be in [1, 32]");
  if (o.rays_per_thread < 0 || o.rays_per_thread > 128)
    return bad(BH_ERR_INVALID_ARGUMENT, "rays_per_thread must be in [0, 128]");
  return BH_OK;
}

// GRID / HYBRID blocks of a frame: block_x columns by rays_per_thread tiles of
// block_y rows.
inline int64_t grid_blocks_x(int w, int bx) { return (int64_t(w) + bx - 1) / bx; }
inline int64_t grid_blocks_y(int h, int by, int rpt) {
  const int64_t rows = int64_t(by) * (rpt > 0 ? rpt : 1);
  return (int64_t(h) + rows - 1) / rows;
}
inline int64_t grid_blocks(int w, int h, int bx, int by, int rpt) {
  return grid_blocks_x(w, bx) * grid_blocks_y(h, by, rpt);
}
// Numbers the frames' GRID blocks back to back, so that a launch over frames
// of uneven sizes has no empty blocks (block_begin, blocks_x of each record);
// returns the launch's block count, which launch_grid computes the same way.
inline int64_t assign_grid_blocks(DevScene* d, int n, int bx, int by, int rpt) {
  int64_t total = 0;
  for (int i = 0; i < n; ++i) {
    d[i].blocks_x = int32_t(grid_blocks_x(d[i].width, bx));
    d[i].block_begin = total;
    total += grid_blocks(d[i].width, d[i].height, bx, by, rpt);
  }
  return total;
}

// Launchers (bh_kernels.cu). All enqueue on `stream` and return a cudaError_t.
// objects: the FLAT integrator or a scene with objects (grid_objects_kernel).
cudaError_t launch_grid(const LaunchParams& p, const int32_t* scene_w, const int32_t* scene_h,
                        int block_x, int block_y, cudaStream_t stream, bool objects = false);
// MIXED: classifies the FP64-band rays, runs the FP64 pass, which launches
// the FP32 pass from the device once all its blocks are resident, then a
// host-launched FP32 pass that drains what is left of the ray queue
// (band_serial 1: the FP32 pass, then the FP64 pass, both from the host;
// 2: the FP64 pass without its device-side launch, then the FP32 pass).
cudaError_t launch_persistent(const LaunchParams& p, int threads, int blocks, cudaStream_t stream);
// HYBRID: as launch_persistent, with the FP32 pass on the GRID schedule
// (rays_per_thread block tiles per block, band rays deferred); the host's
// launch after the FP64 pass, one wave of blocks looping over the frame
// blocks, traces only if the FP64 pass did not launch the FP32 pass.
// FP32 precision: launch_grid.
cudaError_t launch_hybrid(const LaunchParams& p, const int32_t* scene_w, const int32_t* scene_h, int block_x,
                          int block_y, int band_threads, cudaStream_t stream);
cudaError_t persistent_occupancy(const LaunchParams& p, int threads, int* blocks_per_sm);
cudaError_t launch_fp32_probe(float* sink, int blocks, int threads, int iters, cudaStream_t stream);
cudaError_t launch_fp64_probe(double* sink, int blocks, int threads, int iters, cudaStream_t stream);

}  // namespace bhgb
