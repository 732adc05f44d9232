// C ABI of the GB300 geodesic ray tracer (declared in include/bh_gb300.h).
//
// Host side of the drop-in for the reference's frame body
// (blackhole_solution_test.cc:161-298): validates POD scenes, resolves them
// into DevScene records (positions relative to the hole, FP64 + FP32 copies),
// stages them through pinned memory, launches the kernels on the context's
// stream and, for bh_render, copies the frames back.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "bh_adjoint.h"
#include "bh_internal.h"

using bhgb::DevCounters;
using bhgb::DevObject;
using bhgb::DevScene;
using bhgb::DevTexture;
using bhgb::LaunchParams;

namespace {

struct TexEntry {
  uchar4* texels = nullptr;
  int32_t width = 0, height = 0;
  bool alive = false;
};

template <typename T>
struct PinnedBuf {
  T* ptr = nullptr;
  size_t cap = 0;
};

template <typename T>
struct DevBuf {
  T* ptr = nullptr;
  size_t cap = 0;
};

}  // namespace

// bh_render with host frames: chunks of scenes whose copy-back overlaps the
// next chunk's render.
constexpr int kMaxChunks = 4;

struct bh_ctx {
  bool direct_host = false;  // the last render wrote its frames into host memory from the kernels
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  std::vector<TexEntry> textures;
  PinnedBuf<DevScene> h_scenes;
  DevBuf<DevScene> d_scenes;
  PinnedBuf<DevObject> h_objects;
  DevBuf<DevObject> d_objects;
  DevCounters* d_counters = nullptr;
  DevCounters* h_counters = nullptr;
  DevBuf<uint32_t> band_list;
  DevBuf<uint8_t> out_arena;
  cudaEvent_t ev_start = nullptr, ev_stop = nullptr, ev_staged = nullptr;
  cudaStream_t copy_stream = nullptr;   // bh_render: frame copy-back beside the next chunk's render
  cudaEvent_t ev_chunk[kMaxChunks] = {};
  bool staged_pending = false;
  bool stats_valid = false;
  uint64_t h2d_bytes = 0, d2h_bytes = 0;
  bh_render_stats last{};
  // differentiable render
  PinnedBuf<bhgb::adj::AdjScene> h_adj;
  DevBuf<bhgb::adj::AdjScene> d_adj;
  DevBuf<uint8_t> adj_ckpt, adj_ckpt_band;
  DevBuf<uint2> adj_band;
  DevBuf<double> adj_acc;
  PinnedBuf<double> h_adj_acc;
  DevBuf<unsigned long long> adj_counters;
  cudaStream_t side_stream = nullptr;   // MIXED adjoint: the band pass
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
};

struct bh_sequence {
  bh_ctx* ctx = nullptr;
  int32_t n = 0;
  bh_render_options opts{};
  std::vector<bh_scene> scenes;
  std::vector<bh_frame> frames;
  DevScene* h_scenes = nullptr;   // pinned, owned
  DevScene* d_scenes = nullptr;   // owned
  DevObject* h_objects = nullptr; // pinned, owned (n_objects_total of them)
  DevObject* d_objects = nullptr; // owned
  int32_t n_objects_total = 0;
  DevCounters* d_counters = nullptr;
  uint32_t* band_list = nullptr;
  uint32_t band_capacity = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t ev_done = nullptr;
  bool launched = false;
};

namespace {

int set_err(bh_ctx* ctx, int code, const char* fmt, ...) {
  if (ctx) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    ctx->err = buf;
  }
  return code;
}

int cuda_err(bh_ctx* ctx, cudaError_t e, const char* what) {
  int code = BH_ERR_CUDA;
  if (e == cudaErrorMemoryAllocation) code = BH_ERR_OUT_OF_MEMORY;
  if (e == cudaErrorIllegalAddress || e == cudaErrorLaunchFailure || e == cudaErrorIllegalInstruction ||
      e == cudaErrorMisalignedAddress || e == cudaErrorHardwareStackError)
    code = BH_ERR_DEVICE_FAULT;
  return set_err(ctx, code, "%s: %s", what, cudaGetErrorString(e));
}

#define BH_CUDA(ctx, call)                                   \
  do {                                                       \
    cudaError_t e_ = (call);                                 \
    if (e_ != cudaSuccess) return cuda_err(ctx, e_, #call);  \
  } while (0)

template <typename T>
int ensure_dev(bh_ctx* ctx, DevBuf<T>& b, size_t n) {
  if (b.cap >= n) return BH_OK;
  if (b.ptr) cudaFree(b.ptr);
  b.ptr = nullptr;
  b.cap = 0;
  BH_CUDA(ctx, cudaMalloc(&b.ptr, n * sizeof(T)));
  b.cap = n;
  return BH_OK;
}

template <typename T>
int ensure_pinned(bh_ctx* ctx, PinnedBuf<T>& b, size_t n) {
  if (b.cap >= n) return BH_OK;
  if (b.ptr) cudaFreeHost(b.ptr);
  b.ptr = nullptr;
  b.cap = 0;
  BH_CUDA(ctx, cudaMallocHost(&b.ptr, n * sizeof(T)));
  b.cap = n;
  return BH_OK;
}

bool finite3(const double* v) { return std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]); }
double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
void cross3(const double* a, const double* b, double* c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

int bytes_per_pixel(int32_t format) { return format == BH_FORMAT_BGR8 ? 3 : 4; }

void resolve_defaults(const bh_render_options* in, bh_render_options* out) {
  bh_default_options(out);
  if (!in) return;
  *out = *in;
  bh_render_options d;
  bh_default_options(&d);
  if (out->max_steps == 0) out->max_steps = d.max_steps;
  if (out->step == 0) out->step = d.step;
  if (out->r_escape == 0) out->r_escape = d.r_escape;
  if (out->band < 0) out->band = d.band;
  if (out->block_x == 0) out->block_x = d.block_x;
  if (out->block_y == 0) out->block_y = d.block_y;
  if (out->threads_per_block == 0) out->threads_per_block = d.threads_per_block;
  if (out->refill_threshold == 0) out->refill_threshold = d.refill_threshold;
  if (out->band_step == 0) out->band_step = d.band_step;
  if (out->setup_band < 0) out->setup_band = d.setup_band;
  if (out->slice_steps == 0) out->slice_steps = d.slice_steps;
  if (out->band_lanes == 0) out->band_lanes = d.band_lanes;
  if (out->rays_per_thread == 0) out->rays_per_thread = d.rays_per_thread;
}

int validate_options(bh_ctx* ctx, const bh_render_options& o) {
  char msg[160];
  if (int rc = bhgb::render_options_problem(o, msg, sizeof(msg))) return set_err(ctx, rc, "%s", msg);
  return BH_OK;
}

int texture_ok(bh_ctx* ctx, int32_t id) {
  return id >= 0 && id < (int32_t)ctx->textures.size() && ctx->textures[id].alive;
}

int validate_objects(bh_ctx* ctx, const bh_scene& s, int i, const bh_render_options& o) {
  if (s.n_objects < 0 || s.n_objects > BH_MAX_OBJECTS)
    return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "scene %d: n_objects must be in [0, %d]", i, BH_MAX_OBJECTS);
  if (s.n_objects == 0) return BH_OK;
  if (!s.objects) return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "scene %d: objects is NULL", i);
  if (o.schedule != BH_SCHEDULE_GRID || o.precision == BH_PRECISION_MIXED)
    return set_err(ctx, BH_ERR_UNSUPPORTED, "scene %d: objects need the GRID schedule in FP32 or FP64", i);
  for (int j = 0; j < s.n_objects; ++j) {
    const bh_object& b = s.objects[j];
    if (!finite3(b.v[0]) || !finite3(b.v[1]) || !finite3(b.v[2]) || !finite3(b.v[3]) || !finite3(b.axis_x) ||
        !finite3(b.axis_y) || !finite3(b.axis_z) || !std::isfinite(b.pattern_size))
      return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "scene %d object %d: non-finite value", i, j);
    if (b.type == BH_OBJECT_RECTANGLE) {
      if (b.texture != -1 && !texture_ok(ctx, b.texture))
        return set_err(ctx, BH_ERR_BAD_TEXTURE, "scene %d object %d: texture %d is not valid", i, j, b.texture);
      double e1[3], e2[3], n[3];
      for (int k = 0; k < 3; ++k) {
        e1[k] = b.v[1][k] - b.v[0][k];
        e2[k] = b.v[3][k] - b.v[0][k];
      }
      cross3(e1, e2, n);
      if (!(dot3(n, n) > 0))
        return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "scene %d object %d: degenerate rectangle", i, j);
    } else if (b.type == BH_OBJECT_PLANE) {
      const double* ax[3] = {b.axis_x, b.axis_y, b.axis_z};
      for (const double* a : ax)
        if (!(std::fabs(dot3(a, a) - 1.0) < 1e-6))
          return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "scene %d object %d: plane axes must be unit vectors", i, j);
      // ChessPattern2D divides by (int)(2 * size)
      if (b.pattern_size != 0 && !(b.pattern_size >= 0.5))
        return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "scene %d object %d: pattern_size must be 0 or >= 0.5", i, j);
    } else if (b.type != BH_OBJECT_TRIANGLE) {
      return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "scene %d object %d: unknown type %d", i, j, b.type);
    }
  }
  return BH_OK;
}

// The holes of a MULTI scene relative to the scene's hole: hole 0 is the
// scene's own. Centre of mass and total mass into cen / mtot.
int scene_holes(const bh_scene& s, double (*pos)[3], double* mass, double cen[3], double* mtot) {
  const int n = 1 + (s.n_extra_holes > 0 ? s.n_extra_holes : 0);
  *mtot = 0;
  cen[0] = cen[1] = cen[2] = 0;
  for (int j = 0; j < n; ++j) {
    const bh_hole& b = j == 0 ? s.hole : s.extra_holes[j - 1];
    for (int k = 0; k < 3; ++k) pos[j][k] = b.position[k] - s.hole.position[k];
    mass[j] = b.mass;
    *mtot += b.mass;
    for (int k = 0; k < 3; ++k) cen[k] += b.mass * pos[j][k];
  }
  for (int k = 0; k < 3; ++k) cen[k] /= *mtot;
  return n;
}

int validate_holes(bh_ctx* ctx, const bh_scene& s, int i, const bh_render_options& o) {
  if (s.n_extra_holes < 0 || s.n_extra_holes > BH_MAX_HOLES - 1)
    return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "scene %d: n_extra_holes must be in [0, %d]", i, BH_MAX_HOLES - 1);
  if (s.n_extra_holes > 0) {
    if (!s.extra_holes) return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "scene %d: extra_holes is NULL", i);
    if (o.integrator != BH_INTEGRATOR_MULTI)
      return set_err(ctx, BH_ERR_UNSUPPORTED, "scene %d: extra holes need the MULTI integrator", i);
    for (int j = 0; j < s.n_extra_holes; ++j) {
      const bh_hole& b = s.extra_holes[j];
      if (!finite3(b.position) || !(b.mass > 0) || !std::isfinite(b.mass))
        return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "scene %d extra hole %d: mass must be positive and finite", i, j);
    }
  }
  if (o.integrator != BH_INTEGRATOR_MULTI) return BH_OK;
  double pos[BH_MAX_HOLES][3], mass[BH_MAX_HOLES], cen[3], mtot;
  const int n = scene_holes(s, pos, mass, cen, &mtot);
  const double R = o.r_escape * mtot;
  auto dist = [&](const double* a) {
    const double d[3] = {a[0] - s.hole.position[0] - cen[0], a[1] - s.hole.position[1] - cen[1],
                         a[2] - s.hole.position[2] - cen[2]};
    return std::sqrt(dot3(d, d));
  };
  for (int j = 0; j < n; ++j) {
    const double d[3] = {pos[j][0] - cen[0], pos[j][1] - cen[1], pos[j][2] - cen[2]};
    if (std::sqrt(dot3(d, d)) + 2 * mass[j] >= R)
      return set_err(ctx, BH_ERR_UNSUPPORTED, "scene %d: hole %d reaches the escape sphere", i, j);
  }
  if (dist(s.camera.position) >= R)
    return set_err(ctx, BH_ERR_UNSUPPORTED, "scene %d: camera lies outside the escape sphere", i);
  if (s.disc.enabled && dist(s.disc.center) + s.disc.r_outer >= R)
    return set_err(ctx, BH_ERR_UNSUPPORTED, "scene %d: disc extends past the escape sphere", i);
  return BH_OK;
}

int validate_scene(bh_ctx* ctx, const bh_scene& s, int i, const bh_render_options& o) {
  const bh_camera& c = s.camera;
  if (c.width < 1 || c.height < 1 || c.width > 32768 || c.height > 32768)
    return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "scene %d: image size %dx%d out of range", i, c.width, c.height);
  if (!finite3(c.position) || !finite3(c.axis_x) || !finite3(c.axis_y) || !finite3(c.axis_z) ||
      !std::isfinite(c.focus_len))
    return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "scene %d: camera has a non-finite value", i);
  if (!finite3(s.hole.position) || !(s.hole.mass > 0) || !std::isfinite(s.hole.mass))
    return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "scene %d: hole mass must be positive and finite", i);
  if (s.background != -1 && !texture_ok(ctx, s.background))
    return set_err(ctx, BH_ERR_BAD_TEXTURE, "scene %d: background texture %d is not valid", i, s.background);
  if (int rc = validate_objects(ctx, s, i, o)) return rc;
  if (int rc = validate_holes(ctx, s, i, o)) return rc;
  const double rel[3] = {c.position[0] - s.hole.position[0], c.position[1] - s.hole.position[1],
                         c.position[2] - s.hole.position[2]};
  if (o.integrator == BH_INTEGRATOR_RK4 && std::sqrt(dot3(rel, rel)) >= o.r_escape * s.hole.mass)
    return set_err(ctx, BH_ERR_UNSUPPORTED, "scene %d: camera lies outside the escape radius", i);
  if (s.disc.enabled) {
    const bh_disc& d = s.disc;
    if (!texture_ok(ctx, d.texture))
      return set_err(ctx, BH_ERR_BAD_TEXTURE, "scene %d: disc texture %d is not valid", i, d.texture);
    if (!finite3(d.center) || !finite3(d.normal) || !finite3(d.corner) || !finite3(d.edge_s1) ||
        !finite3(d.edge_s2) || !std::isfinite(d.r_inner) || !std::isfinite(d.r_outer))
      return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "scene %d: disc has a non-finite value", i);
    if (!(d.r_inner >= 0) || !(d.r_outer > d.r_inner))
      return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "scene %d: disc needs 0 <= r_inner < r_outer", i);
    if (d.mapping != BH_DISC_MAP_REF_PLANAR && d.mapping != BH_DISC_MAP_POLAR)
      return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "scene %d: unknown disc mapping %d", i, d.mapping);
    const double nn = dot3(d.normal, d.normal);
    if (!(std::fabs(nn - 1.0) < 1e-6))
      return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "scene %d: disc normal must be a unit vector", i);
    if (!(dot3(d.edge_s1, d.edge_s1) > 0) || !(dot3(d.edge_s2, d.edge_s2) > 0))
      return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "scene %d: disc quad edges must be non-zero", i);
    if (o.integrator == BH_INTEGRATOR_RK4) {
      const double off[3] = {d.center[0] - s.hole.position[0], d.center[1] - s.hole.position[1],
                             d.center[2] - s.hole.position[2]};
      const double scale = std::max(1.0, std::sqrt(dot3(off, off)) + s.hole.mass);
      if (std::fabs(dot3(d.normal, off)) > 1e-9 * scale)
        return set_err(ctx, BH_ERR_UNSUPPORTED,
                       "scene %d: the RK4 integrator needs the disc plane to contain the hole", i);
      if (d.r_outer >= o.r_escape * s.hole.mass)
        return set_err(ctx, BH_ERR_UNSUPPORTED, "scene %d: disc extends past the escape radius", i);
    }
  }
  return BH_OK;
}

void set3(double* dst, float* dstf, double a, double b, double c) {
  dst[0] = a; dst[1] = b; dst[2] = c;
  dstf[0] = float(a); dstf[1] = float(b); dstf[2] = float(c);
}

void resolve_scene(bh_ctx* ctx, const bh_scene& s, const bh_frame& f, const bh_render_options& o,
                   int64_t ray_begin, DevScene* d) {
  std::memset(d, 0, sizeof(*d));
  const bh_camera& c = s.camera;
  const double* h = s.hole.position;
  const double fv[3] = {c.axis_x[0] * c.focus_len, c.axis_x[1] * c.focus_len, c.axis_x[2] * c.focus_len};
  set3(d->F, d->F_f, c.position[0] - h[0], c.position[1] - h[1], c.position[2] - h[2]);
  if (o.raygen == BH_RAYGEN_REF)
    set3(d->E0, d->E0_f, c.position[0] - fv[0], c.position[1] - fv[1], c.position[2] - fv[2]);
  else
    set3(d->E0, d->E0_f, -fv[0], -fv[1], -fv[2]);
  set3(d->vy, d->vy_f, c.axis_y[0], c.axis_y[1], c.axis_y[2]);
  set3(d->vz, d->vz_f, c.axis_z[0], c.axis_z[1], c.axis_z[2]);
  const double M = s.hole.mass;
  d->mass = M;
  d->b_c = 3.0 * std::sqrt(3.0) * M;  // blackhole_solution.h:25
  d->r_h = 2.0 * M;                    // blackhole_solution.h:57
  d->half_w = c.width / 2.0;
  d->half_h = c.height / 2.0;
  d->width = c.width;
  d->height = c.height;
  d->tiles_x = (c.width + 7) / 8;
  {
    const bhgb::DivMagic dm = bhgb::div_magic(uint32_t(d->tiles_x));
    d->tiles_x_magic = dm.m;
    d->tiles_x_shift = dm.s;
  }
  d->ray_begin = ray_begin;
  d->disc_on = s.disc.enabled ? 1 : 0;
  if (s.disc.enabled) {
    const bh_disc& q = s.disc;
    set3(d->dc, d->dc_f, q.center[0] - h[0], q.center[1] - h[1], q.center[2] - h[2]);
    set3(d->dn, d->dn_f, q.normal[0], q.normal[1], q.normal[2]);
    set3(d->dv1, d->dv1_f, q.corner[0] - h[0], q.corner[1] - h[1], q.corner[2] - h[2]);
    set3(d->ds1, d->ds1_f, q.edge_s1[0], q.edge_s1[1], q.edge_s1[2]);
    set3(d->ds2, d->ds2_f, q.edge_s2[0], q.edge_s2[1], q.edge_s2[2]);
    d->s1_len = std::sqrt(dot3(q.edge_s1, q.edge_s1));
    d->s2_len = std::sqrt(dot3(q.edge_s2, q.edge_s2));
    const double e1[3] = {q.edge_s1[0] / d->s1_len, q.edge_s1[1] / d->s1_len, q.edge_s1[2] / d->s1_len};
    double e2[3] = {q.normal[1] * e1[2] - q.normal[2] * e1[1], q.normal[2] * e1[0] - q.normal[0] * e1[2],
                    q.normal[0] * e1[1] - q.normal[1] * e1[0]};
    const double l2 = std::sqrt(dot3(e2, e2));
    if (l2 > 0) { e2[0] /= l2; e2[1] /= l2; e2[2] /= l2; }
    set3(d->de1, d->de1_f, e1[0], e1[1], e1[2]);
    set3(d->de2, d->de2_f, e2[0], e2[1], e2[2]);
    d->r_in = q.r_inner;
    d->r_out = q.r_outer;
    d->disc_map = q.mapping;
    const TexEntry& t = ctx->textures[q.texture];
    d->disc_tex = DevTexture{t.texels, t.width, t.height};
  }
  d->has_bg = s.background >= 0 ? 1 : 0;
  if (s.background >= 0) {
    const TexEntry& t = ctx->textures[s.background];
    d->bg_tex = DevTexture{t.texels, t.width, t.height};
  }
  d->mass_f = float(d->mass);
  d->b_c_f = float(d->b_c);
  d->r_h_f = float(d->r_h);
  d->r_in_f = float(d->r_in);
  d->r_out_f = float(d->r_out);
  d->s1_len_f = float(d->s1_len);
  d->s2_len_f = float(d->s2_len);
  d->half_w_f = float(d->half_w);
  d->half_h_f = float(d->half_h);
  d->inv_mass_f = float(1.0 / d->mass);
  d->b_lip = bhgb::row_b_lipschitz(d->F, d->E0, d->vy, d->vz, d->mass);
  bhgb::resolve_rk4_constants(d->Fhat, d->Fhat_f, &d->Flen, &d->Flen_f, &d->x0, &d->x0_f, d->F, d->mass);
  bhgb::resolve_derived(d);
  {
    double pos[BH_MAX_HOLES][3], mass[BH_MAX_HOLES], cen[3], mtot;
    d->n_holes = scene_holes(s, pos, mass, cen, &mtot);
    for (int j = 0; j < d->n_holes; ++j) {
      bhgb::DevHole& t = d->holes[j];
      for (int k = 0; k < 3; ++k) {
        t.p[k] = pos[j][k];
        t.p_f[k] = float(pos[j][k]);
      }
      t.hm = 0.5 * mass[j];
      t.hm_f = float(t.hm);
    }
    set3(d->mcen, d->mcen_f, cen[0], cen[1], cen[2]);
    d->r_esc = o.r_escape * mtot;
    d->r_esc_f = float(d->r_esc);
  }
  d->pixels = static_cast<uint8_t*>(f.pixels);
  d->cls = f.hit_class;
  d->aux = f.aux;
  bhgb::resolve_frame_flags(d);
}

int32_t count_objects(const bh_scene* scenes, int32_t n) {
  int32_t t = 0;
  for (int i = 0; i < n; ++i) t += scenes[i].n_objects;
  return t;
}

// Resolves the objects of all scenes, in table order, into h and points each
// scene record at its own run of them in d.
void resolve_objects(bh_ctx* ctx, const bh_scene* scenes, int32_t n, DevObject* h, const DevObject* d,
                     DevScene* recs) {
  int32_t at = 0;
  for (int i = 0; i < n; ++i) {
    recs[i].objects = scenes[i].n_objects > 0 ? d + at : nullptr;
    recs[i].n_objects = scenes[i].n_objects;
    for (int j = 0; j < scenes[i].n_objects; ++j, ++at) {
      const bh_object& b = scenes[i].objects[j];
      DevTexture t{nullptr, 0, 0};
      if (b.type == BH_OBJECT_RECTANGLE && b.texture >= 0) {
        const TexEntry& e = ctx->textures[b.texture];
        t = DevTexture{e.texels, e.width, e.height};
      }
      bhgb::resolve_object(b, scenes[i].hole.position, t, h + at);
    }
  }
}

int64_t padded_rays(const bh_camera& c) {
  return int64_t((c.width + 7) / 8) * int64_t((c.height + 3) / 4) * 32;
}

int check_inputs(bh_ctx* ctx, const bh_scene* scenes, int32_t n, const bh_frame* frames,
                 const bh_render_options* opts_in, bh_render_options* o) {
  if (!ctx) return BH_ERR_INVALID_ARGUMENT;
  if (!scenes || !frames || n < 1 || n > 65535)
    return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "need 1..65535 scenes with frames");
  resolve_defaults(opts_in, o);
  int rc = validate_options(ctx, *o);
  if (rc) return rc;
  int64_t total = 0;
  for (int i = 0; i < n; ++i) {
    rc = validate_scene(ctx, scenes[i], i, *o);
    if (rc) return rc;
    if (!frames[i].pixels) return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "frame %d has no pixel buffer", i);
    if (frames[i].aux && o->integrator == BH_INTEGRATOR_REF_TRAPEZOID)
      return set_err(ctx, BH_ERR_UNSUPPORTED, "frame %d: aux output needs the RK4 or FLAT integrator", i);
    total += padded_rays(scenes[i].camera);
  }
  if (total >= (int64_t(1) << 32)) return set_err(ctx, BH_ERR_UNSUPPORTED, "too many rays in one call");
  return BH_OK;
}

// Waits until the pinned staging buffer may be rewritten.
int wait_staging(bh_ctx* ctx) {
  if (ctx->staged_pending) {
    BH_CUDA(ctx, cudaEventSynchronize(ctx->ev_staged));
    ctx->staged_pending = false;
  }
  return BH_OK;
}

LaunchParams base_params(const bh_render_options& o) {
  LaunchParams p{};
  p.integrator = o.integrator;
  p.precision = o.precision;
  p.format = o.format;
  p.raygen = o.raygen;
  p.max_steps = o.max_steps;
  p.c32 = bhgb::make_rk4_consts<float>(o.step, 1.0 / o.r_escape, o.max_steps);
  p.c64 = bhgb::make_rk4_consts<double>(o.step, 1.0 / o.r_escape, o.max_steps);
  p.cband = bhgb::make_rk4_consts<double>(o.band_step, 1.0 / o.r_escape, o.max_steps);
  bhgb::split_band_consts(p.cband, p.band_df);
  p.setup_band = bhgb::setup_band_for(o.band, o.setup_band);
  p.class_band = bhgb::class_band_for(o.band);
  bhgb::set_band_eps(o.band, &p.eps_band_lo, &p.eps_band_hi, &p.band_key_scale, p.eps_band_df);
  p.refill_threshold = o.refill_threshold;
  p.slice_steps = o.slice_steps;
  p.band_lanes = o.band_lanes;
  p.band_serial = o.band_serial;
  p.rays_per_thread = o.rays_per_thread > 0 ? o.rays_per_thread : 1;
  return p;
}

// The band list holds one entry per ray of the call, so it cannot overflow
// (4 bytes per ray, as much as a BGRA8 frame).
uint32_t band_capacity_for(int64_t total) { return uint32_t(total); }

int persistent_blocks(bh_ctx* ctx, const LaunchParams& p, const bh_render_options& o, int* blocks) {
  int per_sm = o.blocks_per_sm;
  if (per_sm == 0) {
    BH_CUDA(ctx, bhgb::persistent_occupancy(p, o.threads_per_block, &per_sm));
    if (per_sm < 1) per_sm = 1;
  }
  *blocks = per_sm * ctx->sm_count;
  return BH_OK;
}

// Enqueues the kernels of one render (scenes already on the device).
int enqueue_kernels(bh_ctx* ctx, LaunchParams& p, const bh_render_options& o, const bh_scene* scenes,
                    int32_t n, cudaStream_t st) {
  if (o.schedule == BH_SCHEDULE_GRID) {
    std::vector<int32_t> w(n), h(n);
    for (int i = 0; i < n; ++i) {
      w[i] = scenes[i].camera.width;
      h[i] = scenes[i].camera.height;
    }
    const bool objects = o.integrator == BH_INTEGRATOR_FLAT || o.integrator == BH_INTEGRATOR_MULTI ||
                         count_objects(scenes, n) > 0;
    BH_CUDA(ctx, bhgb::launch_grid(p, w.data(), h.data(), o.block_x, o.block_y, st, objects));
  } else if (o.schedule == BH_SCHEDULE_HYBRID) {
    std::vector<int32_t> w(n), h(n);
    for (int i = 0; i < n; ++i) {
      w[i] = scenes[i].camera.width;
      h[i] = scenes[i].camera.height;
    }
    BH_CUDA(ctx, bhgb::launch_hybrid(p, w.data(), h.data(), o.block_x, o.block_y, o.threads_per_block, st));
  } else {
    int blocks = 0;
    int rc = persistent_blocks(ctx, p, o, &blocks);
    if (rc) return rc;
    BH_CUDA(ctx, bhgb::launch_persistent(p, o.threads_per_block, blocks, st));
  }
  return BH_OK;
}

// Stages the scenes, launches, and leaves the counters copy enqueued. A
// later chunk of the same call (first = false) resets only the work queues:
// the statistics and the start event run on over the whole call.
int render_on_device(bh_ctx* ctx, const bh_scene* scenes, int32_t n, const bh_frame* dframes,
                     const bh_render_options& o, cudaStream_t st, bool first = true) {
  if (first) ctx->direct_host = false;
  int rc = wait_staging(ctx);
  if (rc) return rc;
  if ((rc = ensure_pinned(ctx, ctx->h_scenes, n))) return rc;
  if ((rc = ensure_dev(ctx, ctx->d_scenes, n))) return rc;
  int64_t total = 0;
  for (int i = 0; i < n; ++i) {
    resolve_scene(ctx, scenes[i], dframes[i], o, total, ctx->h_scenes.ptr + i);
    total += padded_rays(scenes[i].camera);
  }
  bhgb::assign_grid_blocks(ctx->h_scenes.ptr, n, o.block_x, o.block_y, o.rays_per_thread);
  const int32_t nobj = count_objects(scenes, n);
  if (nobj > 0) {
    if ((rc = ensure_pinned(ctx, ctx->h_objects, nobj))) return rc;
    if ((rc = ensure_dev(ctx, ctx->d_objects, nobj))) return rc;
    resolve_objects(ctx, scenes, n, ctx->h_objects.ptr, ctx->d_objects.ptr, ctx->h_scenes.ptr);
  }
  LaunchParams p = base_params(o);
  p.scenes = ctx->d_scenes.ptr;
  p.n_scenes = n;
  p.total_rays = total;
  p.counters = ctx->d_counters;
  if (bhgb::uses_band_pass(o)) {
    const uint32_t cap = band_capacity_for(total);
    if ((rc = ensure_dev(ctx, ctx->band_list, bhgb::band_words(cap)))) return rc;
    bhgb::carve_band(ctx->band_list.ptr, cap, &p.band_list, &p.band_tmp, &p.band_key);
    p.band_capacity = cap;
  }
  if (nobj > 0)
    BH_CUDA(ctx, cudaMemcpyAsync(ctx->d_objects.ptr, ctx->h_objects.ptr, sizeof(DevObject) * nobj,
                                 cudaMemcpyHostToDevice, st));
  BH_CUDA(ctx, cudaMemcpyAsync(ctx->d_scenes.ptr, ctx->h_scenes.ptr, sizeof(DevScene) * n,
                               cudaMemcpyHostToDevice, st));
  if (first) {
    ctx->h2d_bytes = 0;
    ctx->d2h_bytes = 0;
  }
  ctx->h2d_bytes += sizeof(DevScene) * size_t(n) + sizeof(DevObject) * size_t(nobj);
  BH_CUDA(ctx, cudaEventRecord(ctx->ev_staged, st));
  ctx->staged_pending = true;
  if (first) {
    BH_CUDA(ctx, cudaMemsetAsync(ctx->d_counters, 0, sizeof(DevCounters), st));
    BH_CUDA(ctx, cudaEventRecord(ctx->ev_start, st));
  } else {
    DevCounters* c = ctx->d_counters;
    BH_CUDA(ctx, cudaMemsetAsync(c, 0, offsetof(DevCounters, steps), st));  // queue heads
    BH_CUDA(ctx, cudaMemsetAsync(&c->blocks_started, 0, sizeof(c->blocks_started), st));
    BH_CUDA(ctx, cudaMemsetAsync(c->band_hist, 0, sizeof(c->band_hist) + sizeof(c->band_cursor), st));
  }
  if ((rc = enqueue_kernels(ctx, p, o, scenes, n, st))) return rc;
  BH_CUDA(ctx, cudaEventRecord(ctx->ev_stop, st));
  BH_CUDA(ctx, cudaMemcpyAsync(ctx->h_counters, ctx->d_counters, sizeof(DevCounters), cudaMemcpyDeviceToHost, st));
  ctx->stats_valid = true;
  return BH_OK;
}

}  // namespace

extern "C" {

int bh_abi_version(void) { return BH_ABI_VERSION; }

void bh_default_options(bh_render_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->integrator = BH_INTEGRATOR_RK4;
  o->precision = BH_PRECISION_FP32;
  o->raygen = BH_RAYGEN_REF;
  o->format = BH_FORMAT_BGRA8;
  o->schedule = BH_SCHEDULE_GRID;
  o->max_steps = 4000;
  o->step = 0.01;
  o->r_escape = 100.0;
  o->band = 5e-4;
  o->band_step = 0.01;
  o->setup_band = 0.1;
  o->slice_steps = 256;
  o->band_lanes = 32;
  o->block_x = 8;  // each warp an 8 x 4 pixel tile: its rays end closer together than a 32-pixel
  o->block_y = 16; // row's (measured 4-5 % faster than 32 x 4 on RK4, objects and MULTI renders)
  o->threads_per_block = 256;
  o->blocks_per_sm = 0;
  o->refill_threshold = 32;
  o->rays_per_thread = 1;
}

int bh_create(bh_ctx** out, int device) {
  if (!out) return BH_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return BH_ERR_NO_DEVICE;
  if (device < 0 || device >= count) return BH_ERR_INVALID_ARGUMENT;
  bh_ctx* ctx = new (std::nothrow) bh_ctx();
  if (!ctx) return BH_ERR_OUT_OF_MEMORY;
  ctx->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev_start);
  if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev_stop);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_staged, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking);
  for (int c = 0; c < kMaxChunks && e == cudaSuccess; ++c)
    e = cudaEventCreateWithFlags(&ctx->ev_chunk[c], cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaMalloc(&ctx->d_counters, sizeof(DevCounters));
  if (e == cudaSuccess) e = cudaMallocHost(&ctx->h_counters, sizeof(DevCounters));
  if (e != cudaSuccess) {
    bh_destroy(ctx);
    return e == cudaErrorMemoryAllocation ? BH_ERR_OUT_OF_MEMORY : BH_ERR_CUDA;
  }
  *out = ctx;
  return BH_OK;
}

void bh_destroy(bh_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (auto& t : ctx->textures)
    if (t.texels) cudaFree(t.texels);
  if (ctx->h_scenes.ptr) cudaFreeHost(ctx->h_scenes.ptr);
  if (ctx->d_scenes.ptr) cudaFree(ctx->d_scenes.ptr);
  if (ctx->h_objects.ptr) cudaFreeHost(ctx->h_objects.ptr);
  if (ctx->d_objects.ptr) cudaFree(ctx->d_objects.ptr);
  if (ctx->band_list.ptr) cudaFree(ctx->band_list.ptr);
  if (ctx->out_arena.ptr) cudaFree(ctx->out_arena.ptr);
  if (ctx->d_counters) cudaFree(ctx->d_counters);
  if (ctx->h_counters) cudaFreeHost(ctx->h_counters);
  if (ctx->h_adj.ptr) cudaFreeHost(ctx->h_adj.ptr);
  if (ctx->d_adj.ptr) cudaFree(ctx->d_adj.ptr);
  if (ctx->adj_ckpt.ptr) cudaFree(ctx->adj_ckpt.ptr);
  if (ctx->adj_ckpt_band.ptr) cudaFree(ctx->adj_ckpt_band.ptr);
  if (ctx->adj_band.ptr) cudaFree(ctx->adj_band.ptr);
  if (ctx->adj_acc.ptr) cudaFree(ctx->adj_acc.ptr);
  if (ctx->h_adj_acc.ptr) cudaFreeHost(ctx->h_adj_acc.ptr);
  if (ctx->adj_counters.ptr) cudaFree(ctx->adj_counters.ptr);
  if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
  if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
  if (ctx->side_stream) cudaStreamDestroy(ctx->side_stream);
  if (ctx->copy_stream) {
    cudaStreamSynchronize(ctx->copy_stream);
    cudaStreamDestroy(ctx->copy_stream);
  }
  for (cudaEvent_t ev : ctx->ev_chunk)
    if (ev) cudaEventDestroy(ev);
  if (ctx->ev_start) cudaEventDestroy(ctx->ev_start);
  if (ctx->ev_stop) cudaEventDestroy(ctx->ev_stop);
  if (ctx->ev_staged) cudaEventDestroy(ctx->ev_staged);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

const char* bh_last_error(const bh_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

void* bh_stream(bh_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int bh_texture_create(bh_ctx* ctx, const uint8_t* texels, int32_t width, int32_t height, int32_t layout,
                      int64_t row_stride, int32_t* out_id) {
  if (!ctx || !out_id) return BH_ERR_INVALID_ARGUMENT;
  if (!texels || width <= 0 || height <= 0)
    return set_err(ctx, BH_ERR_EMPTY_TEXTURE, "empty texture (the reference terminates here)");
  if ((int64_t)width * height > (int64_t(1) << 28))
    return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "texture larger than 2^28 texels");
  int cpp = 0;
  switch (layout) {
    case BH_TEXEL_BGR8: case BH_TEXEL_RGB8: cpp = 3; break;
    case BH_TEXEL_BGRA8: case BH_TEXEL_RGBA8: cpp = 4; break;
    default: return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "unknown texel layout %d", layout);
  }
  if (row_stride == 0) row_stride = int64_t(width) * cpp;
  if (row_stride < int64_t(width) * cpp) return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "row stride too small");
  std::vector<uchar4> host(size_t(width) * height);
  for (int32_t y = 0; y < height; ++y) {
    const uint8_t* row = texels + y * row_stride;
    for (int32_t x = 0; x < width; ++x) {
      const uint8_t* p = row + x * cpp;
      uchar4 t;
      if (layout == BH_TEXEL_BGR8) t = make_uchar4(p[0], p[1], p[2], 255);
      else if (layout == BH_TEXEL_RGB8) t = make_uchar4(p[2], p[1], p[0], 255);
      else if (layout == BH_TEXEL_BGRA8) t = make_uchar4(p[0], p[1], p[2], p[3]);
      else t = make_uchar4(p[2], p[1], p[0], p[3]);
      host[size_t(y) * width + x] = t;
    }
  }
  BH_CUDA(ctx, cudaSetDevice(ctx->device));
  TexEntry e;
  BH_CUDA(ctx, cudaMalloc(&e.texels, host.size() * sizeof(uchar4)));
  cudaError_t ce = cudaMemcpy(e.texels, host.data(), host.size() * sizeof(uchar4), cudaMemcpyHostToDevice);
  if (ce != cudaSuccess) {
    cudaFree(e.texels);
    return cuda_err(ctx, ce, "texture upload");
  }
  e.width = width;
  e.height = height;
  e.alive = true;
  for (size_t i = 0; i < ctx->textures.size(); ++i) {
    if (!ctx->textures[i].alive && !ctx->textures[i].texels) {
      ctx->textures[i] = e;
      *out_id = int32_t(i);
      return BH_OK;
    }
  }
  ctx->textures.push_back(e);
  *out_id = int32_t(ctx->textures.size() - 1);
  return BH_OK;
}

int bh_texture_destroy(bh_ctx* ctx, int32_t id) {
  if (!ctx) return BH_ERR_INVALID_ARGUMENT;
  if (!texture_ok(ctx, id)) return set_err(ctx, BH_ERR_BAD_TEXTURE, "texture %d is not valid", id);
  BH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  cudaFree(ctx->textures[id].texels);
  ctx->textures[id] = TexEntry{};
  return BH_OK;
}

int bh_render_device(bh_ctx* ctx, const bh_scene* scenes, int32_t n, const bh_frame* frames,
                     const bh_render_options* opts, void* stream) {
  bh_render_options o;
  int rc = check_inputs(ctx, scenes, n, frames, opts, &o);
  if (rc) return rc;
  BH_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  return render_on_device(ctx, scenes, n, frames, o, st);
}

namespace {

// The device address of host memory the device can reach (page-locked and
// mapped: cudaHostAlloc, cudaMallocHost, cudaHostRegister), or null for
// anything else (pageable or device memory).
void* mapped_host_address(void* p) {
  if (!p) return nullptr;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// bh_render into host frames the kernels can write directly: one render, no
// copy-back. The GRID and HYBRID schedules store whole warp rows (BGR8:
// packed words, blocks widened to 32 pixels so that a warp's 96 bytes are
// one row segment); the persistent schedule's scattered per-pixel stores
// would cross the host link one pixel at a time, so it keeps the copy-back.
// Returns 1 (not taken) when a buffer is not mapped host memory.
int render_direct_to_host(bh_ctx* ctx, const bh_scene* scenes, int32_t n, const bh_frame* frames,
                          const bh_render_options& o) {
  if (o.schedule == BH_SCHEDULE_PERSISTENT) return 1;
  std::vector<bh_frame> hf(n);
  uint64_t bytes = 0;
  const int bpp = bytes_per_pixel(o.format);
  for (int i = 0; i < n; ++i) {
    hf[i].pixels = mapped_host_address(frames[i].pixels);
    hf[i].hit_class = static_cast<uint8_t*>(mapped_host_address(frames[i].hit_class));
    hf[i].aux = static_cast<float*>(mapped_host_address(frames[i].aux));
    if (!hf[i].pixels || (frames[i].hit_class && !hf[i].hit_class) || (frames[i].aux && !hf[i].aux)) return 1;
    const uint64_t px = uint64_t(scenes[i].camera.width) * scenes[i].camera.height;
    bytes += px * bpp + (frames[i].hit_class ? px : 0) + (frames[i].aux ? px * sizeof(float) : 0);
  }
  bh_render_options od = o;
  if (od.format == BH_FORMAT_BGR8 && od.block_x < 32) {
    od.block_y = std::max(1, od.block_x * od.block_y / 32);
    od.block_x = 32;
    // and at most 32 tiles per thread: on the 120-frame 1080p fly-through
    // into pinned frames 4 / 8 / 16 / 32 / 64 / 128 took 6.1 / 5.7 / 5.55 /
    // 5.57 / 5.67 / 5.79 ms, where the device-frame optimum is 32-64
    od.rays_per_thread = std::min(od.rays_per_thread, 32);
  }
  int rc = render_on_device(ctx, scenes, n, hf.data(), od, ctx->stream, true);
  if (rc) return rc;
  ctx->d2h_bytes = bytes;
  ctx->direct_host = true;
  BH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return bh_get_stats(ctx, &ctx->last);
}

}  // namespace

int bh_render(bh_ctx* ctx, const bh_scene* scenes, int32_t n, const bh_frame* frames,
              const bh_render_options* opts) {
  bh_render_options o;
  int rc = check_inputs(ctx, scenes, n, frames, opts, &o);
  if (rc) return rc;
  BH_CUDA(ctx, cudaSetDevice(ctx->device));
  if ((rc = render_direct_to_host(ctx, scenes, n, frames, o)) != 1) return rc;
  // device arena: pixels | classes | aux for every frame, 256-byte aligned
  const int bpp = bytes_per_pixel(o.format);
  std::vector<bh_frame> dframes(n);
  std::vector<size_t> off_pix(n), off_cls(n), off_aux(n);
  size_t total = 0;
  auto take = [&](size_t bytes) {
    const size_t at = total;
    total += (bytes + 255) & ~size_t(255);
    return at;
  };
  for (int i = 0; i < n; ++i) {
    const size_t px = size_t(scenes[i].camera.width) * scenes[i].camera.height;
    off_pix[i] = take(px * bpp);
    off_cls[i] = frames[i].hit_class ? take(px) : 0;
    off_aux[i] = frames[i].aux ? take(px * sizeof(float)) : 0;
  }
  if ((rc = ensure_dev(ctx, ctx->out_arena, total))) return rc;
  uint8_t* base = ctx->out_arena.ptr;
  for (int i = 0; i < n; ++i) {
    dframes[i].pixels = base + off_pix[i];
    dframes[i].hit_class = frames[i].hit_class ? base + off_cls[i] : nullptr;
    dframes[i].aux = frames[i].aux ? reinterpret_cast<float*>(base + off_aux[i]) : nullptr;
  }
  // Large calls render in chunks of scenes: each chunk's copy-back (one
  // cudaMemcpyAsync per buffer, on the copy stream) overlaps the next
  // chunk's render. The copy engine moves ~190 GB/s device -> host here, so
  // 120 BGR8 1080p frames (746 MB) take ~4 ms, 40 % of their render. (The
  // kernels writing mapped host frames directly over NVLink-C2C measured
  // 16.4 ms against 9.7 ms: the frame's 3-byte pixels go as byte stores. A
  // per-frame completion flag that let each frame be copied as soon as it
  // was done cost the kernels 0.7-1.6 ms in per-tile atomics.)
  int64_t pixels = 0;
  for (int i = 0; i < n; ++i) pixels += int64_t(scenes[i].camera.width) * scenes[i].camera.height;
  const int chunks = (pixels >= (int64_t(64) << 20) && n >= 2 * kMaxChunks) ? kMaxChunks : 1;
  cudaStream_t cp = chunks > 1 ? ctx->copy_stream : ctx->stream;
  for (int c = 0, i0 = 0; c < chunks; ++c) {
    // Shrinking chunks (38 / 32 / 22 / 8 % of the scenes): only the last
    // chunk's copy-back follows the render. On 120 BGR8 1080p frames this
    // measured 10.52 ms per call against 11.02 ms for equal quarters.
    static const int kShare[kMaxChunks] = {38, 70, 92, 100};
    const int i1 = c + 1 == chunks ? n : std::max(i0 + 1, int((int64_t(n) * kShare[c]) / 100));
    if ((rc = render_on_device(ctx, scenes + i0, i1 - i0, dframes.data() + i0, o, ctx->stream, c == 0))) return rc;
    if (chunks > 1) {
      BH_CUDA(ctx, cudaEventRecord(ctx->ev_chunk[c], ctx->stream));
      BH_CUDA(ctx, cudaStreamWaitEvent(cp, ctx->ev_chunk[c], 0));
    }
    for (int i = i0; i < i1; ++i) {
      const size_t px = size_t(scenes[i].camera.width) * scenes[i].camera.height;
      ctx->d2h_bytes += px * bpp + (frames[i].hit_class ? px : 0) + (frames[i].aux ? px * sizeof(float) : 0);
      BH_CUDA(ctx, cudaMemcpyAsync(frames[i].pixels, dframes[i].pixels, px * bpp, cudaMemcpyDeviceToHost, cp));
      if (frames[i].hit_class)
        BH_CUDA(ctx, cudaMemcpyAsync(frames[i].hit_class, dframes[i].hit_class, px, cudaMemcpyDeviceToHost, cp));
      if (frames[i].aux)
        BH_CUDA(ctx, cudaMemcpyAsync(frames[i].aux, dframes[i].aux, px * sizeof(float), cudaMemcpyDeviceToHost,
                                     cp));
    }
    i0 = i1;
  }
  BH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (chunks > 1) BH_CUDA(ctx, cudaStreamSynchronize(cp));
  return bh_get_stats(ctx, &ctx->last);
}

int bh_get_stats(bh_ctx* ctx, bh_render_stats* out) {
  if (!ctx || !out) return BH_ERR_INVALID_ARGUMENT;
  if (!ctx->stats_valid) return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "no render on this context yet");
  BH_CUDA(ctx, cudaSetDevice(ctx->device));
  BH_CUDA(ctx, cudaEventSynchronize(ctx->ev_stop));
  BH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  const DevCounters& c = *ctx->h_counters;
  bh_render_stats s{};
  s.rays = c.rays;
  s.steps = c.steps;
  s.band_rays = c.band_rays;
  s.band_steps = c.band_steps;
  s.band_overflow = c.band_overflow;
  s.flags = c.flags;
  float ms = 0;
  BH_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop));
  s.kernel_ms = ms;
  s.h2d_bytes = ctx->h2d_bytes;
  s.d2h_bytes = ctx->d2h_bytes;
  if (ctx->direct_host) s.flags |= BH_STATS_DIRECT_HOST;
  *out = s;
  ctx->last = s;
  return BH_OK;
}

// ---- sequences ------------------------------------------------------------------
int bh_sequence_create(bh_ctx* ctx, const bh_scene* scenes, int32_t n, const bh_frame* frames,
                       const bh_render_options* opts, bh_sequence** out) {
  if (!out) return BH_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  bh_render_options o;
  int rc = check_inputs(ctx, scenes, n, frames, opts, &o);
  if (rc) return rc;
  BH_CUDA(ctx, cudaSetDevice(ctx->device));
  bh_sequence* q = new (std::nothrow) bh_sequence();
  if (!q) return set_err(ctx, BH_ERR_OUT_OF_MEMORY, "sequence allocation");
  q->ctx = ctx;
  q->n = n;
  q->opts = o;
  q->scenes.assign(scenes, scenes + n);
  q->frames.assign(frames, frames + n);
  auto fail = [&](int code) {
    bh_sequence_destroy(q);
    return code;
  };
  cudaError_t e = cudaMallocHost(&q->h_scenes, sizeof(DevScene) * n);
  if (e == cudaSuccess) e = cudaMalloc(&q->d_scenes, sizeof(DevScene) * n);
  if (e == cudaSuccess) e = cudaMalloc(&q->d_counters, sizeof(DevCounters));
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&q->ev_done, cudaEventDisableTiming);
  q->n_objects_total = count_objects(scenes, n);
  if (e == cudaSuccess && q->n_objects_total > 0) {
    e = cudaMallocHost(&q->h_objects, sizeof(DevObject) * q->n_objects_total);
    if (e == cudaSuccess) e = cudaMalloc(&q->d_objects, sizeof(DevObject) * q->n_objects_total);
  }
  if (e != cudaSuccess) return fail(cuda_err(ctx, e, "sequence buffers"));
  int64_t total = 0;
  for (int i = 0; i < n; ++i) {
    resolve_scene(ctx, scenes[i], frames[i], o, total, q->h_scenes + i);
    total += padded_rays(scenes[i].camera);
  }
  bhgb::assign_grid_blocks(q->h_scenes, n, o.block_x, o.block_y, o.rays_per_thread);
  if (q->n_objects_total > 0) resolve_objects(ctx, scenes, n, q->h_objects, q->d_objects, q->h_scenes);
  LaunchParams p = base_params(o);
  p.scenes = q->d_scenes;
  p.n_scenes = n;
  p.total_rays = total;
  p.counters = q->d_counters;
  if (bhgb::uses_band_pass(o)) {
    q->band_capacity = band_capacity_for(total);
    e = cudaMalloc(&q->band_list, sizeof(uint32_t) * bhgb::band_words(q->band_capacity));
    if (e != cudaSuccess) return fail(cuda_err(ctx, e, "band list"));
    bhgb::carve_band(q->band_list, q->band_capacity, &p.band_list, &p.band_tmp, &p.band_key);
    p.band_capacity = q->band_capacity;
  }
  int blocks = 0;
  if (o.schedule == BH_SCHEDULE_PERSISTENT && (rc = persistent_blocks(ctx, p, o, &blocks))) return fail(rc);
  cudaStream_t cs = nullptr;
  e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  if (e != cudaSuccess) return fail(cuda_err(ctx, e, "capture stream"));
  e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess && q->n_objects_total > 0)
    e = cudaMemcpyAsync(q->d_objects, q->h_objects, sizeof(DevObject) * q->n_objects_total, cudaMemcpyHostToDevice,
                        cs);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(q->d_scenes, q->h_scenes, sizeof(DevScene) * n, cudaMemcpyHostToDevice, cs);
  if (e == cudaSuccess) e = cudaMemsetAsync(q->d_counters, 0, sizeof(DevCounters), cs);
  if (e == cudaSuccess) {
    if (o.schedule == BH_SCHEDULE_GRID) {
      std::vector<int32_t> w(n), h(n);
      for (int i = 0; i < n; ++i) {
        w[i] = scenes[i].camera.width;
        h[i] = scenes[i].camera.height;
      }
      e = bhgb::launch_grid(p, w.data(), h.data(), o.block_x, o.block_y, cs,
                            o.integrator == BH_INTEGRATOR_FLAT || o.integrator == BH_INTEGRATOR_MULTI ||
                                q->n_objects_total > 0);
    } else if (o.schedule == BH_SCHEDULE_HYBRID) {
      std::vector<int32_t> w(n), h(n);
      for (int i = 0; i < n; ++i) {
        w[i] = scenes[i].camera.width;
        h[i] = scenes[i].camera.height;
      }
      e = bhgb::launch_hybrid(p, w.data(), h.data(), o.block_x, o.block_y, o.threads_per_block, cs);
    } else {
      e = bhgb::launch_persistent(p, o.threads_per_block, blocks, cs);
    }
  }
  cudaGraph_t g = nullptr;
  const cudaError_t e2 = cudaStreamEndCapture(cs, &g);
  cudaStreamDestroy(cs);
  if (e == cudaSuccess) e = e2;
  if (e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return fail(cuda_err(ctx, e, "sequence capture"));
  }
  q->graph = g;
  e = cudaGraphInstantiate(&q->exec, g, 0);
  if (e != cudaSuccess) return fail(cuda_err(ctx, e, "graph instantiate"));
  *out = q;
  return BH_OK;
}

int bh_sequence_update(bh_sequence* q, const bh_scene* scenes, int32_t n) {
  if (!q || !scenes) return BH_ERR_INVALID_ARGUMENT;
  bh_ctx* ctx = q->ctx;
  if (n != q->n) return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "sequence holds %d scenes, got %d", q->n, n);
  for (int i = 0; i < n; ++i) {
    const bh_scene& a = scenes[i];
    const bh_scene& b = q->scenes[i];
    if (a.camera.width != b.camera.width || a.camera.height != b.camera.height ||
        a.background != b.background || a.disc.enabled != b.disc.enabled ||
        (a.disc.enabled && a.disc.texture != b.disc.texture) || a.n_objects != b.n_objects)
      return set_err(ctx, BH_ERR_INVALID_ARGUMENT,
                     "scene %d changes sizes, textures or the object count of the sequence", i);
    int rc = validate_scene(ctx, a, i, q->opts);
    if (rc) return rc;
  }
  BH_CUDA(ctx, cudaSetDevice(ctx->device));
  if (q->launched) BH_CUDA(ctx, cudaEventSynchronize(q->ev_done));
  int64_t total = 0;
  for (int i = 0; i < n; ++i) {
    resolve_scene(ctx, scenes[i], q->frames[i], q->opts, total, q->h_scenes + i);
    total += padded_rays(scenes[i].camera);
    q->scenes[i] = scenes[i];
  }
  bhgb::assign_grid_blocks(q->h_scenes, n, q->opts.block_x, q->opts.block_y, q->opts.rays_per_thread);
  if (q->n_objects_total > 0) resolve_objects(ctx, scenes, n, q->h_objects, q->d_objects, q->h_scenes);
  return BH_OK;
}

int bh_sequence_launch(bh_sequence* q, void* stream) {
  if (!q) return BH_ERR_INVALID_ARGUMENT;
  bh_ctx* ctx = q->ctx;
  BH_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
  BH_CUDA(ctx, cudaGraphLaunch(q->exec, st));
  BH_CUDA(ctx, cudaEventRecord(q->ev_done, st));
  q->launched = true;
  return BH_OK;
}

int bh_sequence_stats(bh_sequence* q, bh_render_stats* out) {
  if (!q || !out) return BH_ERR_INVALID_ARGUMENT;
  bh_ctx* ctx = q->ctx;
  if (!q->launched) return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "sequence not launched yet");
  BH_CUDA(ctx, cudaSetDevice(ctx->device));
  BH_CUDA(ctx, cudaEventSynchronize(q->ev_done));
  DevCounters c;
  BH_CUDA(ctx, cudaMemcpy(&c, q->d_counters, sizeof(c), cudaMemcpyDeviceToHost));
  bh_render_stats s{};
  s.rays = c.rays;
  s.steps = c.steps;
  s.band_rays = c.band_rays;
  s.band_steps = c.band_steps;
  s.band_overflow = c.band_overflow;
  s.flags = c.flags;
  *out = s;
  return BH_OK;
}

void bh_sequence_destroy(bh_sequence* q) {
  if (!q) return;
  if (q->ctx) cudaSetDevice(q->ctx->device);
  if (q->launched && q->ev_done) cudaEventSynchronize(q->ev_done);
  if (q->exec) cudaGraphExecDestroy(q->exec);
  if (q->graph) cudaGraphDestroy(q->graph);
  if (q->h_scenes) cudaFreeHost(q->h_scenes);
  if (q->d_scenes) cudaFree(q->d_scenes);
  if (q->h_objects) cudaFreeHost(q->h_objects);
  if (q->d_objects) cudaFree(q->d_objects);
  if (q->d_counters) cudaFree(q->d_counters);
  if (q->band_list) cudaFree(q->band_list);
  if (q->ev_done) cudaEventDestroy(q->ev_done);
  delete q;
}

// ---- autotuner --------------------------------------------------------------------
}  // extern "C"

namespace {

// Device buffers owned by one tuning run.
struct TuneBuffers {
  std::vector<void*> ptrs;
  ~TuneBuffers() {
    for (void* p : ptrs) cudaFree(p);
  }
  void* get(size_t bytes, cudaError_t* e) {
    void* p = nullptr;
    *e = cudaMalloc(&p, bytes);
    if (*e == cudaSuccess) ptrs.push_back(p);
    return p;
  }
};

struct SampleOut {
  std::vector<uint8_t> cls;
  std::vector<float> aux;
};

// Renders the sample scenes with `o` into device frames and copies class and
// aux back.
int render_sample(bh_ctx* ctx, const std::vector<bh_scene>& s, const std::vector<bh_frame>& f,
                  const bh_render_options& o, std::vector<SampleOut>* out) {
  int rc = render_on_device(ctx, s.data(), int32_t(s.size()), f.data(), o, ctx->stream);
  if (rc) return rc;
  out->resize(s.size());
  for (size_t i = 0; i < s.size(); ++i) {
    const size_t px = size_t(s[i].camera.width) * s[i].camera.height;
    (*out)[i].cls.resize(px);
    (*out)[i].aux.resize(px);
    BH_CUDA(ctx, cudaMemcpyAsync((*out)[i].cls.data(), f[i].hit_class, px, cudaMemcpyDeviceToHost, ctx->stream));
    BH_CUDA(ctx, cudaMemcpyAsync((*out)[i].aux.data(), f[i].aux, px * sizeof(float), cudaMemcpyDeviceToHost,
                                 ctx->stream));
  }
  BH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return BH_OK;
}

void compare_sample(const std::vector<SampleOut>& ref, const std::vector<SampleOut>& got, double* defl,
                    double* radius, double* mismatch) {
  size_t total = 0, bad = 0;
  double d = 0, r = 0;
  for (size_t i = 0; i < ref.size(); ++i) {
    for (size_t k = 0; k < ref[i].cls.size(); ++k) {
      ++total;
      if (ref[i].cls[k] != got[i].cls[k]) {
        ++bad;
        continue;
      }
      const double e = std::fabs(double(ref[i].aux[k]) - double(got[i].aux[k]));
      if (ref[i].cls[k] == BH_CLASS_MISS) d = std::max(d, e);
      else if (ref[i].cls[k] == BH_CLASS_DISC) r = std::max(r, e);
    }
  }
  *defl = d;
  *radius = r;
  *mismatch = total ? double(bad) / double(total) : 0.0;
}

std::string tune_key(bh_ctx* ctx, const bh_scene* scenes, int32_t n, double max_error) {
  cudaDeviceProp prop{};
  cudaGetDeviceProperties(&prop, ctx->device);
  int64_t rays = 0;
  for (int i = 0; i < n; ++i) rays += padded_rays(scenes[i].camera);
  char buf[512];
  std::snprintf(buf, sizeof(buf), "%s|sms=%d|n=%d|rays=%lld|w=%d|h=%d|err=%.3g", prop.name, ctx->sm_count, n,
                (long long)rays, scenes[0].camera.width, scenes[0].camera.height, max_error);
  for (char* c = buf; *c; ++c)
    if (*c == ' ') *c = '_';
  return buf;
}

bool cache_lookup(const char* path, const std::string& key, bh_render_options* o, bh_tune_report* rep) {
  if (!path) return false;
  FILE* f = std::fopen(path, "r");
  if (!f) return false;
  char line[1024];
  bool found = false;
  while (std::fgets(line, sizeof(line), f)) {
    char k[600];
    double step, band, defl, rad, mis, ms;
    int threads, refill, slice, schedule, bx, by, rpt;
    if (std::sscanf(line, "%599s %lf %lf %d %d %d %d %d %d %d %lf %lf %lf %lf", k, &step, &band, &threads, &refill,
                    &slice, &schedule, &bx, &by, &rpt, &defl, &rad, &mis, &ms) == 14 &&
        key == k) {
      o->step = step;
      o->band = band;
      o->threads_per_block = threads;
      o->refill_threshold = refill;
      o->slice_steps = slice;
      o->schedule = schedule;
      o->block_x = bx;
      o->block_y = by;
      o->rays_per_thread = rpt;
      rep->step = step;
      rep->max_deflection = defl;
      rep->max_radius_error = rad;
      rep->class_mismatch = mis;
      rep->kernel_ms = ms;
      found = true;  // the last matching line wins
    }
  }
  std::fclose(f);
  return found;
}

void cache_store(const char* path, const std::string& key, const bh_render_options& o, const bh_tune_report& rep) {
  if (!path) return;
  FILE* f = std::fopen(path, "a");
  if (!f) return;
  std::fprintf(f, "%s %.17g %.17g %d %d %d %d %d %d %d %.6g %.6g %.6g %.6g\n", key.c_str(), o.step, o.band,
               o.threads_per_block, o.refill_threshold, o.slice_steps, o.schedule, o.block_x, o.block_y,
               o.rays_per_thread, rep.max_deflection, rep.max_radius_error, rep.class_mismatch, rep.kernel_ms);
  std::fclose(f);
}

}  // namespace

extern "C" {

int bh_autotune(bh_ctx* ctx, const bh_scene* scenes, int32_t n, bh_render_options* opts, double max_error,
                const char* cache_path, bh_tune_report* report) {
  if (!ctx || !opts || !report) return BH_ERR_INVALID_ARGUMENT;
  if (!(max_error > 0)) return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "max_error must be positive");
  *report = bh_tune_report{};
  bh_render_options base;
  resolve_defaults(opts, &base);
  if (base.integrator != BH_INTEGRATOR_RK4)
    return set_err(ctx, BH_ERR_UNSUPPORTED, "the autotuner tunes the RK4 tracer");
  base.precision = BH_PRECISION_MIXED;
  base.schedule = BH_SCHEDULE_PERSISTENT;
  // validate the batch once (frames are the tuner's own)
  {
    std::vector<bh_frame> dummy(size_t(n > 0 ? n : 1), bh_frame{reinterpret_cast<void*>(1), nullptr, nullptr});
    bh_render_options chk;
    int rc = check_inputs(ctx, scenes, n, dummy.data(), &base, &chk);
    if (rc) return rc;
  }
  BH_CUDA(ctx, cudaSetDevice(ctx->device));
  const std::string key = tune_key(ctx, scenes, n, max_error);
  bh_render_options chosen = base;
  if (cache_lookup(cache_path, key, &chosen, report)) {
    report->from_cache = 1;
    *opts = chosen;
    return BH_OK;
  }

  TuneBuffers mem;
  cudaError_t e = cudaSuccess;
  // sample, with class and aux outputs: up to 16 evenly spaced scenes, fewer
  // (down to 4) while they hold more than eight 1920x1080 frames of pixels
  auto pick = [n](int k, int i) -> int32_t { return k == 1 ? 0 : int32_t(int64_t(i) * (n - 1) / (k - 1)); };
  int ns = std::min<int32_t>(n, 16);
  for (; ns > 4; --ns) {
    double px = 0;
    for (int i = 0; i < ns; ++i) px += double(scenes[pick(ns, i)].camera.width) * scenes[pick(ns, i)].camera.height;
    if (px <= 8.0 * 1920 * 1080) break;
  }
  std::vector<bh_scene> sample;
  for (int i = 0; i < ns; ++i) sample.push_back(scenes[pick(ns, i)]);
  std::vector<bh_frame> sf(sample.size());
  for (size_t i = 0; i < sample.size(); ++i) {
    const size_t px = size_t(sample[i].camera.width) * sample[i].camera.height;
    sf[i].pixels = mem.get(px * 4, &e);
    if (e == cudaSuccess) sf[i].hit_class = static_cast<uint8_t*>(mem.get(px, &e));
    if (e == cudaSuccess) sf[i].aux = static_cast<float*>(mem.get(px * sizeof(float), &e));
    if (e != cudaSuccess) return cuda_err(ctx, e, "tuner sample buffers");
  }
  std::vector<SampleOut> ref, got;
  bh_render_options ro = base;
  ro.precision = BH_PRECISION_FP64;
  ro.schedule = BH_SCHEDULE_GRID;
  ro.format = BH_FORMAT_BGRA8;
  int rc = render_sample(ctx, sample, sf, ro, &ref);
  if (rc) return rc;

  // 1) the largest step that keeps the sample within max_error / 2
  std::vector<double> steps;
  for (double h : {0.2, 0.175, 0.15, 0.125, 0.1, 0.08, 0.05, 0.04, 0.03, 0.02})
    if (h > base.step) steps.push_back(h);
  steps.push_back(base.step);  // the reference step itself is the last resort
  auto meets = [&](const bh_render_options& c, bool* ok) -> int {
    int r = render_sample(ctx, sample, sf, c, &got);
    if (r) return r;
    report->candidates++;
    double d, rr, m;
    compare_sample(ref, got, &d, &rr, &m);
    *ok = d <= 0.5 * max_error && m <= 1e-4;
    if (*ok) {
      report->max_deflection = d;
      report->max_radius_error = rr;
      report->class_mismatch = m;
    }
    return BH_OK;
  };
  bool ok = false;
  for (double h : steps) {
    bh_render_options c = base;
    c.step = h;
    c.format = BH_FORMAT_BGRA8;
    if ((rc = meets(c, &ok))) return rc;
    if (ok) {
      chosen.step = h;
      report->step = h;
      break;
    }
  }
  if (!ok) return set_err(ctx, BH_ERR_UNSUPPORTED, "no candidate step meets the deflection bound");

  // 2) the narrowest FP64 band (never below 2e-5 M, where FP32 with the FP64
  // first integral and the energy projection stays within 2e-5 rad of FP64
  // on an impact-parameter grid) that keeps the sample within the same bound
  for (double band : {2e-5, 1e-4}) {
    if (!(band < base.band)) break;
    bh_render_options c = chosen;
    c.band = band;
    c.format = BH_FORMAT_BGRA8;
    if ((rc = meets(c, &ok))) return rc;
    if (ok) {
      chosen.band = band;
      break;
    }
  }

  // 3) the fastest schedule on the whole batch (pixels only)
  std::vector<bh_frame> bf(static_cast<size_t>(n));
  for (int i = 0; i < n; ++i) {
    bf[i].pixels = mem.get(size_t(scenes[i].camera.width) * scenes[i].camera.height * 4, &e);
    bf[i].hit_class = nullptr;
    bf[i].aux = nullptr;
    if (e != cudaSuccess) return cuda_err(ctx, e, "tuner batch buffers");
  }
  double best = 1e30;
  bh_render_options best_o = chosen;
  auto time_candidate = [&](const bh_render_options& c) -> int {
    double ms = 1e30;
    for (int rep = 0; rep < 2; ++rep) {
      if ((rc = render_on_device(ctx, scenes, n, bf.data(), c, ctx->stream))) return rc;
      bh_render_stats st;
      if ((rc = bh_get_stats(ctx, &st))) return rc;
      ms = std::min(ms, st.kernel_ms);
    }
    report->candidates++;
    if (ms < best) {
      best = ms;
      best_o = c;
    }
    return BH_OK;
  };
  // persistent: block size, refill threshold, slice
  for (int threads : {128, 256})
    for (int refill : {16, 32})
      for (int slice : {128, 256, 512}) {
        bh_render_options c = chosen;
        c.schedule = BH_SCHEDULE_PERSISTENT;
        c.threads_per_block = threads;
        c.refill_threshold = refill;
        c.slice_steps = slice;
        c.format = BH_FORMAT_BGRA8;
        if ((rc = time_candidate(c))) return rc;
      }
  // hybrid (grid FP32 pass beside the persistent FP64 band pass) and grid
  // (band rays inline): block shape and rays per thread (tall blocks: on the
  // 120-frame 1080p fly-through 8x16 blocks took 5.64 / 5.55 / 5.50 / 5.45 ms
  // with 8 / 16 / 32 / 68 tiles per block)
  static const int kShapes[][2] = {{8, 16}, {8, 8}, {16, 8}, {32, 4}};
  for (const auto& sh : kShapes)
    for (int rpt : {8, 16, 32, 64}) {
      bh_render_options c = chosen;
      c.schedule = BH_SCHEDULE_HYBRID;
      c.block_x = sh[0];
      c.block_y = sh[1];
      c.rays_per_thread = rpt;
      // the band pass's block: 256 threads took the impact-parameter grid
      // (20 % band rays) from 57.9 to 43.6 ms against 128, the fly-through alike
      c.threads_per_block = 256;
      c.format = BH_FORMAT_BGRA8;
      if ((rc = time_candidate(c))) return rc;
    }
  // the band pass's block for the fastest hybrid candidate: 512 threads (16
  // warps per SM) suit a band of many double-float rays (impact-parameter
  // grid 43.6 -> 40.9 ms), 256 a few long chains, which the band pass's other
  // warps slow (photon ring 1.98 against 2.13 ms)
  if (best_o.schedule == BH_SCHEDULE_HYBRID) {
    bh_render_options c = best_o;
    c.threads_per_block = 512;
    c.format = BH_FORMAT_BGRA8;
    if ((rc = time_candidate(c))) return rc;
  }
  for (int rpt : {1, 4, 16}) {
    bh_render_options c = chosen;
    c.schedule = BH_SCHEDULE_GRID;
    c.block_x = 8;
    c.block_y = 16;
    c.rays_per_thread = rpt;
    c.format = BH_FORMAT_BGRA8;
    if ((rc = time_candidate(c))) return rc;
  }
  best_o.format = opts->format;
  report->kernel_ms = best;
  *opts = best_o;
  cache_store(cache_path, key, best_o, *report);
  return BH_OK;
}

// ---- probes ----------------------------------------------------------------------
int bh_probe_fp32_peak(bh_ctx* ctx, double* tflops, int32_t* sm_count) {
  if (!ctx || !tflops) return BH_ERR_INVALID_ARGUMENT;
  BH_CUDA(ctx, cudaSetDevice(ctx->device));
  float* sink = nullptr;
  BH_CUDA(ctx, cudaMalloc(&sink, sizeof(float) * 65536));
  const int threads = 256, blocks = ctx->sm_count * 8, iters = 4096;
  double best = 0;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(ctx->ev_start, ctx->stream);
    cudaError_t e = bhgb::launch_fp32_probe(sink, blocks, threads, iters, ctx->stream);
    cudaEventRecord(ctx->ev_stop, ctx->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(ctx->ev_stop);
    if (e != cudaSuccess) {
      cudaFree(sink);
      return cuda_err(ctx, e, "fp32 probe");
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop);
    const double flops = double(blocks) * threads * iters * 16 * 8 * 2;
    if (rep > 0) best = std::max(best, flops / (ms * 1e-3) / 1e12);
  }
  cudaFree(sink);
  *tflops = best;
  if (sm_count) *sm_count = ctx->sm_count;
  return BH_OK;
}

int bh_probe_fp64_peak(bh_ctx* ctx, double* tflops) {
  if (!ctx || !tflops) return BH_ERR_INVALID_ARGUMENT;
  BH_CUDA(ctx, cudaSetDevice(ctx->device));
  double* sink = nullptr;
  BH_CUDA(ctx, cudaMalloc(&sink, sizeof(double) * 65536));
  const int threads = 256, blocks = ctx->sm_count * 4, iters = 64;
  double best = 0;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(ctx->ev_start, ctx->stream);
    cudaError_t e = bhgb::launch_fp64_probe(sink, blocks, threads, iters, ctx->stream);
    cudaEventRecord(ctx->ev_stop, ctx->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(ctx->ev_stop);
    if (e != cudaSuccess) {
      cudaFree(sink);
      return cuda_err(ctx, e, "fp64 probe");
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop);
    const double flops = double(blocks) * threads * iters * 8 * 4 * 2;
    if (rep > 0) best = std::max(best, flops / (ms * 1e-3) / 1e12);
  }
  cudaFree(sink);
  *tflops = best;
  return BH_OK;
}

}  // extern "C"

// ---- differentiable render and its adjoint ----------------------------------------
namespace {

bool finite_n(const double* v, int n) {
  for (int i = 0; i < n; ++i)
    if (!std::isfinite(v[i])) return false;
  return true;
}

// Rodrigues rotation of v about the unit axis a by th (FP64, in place).
void rotate3(double* v, const double* a, double th) {
  const double c = std::cos(th), s = std::sin(th);
  const double k = dot3(a, v) * (1 - c);
  const double x[3] = {a[1] * v[2] - a[2] * v[1], a[2] * v[0] - a[0] * v[2], a[0] * v[1] - a[1] * v[0]};
  for (int i = 0; i < 3; ++i) v[i] = v[i] * c + x[i] * s + a[i] * k;
}

int scene_at_theta(const bh_scene& in, const double* th, bh_scene* out) {
  bh_scene s = in;
  const bh_camera& c0 = in.camera;
  auto rot = [&](double* v) {
    rotate3(v, c0.axis_x, th[BH_GRAD_ROLL]);
    rotate3(v, c0.axis_y, th[BH_GRAD_PITCH]);
    rotate3(v, c0.axis_z, th[BH_GRAD_YAW]);
  };
  rot(s.camera.axis_x);
  rot(s.camera.axis_y);
  rot(s.camera.axis_z);
  for (int i = 0; i < 3; ++i) s.camera.position[i] += th[BH_GRAD_CAM_X + i];
  s.hole.mass = th[BH_GRAD_MASS];
  bh_disc& d = s.disc;
  const double l1 = std::sqrt(dot3(in.disc.edge_s1, in.disc.edge_s1));
  if (l1 > 0) {
    const double e1[3] = {in.disc.edge_s1[0] / l1, in.disc.edge_s1[1] / l1, in.disc.edge_s1[2] / l1};
    // tilt about e1 through the centre; the bounding quad follows r_outer
    const double scale = in.disc.r_outer > 0 ? th[BH_GRAD_R_OUTER] / in.disc.r_outer : 1.0;
    double corner[3];
    for (int i = 0; i < 3; ++i) corner[i] = (in.disc.corner[i] - in.disc.center[i]) * scale;
    rotate3(corner, e1, th[BH_GRAD_TILT]);
    for (int i = 0; i < 3; ++i) {
      d.corner[i] = in.disc.center[i] + corner[i];
      d.edge_s1[i] = in.disc.edge_s1[i] * scale;
      d.edge_s2[i] = in.disc.edge_s2[i] * scale;
    }
    rotate3(d.edge_s1, e1, th[BH_GRAD_TILT]);
    rotate3(d.edge_s2, e1, th[BH_GRAD_TILT]);
    rotate3(d.normal, e1, th[BH_GRAD_TILT]);
  }
  d.r_inner = th[BH_GRAD_R_INNER];
  d.r_outer = th[BH_GRAD_R_OUTER];
  *out = s;
  return BH_OK;
}

int validate_adjoint_options(bh_ctx* ctx, const bh_adjoint_options& o) {
  if (o.precision < BH_PRECISION_FP32 || o.precision > BH_PRECISION_MIXED)
    return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "unknown precision %d", o.precision);
  if (!(o.step > 0 && o.step <= 0.3)) return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "step must be in (0, 0.3]");
  if (o.max_steps < 1 || o.max_steps > 1000000)
    return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "max_steps must be in [1, 1e6]");
  if (!(o.r_escape > 2.0) || !std::isfinite(o.r_escape))
    return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "r_escape must exceed the horizon (2 M)");
  if (!(o.softness > 0) || !std::isfinite(o.softness))
    return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "softness must be positive");
  if (!(o.band >= 0) || !std::isfinite(o.band)) return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "band must be >= 0");
  if (o.checkpoint_every != bhgb::adj::kSeg)
    return set_err(ctx, BH_ERR_UNSUPPORTED, "checkpoint_every must be %d", bhgb::adj::kSeg);
  if (o.threads_per_block != bhgb::adj::kAdjThreads)
    return set_err(ctx, BH_ERR_UNSUPPORTED, "threads_per_block must be %d", bhgb::adj::kAdjThreads);
  return BH_OK;
}

}  // namespace

extern "C" {

void bh_adjoint_default_options(bh_adjoint_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->precision = BH_PRECISION_MIXED;
  o->max_steps = 4000;
  o->step = 0.01;
  o->r_escape = 100.0;
  o->softness = 0.1;
  o->band = 0.3;
  o->checkpoint_every = bhgb::adj::kSeg;
  o->threads_per_block = bhgb::adj::kAdjThreads;
}

int bh_scene_at_theta(const bh_scene* scene, const double* theta, bh_scene* out) {
  if (!scene || !theta || !out) return BH_ERR_INVALID_ARGUMENT;
  if (!finite_n(theta, BH_GRAD_COUNT)) return BH_ERR_INVALID_ARGUMENT;
  return scene_at_theta(*scene, theta, out);
}

int bh_render_adjoint(bh_ctx* ctx, const bh_scene* scenes, int32_t n, const double* theta,
                      const bh_adjoint_frame* frames, const bh_adjoint_options* opts, bh_adjoint_result* results) {
  using namespace bhgb::adj;
  if (!ctx) return BH_ERR_INVALID_ARGUMENT;
  if (!scenes || !frames || n < 1 || n > 65535)
    return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "need 1..65535 scenes with frames");
  bh_adjoint_options o;
  bh_adjoint_default_options(&o);
  if (opts) {
    o = *opts;
    if (o.max_steps == 0) o.max_steps = 4000;
    if (o.step == 0) o.step = 0.01;
    if (o.r_escape == 0) o.r_escape = 100.0;
    if (o.softness == 0) o.softness = 0.1;
    if (o.band < 0) o.band = 0.3;
    if (o.checkpoint_every == 0) o.checkpoint_every = kSeg;
    if (o.threads_per_block == 0) o.threads_per_block = kAdjThreads;
  }
  int rc = validate_adjoint_options(ctx, o);
  if (rc) return rc;
  bh_render_options ro;
  bh_default_options(&ro);
  ro.integrator = BH_INTEGRATOR_RK4;
  ro.r_escape = o.r_escape;
  BH_CUDA(ctx, cudaSetDevice(ctx->device));
  if ((rc = ensure_pinned(ctx, ctx->h_adj, size_t(n)))) return rc;
  int64_t total_blocks = 0, total_rays = 0;
  for (int i = 0; i < n; ++i) {
    double th[BH_GRAD_COUNT];
    if (theta) {
      std::memcpy(th, theta + (size_t)i * BH_GRAD_COUNT, sizeof(th));
      if (!finite_n(th, BH_GRAD_COUNT))
        return set_err(ctx, BH_ERR_INVALID_ARGUMENT, "scene %d: theta has a non-finite value", i);
    } else {
      base_theta(scenes[i], th);
    }
    if (scenes[i].n_objects != 0)
      return set_err(ctx, BH_ERR_UNSUPPORTED, "scene %d: the differentiable render draws no objects", i);
    if (scenes[i].n_extra_holes != 0)
      return set_err(ctx, BH_ERR_UNSUPPORTED, "scene %d: the differentiable render traces one hole", i);
    bh_scene posed;
    scene_at_theta(scenes[i], th, &posed);
    if ((rc = validate_scene(ctx, posed, i, ro))) return rc;
    if (posed.disc.enabled && posed.disc.mapping != BH_DISC_MAP_POLAR)
      return set_err(ctx, BH_ERR_UNSUPPORTED, "scene %d: the differentiable render maps the disc POLAR", i);
    const double* hp = scenes[i].hole.position;
    const double* dc = scenes[i].disc.center;
    if (posed.disc.enabled &&
        std::sqrt((dc[0] - hp[0]) * (dc[0] - hp[0]) + (dc[1] - hp[1]) * (dc[1] - hp[1]) +
                  (dc[2] - hp[2]) * (dc[2] - hp[2])) > 1e-9 * std::max(1.0, posed.hole.mass))
      return set_err(ctx, BH_ERR_UNSUPPORTED, "scene %d: the differentiable render needs the disc centred on the hole", i);
    AdjScene* a = ctx->h_adj.ptr + i;
    std::memset(a, 0, sizeof(*a));
    build_adj_scene(scenes[i], th, o.softness, a);
    a->tex32 = o.precision == BH_PRECISION_MIXED ? 1 : 0;
    a->disc_on = posed.disc.enabled ? 1 : 0;
    if (a->disc_on) {
      const TexEntry& t = ctx->textures[posed.disc.texture];
      a->disc_tex = bhgb::DevTexture{t.texels, t.width, t.height};
    }
    a->has_bg = posed.background >= 0 ? 1 : 0;
    if (a->has_bg) {
      const TexEntry& t = ctx->textures[posed.background];
      a->bg_tex = bhgb::DevTexture{t.texels, t.width, t.height};
    }
    a->scene = i;
    a->block_begin = total_blocks;
    a->ray_begin = total_rays;
    a->target = frames[i].target;
    a->image = frames[i].image;
    a->pixel_grad = frames[i].pixel_grad;
    const int64_t tiles = int64_t(a->tiles_x) * ((posed.camera.height + 3) / 4);
    total_blocks += (tiles + 3) / 4;
    total_rays += int64_t(posed.camera.width) * posed.camera.height;
  }
  int main_grid = 0, band_grid = 0;
  BH_CUDA(ctx, plan_adjoint(o.precision, ctx->sm_count, total_blocks, &main_grid, &band_grid));
  const int64_t nseg = (o.max_steps - 1) / kSeg + 1;
  const bool any_target = [&] {
    for (int i = 0; i < n; ++i)
      if (frames[i].target) return true;
    return false;
  }();
  AdjLaunch L{};
  L.scenes = nullptr;
  L.n_scenes = n;
  L.precision = o.precision;
  L.p.c32 = exact_rk4_consts_f32(o.step, 1.0 / o.r_escape, o.max_steps);
  L.p.c64 = bhgb::make_rk4_consts<double>(o.step, 1.0 / o.r_escape, o.max_steps);
  L.p.inv_h32 = 1.0 / double(L.p.c32.h);
  L.p.inv_h64 = 1.0 / o.step;
  L.p.hstep32 = double(L.p.c32.h);
  L.p.hstep64 = o.step;
  set_df_consts(&L.p);
  L.pband = band_view(L.p);
  L.max_cross = max_crossings(o.max_steps, o.step);
  L.p.softness = o.softness;
  L.p.band = o.band;
  L.p.kmax = o.max_steps;
  L.p.want_grad = any_target ? 1 : 0;
  L.total_blocks = total_blocks;
  L.total_rays = total_rays;
  L.ckpt_slots = int64_t(main_grid) * kAdjThreads;
  L.band_slots = int64_t(band_grid) * kAdjThreads;
  const size_t ck_bytes = any_target ? size_t(L.ckpt_slots) * nseg * checkpoint_bytes(o.precision) : 16;
  const size_t traj_bytes = any_target && band_grid ? size_t(L.band_slots) * (o.max_steps + 1) * sizeof(float2) : 16;
  const size_t cross_bytes = any_target && band_grid ? size_t(L.band_slots) * L.max_cross * sizeof(float) : 16;
  const size_t xw_bytes = any_target && band_grid ? size_t(L.band_slots) * L.max_cross * sizeof(double2) : 16;
  const size_t xw_off = (traj_bytes + cross_bytes + 15) / 16 * 16;
  if ((rc = ensure_dev(ctx, ctx->d_adj, size_t(n)))) return rc;
  if ((rc = ensure_dev(ctx, ctx->adj_ckpt, ck_bytes))) return rc;
  if ((rc = ensure_dev(ctx, ctx->adj_ckpt_band, xw_off + xw_bytes))) return rc;
  if ((rc = ensure_dev(ctx, ctx->adj_acc, size_t(n) * kAccStride))) return rc;
  if ((rc = ensure_pinned(ctx, ctx->h_adj_acc, size_t(n) * kAccStride))) return rc;
  if ((rc = ensure_dev(ctx, ctx->adj_counters, size_t(kCounters)))) return rc;
  const uint32_t band_cap =
      o.precision == BH_PRECISION_MIXED ? uint32_t(std::min<int64_t>(total_rays, int64_t(1) << 30)) : 1u;
  if ((rc = ensure_dev(ctx, ctx->adj_band, size_t(band_cap)))) return rc;
  L.scenes = ctx->d_adj.ptr;
  L.ckpt = ctx->adj_ckpt.ptr;
  L.band_traj = reinterpret_cast<float2*>(ctx->adj_ckpt_band.ptr);
  L.band_cross = reinterpret_cast<float*>(ctx->adj_ckpt_band.ptr + traj_bytes);
  L.band_cross_xw = reinterpret_cast<double2*>(ctx->adj_ckpt_band.ptr + xw_off);
  L.band_list = ctx->adj_band.ptr;
  L.band_capacity = band_cap;
  L.counters = ctx->adj_counters.ptr;
  L.acc = ctx->adj_acc.ptr;
  cudaStream_t st = ctx->stream;
  BH_CUDA(ctx, cudaMemcpyAsync(ctx->d_adj.ptr, ctx->h_adj.ptr, sizeof(AdjScene) * n, cudaMemcpyHostToDevice, st));
  BH_CUDA(ctx, cudaMemsetAsync(ctx->adj_acc.ptr, 0, sizeof(double) * n * kAccStride, st));
  BH_CUDA(ctx, cudaMemsetAsync(ctx->adj_counters.ptr, 0, sizeof(unsigned long long) * kCounters, st));
  BH_CUDA(ctx, cudaEventRecord(ctx->ev_start, st));
  if (o.precision == BH_PRECISION_MIXED && !ctx->side_stream) {
    BH_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->side_stream, cudaStreamNonBlocking));
    BH_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming));
    BH_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming));
  }
  BH_CUDA(ctx, launch_adjoint(L, main_grid, band_grid, st, ctx->side_stream, ctx->ev_fork, ctx->ev_join));
  BH_CUDA(ctx, cudaEventRecord(ctx->ev_stop, st));
  BH_CUDA(ctx, cudaMemcpyAsync(ctx->h_adj_acc.ptr, ctx->adj_acc.ptr, sizeof(double) * n * kAccStride,
                               cudaMemcpyDeviceToHost, st));
  BH_CUDA(ctx, cudaStreamSynchronize(st));
  float ms = 0;
  BH_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop));
  if (results) {
    for (int i = 0; i < n; ++i) {
      const double* a = ctx->h_adj_acc.ptr + (size_t)i * kAccStride;
      const double norm = 3.0 * double(scenes[i].camera.width) * double(scenes[i].camera.height);
      bh_adjoint_result& r = results[i];
      std::memset(&r, 0, sizeof(r));
      r.loss = a[0] / norm;
      for (int k = 0; k < BH_GRAD_COUNT; ++k) r.grad[k] = a[1 + k] / norm;
      r.steps = uint64_t(a[kAccSteps] + 0.5);
      r.band_rays = uint64_t(a[kAccBandRays] + 0.5);
      r.kernel_ms = ms;
    }
  }
  return BH_OK;
}

}  // extern "C"
