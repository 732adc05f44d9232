// bh_render_noalloc: the render entry point for callers that must not
// allocate memory at render time.
//
// Some hosts embed the tracer where allocation is not allowed or not safe:
// a real-time frame loop with a fixed memory budget, an engine that hands
// the library only pre-allocated device buffers, or code that runs while
// the device allocator is off limits. Such callers cannot use bh_render or
// bh_render_device, which grow their context's buffers with cudaMalloc when
// a call needs more room. This entry point takes everything from the caller
// (textures and frames in device memory, scenes on the host) and keeps its
// own scratch -- the work-queue counters, the resolved scene records and the
// FP64 band list of the mixed tracer -- in one file-scope device array of
// fixed size. It calls no cudaMalloc, cudaFree, cudaMallocHost or other
// allocating routine.
//
// The array (kScratchBytes, about 34 MiB: nearly all of it the band list,
// 9 bytes per ray for BH_NOALLOC_MAX_RAYS rays) belongs to every device that
// loads this library, for the life of the process. With lazy module loading
// (the CUDA default) the device reserves it when the module is first loaded
// on that device, which happens inside the first call of this entry point
// there; that first call also takes the array's device address with
// cudaGetSymbolAddress (with that device current) and keeps it for later
// calls. Make that first call during set-up, before any stream capture. The
// kept address is no longer valid after cudaDeviceReset on that device.
// Each call stages its scene records from a static host array into the device
// array with cudaMemcpyAsync; a call on a stream that is capturing is refused
// (BH_ERR_UNSUPPORTED), since the recorded copy would read that host array
// after later calls rewrote it. All calls share the array and it keeps the last
// call's contents: the counters are cleared on the caller's stream at the
// start of each call, and two calls whose work overlaps on the GPU
// (different streams, or the same stream from different host threads
// without ordering) race on it.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "bh_internal.h"

namespace {

using bhgb::DevCounters;
using bhgb::DevScene;
using bhgb::DevTexture;
using bhgb::LaunchParams;

constexpr size_t kAlign = 256;
constexpr size_t round_up(size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }
constexpr size_t kCountersOffset = 0;
constexpr size_t kScenesOffset = round_up(sizeof(DevCounters));
constexpr size_t kBandOffset = kScenesOffset + round_up(sizeof(DevScene) * BH_NOALLOC_MAX_SCENES);
constexpr size_t kScratchBytes = kBandOffset + sizeof(uint32_t) * bhgb::band_words(BH_NOALLOC_MAX_RAYS);
// The size the header states ("about 34 MiB").
static_assert(kScratchBytes > (33u << 20) && kScratchBytes < (35u << 20), "no-alloc scratch is about 34 MiB");

// The scratch: counters | scene records | band list.
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
unsigned char* g_scratch_ptr[kMaxDevices] = {};  // device address per device, 0 until set up
DevScene g_host_scenes[BH_NOALLOC_MAX_SCENES];   // host staging (static: nothing allocated)

int fail(char* err, int32_t len, int code, const char* fmt, ...) {
  if (err && len > 0) {
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(err, size_t(len), fmt, ap);
    va_end(ap);
  }
  return code;
}

bool finite3(const double* v) { return std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]); }
double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

void set3(double* d, float* f, double a, double b, double c) {
  d[0] = a; d[1] = b; d[2] = c;
  f[0] = float(a); f[1] = float(b); f[2] = float(c);
}

bool texture_ok(const bh_device_texture* t, int32_t n, int32_t id) {
  return id >= 0 && id < n && t[id].texels != nullptr && t[id].width > 0 && t[id].height > 0;
}

int64_t padded_rays(const bh_camera& c) { return int64_t((c.width + 7) / 8) * int64_t((c.height + 3) / 4) * 32; }

// Scene record of one scene (the same resolution as the context entry points).
void resolve(const bh_scene& s, const bh_frame& f, const bh_render_options& o, const bh_device_texture* tex,
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
  d->mass = s.hole.mass;
  d->b_c = 3.0 * std::sqrt(3.0) * s.hole.mass;
  d->r_h = 2.0 * s.hole.mass;
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
    d->disc_tex = DevTexture{static_cast<const uchar4*>(tex[q.texture].texels), tex[q.texture].width,
                             tex[q.texture].height};
  }
  d->has_bg = s.background >= 0 ? 1 : 0;
  if (s.background >= 0)
    d->bg_tex = DevTexture{static_cast<const uchar4*>(tex[s.background].texels), tex[s.background].width,
                           tex[s.background].height};
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
  d->pixels = static_cast<uint8_t*>(f.pixels);
  d->cls = f.hit_class;
  d->aux = f.aux;
  bhgb::resolve_frame_flags(d);
}

int check(const bh_scene* scenes, int32_t n, const bh_device_texture* tex, int32_t n_tex, const bh_frame* frames,
          const bh_render_options& o, int64_t* total, char* err, int32_t len) {
  if (!scenes || !frames || n < 1 || n > BH_NOALLOC_MAX_SCENES)
    return fail(err, len, BH_ERR_INVALID_ARGUMENT, "need 1..%d scenes with frames", BH_NOALLOC_MAX_SCENES);
  if (o.integrator == BH_INTEGRATOR_FLAT || o.integrator == BH_INTEGRATOR_MULTI)
    return fail(err, len, BH_ERR_UNSUPPORTED, "the no-alloc render has no FLAT or MULTI integrator");
  {
    char msg[160];
    if (int rc = bhgb::render_options_problem(o, msg, sizeof(msg))) return fail(err, len, rc, "%s", msg);
  }
  int64_t rays = 0;
  for (int i = 0; i < n; ++i) {
    const bh_scene& s = scenes[i];
    const bh_camera& c = s.camera;
    if (c.width < 1 || c.height < 1 || c.width > 32768 || c.height > 32768 || !frames[i].pixels)
      return fail(err, len, BH_ERR_INVALID_ARGUMENT, "scene %d: bad image size or no pixel buffer", i);
    if (!finite3(c.position) || !finite3(c.axis_x) || !finite3(c.axis_y) || !finite3(c.axis_z) ||
        !std::isfinite(c.focus_len) || !finite3(s.hole.position) || !(s.hole.mass > 0) ||
        !std::isfinite(s.hole.mass))
      return fail(err, len, BH_ERR_INVALID_ARGUMENT, "scene %d: non-finite camera or hole", i);
    if (s.background != -1 && !texture_ok(tex, n_tex, s.background))
      return fail(err, len, BH_ERR_BAD_TEXTURE, "scene %d: background texture %d is not valid", i, s.background);
    if (s.n_objects != 0)
      return fail(err, len, BH_ERR_UNSUPPORTED, "scene %d: the no-alloc render draws no objects", i);
    if (s.n_extra_holes != 0)
      return fail(err, len, BH_ERR_UNSUPPORTED, "scene %d: the no-alloc render traces one hole", i);
    if (frames[i].aux && o.integrator != BH_INTEGRATOR_RK4)
      return fail(err, len, BH_ERR_UNSUPPORTED, "frame %d: aux output needs the RK4 integrator", i);
    const double rel[3] = {c.position[0] - s.hole.position[0], c.position[1] - s.hole.position[1],
                           c.position[2] - s.hole.position[2]};
    if (o.integrator == BH_INTEGRATOR_RK4 && std::sqrt(dot3(rel, rel)) >= o.r_escape * s.hole.mass)
      return fail(err, len, BH_ERR_UNSUPPORTED, "scene %d: camera lies outside the escape radius", i);
    if (s.disc.enabled) {
      const bh_disc& d = s.disc;
      if (!texture_ok(tex, n_tex, d.texture))
        return fail(err, len, BH_ERR_BAD_TEXTURE, "scene %d: disc texture %d is not valid", i, d.texture);
      if (!finite3(d.center) || !finite3(d.normal) || !finite3(d.corner) || !finite3(d.edge_s1) ||
          !finite3(d.edge_s2) || !(d.r_inner >= 0) || !(d.r_outer > d.r_inner) || !std::isfinite(d.r_outer) ||
          (d.mapping != BH_DISC_MAP_REF_PLANAR && d.mapping != BH_DISC_MAP_POLAR) ||
          !(std::fabs(dot3(d.normal, d.normal) - 1.0) < 1e-6) || !(dot3(d.edge_s1, d.edge_s1) > 0) ||
          !(dot3(d.edge_s2, d.edge_s2) > 0))
        return fail(err, len, BH_ERR_INVALID_ARGUMENT, "scene %d: invalid disc", i);
      if (o.integrator == BH_INTEGRATOR_RK4) {
        const double off[3] = {d.center[0] - s.hole.position[0], d.center[1] - s.hole.position[1],
                               d.center[2] - s.hole.position[2]};
        const double scale = std::fmax(1.0, std::sqrt(dot3(off, off)) + s.hole.mass);
        if (std::fabs(dot3(d.normal, off)) > 1e-9 * scale || d.r_outer >= o.r_escape * s.hole.mass)
          return fail(err, len, BH_ERR_UNSUPPORTED, "scene %d: disc placement not supported by RK4", i);
      }
    }
    rays += padded_rays(c);
  }
  if (rays > BH_NOALLOC_MAX_RAYS)
    return fail(err, len, BH_ERR_INVALID_ARGUMENT,
                "%lld rays (scenes padded to 8x4 tiles) exceed the no-alloc maximum of %d per call",
                (long long)rays, BH_NOALLOC_MAX_RAYS);
  *total = rays;
  return BH_OK;
}

}  // namespace

extern "C" int bh_render_noalloc(int device, const bh_scene* scenes, int32_t n, const bh_device_texture* textures,
                                 int32_t n_textures, const bh_frame* frames, const bh_render_options* opts,
                                 void* stream, char* error, int32_t error_len) {
  if (error && error_len > 0) error[0] = '\0';
  bh_render_options o;
  bh_default_options(&o);
  if (opts) o = *opts;
  int64_t total = 0;
  int rc = check(scenes, n, textures, n_textures, frames, o, &total, error, error_len);
  if (rc) return rc;
  if (device < 0 || device >= kMaxDevices)
    return fail(error, error_len, BH_ERR_INVALID_ARGUMENT, "device %d out of range", device);

  std::lock_guard<std::mutex> lock(g_mutex);
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return fail(error, error_len, BH_ERR_NO_DEVICE, "cudaSetDevice: %s", cudaGetErrorString(e));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  {
    // A captured call would record a copy from g_host_scenes, which the next
    // call rewrites before the graph replays: refused before any device work.
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(st, &cap);
    if (e != cudaSuccess)
      return fail(error, error_len, BH_ERR_CUDA, "cudaStreamIsCapturing: %s", cudaGetErrorString(e));
    if (cap != cudaStreamCaptureStatusNone)
      return fail(error, error_len, BH_ERR_UNSUPPORTED,
                  "the stream is capturing: a call stages its scenes from a host array that the next call rewrites");
  }
  if (!g_scratch_ptr[device]) {  // once per device, with that device current
    void* ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_scratch);
    if (e != cudaSuccess || !ptr)
      return fail(error, error_len, BH_ERR_CUDA, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    g_scratch_ptr[device] = static_cast<unsigned char*>(ptr);
  }
  unsigned char* base = g_scratch_ptr[device];

  int64_t begin = 0;
  for (int i = 0; i < n; ++i) {
    resolve(scenes[i], frames[i], o, textures, begin, &g_host_scenes[i]);
    begin += padded_rays(scenes[i].camera);
  }
  bhgb::assign_grid_blocks(g_host_scenes, n, o.block_x, o.block_y, o.rays_per_thread);
  // From pageable host memory: returns once the records are staged by the
  // driver, so the static host array may be rewritten by the next call.
  e = cudaMemcpyAsync(base + kScenesOffset, g_host_scenes, sizeof(DevScene) * size_t(n), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(base + kCountersOffset, 0, sizeof(DevCounters), st);
  if (e != cudaSuccess) return fail(error, error_len, BH_ERR_CUDA, "staging: %s", cudaGetErrorString(e));

  LaunchParams p{};
  p.scenes = reinterpret_cast<const DevScene*>(base + kScenesOffset);
  p.n_scenes = n;
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
  p.total_rays = total;
  p.counters = reinterpret_cast<DevCounters*>(base + kCountersOffset);
  bhgb::carve_band(reinterpret_cast<uint32_t*>(base + kBandOffset), uint32_t(BH_NOALLOC_MAX_RAYS), &p.band_list,
                   &p.band_tmp, &p.band_key);
  p.band_capacity = uint32_t(BH_NOALLOC_MAX_RAYS);
  p.refill_threshold = o.refill_threshold;
  p.rays_per_thread = o.rays_per_thread > 0 ? o.rays_per_thread : 1;
  p.slice_steps = o.slice_steps;
  p.band_lanes = o.band_lanes;
  p.band_serial = o.band_serial;

  if (o.schedule == BH_SCHEDULE_GRID) {
    int32_t w[BH_NOALLOC_MAX_SCENES], h[BH_NOALLOC_MAX_SCENES];
    for (int i = 0; i < n; ++i) {
      w[i] = scenes[i].camera.width;
      h[i] = scenes[i].camera.height;
    }
    e = bhgb::launch_grid(p, w, h, o.block_x, o.block_y, st);
  } else if (o.schedule == BH_SCHEDULE_HYBRID) {
    int32_t w[BH_NOALLOC_MAX_SCENES], h[BH_NOALLOC_MAX_SCENES];
    for (int i = 0; i < n; ++i) {
      w[i] = scenes[i].camera.width;
      h[i] = scenes[i].camera.height;
    }
    e = bhgb::launch_hybrid(p, w, h, o.block_x, o.block_y, o.threads_per_block, st);
  } else {
    int per_sm = o.blocks_per_sm, sms = 0;
    if (per_sm == 0) {
      e = bhgb::persistent_occupancy(p, o.threads_per_block, &per_sm);
      if (e != cudaSuccess) return fail(error, error_len, BH_ERR_CUDA, "occupancy: %s", cudaGetErrorString(e));
      if (per_sm < 1) per_sm = 1;
    }
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = bhgb::launch_persistent(p, o.threads_per_block, per_sm * sms, st);
  }
  if (e != cudaSuccess) return fail(error, error_len, BH_ERR_CUDA, "launch: %s", cudaGetErrorString(e));
  return BH_OK;
}
