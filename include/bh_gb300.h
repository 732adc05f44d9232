/*
 * bh_gb300.h -- C ABI of the GB300 (sm_103a) geodesic ray tracer.
 *
 * This is the drop-in boundary for the per-pixel Schwarzschild geodesic render
 * of lackhole/blackhole_8. In the reference that render is not a library call:
 * it is the body of the frame loop in
 * include/blackhole/blackhole_solution_test.cc:161-298, fed by
 *   - Camera<double>            (camera.h:21-71)
 *   - StaticBlackhole<double>   (blackhole_solution.h:16-96)
 *   - Annulus<double> + texture (object/vector_object.h:306-356,
 *                                object/material.h:29-35)
 *   - ObjectManager<double>     (object/object_manager.h:69-85)
 * and it writes a CV_8UC3 (BGR) cv::Mat (blackhole_solution_test.cc:117,
 * 214, 229-233). This header replaces that loop with plain C entry points:
 * scenes are POD structs of resolved world-space poses, textures are uploaded
 * once, frames are written to caller-owned buffers.
 *
 * Conventions
 *   - Every function returns an int status: BH_OK (0) or a negative BH_ERR_*;
 *     bh_last_error() gives the message. Nothing aborts the process (the
 *     reference calls std::terminate on an empty texture, material.h:30-33).
 *   - The caller owns every host buffer. Textures are copied at upload.
 *   - One context = one CUDA device + one CUDA stream. A context is not
 *     re-entrant: use one per host thread.
 *   - Lengths are world units; angles are radians.
 */
#ifndef BH_GB300_H_
#define BH_GB300_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BH_ABI_VERSION 3

/* ---- status codes -------------------------------------------------------- */
enum {
  BH_OK = 0,
  BH_ERR_INVALID_ARGUMENT = -1,
  BH_ERR_EMPTY_TEXTURE = -2,
  BH_ERR_BAD_TEXTURE = -3,
  BH_ERR_CUDA = -4,
  BH_ERR_OUT_OF_MEMORY = -5,
  BH_ERR_UNSUPPORTED = -6,
  BH_ERR_TIMEOUT = -7,
  BH_ERR_NO_DEVICE = -8,
  BH_ERR_DEVICE_FAULT = -9
};

/* ---- enumerations --------------------------------------------------------- */
/* Integrator. REF_TRAPEZOID is the reference's own scheme: dphi/du = 1/sqrt(G)
 * by a 20+20-segment trapezoid rule in u with straight-chord collision tests
 * (blackhole_solution_test.cc:185-296). RK4 integrates u'' = -u + 3 M u^2 in
 * phi with a fixed step of a fourth-order method and exact horizon / escape /
 * disc-plane events: classical RK4 in FP64 (the oracle's scheme), Nystrom's
 * three-stage method for y'' = f(y) in FP32 (fewer instructions, a smaller
 * error constant on this equation); the scene's objects are tested on the
 * chord of every step. FLAT is the
 * reference's flat-space RayTracer (ray_tracer.h:52-96 with
 * BasicLinearRayRecurrence, driven as in ray_tracer_test.cc:140-155): ten
 * straight chords from the focus through the PixelVector point, the step
 * scaled by 100 / |step|^2 when |step|^2 < 100, tested against the objects
 * and the disc; the hole does not bend or stop it (GRID schedule only).
 * MULTI traces the scene's hole and its extra_holes together (the reference
 * only sketches this, multiple_blackhole_solution_test.cc:149-262, by
 * averaging per-hole plane solutions): null rays of the static metric
 *   ds^2 = -a^2 dt^2 + p^4 (dx^2 + dy^2 + dz^2),
 *   p = 1 + S, a = (1 - S) / (1 + S), S = sum_i m_i / (2 |x - x_i|),
 * with every position taken as an isotropic coordinate. For one hole this is
 * Schwarzschild (areal radius r = rho (1 + m / 2 rho)^2); p is the
 * Brill-Lindquist conformal factor of several holes. Rays follow Fermat's
 * principle with index n = p^2 / a, integrated by RK4 in Euclidean arc
 * length with step `step` times the distance to the nearest hole. A ray is
 * captured where S reaches 0.9, escapes through the sphere of radius
 * r_escape * (sum of masses) about the holes' centre of mass, and is tested
 * against the disc (the curved step, Hermite-interpolated) and the objects
 * (the step's chord) on every step (GRID schedule, FP32 or FP64). */
enum { BH_INTEGRATOR_REF_TRAPEZOID = 0, BH_INTEGRATOR_RK4 = 1, BH_INTEGRATOR_FLAT = 2, BH_INTEGRATOR_MULTI = 3 };

/* Arithmetic. MIXED (RK4 only): FP32 bulk; rays whose impact parameter lies
 * within `band` of 3*sqrt(3)*M integrate with FP64 accuracy (double-float on
 * the FP32 pipe, FP64 for the few within ~1e-7 M and for their events); the
 * first integral of rays within `setup_band` and disc-crossing refinement near
 * the disc edges exact to double-float. */
enum { BH_PRECISION_FP32 = 0, BH_PRECISION_FP64 = 1, BH_PRECISION_MIXED = 2 };

/* Ray generation. REF reproduces the reference: the ray runs from the focus
 * toward the point Camera::PixelVector(x, y) (a direction, camera.h:55-59,
 * used as a point at blackhole_solution_test.cc:167-170). PINHOLE runs it
 * along PixelVector(x, y) from the focus. */
enum { BH_RAYGEN_REF = 0, BH_RAYGEN_PINHOLE = 1 };

/* Disc texture mapping. REF_PLANAR is Rectangle::color (vector_object.h:
 * 159-179): nearest texel on the quad basis s1 = v2 - v1, s2 = v4 - v1.
 * POLAR: x = (r - r_inner) / (r_outer - r_inner), y = azimuth / 2pi about
 * e1 = s1/|s1|, e2 = normal x e1. */
enum { BH_DISC_MAP_REF_PLANAR = 0, BH_DISC_MAP_POLAR = 1 };

/* Framebuffer formats. BGR8 is the reference's CV_8UC3 layout. */
enum { BH_FORMAT_BGRA8 = 0, BH_FORMAT_BGR8 = 1, BH_FORMAT_RGBA8 = 2 };

/* Texture layouts accepted by bh_texture_create. BGR8 is cv::Mat CV_8UC3. */
enum { BH_TEXEL_BGR8 = 0, BH_TEXEL_RGB8 = 1, BH_TEXEL_BGRA8 = 2, BH_TEXEL_RGBA8 = 3 };

/* Work schedule. GRID: one thread per pixel of rays_per_thread block tiles
 * over a 2-D grid per frame (MIXED: FP64 band rays traced inline).
 * PERSISTENT: one work-stealing launch over every frame of the call, warps
 * refill finished lanes with new rays; FP64 band rays are deferred to a
 * second persistent pass. HYBRID (RK4, FP32 or MIXED): MIXED runs the FP32
 * pass on the GRID schedule with the FP64 band rays deferred to the
 * persistent FP64 pass, which runs beside it; FP32 is the GRID schedule. */
enum { BH_SCHEDULE_GRID = 0, BH_SCHEDULE_PERSISTENT = 1, BH_SCHEDULE_HYBRID = 2 };

/* Per-pixel hit classes written to bh_frame.hit_class. OBJECT: one of the
 * scene's bh_objects (aux holds its index). */
enum { BH_CLASS_MISS = 0, BH_CLASS_HORIZON = 1, BH_CLASS_DISC = 2, BH_CLASS_MAXSTEPS = 3, BH_CLASS_OBJECT = 4 };

/* Ordinary objects (object/vector_object.h, object/pattern.h). Each is drawn
 * where a chord of the ray crosses it, the hit nearest the chord's start
 * first, as ObjectManager::FindCollision (object_manager.h:69-85). On exact
 * distance ties the reference keeps the first object its map visits; with
 * the disc inserted first, the hole second and the objects after them in
 * table order, libstdc++ visits the objects from last to first, then the
 * hole, then the disc, and so does the tracer.
 * RECTANGLE: Rectangle<T> (vector_object.h:80-183) with vertex()[1..4] =
 *   v[0..3]: the chord crosses the plane of v1, v2, v4 inside the quad;
 *   colour by Rectangle::color from `texture` (nearest texel, truncating
 *   casts; indices clamped to the texture where the reference reads
 *   outside it), or black with texture -1.
 * TRIANGLE: Triangle<T> (vector_object.h:18-77), Moller-Trumbore on
 *   vertex()[1..3] = v[0..2] with epsilon 10 * machine epsilon of the
 *   arithmetic; drawn black (it has no colour of its own, material.h:54).
 * PLANE: InfinitePlane<T> (vector_object.h:187-238) through position() =
 *   v[0] with unit axes axis_x, axis_y and normal axis_z (Object<T> axes);
 *   colour ChessPattern2D<T>{pattern_size} (pattern.h:14-46) at the plane
 *   coordinates InfinitePlane::color derives from the hit's world x and y,
 *   or black with pattern_size <= 0. */
enum { BH_OBJECT_RECTANGLE = 1, BH_OBJECT_TRIANGLE = 2, BH_OBJECT_PLANE = 3 };

typedef struct bh_object {
  int32_t type;        /* BH_OBJECT_* */
  int32_t texture;     /* RECTANGLE: texture id from bh_texture_create, or -1 */
  double v[4][3];      /* vertices (world coordinates), see above */
  double axis_x[3];    /* PLANE: vector_x(), vector_y(), vector_z() */
  double axis_y[3];
  double axis_z[3];
  double pattern_size; /* PLANE: ChessPattern2D pattern size */
} bh_object;

/* Objects per scene accepted by the render calls. */
#define BH_MAX_OBJECTS 64
/* Holes per scene (the scene's hole and its extra holes) of the MULTI integrator. */
#define BH_MAX_HOLES 8

/* ---- scene ------------------------------------------------------------------ */
/* Camera<T> state (camera.h:21-71 on Object<T>, object/object.h:23-118). */
typedef struct bh_camera {
  double position[3];  /* focus() = Object::position() */
  double axis_x[3];    /* vector_x(): viewing direction */
  double axis_y[3];    /* vector_y(): +x image direction */
  double axis_z[3];    /* vector_z(): +y image direction */
  double focus_len;    /* width / (2 tan(fov/2)), camera.h:37-41 */
  int32_t width;
  int32_t height;
} bh_camera;

/* StaticBlackhole<T> (blackhole_solution.h:24-25). */
typedef struct bh_hole {
  double position[3];
  double mass;
} bh_hole;

/* Annulus<T> (vector_object.h:306-356) and its texture. */
typedef struct bh_disc {
  double center[3];    /* vertex()[0] */
  double normal[3];    /* norm_: fixed at construction, vector_object.h:325 */
  double corner[3];    /* vertex()[1] */
  double edge_s1[3];   /* vertex()[2] - vertex()[1] */
  double edge_s2[3];   /* vertex()[4] - vertex()[1] */
  double r_inner;
  double r_outer;
  int32_t texture;     /* id from bh_texture_create; must be valid if enabled */
  int32_t mapping;     /* BH_DISC_MAP_* */
  int32_t enabled;     /* 0: scene has no disc */
  int32_t reserved;
} bh_disc;

typedef struct bh_scene {
  bh_camera camera;
  bh_hole hole;
  bh_disc disc;
  int32_t background;  /* equirectangular texture id, or -1: escaped rays stay
                          black as in the reference (screen is zeroed,
                          blackhole_solution_test.cc:140) */
  int32_t n_objects;   /* entries of `objects` (0..BH_MAX_OBJECTS) */
  const bh_object* objects; /* host memory, read during the call; NULL when
                          n_objects is 0. Objects need the GRID schedule and
                          FP32 or FP64 (not MIXED), and no differentiable
                          render. */
  int32_t n_extra_holes; /* entries of `extra_holes` (0..BH_MAX_HOLES - 1);
                          non-zero only with the MULTI integrator */
  int32_t reserved_holes;
  const bh_hole* extra_holes; /* host memory, read during the call; NULL when
                          n_extra_holes is 0 */
} bh_scene;

/* One output frame; width and height come from the scene's camera. */
typedef struct bh_frame {
  void* pixels;        /* width*height*bytes_per_pixel(format), row-major */
  uint8_t* hit_class;  /* optional (NULL): width*height BH_CLASS_* */
  float* aux;          /* optional (NULL): width*height. RK4: deflection
                          angle (rad) of escaped rays, hit radius (units of M)
                          of disc hits; MULTI: the angle (rad) between the
                          ray's first and last direction of escaped rays, the
                          hit's distance from the disc centre (units of the
                          scene hole's mass) of disc hits; RK4, MULTI and
                          FLAT: the object's index of object hits; 0
                          otherwise (not REF_TRAPEZOID) */
} bh_frame;

typedef struct bh_render_options {
  int32_t integrator;        /* BH_INTEGRATOR_* (default RK4) */
  int32_t precision;         /* BH_PRECISION_* (default FP32) */
  int32_t raygen;            /* BH_RAYGEN_* (default REF) */
  int32_t format;            /* BH_FORMAT_* (default BGRA8) */
  int32_t schedule;          /* BH_SCHEDULE_* (default GRID) */
  int32_t max_steps;         /* RK4 / MULTI step cap (default 4000) */
  double step;               /* RK4 step in phi (default 0.01); MULTI: step
                                length per unit distance to the nearest hole */
  double r_escape;           /* RK4 escape radius in units of M (default 100);
                                MULTI: in units of the holes' total mass */
  double band;               /* MIXED: rays with |b - 3 sqrt(3) M| < band * M are
                                traced with FP64 accuracy (double-float, FP64
                                within ~1e-7 M) with step band_step
                                (default 5e-4) */
  int32_t block_x;           /* GRID block shape (default 8 x 16: each warp an
                                8 x 4 pixel tile) */
  int32_t block_y;
  int32_t threads_per_block; /* PERSISTENT block size (32..256); HYBRID: the
                                band pass's block size (32..512, default 256) */
  int32_t blocks_per_sm;     /* PERSISTENT CTAs per SM (default: occupancy) */
  int32_t refill_threshold;  /* PERSISTENT: refill a warp once this many lanes
                                are idle (default 32) */
  double band_step;          /* MIXED: RK4 step of the band (default 0.01) */
  double setup_band;         /* MIXED: rays with |b - 3 sqrt(3) M| < setup_band * M
                                take their first integral 1/b^2 - 1/27 exactly
                                (double-float)
                                (default 0.1; raised to band + 2e-3 when
                                smaller) */
  int32_t slice_steps;       /* PERSISTENT: integration steps between refill
                                checks (default 256) */
  int32_t band_lanes;        /* MIXED + PERSISTENT: lanes per warp that trace
                                FP64 band rays (1..32, default 32) */
  int32_t band_serial;       /* MIXED + PERSISTENT or HYBRID: 0 (default) = the
                                FP64 band pass runs beside the FP32 pass from
                                its start and launches it from the device;
                                1 = the FP32 pass, then the FP64 pass, both
                                launched by the host (each pass on its own,
                                e.g. to profile); 2 = the FP64 pass, then the
                                FP32 pass, both launched by the host (no
                                launch from the device) */
  int32_t rays_per_thread;   /* GRID / HYBRID: pixels each thread traces, from
                                that many consecutive block tiles down the
                                image, one after the other (1..128; 0 = 1, the
                                default) */
  int32_t reserved[2];
} bh_render_options;

/* Counters of the most recent render on a context. */
#define BH_STATS_DIRECT_HOST 256u
typedef struct bh_render_stats {
  uint64_t rays;          /* pixels traced */
  uint64_t steps;         /* integration steps summed over rays */
  uint64_t band_rays;     /* rays traced in FP64 because of the band */
  uint64_t band_steps;    /* steps of those rays */
  uint64_t band_overflow; /* band rays that found no slot in the band list
                             (0: the list holds one slot per ray) */
  uint64_t flags;         /* device bits (0 = none): 1 = band list full,
                             2 = MIXED + PERSISTENT or HYBRID: the
                             device-side launch of the FP32 pass failed and
                             the host's launch after it traced the bulk
                             (image still complete); host bit
                             BH_STATS_DIRECT_HOST: bh_render's kernels wrote
                             the frames into host memory directly */
  double kernel_ms;       /* device time of the launches, CUDA events */
  uint64_t h2d_bytes;     /* bytes copied host -> device by the call */
  uint64_t d2h_bytes;     /* bytes copied device -> host by the call
                             (frames; the counters excluded) */
} bh_render_stats;

typedef struct bh_ctx bh_ctx;
typedef struct bh_sequence bh_sequence;

/* ---- context ---------------------------------------------------------------- */
int bh_abi_version(void);
void bh_default_options(bh_render_options* opts);
int bh_create(bh_ctx** out, int device);
void bh_destroy(bh_ctx* ctx);
const char* bh_last_error(const bh_ctx* ctx);
/* Stream used by the context (a cudaStream_t). */
void* bh_stream(bh_ctx* ctx);

/* ---- textures (Material<T>::SetTexture, material.h:29-35) --------------------
 * Copies a width x height texture to the device. An empty texture returns
 * BH_ERR_EMPTY_TEXTURE where the reference terminates. row_stride in bytes
 * (0 = packed). */
int bh_texture_create(bh_ctx* ctx, const uint8_t* texels, int32_t width, int32_t height,
                      int32_t layout, int64_t row_stride, int32_t* out_id);
int bh_texture_destroy(bh_ctx* ctx, int32_t id);

/* ---- render ---------------------------------------------------------------
 * Replaces the frame body blackhole_solution_test.cc:161-298 for n scenes.
 * bh_render: host frames; uploads the scenes, renders, copies the frames back
 * and returns when they are in host memory. When every buffer of every frame
 * is page-locked host memory the device can address (cudaHostAlloc,
 * cudaMallocHost or cudaHostRegister) and the schedule is GRID or HYBRID,
 * the kernels write the frames there directly (no device copy, no
 * copy-back; stats flag BH_STATS_DIRECT_HOST); BGR8 frames are then written
 * with blocks 32 pixels wide (same threads per block) and at most 32 tiles
 * per thread, so that each warp stores whole 96-byte row segments over the
 * host link.
 * bh_render_device: frames in device memory; enqueued on `stream` (a
 * cudaStream_t, NULL = the context's stream) and returns without waiting. */
int bh_render(bh_ctx* ctx, const bh_scene* scenes, int32_t n, const bh_frame* frames,
              const bh_render_options* opts);
int bh_render_device(bh_ctx* ctx, const bh_scene* scenes, int32_t n, const bh_frame* frames,
                     const bh_render_options* opts, void* stream);
/* Waits for the context's work and returns the counters of the last render. */
int bh_get_stats(bh_ctx* ctx, bh_render_stats* out);

/* ---- captured sequences (camera fly-through as one CUDA graph) --------------
 * Captures the render of n scenes into device frames as a CUDA graph. The
 * scenes can be replaced between launches (same count, sizes and textures);
 * the new poses are copied into the graph's own device buffer by the launch.*/
int bh_sequence_create(bh_ctx* ctx, const bh_scene* scenes, int32_t n, const bh_frame* frames,
                       const bh_render_options* opts, bh_sequence** out);
int bh_sequence_update(bh_sequence* seq, const bh_scene* scenes, int32_t n);
int bh_sequence_launch(bh_sequence* seq, void* stream);
/* Waits for the last launch of the sequence and returns its counters
 * (kernel_ms is not measured for sequences and reads 0). */
int bh_sequence_stats(bh_sequence* seq, bh_render_stats* out);
void bh_sequence_destroy(bh_sequence* seq);

/* ---- autotuner -----------------------------------------------------------------------
 * No counterpart in the reference. Chooses the mixed-precision batched
 * tracer's RK4 step, FP64 band width, schedule and its shape (persistent:
 * block size, refill threshold, slice length; grid: block shape and rays per
 * thread) for a batch of scenes:
 *   1. renders a sample of the scenes (up to 16, evenly spaced, fewer while
 *      they hold more than eight 1920x1080 frames of pixels; at least 4) in
 *      FP64 with the options' step as the reference (the oracle's scheme);
 *   2. takes the largest step in {0.2, 0.175, 0.15, 0.125, 0.1, 0.08, 0.05,
 *      0.04, 0.03, 0.02, 0.01} whose MIXED render of the sample stays within
 *      max_error / 2 rad of the reference deflection on every escaped ray
 *      with an agreeing class, with classes agreeing on >= 99.99 % of pixels;
 *   3. takes the narrowest FP64 band in {2e-5, 1e-4} (when below the
 *      options' band) whose MIXED render of the sample meets the same bound;
 *   4. times the schedule candidates on the whole batch and keeps the
 *      fastest: PERSISTENT with threads {128, 256} x refill {16, 32} x
 *      slice {128, 256, 512}; HYBRID with block shapes {8x16, 8x8, 16x8,
 *      32x4} x rays per thread {2, 4, 8}; GRID 8x16 with rays per thread
 *      {1, 4}.
 * `opts` is read as the base (integrator must be RK4) and overwritten with
 * the choice (precision MIXED). When cache_path is not
 * NULL the choice is looked up there first (key: device, batch shape,
 * max_error) and appended after tuning. The sample's renders and the timing
 * frames use the context's device buffers. */
typedef struct bh_tune_report {
  double step;             /* chosen RK4 step */
  double max_deflection;   /* max |deflection - FP64 reference| at that step (rad) */
  double max_radius_error; /* max |disc hit radius - FP64 reference| (units of M) */
  double class_mismatch;   /* fraction of sample pixels whose class differs */
  double kernel_ms;        /* device time of the chosen configuration on the batch */
  int32_t candidates;      /* configurations rendered */
  int32_t from_cache;      /* 1 when the choice came from the cache file */
} bh_tune_report;
int bh_autotune(bh_ctx* ctx, const bh_scene* scenes, int32_t n, bh_render_options* opts, double max_error,
                const char* cache_path, bh_tune_report* report);

/* ---- render without allocating -------------------------------------------------
 * No counterpart in the reference (it renders on the CPU and never allocates
 * device memory). For callers that may not allocate at render time -- a
 * real-time frame loop with a fixed memory budget, or a host that gives the
 * library only pre-allocated device buffers -- and so cannot use bh_render or
 * bh_render_device, whose contexts grow their buffers with cudaMalloc.
 * Textures (BGRA8, caller-owned device memory, indexed by the scenes'
 * texture ids) and frames are in device memory; scenes are on the host and
 * carry no objects (n_objects 0; the FLAT integrator is not offered). The
 * library's own scratch (counters, scene records, the FP64 band list) lives
 * in one fixed device array of about 34 MiB that every device loading the
 * library holds until exit; calls are limited to BH_NOALLOC_MAX_SCENES scenes
 * and BH_NOALLOC_MAX_RAYS rays (scenes padded to 8x4 tiles) and are rejected
 * with BH_ERR_INVALID_ARGUMENT above that. The first call on a device loads
 * the library's device code there, which reserves the array, and takes the
 * array's address: make that first call during set-up, before any stream
 * capture. The address is kept for later calls and is no longer valid after
 * cudaDeviceReset. Each call copies its scene records from a static host
 * array with cudaMemcpyAsync; a call on a stream that is capturing is refused
 * with BH_ERR_UNSUPPORTED (the recorded copy would read that host array after
 * later calls rewrote it). All calls share the array: calls whose work
 * overlaps on the GPU race. Enqueued on `stream`
 * (a cudaStream_t, NULL = the legacy default stream); returns without
 * waiting. `error` (may be NULL) receives a message of at most error_len
 * bytes. */
#define BH_NOALLOC_MAX_SCENES 64
#define BH_NOALLOC_MAX_RAYS 4000000
typedef struct bh_device_texture {
  const void* texels;  /* width*height BGRA8 texels in device memory */
  int32_t width;
  int32_t height;
} bh_device_texture;
int bh_render_noalloc(int device, const bh_scene* scenes, int32_t n, const bh_device_texture* textures,
                      int32_t n_textures, const bh_frame* frames, const bh_render_options* opts, void* stream,
                      char* error, int32_t error_len);

/* ---- differentiable render and its adjoint -------------------------------------
 * No counterpart in the reference (it has no gradients and no smooth mode).
 * A smooth variant of the RK4 render, so that an image loss has gradients:
 *   - disc: bilinear texture in (radius, azimuth), texel x over [r_in, r_out]
 *     (POLAR mapping about the hole), opacity
 *     alpha = s((R - r_in)/w) s((r_out - R)/w), s the logistic function,
 *     w = softness * M; crossings composite front to back
 *     (C += T alpha C_disc, T *= 1 - alpha); the ray stops once T < 1e-4;
 *   - sky: bilinear equirectangular background at the escape direction;
 *   - horizon and step cap: black.
 * Colours are linear RGB in [0, 1] (texel / 255), float32, H*W*3 row-major.
 * The parameters theta (BH_GRAD_COUNT doubles per scene) are taken about the
 * scene: M; camera position offset (x, y, z); camera yaw, pitch and roll,
 * rotations of the camera axes about the scene camera's own axis_z, axis_y
 * and axis_x, applied as R(z, yaw) R(y, pitch) R(x, roll); disc tilt, a
 * rotation of the disc normal about the disc's in-plane axis edge_s1/|s1|;
 * r_inner; r_outer. theta = NULL means the scene itself (M, zeros, its radii).
 * bh_render_adjoint renders every scene at its theta and, for frames with a
 * target, returns loss = mean over H*W*3 of (C - target)^2 and its gradient
 * with respect to theta. The gradient is reverse mode through the fixed-step
 * RK4 integrator with a checkpoint of the trajectory every
 * checkpoint_every steps (recomputed in 8-step pieces on the way back).
 * Buffers in `frames` are device memory; results are written to the host
 * array `results` (may be NULL) when the call returns. Enqueued on the
 * context's stream; the call waits for it. */
enum {
  BH_GRAD_MASS = 0,
  BH_GRAD_CAM_X = 1,
  BH_GRAD_CAM_Y = 2,
  BH_GRAD_CAM_Z = 3,
  BH_GRAD_YAW = 4,
  BH_GRAD_PITCH = 5,
  BH_GRAD_ROLL = 6,
  BH_GRAD_TILT = 7,
  BH_GRAD_R_INNER = 8,
  BH_GRAD_R_OUTER = 9,
  BH_GRAD_COUNT = 10
};

typedef struct bh_adjoint_options {
  int32_t precision;         /* FP64; FP32 (plain FP32 throughout); MIXED (default):
                                FP64 ray setup and crossing phases, FP32 integration
                                with compensated state updates, and rays with
                                |b/M - 3 sqrt 3| < band entirely in FP64 */
  int32_t max_steps;         /* default 4000 */
  double step;               /* RK4 step in phi, default 0.01 (at most 0.3) */
  double r_escape;           /* escape radius in units of M, default 100 */
  double softness;           /* disc-edge width in units of M, default 0.1 */
  double band;               /* MIXED FP64 band in units of M, default 0.3 */
  int32_t checkpoint_every;  /* steps between trajectory checkpoints: 64 */
  int32_t threads_per_block; /* 0 = default (128, a multiple of 32 up to 256) */
  int32_t reserved[8];
} bh_adjoint_options;

typedef struct bh_adjoint_frame {
  const float* target;  /* device, H*W*3 RGB; NULL renders without gradient */
  float* image;         /* device, H*W*3 RGB, or NULL */
  float* pixel_grad;    /* device, H*W*BH_GRAD_COUNT, or NULL: per pixel the
                           gradient of sum_c (C_c - target_c)^2 (not divided
                           by H*W*3) */
} bh_adjoint_frame;

typedef struct bh_adjoint_result {
  double loss;                 /* mean over H*W*3 of (C - target)^2 */
  double grad[BH_GRAD_COUNT];  /* d loss / d theta */
  uint64_t steps;              /* RK4 steps of the forward pass */
  uint64_t band_rays;          /* MIXED: rays traced in FP64 */
  double kernel_ms;            /* device time of the call's kernels (all scenes) */
} bh_adjoint_result;

void bh_adjoint_default_options(bh_adjoint_options* opts);
int bh_render_adjoint(bh_ctx* ctx, const bh_scene* scenes, int32_t n, const double* theta,
                      const bh_adjoint_frame* frames, const bh_adjoint_options* opts, bh_adjoint_result* results);
/* The scene moved to theta (pose, disc normal, M and radii replaced): what
 * bh_render_adjoint renders for theta, as a scene for the other renders. */
int bh_scene_at_theta(const bh_scene* scene, const double* theta, bh_scene* out);

/* ---- device probes ------------------------------------------------------------
 * Measured FP32 FMA throughput of the device (TFLOP/s, FMA = 2 flops) and its
 * multiprocessor count; used as the roofline denominator. */
int bh_probe_fp32_peak(bh_ctx* ctx, double* tflops, int32_t* sm_count);
int bh_probe_fp64_peak(bh_ctx* ctx, double* tflops);

/* Algorithmic FP32 flops of one RK4-in-phi step of the orbit u'' = -u + 3Mu^2
 * (FMA = 2): four evaluations of f = (w, 3Mu^2 - u) at 3 flops, three stage
 * states at 2 FMA, the final combination (4 FMA for each of u and w), and
 * about 10 for the phi advance, the node / horizon / escape compares and the
 * (cos, sin) rotation recurrence of the 3-D position. The roofline unit. */
#define BH_RK4_ALGO_FLOPS_PER_STEP 50
/* What the FP32 tracers issue per step: Nystrom's three-stage fourth-order
 * method for x'' = x + 3x^2 (x = u - 1/3, no x' term), with events tested by
 * step index, 15 FP32 instructions = 26 flops. (The FP64 tracer takes
 * classical RK4 in Runge-Kutta-Nystrom form, 18 instructions, as the oracle
 * does; both are fourth order in the step.) */
#define BH_RK4_FLOPS_PER_STEP 26
#define BH_RK4_INSTRUCTIONS_PER_STEP 15

#ifdef __cplusplus
}
#endif

#endif /* BH_GB300_H_ */
