/*
 * Test infrastructure: FP64 CPU oracle of the geodesic render. Used only by
 * the tests, by the smoke check and by the CPU-baseline leg of the bench;
 * nothing in the product links it.
 *
 * Two restatements of the reference's per-pixel render, written in plain C
 * from the reference's formulas (all FP64, as the reference's value_type):
 *
 *   orc_render_ref  -- the reference's own scheme, following
 *     include/blackhole/blackhole_solution_test.cc:161-298 literally:
 *       pv, F           :167-168 (Camera::PixelVector, camera.h:55-59)
 *       basis yv zv xv  :170-174 (cv::normalize; zero vector -> zero)
 *       Mre, Mconv      :176-183 (3x3 inverse by adjugate / determinant)
 *       b, SolveG       :185-190 (blackhole_solution.h:35-53)
 *       phi, u, du      :191-206
 *       19 inward steps :217-239, the 0.9 step :240-262, capture :264-272,
 *       19 outward steps:274-296
 *     with FindCollision (object_manager.h:69-85: nearest hit to p1, the hole
 *     first), StaticBlackhole::Collide (blackhole_solution.h:65-88),
 *     Annulus::Collide (vector_object.h:328-347) and Rectangle::color
 *     (vector_object.h:159-179, index clamped where the reference would read
 *     outside the texture).
 *
 *   orc_render_rk4  -- the same ray generation and plane reduction, then RK4
 *     in phi on u'' = -u + 3 u^2 (u = M/r; the first integral is G of
 *     blackhole_solution.h:27-29) with a fixed step, the horizon at u = 1/2,
 *     escape at u = M / r_escape (Hermite-refined), disc-plane crossings at
 *     phi = phi_node + j*pi (partial RK4 step) and the step cap.
 *
 *   orc_render_flat -- the reference's flat-space RayTracer (ray_tracer.h:
 *     52-96, BasicLinearRayRecurrence :17-33) as ray_tracer_test.cc:140-155
 *     drives it: ten chords from the focus through the PixelVector point,
 *     the step scaled by 100 / |step|^2 when |step|^2 < 100.
 *
 *   orc_render_multi -- the MULTI integrator (several holes; see
 *     multi_pixel below): no counterpart in the reference to restate, its
 *     multi-hole experiment being disabled and unfinished.
 *
 *   Ordinary objects (bh_object) take part in every chord test of modes A
 *   and flat, and of each RK4 step of mode B: Rectangle::Collide / color
 *   (vector_object.h:107-180), Triangle::Collide (:39-71, black),
 *   InfinitePlane::Collide / color (:210-232) with ChessPattern2D
 *   (pattern.h:23-46). FindCollision keeps the first object visited on exact
 *   ties, visiting the objects from last to first, then the hole, then the
 *   disc (the reference's map order with the disc and the hole inserted
 *   first).
 *
 * Outputs per pixel: BGRA bytes, hit class, an aux value (deflection angle of
 * escaped rays, hit radius / M of disc hits), margins to the nearest texel
 * edge and disc edge (used by the tests to separate boundary pixels), b / M
 * and the number of RK4 steps.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "bh_gb300.h"

#define ORC_PI 3.14159265358979323846

typedef struct { double x, y, z; } vec3;

static vec3 v3(double x, double y, double z) { vec3 r = {x, y, z}; return r; }
static vec3 v3a(const double* a) { return v3(a[0], a[1], a[2]); }
static vec3 add(vec3 a, vec3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static vec3 sub(vec3 a, vec3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static vec3 scale(vec3 a, double s) { return v3(a.x * s, a.y * s, a.z * s); }
static double dot(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static vec3 cross(vec3 a, vec3 b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static vec3 normalize(vec3 a) {
  double l = sqrt(dot(a, a));
  return scale(a, l != 0.0 ? 1.0 / l : 0.0);
}

typedef struct { double m[3][3]; } mat3;

static vec3 mat_vec(const mat3* a, vec3 v) {
  return v3(a->m[0][0] * v.x + a->m[0][1] * v.y + a->m[0][2] * v.z,
            a->m[1][0] * v.x + a->m[1][1] * v.y + a->m[1][2] * v.z,
            a->m[2][0] * v.x + a->m[2][1] * v.y + a->m[2][2] * v.z);
}

static mat3 mat_inv(const mat3* a) {
  mat3 r;
  const double (*m)[3] = a->m;
  double c00 = m[1][1] * m[2][2] - m[1][2] * m[2][1];
  double c01 = m[1][2] * m[2][0] - m[1][0] * m[2][2];
  double c02 = m[1][0] * m[2][1] - m[1][1] * m[2][0];
  double det = m[0][0] * c00 + m[0][1] * c01 + m[0][2] * c02;
  memset(&r, 0, sizeof(r));
  if (det == 0.0) return r;
  double k = 1.0 / det;
  r.m[0][0] = c00 * k;
  r.m[1][0] = c01 * k;
  r.m[2][0] = c02 * k;
  r.m[0][1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) * k;
  r.m[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) * k;
  r.m[2][1] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]) * k;
  r.m[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) * k;
  r.m[1][2] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]) * k;
  r.m[2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) * k;
  return r;
}

typedef struct {
  const uint8_t* bgra; /* width*height*4 */
  int32_t width, height;
} orc_texture;

typedef struct {
  double step;
  int32_t max_steps;
  double r_escape; /* units of M */
} orc_rk4_opts;

/* Per-pixel outputs; every pointer except bgra may be NULL. */
typedef struct {
  uint8_t* bgra;
  uint8_t* cls;
  double* aux;
  double* margin_tex; /* distance of the sampling coordinate to a texel edge, texels */
  double* margin_r;   /* disc hits: min(r - r_in, r_out - r) / M */
  double* b_over_m;
  int32_t* steps;
} orc_outputs;

/* ------------------------------------------------------------------------- */
/* scene view: the reference's objects, in world coordinates */
typedef struct {
  vec3 focus, vx, vy, vz;
  double focus_len;
  int W, H;
  vec3 hole;
  double M, b_c, radius;
  int disc_on, disc_map;
  vec3 dcen, dnorm, v1, s1, s2;
  double r_in, r_out;
  orc_texture disc_tex, bg_tex;
  int has_bg;
  int n_obj;
  const bh_object* obj;
  const orc_texture* obj_tex; /* one per object (NULL bgra: none), or NULL */
  int n_holes;                /* MULTI: the scene's hole, then its extra holes */
  vec3 hp[BH_MAX_HOLES];
  double hm[BH_MAX_HOLES];    /* half of each mass */
  vec3 mcen;                  /* centre of mass */
  double mtot;
} view;

static void make_view(const bh_scene* s, const orc_texture* disc_tex, const orc_texture* bg_tex, view* v) {
  memset(v, 0, sizeof(*v));
  v->focus = v3a(s->camera.position);
  v->vx = v3a(s->camera.axis_x);
  v->vy = v3a(s->camera.axis_y);
  v->vz = v3a(s->camera.axis_z);
  v->focus_len = s->camera.focus_len;
  v->W = s->camera.width;
  v->H = s->camera.height;
  v->hole = v3a(s->hole.position);
  v->M = s->hole.mass;
  v->b_c = 3.0 * sqrt(3.0) * v->M;  /* blackhole_solution.h:25 */
  v->radius = 2 * v->M;             /* blackhole_solution.h:57 */
  v->disc_on = s->disc.enabled && disc_tex && disc_tex->bgra;
  if (v->disc_on) {
    v->disc_map = s->disc.mapping;
    v->dcen = v3a(s->disc.center);
    v->dnorm = v3a(s->disc.normal);
    v->v1 = v3a(s->disc.corner);
    v->s1 = v3a(s->disc.edge_s1);
    v->s2 = v3a(s->disc.edge_s2);
    v->r_in = s->disc.r_inner;
    v->r_out = s->disc.r_outer;
    v->disc_tex = *disc_tex;
  }
  v->has_bg = s->background >= 0 && bg_tex && bg_tex->bgra;
  if (v->has_bg) v->bg_tex = *bg_tex;
  v->n_obj = s->n_objects;
  v->obj = s->objects;
  v->n_holes = 1 + (s->n_extra_holes > 0 ? s->n_extra_holes : 0);
  v->mcen = v3(0, 0, 0);
  v->mtot = 0;
  for (int i = 0; i < v->n_holes; ++i) {
    const bh_hole* h = i == 0 ? &s->hole : &s->extra_holes[i - 1];
    v->hp[i] = v3a(h->position);
    v->hm[i] = 0.5 * h->mass;
    v->mtot += h->mass;
    v->mcen = add(v->mcen, scale(v->hp[i], h->mass));
  }
  v->mcen = scale(v->mcen, 1.0 / v->mtot);
}

/* Camera::focus_vector / PixelVector(x, y, fv), camera.h:55-63 */
static vec3 pixel_vector(const view* v, int x, int y, vec3 fv) {
  vec3 r = sub(fv, scale(v->vy, (double)(v->W / 2.0 - x)));
  return sub(r, scale(v->vz, (double)(v->H / 2.0 - y)));
}

static double frac_margin(double f) {
  double d = f - floor(f);
  if (d != d) return 0.0; /* NaN coordinates: no margin */
  return d < 0.5 ? d : 1.0 - d;
}

static void read_texel(const orc_texture* t, long long idx, uint8_t out[4]) {
  long long last = (long long)t->width * t->height - 1;
  if (idx < 0) idx = 0;
  if (idx > last) idx = last;
  memcpy(out, t->bgra + idx * 4, 4);
}

static int trunc_int(double v) {
  if (v != v) return 0;
  if (v > 1073741824.0) v = 1073741824.0;
  if (v < -1073741824.0) v = -1073741824.0;
  return (int)v;
}

/* Rectangle::color, vector_object.h:163-179 */
static void color_planar(const view* v, vec3 p, uint8_t out[4], double* margin) {
  vec3 s1 = v->s1, s2 = v->s2;
  vec3 q = sub(p, v->v1);
  double r = sqrt(dot(q, q));
  double theta = acos(dot(s1, q) / (sqrt(dot(s1, s1)) * r));
  theta = isnan(theta) ? 0 : theta;
  double fw = (r * cos(theta) / sqrt(dot(s1, s1))) * v->disc_tex.width;
  double fh = (r * sin(theta) / sqrt(dot(s2, s2))) * v->disc_tex.height;
  int px_w = trunc_int(fw), px_h = trunc_int(fh);
  read_texel(&v->disc_tex, (long long)px_h * v->disc_tex.width + px_w, out);
  if (margin) {
    double a = frac_margin(fw), b = frac_margin(fh);
    *margin = a < b ? a : b;
  }
}

static void color_polar(const view* v, vec3 p, uint8_t out[4], double* margin) {
  vec3 q = sub(p, v->dcen);
  double r = sqrt(dot(q, q));
  vec3 e1 = normalize(v->s1);
  vec3 e2 = normalize(cross(v->dnorm, e1));
  double fx = (r - v->r_in) / (v->r_out - v->r_in) * v->disc_tex.width;
  double a = atan2(dot(e2, q), dot(e1, q)) / (2.0 * ORC_PI);
  a -= floor(a);
  double fy = a * v->disc_tex.height;
  int tx = (int)floor(fx), ty = (int)floor(fy);
  if (tx < 0) tx = 0;
  if (tx > v->disc_tex.width - 1) tx = v->disc_tex.width - 1;
  if (ty < 0) ty = 0;
  if (ty > v->disc_tex.height - 1) ty = v->disc_tex.height - 1;
  read_texel(&v->disc_tex, (long long)ty * v->disc_tex.width + tx, out);
  if (margin) {
    double ma = frac_margin(fx), mb = frac_margin(fy);
    *margin = ma < mb ? ma : mb;
  }
}

static void color_disc(const view* v, vec3 p, uint8_t out[4], double* margin) {
  if (v->disc_map == BH_DISC_MAP_POLAR) color_polar(v, p, out, margin);
  else color_planar(v, p, out, margin);
}

static void color_background(const view* v, vec3 d, uint8_t out[4], double* margin) {
  int W = v->bg_tex.width, H = v->bg_tex.height;
  double lon = atan2(d.y, d.x);
  double z = d.z > 1 ? 1 : (d.z < -1 ? -1 : d.z);
  double lat = asin(z);
  double fx = (lon + ORC_PI) * (W / (2.0 * ORC_PI));
  double fy = (ORC_PI / 2 - lat) * (H / ORC_PI);
  int tx = (int)floor(fx), ty = (int)floor(fy);
  if (tx >= W) tx -= W;
  if (tx < 0) tx = 0;
  if (ty < 0) ty = 0;
  if (ty > H - 1) ty = H - 1;
  read_texel(&v->bg_tex, (long long)ty * W + tx, out);
  if (margin) {
    double a = frac_margin(fx), b = frac_margin(fy);
    *margin = a < b ? a : b;
  }
}

/* ------------------------------------------------------------------------- */
/* collisions in world coordinates */
static int collide_hole(const view* v, vec3 q1, vec3 q2, vec3* hit) {
  vec3 p1 = sub(q1, v->hole), p2 = sub(q2, v->hole);
  double d1 = sqrt(dot(p1, p1)), d2 = sqrt(dot(p2, p2));
  if (d1 < v->radius && d2 < v->radius) return 0;
  vec3 Q1 = sub(q1, v->hole), Q2 = sub(q2, v->hole);
  vec3 Q = sub(Q2, Q1);
  double qq1 = dot(Q, Q1);
  double c = qq1 * qq1 - dot(Q, Q) * (dot(Q1, Q1) - v->radius * v->radius);
  if (c <= 0) return 0;
  double t = (1.0 / dot(Q, Q)) * (-dot(Q, Q1) - sqrt(c));
  if (t <= 0 || t >= 1) return 0;
  *hit = add(add(Q1, scale(Q, t)), v->hole);
  return 1;
}

static int collide_disc(const view* v, vec3 q1, vec3 q2, vec3* hit) {
  vec3 p1 = sub(q1, v->dcen), p2 = sub(q2, v->dcen);
  if (dot(v->dnorm, p1) * dot(v->dnorm, p2) >= 0) return 0;
  double t1 = dot(v->dnorm, p1), t2 = dot(v->dnorm, p2);
  vec3 c = scale(add(scale(p1, fabs(t2)), scale(p2, fabs(t1))), 1.0 / (fabs(t1) + fabs(t2)));
  if (sqrt(dot(c, c)) > v->r_out) return 0;
  if (sqrt(dot(c, c)) < v->r_in) return 0;
  *hit = add(c, v->dcen);
  return 1;
}

/* Rectangle::Collide, vector_object.h:107-127 */
static int collide_rect(const bh_object* o, vec3 aa, vec3 bb, vec3* hit) {
  vec3 p0 = v3a(o->v[0]);
  vec3 p1 = sub(v3a(o->v[1]), p0);
  vec3 p3 = sub(v3a(o->v[3]), p0);
  vec3 n = normalize(cross(p1, p3));
  vec3 Q1 = sub(aa, p0), Q2 = sub(bb, p0);
  double q1 = dot(n, Q1), q2 = dot(n, Q2);
  if (q1 * q2 >= 0) return 0;
  double a1 = fabs(q1), a2 = fabs(q2), d = a1 + a2;
  vec3 s = add(scale(Q1, a2), scale(Q2, a1));
  vec3 Q = v3(s.x / d, s.y / d, s.z / d);
  if (dot(p1, Q) > 0 && dot(p1, p1) > dot(p1, Q) && dot(p3, Q) > 0 && dot(p3, p3) > dot(p3, Q)) {
    *hit = add(Q, p0);
    return 1;
  }
  return 0;
}

/* Triangle::Collide, vector_object.h:39-71 (Moller-Trumbore; no upper bound
 * on t, as in the reference) */
static int collide_tri(const bh_object* o, vec3 p1, vec3 p2, vec3* hit) {
  const double ep = 2.220446049250313e-16 * 10;
  vec3 rv = sub(p2, p1);
  vec3 v0 = v3a(o->v[0]);
  vec3 e1 = sub(v3a(o->v[1]), v0), e2 = sub(v3a(o->v[2]), v0);
  vec3 h = cross(rv, e2);
  double a = dot(e1, h);
  if (-ep < a && a < ep) return 0;
  double f = 1.0 / a;
  vec3 s = sub(p1, v0);
  double u = f * dot(s, h);
  if (u < 0 || u > 1) return 0;
  vec3 q = cross(s, e1);
  double w = f * dot(rv, q);
  if (w < 0 || u + w > 1) return 0;
  double t = f * dot(e2, q);
  if (t <= ep) return 0;
  *hit = add(p1, scale(rv, t));
  return 1;
}

/* InfinitePlane::Collide, vector_object.h:210-225 */
static int collide_plane(const bh_object* o, vec3 p1, vec3 p2, vec3* hit) {
  const double* z = o->axis_z;
  const double* pos = o->v[0];
  double t1 = z[0] * (p1.x - pos[0]) + z[1] * (p1.y - pos[1]) + z[2] * (p1.z - pos[2]);
  double t2 = z[0] * (p2.x - pos[0]) + z[1] * (p2.y - pos[1]) + z[2] * (p2.z - pos[2]);
  if (t1 * t2 > 0) return 0;
  double d1 = fabs(t1), d2 = fabs(t2), d = d1 + d2;
  vec3 s = add(scale(p1, d2), scale(p2, d1));
  *hit = v3(s.x / d, s.y / d, s.z / d);
  return 1;
}

static int collide_object(const bh_object* o, vec3 p1, vec3 p2, vec3* hit) {
  if (o->type == BH_OBJECT_RECTANGLE) return collide_rect(o, p1, p2, hit);
  if (o->type == BH_OBJECT_TRIANGLE) return collide_tri(o, p1, p2, hit);
  return collide_plane(o, p1, p2, hit);
}

/* ChessPattern2D<T>{size}, pattern.h:23-46 ((int) casts pinned) */
static double chess_axis_margin(double size, int m, double b, double c2) {
  /* the colour changes where c2 crosses 0 or size (c2 in [0, 2 size)), where
   * trunc(|c|) crosses a multiple of m (the cell index) and where c changes
   * sign; the distance to the nearest of these, in units of size */
  double d = fabs(c2);
  if (fabs(c2 - size) < d) d = fabs(c2 - size);
  if (fabs(2 * size - c2) < d) d = fabs(2 * size - c2);
  double k = b / m;
  double dk = fabs(b - floor(k + 0.5) * m);
  if (dk < d) d = dk;
  if (b < d) d = b;
  return d == d ? d / size : 0.0; /* NaN coordinates: no margin */
}

static void chess(double size, double x, double y, uint8_t out[4], double* margin) {
  int m = trunc_int(size * 2);
  int white = 0;
  if (margin) *margin = 1.0;
  if (m != 0) {
    double bx = fabs(x), by = fabs(y);
    double x2 = bx - (double)(trunc_int(bx) / m) * (size * 2);
    double y2 = by - (double)(trunc_int(by) / m) * (size * 2);
    int in = (x2 <= size && y2 <= size) || (size <= x2 && size <= y2);
    white = x * y > 0 ? in : !in;
    if (margin) {
      double a = chess_axis_margin(size, m, bx, x2), b = chess_axis_margin(size, m, by, y2);
      *margin = a < b ? a : b;
    }
  }
  out[0] = out[1] = out[2] = white ? 255 : 0;
}

/* Rectangle::color (vector_object.h:163-180), InfinitePlane::color (:227-232),
 * Material::color for triangles (black) */
static void color_object(const view* v, int i, vec3 p, uint8_t out[4], double* margin) {
  const bh_object* o = &v->obj[i];
  out[0] = out[1] = out[2] = 0;
  if (margin) *margin = 1.0;
  if (o->type == BH_OBJECT_RECTANGLE) {
    const orc_texture* t = v->obj_tex ? &v->obj_tex[i] : NULL;
    if (!t || !t->bgra) return;
    vec3 v1 = v3a(o->v[0]);
    vec3 s1 = sub(v3a(o->v[1]), v1), s2 = sub(v3a(o->v[3]), v1);
    vec3 q = sub(p, v1);
    double r = sqrt(dot(q, q));
    double theta = acos(dot(s1, q) / (sqrt(dot(s1, s1)) * r));
    theta = isnan(theta) ? 0 : theta;
    double fw = (r * cos(theta) / sqrt(dot(s1, s1))) * t->width;
    double fh = (r * sin(theta) / sqrt(dot(s2, s2))) * t->height;
    int px_w = trunc_int(fw), px_h = trunc_int(fh);
    read_texel(t, (long long)px_h * t->width + px_w, out);
    if (margin) {
      double a = frac_margin(fw), b = frac_margin(fh);
      *margin = a < b ? a : b;
    }
  } else if (o->type == BH_OBJECT_PLANE && o->pattern_size > 0) {
    const double* vx = o->axis_x;
    const double* vy = o->axis_y;
    double b = (vx[0] * p.y - vx[1] * p.x) / (vx[0] * vy[1] - vx[1] * vy[0]);
    double a = (p.x - b * vy[0]) / vx[0];
    chess(o->pattern_size, a, b, out, margin);
  }
}

/* Nearest object hit to p1 on the chord (objects visited from last to first,
 * the first keeps ties); -1 when none. */
static int nearest_object(const view* v, vec3 p1, vec3 p2, double* dd_out, vec3* hit) {
  int obj = -1;
  double best = 0;
  for (int i = v->n_obj - 1; i >= 0; --i) {
    vec3 h;
    if (collide_object(&v->obj[i], p1, p2, &h)) {
      vec3 d = sub(p1, h);
      double dd = dot(d, d);
      if (obj < 0 || dd < best) {
        obj = i;
        best = dd;
        *hit = h;
      }
    }
  }
  *dd_out = best;
  return obj;
}

/* ObjectManager::FindCollision: nearest to p1 over the objects, the hole
 * (with_hole) and the disc; returns the class, writes the colour and, for an
 * object, its index. */
/* margin (may be NULL): the colour's distance to a texel or pattern edge. */
static int find_collision_objects(const view* v, vec3 p1, vec3 p2, int with_hole, uint8_t out[4], int* obj_out,
                                  double* margin) {
  int cls = BH_CLASS_MISS, obj = -1;
  double best = 0;
  vec3 hp = v3(0, 0, 0), h;
  obj = nearest_object(v, p1, p2, &best, &hp);
  if (obj >= 0) cls = BH_CLASS_OBJECT;
  if (with_hole && collide_hole(v, p1, p2, &h)) {
    vec3 d = sub(p1, h);
    double dd = dot(d, d);
    if (cls == BH_CLASS_MISS || dd < best) {
      cls = BH_CLASS_HORIZON;
      best = dd;
      hp = h;
    }
  }
  if (v->disc_on && collide_disc(v, p1, p2, &h)) {
    vec3 d = sub(p1, h);
    double dd = dot(d, d);
    if (cls == BH_CLASS_MISS || dd < best) {
      cls = BH_CLASS_DISC;
      best = dd;
      hp = h;
    }
  }
  out[0] = out[1] = out[2] = 0;
  if (cls == BH_CLASS_DISC) color_disc(v, hp, out, margin);
  if (cls == BH_CLASS_OBJECT) color_object(v, obj, hp, out, margin);
  if (obj_out) *obj_out = cls == BH_CLASS_OBJECT ? obj : -1;
  return cls;
}

static int find_collision(const view* v, vec3 p1, vec3 p2, uint8_t out[4], double* margin) {
  return find_collision_objects(v, p1, p2, 1, out, NULL, margin);
}

/* StaticBlackhole::G, InvSqrtG, SolveG (blackhole_solution.h:27-53) */
static double G(double M, double u, double b) { return (u * u * (2.0 * M * u - 1.0)) + (1.0 / (b * b)); }
static double inv_sqrt_G(double M, double u, double b) { return 1.0 / sqrt(G(M, u, b)); }
static double solve_G(double M, double b) {
  double l = 0.0 + cbrt(2.220446049250313e-16); /* epsilon<double>(), utility.h:17-21 */
  double r = 1.0 / (3.0 * M);
  for (int i = 0; i < 20; ++i) {
    double mid = (l + r) / 2.0;
    if (G(M, mid, b) > 0.0) l = mid;
    else r = mid;
  }
  return l;
}

/* Ray generation and plane reduction, blackhole_solution_test.cc:167-193 */
typedef struct {
  vec3 yv, zv, xv;
  mat3 re;
  vec3 Fc;
} plane;

static void reduce(const view* v, int x, int y, plane* p) {
  vec3 fv = scale(v->vx, v->focus_len);
  vec3 pv = sub(pixel_vector(v, x, y, fv), v->hole);
  vec3 F = sub(v->focus, v->hole);
  p->yv = normalize(sub(F, pv));
  p->zv = normalize(cross(pv, p->yv));
  if (isnan(p->zv.x)) p->zv = v3(1, 0, 0);
  p->xv = normalize(cross(p->yv, p->zv));
  mat3 re = {{{p->zv.x, p->yv.x, p->xv.x}, {p->zv.y, p->yv.y, p->xv.y}, {p->zv.z, p->yv.z, p->xv.z}}};
  p->re = re;
  mat3 conv = mat_inv(&re);
  p->Fc = mat_vec(&conv, F);
}

static vec3 back_project(const view* v, const plane* p, double r, double phi) {
  return add(mat_vec(&p->re, v3(0, r * cos(phi), r * sin(phi))), v->hole);
}

/* ------------------------------------------------------------------------- */
static int ref_pixel(const view* v, int x, int y, uint8_t out[4], double* margin) {
  plane p;
  reduce(v, x, y, &p);
  const double b = p.Fc.z;
  double sol = -1;
  if (b >= v->b_c) sol = solve_G(v->M, b);
  const double periapsis = b < v->b_c ? 1.0 / (3 * v->M) : sol;
  double r0 = sqrt(dot(p.Fc, p.Fc));
  double phi = atan(p.Fc.z / p.Fc.y);
  double dphi = 0, dphi_prev = 0;
  double u = 1. / r0;
  const int nstep = 20, nstep_safe = nstep - 1;
  double du = (periapsis - u) * (1.0 / nstep);
  const double du_h = du / 2.;
  vec3 prev = v->focus, cur;
  int cls;
  for (int i = 0; i < nstep_safe; ++i) {
    u += du;
    dphi = inv_sqrt_G(v->M, u, b);
    phi += (dphi_prev + dphi) * du_h;
    cur = back_project(v, &p, 1. / u, phi);
    dphi_prev = dphi;
    if ((cls = find_collision(v, prev, cur, out, margin)) != BH_CLASS_MISS) return cls;
    prev = cur;
  }
  u += du * 0.9;
  dphi = inv_sqrt_G(v->M, u, b);
  phi += (dphi_prev + dphi) * du_h;
  cur = back_project(v, &p, 1. / u, phi);
  dphi_prev = dphi;
  if ((cls = find_collision(v, prev, cur, out, margin)) != BH_CLASS_MISS) return cls;
  prev = cur;
  if (sol < 0) return find_collision(v, prev, v->hole, out, margin);
  for (int i = 0; i < nstep_safe; ++i) {
    u -= du;
    dphi = inv_sqrt_G(v->M, u, b);
    phi += (dphi_prev + dphi) * du_h;
    cur = back_project(v, &p, 1. / u, phi);
    if ((cls = find_collision(v, prev, cur, out, margin)) != BH_CLASS_MISS) return cls;
    dphi_prev = dphi;
    prev = cur;
  }
  return BH_CLASS_MISS;
}

/* ------------------------------------------------------------------------- */
static void rk4(double* u, double* w, double h) {
  double u0 = *u, w0 = *w;
  double k1u = w0, k1w = 3 * u0 * u0 - u0;
  double u2 = u0 + 0.5 * h * k1u, w2 = w0 + 0.5 * h * k1w;
  double k2u = w2, k2w = 3 * u2 * u2 - u2;
  double u3 = u0 + 0.5 * h * k2u, w3 = w0 + 0.5 * h * k2w;
  double k3u = w3, k3w = 3 * u3 * u3 - u3;
  double u4 = u0 + h * k3u, w4 = w0 + h * k3w;
  double k4u = w4, k4w = 3 * u4 * u4 - u4;
  *u = u0 + h / 6 * (k1u + 2 * k2u + 2 * k3u + k4u);
  *w = w0 + h / 6 * (k1w + 2 * k2w + 2 * k3w + k4w);
}

static void hermite(double ua, double ha, double ub, double hb, double t, double* p, double* dp) {
  double t2 = t * t, t3 = t2 * t;
  *p = (2 * t3 - 3 * t2 + 1) * ua + (t3 - 2 * t2 + t) * ha + (-2 * t3 + 3 * t2) * ub + (t3 - t2) * hb;
  *dp = (6 * t2 - 6 * t) * ua + (3 * t2 - 4 * t + 1) * ha + (-6 * t2 + 6 * t) * ub + (3 * t2 - 2 * t) * hb;
}

typedef struct {
  int cls;
  uint8_t bgra[4];
  double aux, margin_tex, margin_r, b_over_m;
  int steps;
} rk4_result;

static void rk4_pixel(const view* v, const orc_rk4_opts* o, int x, int y, rk4_result* res) {
  plane p;
  reduce(v, x, y, &p);
  memset(res, 0, sizeof(*res));
  res->bgra[3] = 255;
  res->margin_tex = 1.0;
  res->margin_r = 1e30;
  const double M = v->M, h = o->step;
  const double b = p.Fc.z, bm = b / M;
  res->b_over_m = bm;
  const double r0 = sqrt(dot(p.Fc, p.Fc));
  double u = M / r0;
  const double phi0 = atan2(p.Fc.z, p.Fc.y);
  if (!(bm > 1e-6)) {
    res->cls = BH_CLASS_HORIZON;
    return;
  }
  double w = copysign(sqrt(fmax(1.0 / (bm * bm) - u * u * (1.0 - 2.0 * u), 0.0)), p.Fc.y);
  const double u_esc = 1.0 / o->r_escape;
  /* disc plane crossings: n.(r cos phi yv + r sin phi xv) = 0 */
  long long kc = -1;
  double dcr = 0;
  if (v->disc_on) {
    double A = dot(v->dnorm, p.yv), B = dot(v->dnorm, p.xv);
    if (A * A + B * B > 1e-24) {
      dcr = fmod(atan2(B, A) + ORC_PI / 2 - phi0, ORC_PI);
      if (dcr <= 0) dcr += ORC_PI;
      kc = (long long)floor(dcr / h);
    }
  }
  for (int k = 0; k < o->max_steps; ++k) {
    if (k == kc) {
      double uc = u, wc = w;
      rk4(&uc, &wc, dcr - kc * h);
      double rc = 1.0 / uc;
      if (uc < 0.5 && rc * M >= v->r_in && rc * M <= v->r_out) {
        double phic = phi0 + dcr;
        vec3 hit = back_project(v, &p, rc * M, phic);
        res->cls = BH_CLASS_DISC;
        res->aux = rc;
        double dr1 = rc - v->r_in / M, dr2 = v->r_out / M - rc;
        res->margin_r = dr1 < dr2 ? dr1 : dr2;
        color_disc(v, hit, res->bgra, &res->margin_tex);
        res->steps = k;
        return;
      }
      dcr += ORC_PI;
      kc = (long long)floor(dcr / h);
    }
    double ua = u, wa = w;
    rk4(&u, &w, h);
    if (!(u < 0.5)) {
      res->cls = BH_CLASS_HORIZON;
      res->steps = k + 1;
      return;
    }
    if (u <= u_esc) {
      double t = (ua - u_esc) / (ua - u), pp, dp;
      for (int i = 0; i < 8; ++i) {
        hermite(ua, h * wa, u, h * w, t, &pp, &dp);
        t -= (pp - u_esc) / dp;
        if (t < 0) t = 0;
        if (t > 1) t = 1;
      }
      hermite(ua, h * wa, u, h * w, t, &pp, &dp);
      double we = dp / h;
      double phie = phi0 + (k + t) * h;
      double psi = phie + atan2(u_esc, -we);
      res->cls = BH_CLASS_MISS;
      res->aux = psi - ORC_PI;
      res->steps = k + 1;
      if (v->has_bg) {
        vec3 d = add(scale(p.yv, cos(psi)), scale(p.xv, sin(psi)));
        color_background(v, d, res->bgra, &res->margin_tex);
      }
      return;
    }
  }
  res->cls = BH_CLASS_MAXSTEPS;
  res->steps = o->max_steps;
}

/* Mode B with objects: each RK4 step's chord between the positions at its
 * ends is tested against the objects; within a step the earlier event wins,
 * a disc crossing at its fraction of the step's angle, an object hit at its
 * fraction of the chord. */
static void rk4_pixel_obj(const view* v, const orc_rk4_opts* o, int x, int y, rk4_result* res) {
  plane p;
  reduce(v, x, y, &p);
  memset(res, 0, sizeof(*res));
  res->bgra[3] = 255;
  res->margin_tex = 1.0;
  res->margin_r = 1e30;
  const double M = v->M, h = o->step;
  const double b = p.Fc.z, bm = b / M;
  res->b_over_m = bm;
  const double r0 = sqrt(dot(p.Fc, p.Fc));
  double u = M / r0;
  const double phi0 = atan2(p.Fc.z, p.Fc.y);
  if (!(bm > 1e-6)) {
    res->cls = BH_CLASS_HORIZON;
    return;
  }
  double w = copysign(sqrt(fmax(1.0 / (bm * bm) - u * u * (1.0 - 2.0 * u), 0.0)), p.Fc.y);
  const double u_esc = 1.0 / o->r_escape;
  long long kc = -1;
  double dcr = 0;
  if (v->disc_on) {
    double A = dot(v->dnorm, p.yv), B = dot(v->dnorm, p.xv);
    if (A * A + B * B > 1e-24) {
      dcr = fmod(atan2(B, A) + ORC_PI / 2 - phi0, ORC_PI);
      if (dcr <= 0) dcr += ORC_PI;
      kc = (long long)floor(dcr / h);
    }
  }
  vec3 prev = v->focus;
  for (int k = 0; k < o->max_steps; ++k) {
    double f_disc = 2, rc_hit = 0;
    if (k == kc) {
      double uc = u, wc = w;
      rk4(&uc, &wc, dcr - kc * h);
      double rc = 1.0 / uc;
      if (uc < 0.5 && rc * M >= v->r_in && rc * M <= v->r_out) {
        double fr = (dcr - kc * h) / h;
        f_disc = fr < 0 ? 0 : fr;
        rc_hit = rc;
      } else {
        dcr += ORC_PI;
        kc = (long long)floor(dcr / h);
      }
    }
    double ua = u, wa = w, un = u, wn = w;
    rk4(&un, &wn, h);
    double f_obj = 2;
    int obj = -1;
    vec3 ohit = v3(0, 0, 0);
    if (un > 0) {
      vec3 next = back_project(v, &p, M / un, phi0 + (k + 1) * h);
      double dd = 0;
      obj = nearest_object(v, prev, next, &dd, &ohit);
      if (obj >= 0) {
        vec3 ch = sub(next, prev);
        f_obj = sqrt(dd / dot(ch, ch));
      }
      prev = next;
    }
    if (f_disc <= 1 && f_disc <= f_obj) {
      vec3 hit = back_project(v, &p, rc_hit * M, phi0 + dcr);
      res->cls = BH_CLASS_DISC;
      res->aux = rc_hit;
      double dr1 = rc_hit - v->r_in / M, dr2 = v->r_out / M - rc_hit;
      res->margin_r = dr1 < dr2 ? dr1 : dr2;
      color_disc(v, hit, res->bgra, &res->margin_tex);
      res->steps = k;
      return;
    }
    if (f_obj <= 1) {
      res->cls = BH_CLASS_OBJECT;
      res->aux = obj;
      color_object(v, obj, ohit, res->bgra, &res->margin_tex);
      res->steps = k + 1;
      return;
    }
    u = un;
    w = wn;
    if (!(u < 0.5)) {
      res->cls = BH_CLASS_HORIZON;
      res->steps = k + 1;
      return;
    }
    if (u <= u_esc) {
      double t = (ua - u_esc) / (ua - u), pp, dp;
      for (int i = 0; i < 8; ++i) {
        hermite(ua, h * wa, u, h * w, t, &pp, &dp);
        t -= (pp - u_esc) / dp;
        if (t < 0) t = 0;
        if (t > 1) t = 1;
      }
      hermite(ua, h * wa, u, h * w, t, &pp, &dp);
      double we = dp / h;
      double psi = phi0 + (k + t) * h + atan2(u_esc, -we);
      res->cls = BH_CLASS_MISS;
      res->aux = psi - ORC_PI;
      res->steps = k + 1;
      if (v->has_bg) {
        vec3 d = add(scale(p.yv, cos(psi)), scale(p.xv, sin(psi)));
        color_background(v, d, res->bgra, &res->margin_tex);
      }
      return;
    }
  }
  res->cls = BH_CLASS_MAXSTEPS;
  res->steps = o->max_steps;
}

/* The flat RayTracer (REF ray generation): ten chords, then a miss. */
static int flat_pixel(const view* v, int x, int y, uint8_t out[4], int* obj, double* margin) {
  vec3 fv = scale(v->vx, v->focus_len);
  vec3 old = v->focus;
  vec3 pres = pixel_vector(v, x, y, fv);
  vec3 vec = sub(pres, old);
  double d2 = dot(vec, vec);
  if (d2 < 100) vec = scale(vec, 100.0 / d2);
  for (int i = 0; i < 10; ++i) {
    int cls = find_collision_objects(v, old, pres, 0, out, obj, margin);
    if (cls != BH_CLASS_MISS) return cls;
    vec3 next = add(pres, vec);
    old = pres;
    pres = next;
  }
  return BH_CLASS_MISS;
}

/* MULTI: null rays of ds^2 = -a^2 dt^2 + p^4 |dx|^2 with p = 1 + S,
 * a = (1 - S) / (1 + S), S = sum m_i / (2 |x - x_i|) (isotropic coordinates;
 * one hole: Schwarzschild). Their spatial paths are the rays of the index
 * n = (1 + S)^3 / (1 - S): dx/ds = T, dT/ds = g - T (T . g), g = grad ln n.
 * RK4 in the Euclidean arc length s with h = step * (distance to the nearest
 * hole); capture at S >= 0.9; escape through the sphere of radius
 * r_escape * (total mass) about the centre of mass, moving outward; per step
 * the disc on the Hermite curve of the step (three Newton steps from the
 * chord's estimate) and the objects on its chord, the earlier winning (the
 * disc on ties). aux: the angle between the first and the last direction of
 * an escaped ray, the distance of a disc hit from the disc centre / m_0, the
 * index of an object hit. No counterpart in the reference, whose
 * multiple_blackhole_solution_test.cc:149-262 averages per-hole plane
 * solutions. */
typedef struct {
  vec3 a;
  double S, d2;
} meval;

static meval multi_eval(const view* v, vec3 x, vec3 T) {
  double S = 0, d2 = 1e300;
  vec3 gS = v3(0, 0, 0);
  for (int i = 0; i < v->n_holes; ++i) {
    vec3 d = sub(x, v->hp[i]);
    double r2 = dot(d, d);
    double ir = 1.0 / sqrt(r2);
    double k = v->hm[i] * ir;
    S += k;
    gS = sub(gS, scale(d, k * ir * ir));
    if (r2 < d2) d2 = r2;
  }
  double f = 3.0 / (1.0 + S) + 1.0 / (1.0 - S);
  vec3 g = scale(gS, f);
  meval e;
  e.a = sub(g, scale(T, dot(T, g)));
  e.S = S;
  e.d2 = d2;
  return e;
}

static void hermite3(vec3 x0, vec3 m0, vec3 x1, vec3 m1, double t, vec3* p, vec3* dp) {
  double t2 = t * t, t3 = t2 * t;
  *p = add(add(scale(x0, 2 * t3 - 3 * t2 + 1), scale(m0, t3 - 2 * t2 + t)),
           add(scale(x1, 3 * t2 - 2 * t3), scale(m1, t3 - t2)));
  *dp = add(add(scale(x0, 6 * t2 - 6 * t), scale(m0, 3 * t2 - 4 * t + 1)),
            add(scale(x1, 6 * t - 6 * t2), scale(m1, 3 * t2 - 2 * t)));
}

static double clamp01(double t) { return t < 0 ? 0 : (t > 1 ? 1 : t); }

static void multi_pixel(const view* v, const orc_rk4_opts* o, int x, int y, rk4_result* res) {
  memset(res, 0, sizeof(*res));
  res->bgra[3] = 255;
  res->margin_tex = 1.0;
  res->margin_r = 1e30;
  vec3 fv = scale(v->vx, v->focus_len);
  vec3 pv = pixel_vector(v, x, y, fv); /* a point, as the reference uses it */
  const vec3 T0 = normalize(sub(pv, v->focus));
  const double resc = o->r_escape * v->mtot;
  vec3 X = v->focus, T = T0;
  meval e = multi_eval(v, X, T);
  {
    vec3 F = sub(v->focus, v->hp[0]);
    double n = pow(1 + e.S, 3) / (1 - e.S);
    res->b_over_m = n * sqrt(dot(cross(F, T0), cross(F, T0))) / (2 * v->hm[0]);
  }
  res->cls = BH_CLASS_MAXSTEPS;
  int k = 0;
  for (;; ++k) {
    if (e.S >= 0.9) {
      res->cls = BH_CLASS_HORIZON;
      break;
    }
    if (k >= o->max_steps) break;
    double h = o->step * sqrt(e.d2), hh = 0.5 * h;
    vec3 t2 = add(T, scale(e.a, hh));
    meval e2 = multi_eval(v, add(X, scale(T, hh)), t2);
    vec3 t3 = add(T, scale(e2.a, hh));
    meval e3 = multi_eval(v, add(X, scale(t2, hh)), t3);
    vec3 t4 = add(T, scale(e3.a, h));
    meval e4 = multi_eval(v, add(X, scale(t3, h)), t4);
    double h6 = h / 6.0;
    vec3 Xn = add(X, scale(add(add(T, scale(add(t2, t3), 2.0)), t4), h6));
    vec3 Tn = normalize(add(T, scale(add(add(e.a, scale(add(e2.a, e3.a), 2.0)), e4.a), h6)));
    double f_disc = 2;
    vec3 dhit = v3(0, 0, 0);
    if (v->disc_on) {
      double g0 = dot(v->dnorm, sub(X, v->dcen)), g1 = dot(v->dnorm, sub(Xn, v->dcen));
      if ((g0 > 0) != (g1 > 0)) {
        double t = g0 != g1 ? g0 / (g0 - g1) : 0.5;
        vec3 p, dp;
        for (int i = 0; i < 3; ++i) {
          hermite3(X, scale(T, h), Xn, scale(Tn, h), t, &p, &dp);
          double dd = dot(v->dnorm, dp);
          if (dd != 0) t = clamp01(t - dot(v->dnorm, sub(p, v->dcen)) / dd);
        }
        hermite3(X, scale(T, h), Xn, scale(Tn, h), t, &p, &dp);
        vec3 q = sub(p, v->dcen);
        double rr = sqrt(dot(q, q));
        if (rr >= v->r_in && rr <= v->r_out) {
          f_disc = t;
          dhit = p;
        }
      }
    }
    double f_obj = 2;
    int obj = -1;
    vec3 ohit = v3(0, 0, 0);
    if (v->n_obj > 0) {
      double dd = 0;
      obj = nearest_object(v, X, Xn, &dd, &ohit);
      if (obj >= 0) {
        vec3 ch = sub(Xn, X);
        f_obj = sqrt(dd / dot(ch, ch));
      }
    }
    if (f_disc <= 1 && f_disc <= f_obj) {
      vec3 q = sub(dhit, v->dcen);
      double rr = sqrt(dot(q, q));
      res->cls = BH_CLASS_DISC;
      res->aux = rr / (2 * v->hm[0]);
      double dr1 = rr - v->r_in, dr2 = v->r_out - rr;
      res->margin_r = (dr1 < dr2 ? dr1 : dr2) / (2 * v->hm[0]);
      color_disc(v, dhit, res->bgra, &res->margin_tex);
      ++k;
      break;
    }
    if (f_obj <= 1) {
      res->cls = BH_CLASS_OBJECT;
      res->aux = obj;
      color_object(v, obj, ohit, res->bgra, &res->margin_tex);
      ++k;
      break;
    }
    vec3 q = sub(Xn, v->mcen);
    if (dot(q, q) >= resc * resc && dot(Tn, q) > 0) {
      vec3 q0 = sub(X, v->mcen);
      double r0 = sqrt(dot(q0, q0)), r1 = sqrt(dot(q, q));
      double t = r1 != r0 ? clamp01((resc - r0) / (r1 - r0)) : 1.0;
      vec3 p, dp;
      for (int i = 0; i < 3; ++i) {
        hermite3(X, scale(T, h), Xn, scale(Tn, h), t, &p, &dp);
        vec3 w = sub(p, v->mcen);
        double dd = 2 * dot(w, dp);
        if (dd != 0) t = clamp01(t - (dot(w, w) - resc * resc) / dd);
      }
      hermite3(X, scale(T, h), Xn, scale(Tn, h), t, &p, &dp);
      vec3 Te = normalize(dp);
      vec3 cr = cross(T0, Te);
      res->cls = BH_CLASS_MISS;
      res->aux = atan2(sqrt(dot(cr, cr)), dot(T0, Te));
      if (v->has_bg) color_background(v, Te, res->bgra, &res->margin_tex);
      ++k;
      break;
    }
    X = Xn;
    T = Tn;
    e = multi_eval(v, X, T);
  }
  res->steps = k;
}

/* ------------------------------------------------------------------------- */
static void set_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
}

/* Mode A over the whole image (pixels == NULL) or a list of npix pixels
 * given as (x, y) pairs. Outputs are indexed like the pixels. */
int orc_render_ref(const bh_scene* s, const orc_texture* disc_tex, const orc_texture* obj_tex,
                   const int32_t* pixels, int64_t npix, const orc_outputs* out, int nthreads) {
  view v;
  make_view(s, disc_tex, NULL, &v);
  v.obj_tex = obj_tex;
  const int64_t n = pixels ? npix : (int64_t)v.W * v.H;
  set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t i = 0; i < n; ++i) {
    int x = pixels ? pixels[2 * i] : (int)(i % v.W);
    int y = pixels ? pixels[2 * i + 1] : (int)(i / v.W);
    uint8_t c[4] = {0, 0, 0, 255};
    double mt = 1.0;
    int cls = ref_pixel(&v, x, y, c, &mt);
    c[3] = 255;
    if (out->bgra) memcpy(out->bgra + 4 * i, c, 4);
    if (out->cls) out->cls[i] = (uint8_t)cls;
    if (out->margin_tex) out->margin_tex[i] = cls == BH_CLASS_DISC || cls == BH_CLASS_OBJECT ? mt : 1.0;
  }
  return 0;
}

int orc_render_rk4(const bh_scene* s, const orc_texture* disc_tex, const orc_texture* bg_tex,
                   const orc_texture* obj_tex, const orc_rk4_opts* o, const int32_t* pixels, int64_t npix,
                   const orc_outputs* out, int nthreads) {
  view v;
  make_view(s, disc_tex, bg_tex, &v);
  v.obj_tex = obj_tex;
  const int64_t n = pixels ? npix : (int64_t)v.W * v.H;
  set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t i = 0; i < n; ++i) {
    int x = pixels ? pixels[2 * i] : (int)(i % v.W);
    int y = pixels ? pixels[2 * i + 1] : (int)(i / v.W);
    rk4_result r;
    if (v.n_obj > 0) rk4_pixel_obj(&v, o, x, y, &r);
    else rk4_pixel(&v, o, x, y, &r);
    if (out->bgra) memcpy(out->bgra + 4 * i, r.bgra, 4);
    if (out->cls) out->cls[i] = (uint8_t)r.cls;
    if (out->aux) out->aux[i] = r.aux;
    if (out->margin_tex) out->margin_tex[i] = r.margin_tex;
    if (out->margin_r) out->margin_r[i] = r.margin_r;
    if (out->b_over_m) out->b_over_m[i] = r.b_over_m;
    if (out->steps) out->steps[i] = r.steps;
  }
  return 0;
}

/* Flat mode over the whole image or a pixel list; aux receives the object
 * index of object hits. */
int orc_render_flat(const bh_scene* s, const orc_texture* disc_tex, const orc_texture* obj_tex,
                    const int32_t* pixels, int64_t npix, const orc_outputs* out, int nthreads) {
  view v;
  make_view(s, disc_tex, NULL, &v);
  v.obj_tex = obj_tex;
  const int64_t n = pixels ? npix : (int64_t)v.W * v.H;
  set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t i = 0; i < n; ++i) {
    int x = pixels ? pixels[2 * i] : (int)(i % v.W);
    int y = pixels ? pixels[2 * i + 1] : (int)(i / v.W);
    uint8_t c[4] = {0, 0, 0, 255};
    int obj = -1;
    double mt = 1.0;
    int cls = flat_pixel(&v, x, y, c, &obj, &mt);
    c[3] = 255;
    if (out->bgra) memcpy(out->bgra + 4 * i, c, 4);
    if (out->cls) out->cls[i] = (uint8_t)cls;
    if (out->aux) out->aux[i] = obj;
    if (out->margin_tex) out->margin_tex[i] = cls == BH_CLASS_DISC || cls == BH_CLASS_OBJECT ? mt : 1.0;
  }
  return 0;
}

/* MULTI over the whole image or a pixel list (REF ray generation). */
int orc_render_multi(const bh_scene* s, const orc_texture* disc_tex, const orc_texture* bg_tex,
                     const orc_texture* obj_tex, const orc_rk4_opts* o, const int32_t* pixels, int64_t npix,
                     const orc_outputs* out, int nthreads) {
  view v;
  make_view(s, disc_tex, bg_tex, &v);
  v.obj_tex = obj_tex;
  const int64_t n = pixels ? npix : (int64_t)v.W * v.H;
  set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t i = 0; i < n; ++i) {
    int x = pixels ? pixels[2 * i] : (int)(i % v.W);
    int y = pixels ? pixels[2 * i + 1] : (int)(i / v.W);
    rk4_result r;
    multi_pixel(&v, o, x, y, &r);
    if (out->bgra) memcpy(out->bgra + 4 * i, r.bgra, 4);
    if (out->cls) out->cls[i] = (uint8_t)r.cls;
    if (out->aux) out->aux[i] = r.aux;
    if (out->margin_tex) out->margin_tex[i] = r.margin_tex;
    if (out->margin_r) out->margin_r[i] = r.margin_r;
    if (out->b_over_m) out->b_over_m[i] = r.b_over_m;
    if (out->steps) out->steps[i] = r.steps;
  }
  return 0;
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
