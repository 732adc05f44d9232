// Test infrastructure (oracle only). Driver program that runs the reference's
// own per-pixel geodesic render loop -- blackhole_solution_test.cc:161-308,
// extracted unmodified at build time by oracle/build_ref.py into
// oracle/_ref/src/ref_render_loop.inc -- on scenes built through the
// reference's own API: Camera<double> (camera.h:30-63), StaticBlackhole<double>
// (blackhole_solution.h:24-88), Annulus<double> (vector_object.h:320-347) and
// ObjectManager<double> (object_manager.h:30-85). It compiles against the
// project-written OpenCV stand-in in oracle/cvshim.
//
// With `mode flat` it runs the reference's flat-space RayTracer instead
// (ray_tracer.h:52-96): per pixel RayTracer(camera.focus(),
// camera.PixelVector(x, y, fv)).Prograde(manager, pixel, 10), the loop of
// ray_tracer_test.cc:140-155; the hole is not inserted then.
//
// The reference draws no class buffer (a horizon hit and a miss are both
// black), so a second "tag" pass replaces the scene objects by subclasses
// that override only the virtual colour (material.h:54) with a class tag:
// 1 = horizon, 2 = disc, 4 = object (channel 1: its index), 0 = nothing hit.
// Collision code is inherited as is.
//
// Usage: ref_runner SCENE_FILE OUT_FILE [--tag] [--threads N] [--time]
// Scene file (whitespace-separated tokens):
//   mode curved|flat          (optional, default curved)
//   image W H
//   fov RADIANS
//   bh X Y Z MASS
//   disc P1x P1y P1z P2x P2y P2z P3x P3y P3z P4x P4y P4z R_OUTER R_INNER (optional)
//   disc_op OP ARGS...        (optional, any number, applied in order)
//   texture PATH COLS ROWS    (raw BGR bytes, row-major; the disc's)
//   rect P1x..P4z PATH COLS ROWS   (Rectangle<double>, textured; PATH - for none)
//   plane Px Py Pz SIZE       (InfinitePlane<double> with ChessPattern2D{SIZE})
//   obj_op OP ARGS...         (pose op on the last object line)
//   frames N
//   frame K OP ARGS... (K ops) (N times; camera ops for that frame)
// Objects are inserted after the disc and the hole, in file order.
// OP is one of MoveTo x y z | Move dx dy dz | MoveX d | MoveY d | MoveZ d |
//              RotateX a | RotateY a | RotateZ a | Fov a
// OUT_FILE receives N frames of W*H*3 bytes (BGR), or the tag per pixel in
// channel 0 with --tag.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "opencv2/opencv.hpp"
#include "blackhole/camera.h"
#include "blackhole/object.h"
#include "blackhole/object/object_manager.h"
#include "blackhole/object/pattern.h"
#include "blackhole/blackhole_solution.h"
#include "blackhole/ray_tracer.h"

namespace {

using value_type = double;
using point_type = cv::Vec<value_type, 3>;
using vector_type = cv::Vec<value_type, 3>;
using matrix_type = cv::Matx<value_type, 3, 3>;

struct TagBlackhole : blackhole::StaticBlackhole<double> {
  using blackhole::StaticBlackhole<double>::StaticBlackhole;
  cv::Vec3b color(double, double, double) const override { return {1, 0, 0}; }
};

struct TagAnnulus : blackhole::Annulus<double> {
  using blackhole::Annulus<double>::Annulus;
  cv::Vec3b color(double, double, double) const override { return {2, 0, 0}; }
};

struct TagRectangle : blackhole::Rectangle<double> {
  using blackhole::Rectangle<double>::Rectangle;
  int idx = 0;
  cv::Vec3b color(double, double, double) const override { return {4, (unsigned char)idx, 0}; }
};

struct TagPlane : blackhole::InfinitePlane<double> {
  using blackhole::InfinitePlane<double>::InfinitePlane;
  int idx = 0;
  cv::Vec3b color(double, double, double) const override { return {4, (unsigned char)idx, 0}; }
};

struct Op {
  std::string name;
  double a[3] = {0, 0, 0};
};

struct ObjSpec {
  std::string kind;
  double v[12] = {0};
  double size = 0;
  std::string tex_path;
  int tex_cols = 0, tex_rows = 0;
  std::vector<Op> ops;
};

int nargs(const std::string& op) {
  if (op == "MoveTo" || op == "Move") return 3;
  if (op == "MoveX" || op == "MoveY" || op == "MoveZ" || op == "RotateX" ||
      op == "RotateY" || op == "RotateZ" || op == "Fov")
    return 1;
  return -1;
}

template <typename Obj>
void apply(Obj& o, const Op& op) {
  if (op.name == "MoveTo") o.MoveTo(op.a[0], op.a[1], op.a[2]);
  else if (op.name == "Move") o.Move(op.a[0], op.a[1], op.a[2]);
  else if (op.name == "MoveX") o.MoveX(op.a[0]);
  else if (op.name == "MoveY") o.MoveY(op.a[0]);
  else if (op.name == "MoveZ") o.MoveZ(op.a[0]);
  else if (op.name == "RotateX") o.RotateX(op.a[0]);
  else if (op.name == "RotateY") o.RotateY(op.a[0]);
  else if (op.name == "RotateZ") o.RotateZ(op.a[0]);
}

[[noreturn]] void fail(const std::string& msg) {
  std::cerr << "ref_runner: " << msg << "\n";
  std::exit(2);
}

Op read_op(std::istream& in) {
  Op op;
  if (!(in >> op.name)) fail("truncated op");
  const int n = nargs(op.name);
  if (n < 0) fail("unknown op " + op.name);
  for (int i = 0; i < n; ++i)
    if (!(in >> op.a[i])) fail("truncated op args");
  return op;
}

// The flat RayTracer over the frame, as ray_tracer_test.cc:140-155 drives it
// (pixels are independent; FindCollision is const).
void render_flat(const blackhole::Camera<value_type>& camera, const blackhole::ObjectManager<value_type>& manager,
                 cv::Mat* screen, const int kScreenWidth, const int kScreenHeight) {
  const auto fv = camera.focus_vector();
#pragma omp parallel for schedule(dynamic, 2)
  for (int x = 0; x < kScreenWidth; ++x) {
    for (int y = 0; y < kScreenHeight; ++y) {
      blackhole::RayTracer ray_tracer(camera.focus(), camera.PixelVector(x, y, fv));
      ray_tracer.Prograde(manager, screen->data + (y * kScreenWidth + x) * 3, 10);
    }
  }
}

cv::Mat read_texture(const std::string& path, int cols, int rows) {
  cv::Mat t(rows, cols, CV_8UC3);
  std::ifstream tf(path, std::ios::binary);
  tf.read(reinterpret_cast<char*>(t.data), std::streamsize(t.total() * 3));
  if (!tf) fail("cannot read texture " + path);
  return t;
}

// One frame of the reference's render loop. The names the loop uses --
// camera, blackhole, manager, screen, kScreenWidth, kScreenHeight and the
// four type aliases -- are bound here exactly as in the reference's main().
template <typename BH>
void render_frame(const blackhole::Camera<value_type>& camera, const BH& blackhole,
                  const blackhole::ObjectManager<value_type>& manager, cv::Mat* screen,
                  const int kScreenWidth, const int kScreenHeight) {
#include "ref_render_loop.inc"
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 3) fail("usage: ref_runner SCENE OUT [--tag] [--threads N] [--time]");
  bool tag = false, timed = false;
  int threads = 0;
  for (int i = 3; i < argc; ++i) {
    std::string a = argv[i];
    if (a == "--tag") tag = true;
    else if (a == "--time") timed = true;
    else if (a == "--threads" && i + 1 < argc) threads = std::atoi(argv[++i]);
    else fail("bad argument " + a);
  }
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
  const int used_threads = omp_get_max_threads();
#else
  const int used_threads = 1;
#endif

  std::ifstream in(argv[1]);
  if (!in) fail("cannot open scene");
  int W = 0, H = 0, nframes = 0;
  double fov = 0, bx = 0, by = 0, bz = 0, mass = 1;
  double dp[12] = {0};
  double r_outer = 0, r_inner = 0;
  std::vector<Op> disc_ops;
  std::string tex_path;
  int tex_cols = 0, tex_rows = 0;
  std::vector<std::vector<Op>> frames;
  std::vector<ObjSpec> objs;
  bool flat = false, have_disc = false;
  std::string key;
  while (in >> key) {
    if (key == "mode") {
      std::string m;
      in >> m;
      if (m == "flat") flat = true;
      else if (m != "curved") fail("unknown mode " + m);
    } else if (key == "tri") {
      // Triangle<T>'s constructors initialize Object<T>, which is not its
      // direct base (vector_object.h:26-36): it does not compile instantiated.
      fail("Triangle<double> does not compile in the reference");
    } else if (key == "rect" || key == "plane") {
      ObjSpec o;
      o.kind = key;
      const int nv = key == "rect" ? 12 : 3;
      for (int i = 0; i < nv; ++i) in >> o.v[i];
      if (key == "rect") in >> o.tex_path >> o.tex_cols >> o.tex_rows;
      if (key == "plane") in >> o.size;
      if (!in) fail("truncated " + key);
      objs.push_back(o);
    } else if (key == "obj_op") {
      if (objs.empty()) fail("obj_op before any object");
      objs.back().ops.push_back(read_op(in));
    } else if (key == "image") in >> W >> H;
    else if (key == "fov") in >> fov;
    else if (key == "bh") in >> bx >> by >> bz >> mass;
    else if (key == "disc") {
      for (double& v : dp) in >> v;
      in >> r_outer >> r_inner;
      have_disc = true;
    } else if (key == "disc_op") disc_ops.push_back(read_op(in));
    else if (key == "texture") in >> tex_path >> tex_cols >> tex_rows;
    else if (key == "frames") in >> nframes;
    else if (key == "frame") {
      int k = 0;
      in >> k;
      std::vector<Op> ops;
      for (int i = 0; i < k; ++i) ops.push_back(read_op(in));
      frames.push_back(ops);
    } else fail("unknown key " + key);
  }
  if (W <= 0 || H <= 0 || int(frames.size()) != nframes || (have_disc && (tex_cols <= 0 || tex_rows <= 0)))
    fail("incomplete scene");

  // Insertion order follows the reference's main(): disc first, then the
  // hole (not in flat mode), then the objects.
  auto& manager = blackhole::ObjectManager<value_type>::GetInstance();
  const point_type p1{dp[0], dp[1], dp[2]}, p2{dp[3], dp[4], dp[5]};
  const point_type p3{dp[6], dp[7], dp[8]}, p4{dp[9], dp[10], dp[11]};
  if (have_disc) {
    const cv::Mat texture = read_texture(tex_path, tex_cols, tex_rows);
    if (tag) {
      auto d = manager.InsertObject(std::make_unique<TagAnnulus>(p1, p2, p3, p4, r_outer, r_inner));
      d.second->SetTexture(texture);
      for (const Op& op : disc_ops) apply(*d.second, op);
    } else {
      auto d = manager.InsertObject<blackhole::Annulus>(p1, p2, p3, p4, r_outer, r_inner);
      d.second->SetTexture(texture);
      for (const Op& op : disc_ops) apply(*d.second, op);
    }
  }
  std::unique_ptr<blackhole::StaticBlackhole<value_type>> own_hole;
  const blackhole::StaticBlackhole<value_type>* hole = nullptr;
  if (flat) {
    own_hole = std::make_unique<blackhole::StaticBlackhole<value_type>>(point_type(bx, by, bz), mass);
    hole = own_hole.get();
  } else if (tag) {
    hole = manager.InsertObject(std::make_unique<TagBlackhole>(point_type(bx, by, bz), mass)).second;
  } else {
    hole = manager.InsertObject<blackhole::StaticBlackhole>(point_type(bx, by, bz), mass).second;
  }
  for (size_t k = 0; k < objs.size(); ++k) {
    const ObjSpec& o = objs[k];
    const double* v = o.v;
    blackhole::DrawableObject<value_type>* obj = nullptr;
    if (o.kind == "rect") {
      const point_type a{v[0], v[1], v[2]}, b{v[3], v[4], v[5]}, c{v[6], v[7], v[8]}, d{v[9], v[10], v[11]};
      if (tag) {
        auto r = manager.InsertObject(std::make_unique<TagRectangle>(a, b, c, d));
        r.second->idx = int(k);
        obj = r.second;
      } else {
        auto r = manager.InsertObject<blackhole::Rectangle>(a, b, c, d);
        if (o.tex_path != "-") r.second->SetTexture(read_texture(o.tex_path, o.tex_cols, o.tex_rows));
        obj = r.second;
      }
    } else {
      const point_type pos{v[0], v[1], v[2]};
      if (tag) {
        auto r = manager.InsertObject(std::make_unique<TagPlane>(pos));
        r.second->idx = int(k);
        obj = r.second;
      } else {
        obj = manager.InsertObject<blackhole::InfinitePlane>(pos, blackhole::ChessPattern2D<value_type>{int(o.size)})
                  .second;
      }
    }
    for (const Op& op : o.ops) apply(*obj, op);
  }

  std::ofstream out(argv[2], std::ios::binary);
  if (!out) fail("cannot open output");
  double seconds = 0;
  for (int f = 0; f < nframes; ++f) {
    blackhole::Camera<value_type> camera(W, H, fov);
    for (const Op& op : frames[f]) {
      if (op.name == "Fov") camera.fov(op.a[0]);
      else apply(camera, op);
    }
    cv::Mat screen(H, W, CV_8UC3, cv::Scalar(0, 0, 0));
    const auto t0 = std::chrono::steady_clock::now();
    if (flat) render_flat(camera, manager, &screen, W, H);
    else render_frame(camera, *hole, manager, &screen, W, H);
    const auto t1 = std::chrono::steady_clock::now();
    seconds += std::chrono::duration<double>(t1 - t0).count();
    out.write(reinterpret_cast<const char*>(screen.data), std::streamsize(screen.total() * 3));
  }
  if (timed) {
    const double rays = double(W) * H * nframes;
    std::printf("{\"seconds\": %.6f, \"rays\": %.0f, \"mrays_per_s\": %.6f, \"threads\": %d}\n",
                seconds, rays, rays / seconds / 1e6, used_threads);
  }
  return 0;
}
