// Test infrastructure (oracle only). Driver program that runs the reference's
// own per-pixel geodesic render loop -- blackhole_solution_test.cc:161-308,
// extracted unmodified at build time by oracle/build_ref.py into
// oracle/_ref/src/ref_render_loop.inc -- on scenes built through the
// reference's own API: Camera<double> (camera.h:30-63), StaticBlackhole<double>
// (blackhole_solution.h:24-88), Annulus<double> (vector_object.h:320-347) and
// ObjectManager<double> (object_manager.h:30-85). It compiles against the
// project-written OpenCV stand-in in oracle/cvshim.
//
// The reference draws no class buffer (a horizon hit and a miss are both
// black), so a second "tag" pass replaces the two scene objects by subclasses
// that override only the virtual colour (material.h:54) with a class tag:
// 1 = horizon, 2 = disc, 0 = nothing hit. Collision code is inherited as is.
//
// Usage: ref_runner SCENE_FILE OUT_FILE [--tag] [--threads N] [--time]
// Scene file (whitespace-separated tokens):
//   image W H
//   fov RADIANS
//   bh X Y Z MASS
//   disc P1x P1y P1z P2x P2y P2z P3x P3y P3z P4x P4y P4z R_OUTER R_INNER
//   disc_op OP ARGS...        (optional, any number, applied in order)
//   texture PATH COLS ROWS    (raw BGR bytes, row-major)
//   frames N
//   frame K OP ARGS... (K ops) (N times; camera ops for that frame)
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
#include "blackhole/blackhole_solution.h"

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

struct Op {
  std::string name;
  double a[3] = {0, 0, 0};
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
  std::string key;
  while (in >> key) {
    if (key == "image") in >> W >> H;
    else if (key == "fov") in >> fov;
    else if (key == "bh") in >> bx >> by >> bz >> mass;
    else if (key == "disc") {
      for (double& v : dp) in >> v;
      in >> r_outer >> r_inner;
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
  if (W <= 0 || H <= 0 || int(frames.size()) != nframes || tex_cols <= 0 || tex_rows <= 0)
    fail("incomplete scene");

  cv::Mat texture(tex_rows, tex_cols, CV_8UC3);
  {
    std::ifstream tf(tex_path, std::ios::binary);
    tf.read(reinterpret_cast<char*>(texture.data), std::streamsize(texture.total() * 3));
    if (!tf) fail("cannot read texture");
  }

  // Insertion order follows the reference's main(): disc first, then the hole.
  auto& manager = blackhole::ObjectManager<value_type>::GetInstance();
  const point_type p1{dp[0], dp[1], dp[2]}, p2{dp[3], dp[4], dp[5]};
  const point_type p3{dp[6], dp[7], dp[8]}, p4{dp[9], dp[10], dp[11]};
  const blackhole::StaticBlackhole<value_type>* hole = nullptr;
  if (tag) {
    auto d = manager.InsertObject(std::make_unique<TagAnnulus>(p1, p2, p3, p4, r_outer, r_inner));
    d.second->SetTexture(texture);
    for (const Op& op : disc_ops) apply(*d.second, op);
    hole = manager.InsertObject(std::make_unique<TagBlackhole>(point_type(bx, by, bz), mass)).second;
  } else {
    auto d = manager.InsertObject<blackhole::Annulus>(p1, p2, p3, p4, r_outer, r_inner);
    d.second->SetTexture(texture);
    for (const Op& op : disc_ops) apply(*d.second, op);
    hole = manager.InsertObject<blackhole::StaticBlackhole>(point_type(bx, by, bz), mass).second;
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
    render_frame(camera, *hole, manager, &screen, W, H);
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
