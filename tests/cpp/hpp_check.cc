// Checks of include/blackhole_gb300.hpp, driven by tests/test_cpp_header.py.
//   hpp_check pod                 the single-scene geometry built with the C++
//                                 classes, printed as the hex of its bh_scene
//   hpp_check objects             the objects of the objects scene (a chess
//                                 plane, two panels, one rotated; a triangle)
//                                 as bh_objects, one hex line each
//   hpp_check errors              error paths that need no GPU
//   hpp_check render W H DISC BG OUT
//                                 renders the scene (disc RGBA8 1024x64 and sky
//                                 RGB8 2048x1024 texels read from files) and
//                                 writes BGR24 pixels then hit classes to OUT
//   hpp_check binary W H DISC BG OUT
//                                 the same for the equal-mass binary (two holes
//                                 of mass 1/2 at y = -+3, disc 8.4-20, camera at
//                                 30 from the origin) with the MULTI integrator
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iterator>
#include <string>
#include <vector>

#include "blackhole_gb300.hpp"

using namespace blackhole;

namespace {

// The single scene: M = 1 at the origin, camera at r = 20 M, 80 degrees from
// the disc normal, FoV 60 degrees; disc 6-20 M (polar mapping).
struct Built {
  Camera<double> cam;
  StaticBlackhole<double> bh;
  Annulus<double> disc;
};

Built build(int w, int h) {
  const double incl = 80 * M_PI / 180, r = 20;
  Camera<double> cam(w, h, 60 * M_PI / 180);
  cam.RotateZ(-0.0);
  cam.RotateY(incl - M_PI / 2);
  cam.MoveTo(-r * std::sin(incl), -0.0, r * std::cos(incl));
  StaticBlackhole<double> bh({0, 0, 0}, 1.0);
  Annulus<double> disc({20, 20, 0}, {-20, 20, 0}, {-20, -20, 0}, {20, -20, 0}, 20, 6);
  disc.mapping(BH_DISC_MAP_POLAR);
  return {cam, bh, disc};
}

std::vector<uint8_t> read_file(const char* path) {
  std::ifstream f(path, std::ios::binary);
  return std::vector<uint8_t>(std::istreambuf_iterator<char>(f), {});
}

int fail(const char* what) {
  std::fprintf(stderr, "FAIL: %s\n", what);
  return 1;
}

}  // namespace

int main(int argc, char** argv) {
  const std::string mode = argc > 1 ? argv[1] : "";
  if (mode == "pod") {
    Built b = build(640, 360);
    const bh_scene s = ToPod(b.cam, b.bh, &b.disc, 0, 1);
    const auto* p = reinterpret_cast<const unsigned char*>(&s);
    for (size_t i = 0; i < sizeof(s); ++i) std::printf("%02x", p[i]);
    std::printf("\n");
    return 0;
  }
  if (mode == "objects") {
    InfinitePlane<double> plane({0, 0, -6}, ChessPattern2D<double>(2));
    Rectangle<double> back({12, 8, 8}, {12, -8, 8}, {12, -8, -4}, {12, 8, -4});
    Rectangle<double> side(-8, -10, 6, 8, -10, 6, 8, -10, -2, -8, -10, -2);
    side.RotateZ(0.3);
    side.MoveX(1.5);
    Triangle<double> tri({10, -6, -3}, {10, 6, -3}, {10, 0, 9});
    const SceneObject<double> objs[] = {&plane, &back, &side, &tri};
    const int32_t tex[] = {-1, 3, 4, -1};
    for (int k = 0; k < 4; ++k) {
      const bh_object o = ToPod(objs[k], tex[k]);
      const auto* p = reinterpret_cast<const unsigned char*>(&o);
      for (size_t i = 0; i < sizeof(o); ++i) std::printf("%02x", p[i]);
      std::printf("\n");
    }
    return 0;
  }
  if (mode == "errors") {
    Annulus<double> disc({1, 1, 0}, {-1, 1, 0}, {-1, -1, 0}, {1, -1, 0}, 1, 0.5);
    try {
      disc.SetTexture(Texture());
      return fail("empty texture accepted");
    } catch (const Error& e) {
      if (e.code() != BH_ERR_EMPTY_TEXTURE) return fail("wrong code for an empty texture");
    }
    Camera<double> cam(100, 50, 10.0);  // fov clamped below pi
    if (!(cam.fov() < M_PI && cam.fov() > 3.14)) return fail("fov clamp");
    const auto pv = cam.PixelVector(0, 0);
    const auto want = cam.focus_vector() - cam.vector_y() * 50.0 - cam.vector_z() * 25.0;
    for (int i = 0; i < 3; ++i)
      if (std::fabs(pv[i] - want[i]) > 1e-12) return fail("PixelVector");
    // without a device, creating a renderer throws BH_ERR_NO_DEVICE
    if (argc > 2 && std::string(argv[2]) == "nodevice") {
      try {
        Renderer r(0);
        return fail("renderer created without a device");
      } catch (const Error& e) {
        if (e.code() != BH_ERR_NO_DEVICE) return fail("wrong code without a device");
      }
    }
    std::printf("ok\n");
    return 0;
  }
  if (mode == "render" && argc == 7) {
    const int w = std::atoi(argv[2]), h = std::atoi(argv[3]);
    Built b = build(w, h);
    const std::vector<uint8_t> dt = read_file(argv[4]), bt = read_file(argv[5]);
    if (dt.size() != 1024 * 64 * 4 || bt.size() != 2048 * 1024 * 3) return fail("texture files");
    b.disc.SetTexture(Texture::FromPixels(1024, 64, BH_TEXEL_RGBA8, dt.data()));
    Background sky(Texture::FromPixels(2048, 1024, BH_TEXEL_RGB8, bt.data()));
    Options o;
    o.want_classes = true;
    Image img;
    Render(b.cam, b.bh, &b.disc, &sky, img, o);
    // a second render reuses the uploaded textures
    Image again = Render(b.cam, b.bh, &b.disc, &sky, o);
    if (again.pixels != img.pixels) return fail("repeat render differs");
    std::ofstream f(argv[6], std::ios::binary);
    f.write(reinterpret_cast<const char*>(img.pixels.data()), std::streamsize(img.pixels.size()));
    f.write(reinterpret_cast<const char*>(img.hit_class.data()), std::streamsize(img.hit_class.size()));
    std::printf("ok %d %d\n", img.width, img.height);
    return 0;
  }
  if (mode == "binary" && argc == 7) {
    const int w = std::atoi(argv[2]), h = std::atoi(argv[3]);
    const double incl = 80 * M_PI / 180, r = 30;
    Camera<double> cam(w, h, 60 * M_PI / 180);
    cam.RotateZ(-0.0);
    cam.RotateY(incl - M_PI / 2);
    cam.MoveTo(-r * std::sin(incl), -0.0, r * std::cos(incl));
    StaticBlackhole<double> h1({0, -3, 0}, 0.5), h2({0, 3, 0}, 0.5);
    Annulus<double> disc({20, 20, 0}, {-20, 20, 0}, {-20, -20, 0}, {20, -20, 0}, 20, 1.4 * 6.0);
    disc.mapping(BH_DISC_MAP_POLAR);
    const std::vector<uint8_t> dt = read_file(argv[4]), bt = read_file(argv[5]);
    if (dt.size() != 1024 * 64 * 4 || bt.size() != 2048 * 1024 * 3) return fail("texture files");
    disc.SetTexture(Texture::FromPixels(1024, 64, BH_TEXEL_RGBA8, dt.data()));
    Background sky(Texture::FromPixels(2048, 1024, BH_TEXEL_RGB8, bt.data()));
    Scene<double> sc{&cam, &h1, &disc, &sky, {}, {&h2}};
    Options o;
    o.want_classes = true;
    o.integrator = BH_INTEGRATOR_MULTI;
    o.precision = BH_PRECISION_FP64;
    o.step = 0.02;
    o.max_steps = 20000;
    std::vector<Image> imgs;
    DefaultRenderer().Render(std::vector<Scene<double>>{sc}, imgs, o);
    const Image& img = imgs[0];
    std::ofstream f(argv[6], std::ios::binary);
    f.write(reinterpret_cast<const char*>(img.pixels.data()), std::streamsize(img.pixels.size()));
    f.write(reinterpret_cast<const char*>(img.hit_class.data()), std::streamsize(img.hit_class.size()));
    std::printf("ok %d %d\n", img.width, img.height);
    return 0;
  }
  return fail("usage");
}
