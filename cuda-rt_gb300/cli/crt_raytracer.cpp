// crt_raytracer -- drop-in for the reference's cuda_bvh executable
// (src/main.cpp:91-332): the same flags and defaults, an OBJ/MTL scene in, a
// 24-bit BMP out, through the reference's call sequence on crt::RayTracer
// (include/crt.hpp): LoadObj, setHostLight, setCamera, setUpDevice, run,
// pullRaytracedImage, writeImage.
//
//   -i, --input <file.obj>         scene (required); its MTL is read from the
//                                  OBJ's directory, as main.cpp passes it
//   -o, --output <file.bmp>        image
//   -w, --width <int>, -h, --height <int>       image size (default 512 x 512)
//   -f, --fstop <float>            camera f-stop (aperture 1/fstop; default 8)
//   -v, --fov <float>              vertical field of view in degrees (default 30)
//   -P, --focalpoint <float>       focal distance (default 10)
//   -p, --position x,y,z           light position (default 1,1,1)
//   -c, --color r,g,b              light colour (default 1,1,1)
//   -a, --attenuation a,b,c        falloff 1/(a + b d + c d^2) (default 0,0.01,0.001)
//   -R, --radius <float>           light radius (default 0.5)
//   -d, --orientation x,y,z        accepted; a positional light ignores it
//   -n, --numeric, -1, --nonempty  accepted and ignored, as in main.cpp
//       --spp <int>                samples per pixel (default 20, the reference's N)
//       --seed <int>               0 (default): the reference's random streams; other
//                                  values give an independent render
//       --depth <int>              levels of reflected and refracted rays (default 0:
//                                  the reference's image, whose traceRay block for
//                                  them is commented out; at most CRT_MAX_DEPTH),
//                                  with kr = Ks and ior = Ni from the MTL
//
// Vectors are parsed per component with float precision and widened to
// double, scalars with double precision, as main.cpp does (stof / stod).
// The reference's RayTracer(h, w, 1) renders an h x h image whatever -w says
// (inc/raytracer.h:36); this tool renders width x height (the same image for
// square sizes).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "crt.hpp"

namespace {

struct Opt {
  char s;
  const char* l;
  bool arg;
};
const Opt kOpts[] = {{'i', "input", true},       {'o', "output", true},      {'w', "width", true},
                     {'h', "height", true},      {'f', "fstop", true},       {'v', "fov", true},
                     {'P', "focalpoint", true},  {'p', "position", true},    {'c', "color", true},
                     {'a', "attenuation", true}, {'R', "radius", true},      {'d', "orientation", true},
                     {'n', "numeric", true},     {'1', "nonempty", true},    {0, "spp", true},
                     {0, "depth", true},         {0, "seed", true},          {0, "help", false}};

void usage() {
  std::printf(
      "USAGE: crt_raytracer -i scene.obj -o image.bmp [-w W] [-h H] [-f fstop] [-v fov] [-P focal]\n"
      "                     [-p x,y,z] [-c r,g,b] [-a a,b,c] [-R radius] [-d x,y,z] [--spp N]\n"
      "                     [--depth N] [--seed N]\n");
}

bool vec3(const std::string& s, double out[3]) {
  // main.cpp's split(',') + stof per component
  size_t at = 0;
  for (int k = 0; k < 3; k++) {
    const size_t e = s.find(',', at);
    const std::string item = s.substr(at, e == std::string::npos ? std::string::npos : e - at);
    char* end = nullptr;
    const float v = std::strtof(item.c_str(), &end);
    if (item.empty() || end == item.c_str()) return false;
    out[k] = (double)v;
    if (e == std::string::npos) return k == 2;
    at = e + 1;
  }
  return true;
}

bool scalar(const std::string& s, double& out) {
  char* end = nullptr;
  out = std::strtod(s.c_str(), &end);
  return end != s.c_str();
}

}  // namespace

int main(int argc, char** argv) {
  std::string input, output;
  int width = 512, height = 512, spp = 20, depth = 0;
  unsigned long seed = 0;
  crt::Camera camera;  // fov 30, f-stop 8, focal point 10 (kernels/camera.cu:10-22)
  crt::Light_h light;  // position and colour (1,1,1), radius 0.5, falloff (0, 0.01, 0.001) (inc/Light.h:28)
  double fov = camera.getFOV(), fstop = 1 / camera.getAperature(), focal = camera.getFocalPoint();
  if (argc <= 1) {
    usage();
    return 0;
  }
  for (int i = 1; i < argc; i++) {
    std::string a = argv[i], val;
    const Opt* o = nullptr;
    if (a.rfind("--", 0) == 0) {
      const size_t eq = a.find('=');
      const std::string name = a.substr(2, eq == std::string::npos ? std::string::npos : eq - 2);
      for (const Opt& c : kOpts)
        if (name == c.l) o = &c;
      if (o && o->arg) {
        if (eq != std::string::npos) val = a.substr(eq + 1);
        else if (i + 1 < argc) val = argv[++i];
        else o = nullptr;
      }
    } else if (a.size() >= 2 && a[0] == '-') {
      for (const Opt& c : kOpts)
        if (c.s && a[1] == c.s) o = &c;
      if (o && o->arg) {
        if (a.size() > 2) val = a.substr(2);
        else if (i + 1 < argc) val = argv[++i];
        else o = nullptr;
      }
    }
    if (!o) {
      std::fprintf(stderr, "crt_raytracer: bad option '%s'\n", a.c_str());
      usage();
      return 1;
    }
    const std::string name = o->l;
    double v[3];
    bool ok = true;
    if (name == "help") {
      usage();
      return 0;
    } else if (name == "input") {
      input = val;
    } else if (name == "output") {
      output = val;
    } else if (name == "width" || name == "height" || name == "spp") {
      char* end = nullptr;
      const long x = std::strtol(val.c_str(), &end, 10);
      ok = end != val.c_str() && x > 0 && x <= (1 << 15);
      (name == "width" ? width : name == "height" ? height : spp) = (int)x;
    } else if (name == "depth") {
      char* end = nullptr;
      const long x = std::strtol(val.c_str(), &end, 10);
      ok = end != val.c_str() && *end == '\0' && x >= 0 && x <= CRT_MAX_DEPTH;
      depth = (int)x;
    } else if (name == "seed") {
      char* end = nullptr;
      seed = std::strtoul(val.c_str(), &end, 10);
      ok = end != val.c_str() && *end == '\0' && seed <= 0xFFFFFFFFul;
    } else if (name == "fstop") {
      ok = scalar(val, fstop);
    } else if (name == "fov") {
      ok = scalar(val, fov);
    } else if (name == "focalpoint") {
      ok = scalar(val, focal);
    } else if (name == "radius") {
      ok = scalar(val, light.radius);
    } else if (name == "position" || name == "color") {
      ok = vec3(val, v);
      if (ok) (name == "position" ? light.position : light.color) = crt::Vec3d{v[0], v[1], v[2]};
    } else if (name == "attenuation") {
      ok = vec3(val, v);
      if (ok) light.constantTerm = v[0], light.linearTerm = v[1], light.quadraticTerm = v[2];
    } else if (name == "orientation") {
      ok = vec3(val, v);  // unused by the positional light
      if (ok) light.orientation = crt::Vec3d{v[0], v[1], v[2]};
    }  // numeric / nonempty: accepted and ignored
    if (!ok) {
      std::fprintf(stderr, "crt_raytracer: bad value '%s' for --%s\n", val.c_str(), o->l);
      return 1;
    }
  }
  if (input.empty()) {
    std::fprintf(stderr, "crt_raytracer: an input OBJ (-i) is required\n");
    return 1;
  }
  camera.setfov(fov);
  camera.setFstop(fstop);
  camera.setFocalPoint(focal);
  try {
    crt::RayTracer rayTracer(width, height, 1);
    rayTracer.setSamples(spp);
    rayTracer.setDepth(depth);
    rayTracer.setSeed((uint32_t)seed);
    rayTracer.LoadObj(input, "");  // the MTL is read from the OBJ's directory
    rayTracer.setHostLight(light);
    rayTracer.setCamera(&camera);
    rayTracer.setUpDevice();
    rayTracer.run();
    rayTracer.pullRaytracedImage();
    if (!output.empty()) rayTracer.writeImage(output);
    std::printf("crt_raytracer: %d triangles, %dx%d, %d spp, depth %d -> %s\n", rayTracer.scene().numTriangles(),
                width, height, spp, depth, output.empty() ? "(no output)" : output.c_str());
  } catch (const std::exception& e) {
    std::fprintf(stderr, "crt_raytracer: %s\n", e.what());
    return 1;
  }
  return 0;
}
