/* crt.hpp -- C++ classes over the C ABI (crt.h) with the reference's class and
 * method names, for host code written against mbartling/cuda-rt:
 *
 *   Camera      inc/camera.h:6-60 (the getters and setters the render reads)
 *   Light_h     inc/Light.h:7-29
 *   Scene       Scene_h::LoadObj + Scene_d = Scene_h (src/scene.cpp:6-160)
 *   BVH         BVH_d::setUp / intersect / intersectAny (inc/bvh.cuh:31-69)
 *   RayTracer   inc/raytracer.h:12-72 (LoadObj, setCamera, setHostLight,
 *               setUpDevice, run, pullRaytracedImage, writeImage)
 *
 * Header only; link with libcrt.so.  Where the reference printed an error and
 * called exit(1) (src/scene.cpp:71-81), these classes throw crt::Error with
 * the library's status and message. */
#ifndef CRT_HPP_
#define CRT_HPP_

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "crt.h"

namespace crt {

class Error : public std::runtime_error {
 public:
  Error(crt_status s, const std::string& what)
      : std::runtime_error(what + ": " + crt_last_error_string()), status(s) {}
  crt_status status;
};

inline void check(crt_status s, const char* what) {
  if (s != CRT_OK) throw Error(s, what);
}

struct Vec3d {
  double x, y, z;
};

/* Camera: the reference's defaults are fov 30, f-stop 8, focal point 10 and
 * the eye at the origin (kernels/camera.cu:10-22). */
class Camera {
 public:
  void setfov(double fov) { fov_ = fov; }
  void setFstop(double fstop) { fstop_ = fstop; }
  void setFocalPoint(double focal_point) { focal_ = focal_point; }
  void setEye(const Vec3d& eye) { eye_ = eye; }
  double getFOV() const { return fov_; }
  double getFocalPoint() const { return focal_; }
  double getAperature() const { return 1 / fstop_; }
  const Vec3d& getEye() const { return eye_; }
  crt_camera to_c() const {
    crt_camera c{};
    c.fov = fov_, c.focal_point = focal_, c.fstop = fstop_;
    c.eye[0] = eye_.x, c.eye[1] = eye_.y, c.eye[2] = eye_.z;
    return c;
  }

 private:
  double fov_ = 30.0, fstop_ = 8.0, focal_ = 10.0;
  Vec3d eye_{0.0, 0.0, 0.0};
};

/* Light_h with the reference's defaults (inc/Light.h:28).  The positional
 * light reads color, position, radius and the falloff terms. */
struct Light_h {
  Vec3d color{1.0, 1.0, 1.0};
  Vec3d position{1.0, 1.0, 1.0};
  Vec3d orientation{0.5, -1.0, -1.0};
  double width = 1.0, height = 1.0, radius = 0.5;
  double constantTerm = 0.0, linearTerm = 0.01, quadraticTerm = 0.001;
  crt_light to_c() const {
    crt_light l{};
    l.color[0] = color.x, l.color[1] = color.y, l.color[2] = color.z;
    l.position[0] = position.x, l.position[1] = position.y, l.position[2] = position.z;
    l.radius = radius, l.constant_term = constantTerm, l.linear_term = linearTerm;
    l.quadratic_term = quadraticTerm;
    return l;
  }
};

/* A mesh loaded from OBJ/MTL (Scene_h::LoadObj) and its device copy with the
 * BVH built (Scene_d = Scene_h).  Not copyable; movable. */
class Scene {
 public:
  Scene() = default;
  Scene(const Scene&) = delete;
  Scene& operator=(const Scene&) = delete;
  Scene(Scene&& o) noexcept { *this = std::move(o); }
  Scene& operator=(Scene&& o) noexcept {
    std::swap(obj_, o.obj_);
    std::swap(dev_, o.dev_);
    std::swap(camera_, o.camera_);
    return *this;
  }
  ~Scene() {
    crt_scene_destroy(dev_);
    crt_obj_free(obj_);
  }

  void LoadObj(const std::string& filename, const std::string& mtl_basepath = std::string()) {
    crt_obj* o = nullptr;
    check(crt_obj_load(filename.c_str(), mtl_basepath.empty() ? nullptr : mtl_basepath.c_str(), &o), "LoadObj");
    crt_obj_free(obj_);
    obj_ = o;
  }
  void setCamera(Camera* camera) { camera_ = camera; }
  Camera* getCamera() const { return camera_; }
  /* Upload and build (Scene_d::operator=(const Scene_h&), src/scene.cpp:82-160). */
  void setUpDevice(void* stream = nullptr) {
    if (!obj_) throw std::logic_error("Scene::setUpDevice before LoadObj");
    crt_mesh_desc d;
    check(crt_obj_mesh(obj_, &d), "setUpDevice");
    crt_scene* s = nullptr;
    check(crt_scene_create(&d, stream, &s), "setUpDevice");
    crt_scene_destroy(dev_);
    dev_ = s;
  }
  int numTriangles() const {
    crt_mesh_desc d;
    return obj_ && crt_obj_mesh(obj_, &d) == CRT_OK ? d.num_triangles : 0;
  }
  /* kr = Ks and ior = Ni per material, as LoadObj fills Material
   * (src/scene.cpp:29-31), for recursive renders. */
  std::vector<crt_optics> optics() const {
    crt_mesh_desc d;
    if (!obj_ || crt_obj_mesh(obj_, &d) != CRT_OK) return {};
    std::vector<crt_optics> o((size_t)d.num_materials);
    check(crt_obj_optics(obj_, o.data()), "optics");
    return o;
  }
  crt_scene* device() const { return dev_; }

 private:
  crt_obj* obj_ = nullptr;
  crt_scene* dev_ = nullptr;
  Camera* camera_ = nullptr;
};

/* BVH_d on a scene's device data (inc/bvh.cuh:31-69). */
class BVH {
 public:
  explicit BVH(const Scene& scene) : s_(scene.device()) {
    if (!s_) throw std::logic_error("BVH of a scene without setUpDevice");
  }
  /* Morton codes, stable sort, hierarchy, refit (src/bvh.cpp:3-32). */
  void setUp(void* stream = nullptr) { check(crt_bvh_build(s_, stream), "BVH::setUp"); }
  /* RefitBounds on the existing topology after new vertex positions. */
  void refit(const float* vertices, void* stream = nullptr) {
    check(crt_scene_set_vertices(s_, vertices, 0, stream), "BVH::refit");
  }
  /* BVH_d::intersect for n rays of 6 doubles (origin, direction). */
  void intersect(const double* rays, int64_t n, int32_t* ids, double* t = nullptr, double* normals = nullptr,
                 void* stream = nullptr) {
    check(crt_trace_closest(s_, rays, n, ids, t, normals, stream), "BVH::intersect");
  }
  /* BVH_d::intersectAny: the first hit in left-first DFS order. */
  void intersectAny(const double* rays, int64_t n, int32_t* ids, double* t = nullptr, void* stream = nullptr) {
    check(crt_trace_shadow(s_, rays, n, ids, t, stream), "BVH::intersectAny");
  }

 private:
  crt_scene* s_;
};

/* RayTracer (inc/raytracer.h:12-72).  The reference's three-argument
 * constructor stores imageWidth as the height too (raytracer.h:36); this one
 * keeps both.  run() takes 20 samples per pixel (raytracer.cu:138) unless
 * setSamples() says otherwise, and depth 0 (the reference's traceRay, whose
 * reflection/refraction block is commented out) unless setDepth() asks for
 * reflected and refracted rays. */
class RayTracer {
 public:
  RayTracer() : RayTracer(512, 512, 1) {}
  RayTracer(int imageWidth, int imageHeight, int superSampling)
      : w_(imageWidth), h_(imageHeight), super_(superSampling), image_((size_t)imageWidth * imageHeight * 3) {}

  void LoadObj(const std::string& filename, const std::string& mtl_basepath) {
    scene_.LoadObj(filename, mtl_basepath);
  }
  void setCamera(Camera* camera) { scene_.setCamera(camera); }
  void setHostLight(const Light_h& light) { light_ = light; }
  void setUpDevice(void* stream = nullptr) { scene_.setUpDevice(stream); }
  void setSamples(int spp) { spp_ = spp; }
  void setDepth(int depth) { depth_ = depth; }
  /* 0 (default): the reference's random streams; other values: an
   * independent render (crt_render_params.seed). */
  void setSeed(uint32_t seed) { seed_ = seed; }
  /* runRayTracerKernelRec over the image (kernels/raytracer.cu:55-92). */
  void run(void* stream = nullptr) {
    if (!scene_.device()) throw std::logic_error("RayTracer::run before setUpDevice");
    const Camera cam = scene_.getCamera() ? *scene_.getCamera() : Camera();
    const crt_camera c = cam.to_c();
    const crt_light l = light_.to_c();
    crt_render_params p{w_, h_, spp_, 0, 0, seed_};
    crt_render_out o{};
    o.rgb8 = image_.data();
    if (depth_ == 0) {
      check(crt_render(scene_.device(), &c, &l, &p, &o, stream), "RayTracer::run");
    } else {
      const std::vector<crt_optics> opt = scene_.optics();
      check(crt_render_recursive(scene_.device(), &c, &l, &p, depth_, opt.data(), &o, stream), "RayTracer::run");
    }
    check(crt_scene_check(scene_.device(), stream), "RayTracer::run");
  }
  /* The image is already in host memory after run(); kept for the
   * reference's call sequence (inc/raytracer.h:53-63). */
  void pullRaytracedImage() {}
  /* writeBMP (src/bitmap.cpp:99-154). */
  void writeImage(const std::string& filename) const {
    check(crt_write_bmp(filename.c_str(), w_, h_, image_.data()), "RayTracer::writeImage");
  }
  /* rgb8, bottom-up rows as the reference's image buffer. */
  const std::vector<uint8_t>& image() const { return image_; }
  int width() const { return w_; }
  int height() const { return h_; }
  int superSampling() const { return super_; }
  const Scene& scene() const { return scene_; }

 private:
  int w_, h_, super_;
  int spp_ = 20, depth_ = 0;
  uint32_t seed_ = 0;
  std::vector<uint8_t> image_;
  Scene scene_;
  Light_h light_;
};

}  // namespace crt

#endif  // CRT_HPP_
