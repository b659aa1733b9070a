"""The C ABI library loads and exports every entry point include/*.h declares
(no compute calls: this runs without a GPU)."""
import glob
import os
import re

from conftest import ROOT


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names.update(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(crt_\w+)\s*\(", src, flags=re.M))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("crt_scene_create", "crt_bvh_build", "crt_bvh_refit", "crt_trace_closest", "crt_trace_shadow",
                 "crt_render", "crt_sort_pairs", "crt_morton", "crt_last_error_string"):
        assert must in names


def test_library_exports_every_declared_symbol(built):
    import crt
    lib = crt.lib()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"
    assert b"sm_103a" in lib.crt_version()


def test_library_is_in_tree_and_built_for_sm103a(built):
    import crt.build as b
    assert os.path.exists(b.LIB) and b.LIB.startswith(ROOT)
    assert "arch=compute_103a,code=sm_103a" in " ".join(b.ARCH)
    assert "-fmad=false" in b.FLAGS


def test_cpp_wrappers_compile_and_link(built, tmp_path):
    """include/crt.hpp (Camera, Light_h, Scene, BVH, RayTracer with the
    reference's method names) compiles warning-free and links against the
    library; a program using it reports a missing OBJ as crt::Error."""
    import subprocess
    src = tmp_path / "use.cpp"
    src.write_text(r'''
#include "crt.hpp"
#include <cstdio>
int main() {
  crt::Camera cam;
  cam.setfov(45); cam.setFstop(16); cam.setFocalPoint(2);
  if (cam.getFOV() != 45 || cam.getAperature() != 1.0 / 16 || cam.getFocalPoint() != 2) return 2;
  crt::Light_h light;
  if (light.radius != 0.5 || light.linearTerm != 0.01) return 3;
  crt::RayTracer rt(64, 32, 1);
  rt.setCamera(&cam);
  rt.setHostLight(light);
  try {
    rt.LoadObj("/nonexistent/scene.obj", "");
  } catch (const crt::Error& e) {
    std::printf("%d %s\n", (int)e.status, e.what());
    return e.status == CRT_INVALID_ARG ? 0 : 4;
  }
  return 5;
}
''')
    lib = os.path.join(ROOT, "cuda-rt_gb300", "lib")
    exe = str(tmp_path / "use")
    subprocess.check_call(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                           str(src), "-L", lib, "-lcrt", "-Wl,-rpath," + lib, "-o", exe])
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "cannot open" in r.stdout, (r.returncode, r.stdout, r.stderr)


def test_cpp_wrappers_host_side(built, tmp_path):
    """The host-only parts of include/crt.hpp: Scene::LoadObj fills the mesh
    (fan-triangulated quad, Ks/Ni optics per material), and the classes
    refuse calls made out of the reference's order (BVH of a scene without
    setUpDevice, RayTracer::run before setUpDevice) with std::logic_error."""
    import subprocess
    (tmp_path / "q.mtl").write_text("newmtl m\nKd 0.5 0.5 0.5\nKs 0.25 0.5 0.75\nNi 1.33\n")
    (tmp_path / "q.obj").write_text("mtllib q.mtl\nv 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvn 0 0 1\n"
                                    "usemtl m\nf 1//1 2//1 3//1 4//1\n")
    src = tmp_path / "host.cpp"
    src.write_text(r'''
#include "crt.hpp"
#include <cstdio>
#include <stdexcept>
int main(int argc, char** argv) {
  (void)argc;
  crt::Scene scene;
  scene.LoadObj(argv[1]);
  if (scene.numTriangles() != 2) return 2;
  const std::vector<crt_optics> o = scene.optics();
  if (o.size() != 1 || o[0].kr[0] != 0.25 || o[0].kr[2] != 0.75 || o[0].ior != 1.33) return 3;
  try {
    crt::BVH bvh(scene);
    return 4;
  } catch (const std::logic_error&) {
  }
  crt::RayTracer rt(16, 8, 1);
  if (rt.width() != 16 || rt.height() != 8 || rt.image().size() != 16 * 8 * 3) return 5;
  try {
    rt.run();
    return 6;
  } catch (const std::logic_error&) {
  }
  crt::Scene moved = std::move(scene);
  if (moved.numTriangles() != 2 || scene.numTriangles() != 0) return 7;
  std::printf("ok\n");
  return 0;
}
''')
    lib = os.path.join(ROOT, "cuda-rt_gb300", "lib")
    exe = str(tmp_path / "host")
    subprocess.check_call(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                           str(src), "-L", lib, "-lcrt", "-Wl,-rpath," + lib, "-o", exe])
    r = subprocess.run([exe, str(tmp_path / "q.obj")], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "ok" in r.stdout, (r.returncode, r.stdout, r.stderr)
