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
