"""The drop-in command-line renderer (crt_raytracer, the reference's cuda_bvh
flags) end to end: OBJ/MTL in, BMP out, against the oracle's render of the
same scene with the same camera and light (flag vectors parsed with float
precision, as main.cpp's stof)."""
import math
import os
import subprocess

import numpy as np
import pytest

from conftest import assert_equal
from test_obj import read_bmp

pytestmark = pytest.mark.gpu


def write_scene(d, mesh):
    with open(os.path.join(d, "soup.mtl"), "w") as f:
        f.write("newmtl matte\nKd 0.8 0.7 0.6\nKs 0 0 0\n")
    with open(os.path.join(d, "soup.obj"), "w") as f:
        f.write("mtllib soup.mtl\n")
        for v in mesh.verts:
            f.write("v %.9g %.9g %.9g\n" % tuple(float(x) for x in v))
        for n in mesh.normals:
            f.write("vn %.9g %.9g %.9g\n" % tuple(float(x) for x in n))
        f.write("usemtl matte\n")
        for a, b in zip(mesh.vidx + 1, mesh.nidx + 1):
            f.write("f %d//%d %d//%d %d//%d\n" % (a[0], b[0], a[1], b[1], a[2], b[2]))
    return os.path.join(d, "soup.obj")


def f32(*xs):
    return tuple(float(np.float32(x)) for x in xs)


@pytest.fixture(scope="module")
def cli_scene(cuda, tmp_path_factory):
    from crt import build, data
    d = str(tmp_path_factory.mktemp("cli"))
    mesh = data.soup(3000, seed=9, scale=0.9, cam_pos=(0.0, 0.0, -3.0))
    obj = write_scene(d, mesh)
    return build.build_cli(), d, obj, data.load_obj(obj)


def run_cli(cli, args):
    r = subprocess.run([cli] + args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return r


def test_cli_pinhole_matches_oracle_bit_exact(cli_scene):
    from crt import data
    from oracle.oracle import OracleScene
    cli, d, obj, mesh = cli_scene
    bmp = os.path.join(d, "pinhole.bmp")
    W, H, spp = 64, 48, 4
    run_cli(cli, ["-i", obj, "-o", bmp, "-w", str(W), "-h", str(H), "-f", "inf", "-v", "45", "-P", "2",
                  "-p", "2.3,1.7,-2.1", "-c", "1,0.9,0.8", "-a", "1,0,0.05", "-R", "0", "--spp", str(spp)])
    got = read_bmp(bmp)
    cam = data.Camera(fov=45.0, focal_point=2.0, fstop=math.inf)
    light = data.Light(position=f32(2.3, 1.7, -2.1), color=f32(1, 0.9, 0.8), radius=0.0, constant_term=1.0,
                       linear_term=0.0, quadratic_term=f32(0.05)[0])
    ref = OracleScene(mesh).render(cam, light, W, H, spp=spp)["rgb"]
    assert_equal(got, ref, "CLI image")
    assert got.any()


def test_cli_reference_defaults_thin_lens(cli_scene):
    """The reference's defaults (fov 30, f-stop 8, focus 10, light at 1,1,1 with
    falloff 0, 0.01, 0.001, 20 samples) with a point light (-R 0): thin-lens
    rays use cos/sin, which may differ from the host's in the last bit, so
    the image is held to 1/255 per channel."""
    from crt import data
    from oracle.oracle import OracleScene
    cli, d, obj, mesh = cli_scene
    bmp = os.path.join(d, "defaults.bmp")
    run_cli(cli, ["--input=" + obj, "--output", bmp, "-w", "32", "-h", "32", "-R0"])
    got = read_bmp(bmp)
    cam = data.Camera(fov=30.0, focal_point=10.0, fstop=8.0)
    light = data.Light(position=(1.0, 1.0, 1.0), color=(1.0, 1.0, 1.0), radius=0.0, constant_term=0.0,
                       linear_term=0.01, quadratic_term=0.001)
    ref = OracleScene(mesh).render(cam, light, 32, 32, spp=20)["rgb"]
    diff = np.abs(got.astype(int) - ref.astype(int))
    assert diff.max() <= 1 and (diff == 0).mean() > 0.99


def test_cli_errors(cli_scene, tmp_path):
    cli, d, obj, mesh = cli_scene
    r = subprocess.run([cli, "-i", str(tmp_path / "absent.obj")], capture_output=True, text=True, timeout=60)
    assert r.returncode != 0 and "cannot open" in r.stderr
    r = subprocess.run([cli, "-i", obj, "-w", "zero"], capture_output=True, text=True, timeout=60)
    assert r.returncode != 0 and "bad value" in r.stderr
    r = subprocess.run([cli, "--bogus"], capture_output=True, text=True, timeout=60)
    assert r.returncode != 0


def write_materials_scene(d, mesh, ior):
    """An OBJ/MTL pair holding `mesh` with one MTL entry per material row
    (Kd, Ks, Kt, Ke, Ns, and Ni from `ior`)."""
    names = [f"m{k}" for k in range(len(mesh.materials))]
    with open(os.path.join(d, "optics.mtl"), "w") as f:
        for name, m, n in zip(names, mesh.materials, ior):
            f.write(f"newmtl {name}\n")
            for key, at in (("Kd", 3), ("Ks", 6), ("Kt", 9), ("Ke", 12)):
                f.write(key + " %.17g %.17g %.17g\n" % tuple(m[at:at + 3]))
            f.write("Ns %.17g\nNi %.17g\n" % (m[15], n))
    with open(os.path.join(d, "optics.obj"), "w") as f:
        f.write("mtllib optics.mtl\n")
        for v in mesh.verts:
            f.write("v %.9g %.9g %.9g\n" % tuple(float(x) for x in v))
        for n in mesh.normals:
            f.write("vn %.9g %.9g %.9g\n" % tuple(float(x) for x in n))
        cur = None
        for a, b, m in zip(mesh.vidx + 1, mesh.nidx + 1, mesh.matid):
            if m != cur:
                f.write(f"usemtl {names[m]}\n")
                cur = m
            f.write("f %d//%d %d//%d %d//%d\n" % (a[0], b[0], a[1], b[1], a[2], b[2]))
    return os.path.join(d, "optics.obj")


def test_cli_depth_reflections_and_refractions(cli_scene, tmp_path):
    """--depth 3 on a mirror, glass and diffuse scene: the CLI takes kr = Ks
    and ior = Ni from the MTL (crt_obj_optics) and renders with
    crt_render_recursive; compared with the oracle's recursive render of the
    same OBJ.  Every material with Ks reflects and has a Phong highlight,
    whose powf may round differently on the host: 8-bit values within 1."""
    from crt import data
    from oracle.oracle import OracleScene
    from test_recursive import optics_scene
    cli = cli_scene[0]
    mesh, optics = optics_scene(specular=True)
    obj = write_materials_scene(str(tmp_path), mesh, optics[:, 3])
    bmp = str(tmp_path / "depth.bmp")
    W, H, spp = 48, 32, 2
    run_cli(cli, ["-i", obj, "-o", bmp, "-w", str(W), "-h", str(H), "-f", "inf", "-v", "50", "-P", "3",
                  "-p", "2.5,3,-1.5", "-a", "1,0.02,0.01", "-R", "0", "--spp", str(spp), "--depth", "3"])
    got = read_bmp(bmp)
    back = data.load_obj(obj)
    cam = data.Camera(fov=50.0, focal_point=3.0, fstop=math.inf)
    light = data.Light(position=f32(2.5, 3, -1.5), radius=0.0, constant_term=1.0, linear_term=f32(0.02)[0],
                       quadratic_term=f32(0.01)[0])
    cli_optics = np.concatenate([back.materials[:, 6:9], optics[:, 3:4]], 1)
    ref = OracleScene(back).render_recursive(cam, light, W, H, spp, 3, cli_optics)["rgb"]
    plain = OracleScene(back).render(cam, light, W, H, spp=spp)["rgb"]
    diff = np.abs(got.astype(int) - ref.astype(int))
    assert diff.max() <= 1 and (diff == 0).mean() > 0.99
    assert (got != plain).any(1).mean() > 0.05  # the reflections and refractions show
    r = subprocess.run([cli, "-i", obj, "--depth", "9"], capture_output=True, text=True, timeout=60)
    assert r.returncode != 0 and "bad value" in r.stderr



def test_cpp_bvh_intersect_matches_oracle(cli_scene, tmp_path):
    """crt::Scene + crt::BVH (include/crt.hpp): BVH_d::intersect and
    intersectAny on random rays through the C++ classes, against the oracle."""
    from oracle.oracle import OracleScene
    cli, d, obj, mesh = cli_scene
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = tmp_path / "bvh.cpp"
    src.write_text(r'''
#include "crt.hpp"
#include <cstdio>
#include <vector>
int main(int argc, char** argv) {
  crt::Scene scene;
  scene.LoadObj(argv[1]);
  scene.setUpDevice();
  crt::BVH bvh(scene);
  bvh.setUp();
  FILE* f = std::fopen(argv[2], "rb");
  std::vector<double> rays;
  double x;
  while (std::fread(&x, sizeof x, 1, f) == 1) rays.push_back(x);
  std::fclose(f);
  const long n = (long)rays.size() / 6;
  std::vector<int> ids(n), any(n);
  std::vector<double> t(n), ta(n);
  bvh.intersect(rays.data(), n, ids.data(), t.data());
  bvh.intersectAny(rays.data(), n, any.data(), ta.data());
  f = std::fopen(argv[3], "wb");
  std::fwrite(ids.data(), sizeof(int), n, f);
  std::fwrite(t.data(), sizeof(double), n, f);
  std::fwrite(any.data(), sizeof(int), n, f);
  std::fclose(f);
  return 0;
}
''')
    lib = os.path.join(root, "cuda-rt_gb300", "lib")
    exe = str(tmp_path / "bvh")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", os.path.join(root, "include"), str(src), "-L", lib,
                           "-lcrt", "-Wl,-rpath," + lib, "-o", exe])
    rng = np.random.default_rng(5)
    n = 4096
    org = rng.uniform(-0.3, 0.3, (n, 3))
    target = mesh.verts[rng.integers(0, len(mesh.verts), n)].astype(np.float64) + rng.normal(0, 0.002, (n, 3))
    dirs = target - org
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    rays = np.concatenate([org, dirs], 1)
    rays.astype(np.float64).tofile(str(tmp_path / "rays.bin"))
    subprocess.run([exe, obj, str(tmp_path / "rays.bin"), str(tmp_path / "out.bin")], check=True, timeout=120)
    raw = open(tmp_path / "out.bin", "rb").read()
    ids = np.frombuffer(raw[:4 * n], np.int32)
    t = np.frombuffer(raw[4 * n:12 * n], np.float64)
    anyh = np.frombuffer(raw[12 * n:16 * n], np.int32)
    o = OracleScene(mesh)
    rid, rt, _ = o.trace(rays)
    aid, _, _ = o.trace(rays, any_hit=True)
    assert_equal(ids, rid, "closest ids")
    assert_equal(t, rt, "closest t")
    assert_equal(anyh, aid, "any-hit ids")
    assert (ids >= 0).sum() > n // 8
