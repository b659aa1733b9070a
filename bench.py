"""Benchmark: the plain large workload, one frame per step.

Workload (the large plain configuration): a 1,003,520-face geodesic
icosphere (nu=224) with seeded radial displacement, FP32; LBVH build from
the resident vertices, then a 1920x1080 render at 16 samples per pixel with
a thin lens (aperture radius 0.05, focus 3.0) on the reference's mrand
stream, Lambert shading and one shadow ray per hit.  A step = crt_bvh_build
+ crt_render (device buffers).  `value` = primary rays per second of the
whole step (1920*1080*16 / step time), in Mrays/s.

`e2e` runs the same step through the C ABI with host buffers: the vertex
upload from pinned memory (crt_scene_set_vertices, rebuild) and the image
download into pinned memory (crt_render with a host rgb8 pointer).

L2 (129 MB) is flushed between timed steps by writing a 512 MB buffer
outside the timed region; each step is timed alone with CUDA events on the
stream the library launches on, and the step times are summed.

`--impl reference` times the reference's algorithm on the host cores: the
reference's own device code compiled for the host (oracle/_ref) where it
was built for this machine, else the oracle port (oracle/crt_oracle.cpp),
with all host threads, on a bounded sample of the same workload (a band of
image rows per step, the BVH built once outside the timed region).

Multi-GPU (torchrun): independent replicas, one frame per rank per step; the
barrier + max-over-ranks timing gives the whole-job rate.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "cuda-rt_gb300"))
sys.path.insert(0, ROOT)

METRIC = "LBVH build Mtris/s; closest-hit Mrays/s; batched+adjoint vs plain, 1 GB300"
W, H, SPP = 1920, 1080, 16
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one timed
# k_pixels launch of this frame (9,606,780,416 read + 2,594,846,720 written),
# and the build's DRAM and L2 (lts__t_bytes.sum) bytes summed over its seven
# kernels, from single-pass ncu captures (profiles/large_frame_step_kernels.md
# gives the commands); the render's fetched bytes (the `achieved` numerator)
# are mostly served by L1 and L2.  Most of the render's DRAM bytes are the
# lens-table lookups (two random loads per sample, each filling whole L2
# lines) and the threads' local memory (traversal stacks and register spills
# of 175,104 resident threads).  Re-captured whenever those kernels change.
RENDER_DRAM_BYTES = 11_957_783_808
BUILD_DRAM_BYTES = 227_666_176
BUILD_L2_BYTES = 869_048_800
TRAFFIC_SOURCE = "ncu 2025.3 single-pass captures, GB300, 2026-12-04"


def build_launches(n):
    """Kernel launches of one crt_bvh_build of n triangles (build.cu): init,
    bounds, Morton, the sort (one cooperative launch from 16,384 triangles
    up to 152 tiles of 8192, else three passes), split search, refit and,
    above one 512-leaf refit block, the spanning-node refit."""
    if n <= 0:
        return 0
    sort = 1 if 2 * 8192 <= n <= 152 * 8192 else 3
    return 3 + sort + (1 if n >= 2 else 0) + 1 + (1 if n > 512 else 0)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """Samples nvidia-smi (every 50 ms) during the timed region: the sampler
    is started, and its first sample awaited, before the region begins; the
    summary keeps the samples read between the region's start and its end."""

    def __init__(self, index=0):
        self.samples, self.proc, self.index = [], None, index
        self.t0 = self.t1 = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            deadline = time.time() + 5.0
            while not self.samples and time.time() < deadline and self.proc.poll() is None:
                time.sleep(0.01)
        except OSError:
            self.proc = None
        self.t0 = time.time()
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                self.samples.append([time.time()] + parts)

    def __exit__(self, *a):
        self.t1 = time.time()
        if self.proc:
            time.sleep(0.06)  # the sample that covers the region's last moments
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        inside = [s[1:] for s in self.samples if self.t0 is not None and self.t0 <= s[0] <= self.t1 + 0.06]
        samples = inside or [s[1:] for s in self.samples[-2:]]
        if not samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(s[0]) for s in samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in samples for i in range(4) if s[3 + i].strip() == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(samples)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        backend = "nccl" if os.environ.get("CRT_BENCH_BACKEND", "nccl") == "nccl" else "gloo"
        dist.init_process_group(backend)
        return dist, rank, ws
    return None, 0, 1


def max_over_ranks(dist, x, device="cpu"):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def run_crt(args, dist, rank, ws):
    import torch

    import crt
    from crt import data

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    sc = data.config1()
    mesh = sc.mesh
    n = mesh.ntri
    scene = crt.Scene(mesh)
    stream = torch.cuda.current_stream()
    rgb = torch.empty((W * H, 3), dtype=torch.uint8, device="cuda")
    out = {"rgb8": rgb}
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")

    def step():
        scene.build(stream=stream)
        scene.render(sc.camera, sc.light, W, H, SPP, out=out, stream=stream)

    # warm-up
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    scene.check()
    # instrumented pass (outside timing): traversal traffic for the roofline
    stats = torch.zeros(2, dtype=torch.int64, device="cuda")
    scene.render(sc.camera, sc.light, W, H, SPP, out={"rgb8": rgb, "traversal_stats": stats}, stream=stream)
    torch.cuda.synchronize()
    nodes_visited, tris_tested = [int(x) for x in stats.cpu()]
    # timed steps: build and render timed separately, L2 flushed before each step
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    barrier(dist)
    torch.cuda.synchronize()
    with Clocks(dev) as clk:
        for k in range(args.steps):
            flush.zero_()
            ev[k][0].record(stream)
            scene.build(stream=stream)
            ev[k][1].record(stream)
            scene.render(sc.camera, sc.light, W, H, SPP, out=out, stream=stream)
            ev[k][2].record(stream)
        torch.cuda.synchronize()
    barrier(dist)
    t_build = sum(e[0].elapsed_time(e[1]) for e in ev) / 1e3
    t_render = sum(e[1].elapsed_time(e[2]) for e in ev) / 1e3
    t_total = max_over_ranks(dist, t_build + t_render, "cuda")
    rays = W * H * SPP
    value = rays * args.steps * ws / t_total / 1e6
    ms_step = t_total / args.steps * 1e3
    hbm, peak_kind = peaks()
    # render roofline (the dominant kernel): the bytes the traversal fetches,
    # 128 B per visited four-wide node + 48 B per tested leaf triangle, per launch
    alg_bytes = nodes_visited * 128 + tris_tested * 48
    render_s = t_render / args.steps
    achieved = alg_bytes / render_s / 1e9
    build_s = t_build / args.steps
    s_in = 12 + 12 * mesh.verts.shape[0] / n
    build_bytes = n * (s_in + 220)
    scene.check()

    # e2e through the C ABI with host (pinned) buffers
    verts_h = torch.from_numpy(mesh.verts).pin_memory()
    rgb_h = torch.empty((W * H, 3), dtype=torch.uint8).pin_memory()
    out_h = {"rgb8": rgb_h}

    def e2e_step():
        scene.set_vertices(verts_h, rebuild=True, stream=stream)
        scene.render(sc.camera, sc.light, W, H, SPP, out=out_h, stream=stream)

    for _ in range(max(1, args.warmup // 2)):
        e2e_step()
    torch.cuda.synchronize()
    e2e_steps = max(3, args.steps // 2)
    barrier(dist)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    torch.cuda.synchronize()
    t_e2e = max_over_ranks(dist, time.perf_counter() - t0, "cuda")
    e2e_value = rays * e2e_steps * ws / t_e2e / 1e6
    ok_img = bool(np.array_equal(rgb_h.numpy(), rgb.cpu().numpy()))

    refit = run_refit_vs_rebuild() if (rank == 0 and not args.no_extras) else None
    batched = run_batched() if (rank == 0 and not args.no_extras) else None
    adjoint = run_adjoint() if (rank == 0 and not args.no_extras) else None
    nextrows = run_next_rows() if (rank == 0 and not args.no_extras) else None
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(sc, args.cpu_seconds)
    if rank != 0:
        return None
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_step, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded icosphere, PCG64)",
        "config": {"workload": "large plain: nu=224 icosphere 1,003,520 tris FP32, LBVH build + 1920x1080 "
                               "16 spp thin-lens render (aperture 0.05, focus 3.0), Lambert + 1 shadow ray/hit",
                   "triangles": n, "width": W, "height": H, "spp": SPP,
                   "l2": "flushed between steps (512 MB write, untimed)", "parallelism": f"replicas x{ws}"},
        "build_mtris_s": round(n / build_s / 1e6, 2), "build_ms": round(build_s * 1e3, 4),
        "render_ms": round(render_s * 1e3, 3), "render_mrays_s": round(rays / render_s / 1e6, 2),
        "build_roofline": {"bound": "hbm", "achieved": round(build_bytes / build_s / 1e9, 1), "peak": hbm,
                           "unit": "GB/s", "frac": round(build_bytes / build_s / 1e9 / hbm, 4),
                           "bytes_per_tri": round(s_in + 220, 1), "peak_kind": peak_kind,
                           "traffic": BUILD_DRAM_BYTES, "l2_bytes": BUILD_L2_BYTES,
                           "l2_gbs": round(BUILD_L2_BYTES / build_s / 1e9, 1), "traffic_source": TRAFFIC_SOURCE},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": hbm, "unit": "GB/s",
                     "frac": round(achieved / hbm, 4), "traffic": RENDER_DRAM_BYTES, "kernel": "k_pixels",
                     "alg_bytes_per_launch": alg_bytes, "nodes_visited": nodes_visited,
                     "tris_tested": tris_tested, "peak_kind": peak_kind, "traffic_source": TRAFFIC_SOURCE},
        "e2e": {"value": round(e2e_value, 3), "unit": "Mrays/s", "h2d_bytes_per_step": int(mesh.verts.nbytes),
                "d2h_bytes_per_step": W * H * 3, "image_matches_device_run": ok_img},
        "gpu_launches": (build_launches(n) + 1) * args.steps,
        "clocks": clk.summary(),
    }
    if refit is not None:
        line["refit_vs_rebuild"] = refit
    if batched is not None:
        line["batched_vs_plain"] = batched
    if adjoint is not None:
        line["adjoint"] = adjoint
    if nextrows is not None:
        line["next_rows"] = nextrows
    if cpu is not None:
        line["cpu_baseline"] = cpu
    return line


def run_build_only(args):
    """crt_bvh_build of the large mesh, W untimed then K timed back to back
    (CUDA events on the library's stream); the device holds the scene only
    (about 300 MB), which keeps ncu captures of the build kernels small."""
    import torch

    import crt
    from crt import data
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    sc = data.config1()
    scene = crt.Scene(sc.mesh)
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        scene.build(stream=stream)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        scene.build(stream=stream)
    e1.record(stream)
    torch.cuda.synchronize()
    scene.check()
    ms = e0.elapsed_time(e1) / max(args.steps, 1)
    n = sc.mesh.ntri
    return {"metric": "LBVH build ms (large mesh, back to back)", "value": round(ms, 4), "unit": "ms",
            "higher_is_better": False, "steps": args.steps, "warmup": args.warmup, "triangles": n,
            "build_mtris_s": round(n / ms / 1e3, 1), "gpu_launches": build_launches(n) * args.steps}


def run_render_only(args, width, height):
    """crt_render of the large mesh (thin lens, 16 spp) at width x height with
    a device output, W untimed then K timed back to back: a smaller frame of
    the same kernel, for multi-pass profiling (about 2.4 GB on the device
    with the lens tables)."""
    import torch

    import crt
    from crt import data
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    sc = data.config1()
    scene = crt.Scene(sc.mesh)
    stream = torch.cuda.current_stream()
    rgb = torch.empty((width * height, 3), dtype=torch.uint8, device="cuda")
    for _ in range(max(args.warmup, 1)):
        scene.render(sc.camera, sc.light, width, height, SPP, out={"rgb8": rgb}, stream=stream)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        scene.render(sc.camera, sc.light, width, height, SPP, out={"rgb8": rgb}, stream=stream)
    e1.record(stream)
    torch.cuda.synchronize()
    scene.check()
    ms = e0.elapsed_time(e1) / max(args.steps, 1)
    rays = width * height * SPP
    return {"metric": "render ms (large mesh, back to back)", "value": round(ms, 4), "unit": "ms",
            "higher_is_better": False, "steps": args.steps, "warmup": args.warmup, "width": width, "height": height,
            "spp": SPP, "mrays_s": round(rays / ms / 1e3, 1), "gpu_launches": args.steps}


def run_batched_only(count):
    """The first `count` meshes of the batched workload, built and rendered
    twice in the two-launch form with a fixed shape; the second run timed."""
    import torch

    import crt
    from crt import data
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    scs = data.config3(count=count)
    b = crt.Batch([s.mesh for s in scs], [(s.camera, s.light, s.width, s.height, s.spp) for s in scs])
    img = torch.empty((int(b.offsets[-1]), 3), dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    b.set_tuning(256, 1, 16, 2)
    b.run(img, graph=False, stream=stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    b.run(img, graph=False, stream=stream)
    e1.record(stream)
    torch.cuda.synchronize()
    b.check()
    ms = e0.elapsed_time(e1)
    return {"metric": "batched build + render ms", "value": round(ms, 3), "unit": "ms", "higher_is_better": False,
            "meshes": count, "triangles": sum(b.ntri), "rays": b.rays, "mrays_s": round(b.rays / ms / 1e3, 1)}


def run_refit_vs_rebuild(frames=60, W2=1280, H2=720, spp=4):
    """The dynamic workload: the large mesh animated over `frames` frames, each
    frame traced at W2 x H2 x spp; per frame either an atomic bottom-up refit on
    frame 0's topology or a full LBVH rebuild.  Vertex arrays of all frames are
    resident on the device before timing; each frame's update (vertex copy +
    refit or rebuild) and render are timed with CUDA events."""
    import torch

    import crt
    from crt import data
    anim = data.Animation(frames=frames)
    sc = anim.scene(W2, H2, spp)
    allv = torch.from_numpy(np.stack([anim.vertices(f) for f in range(frames)])).cuda()
    stream = torch.cuda.current_stream()
    rgb = torch.empty((W2 * H2, 3), dtype=torch.uint8, device="cuda")
    out = {"rgb8": rgb}
    res = {}
    for mode in ("refit", "rebuild"):
        scene = crt.Scene(anim.mesh0)
        scene.render(sc.camera, sc.light, W2, H2, spp, out=out, stream=stream)  # warm-up
        ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(frames)]
        torch.cuda.synchronize()
        for f in range(frames):
            ev[f][0].record(stream)
            scene.set_vertices(allv[f], rebuild=(mode == "rebuild" or f == 0), stream=stream)
            ev[f][1].record(stream)
            scene.render(sc.camera, sc.light, W2, H2, spp, out=out, stream=stream)
            ev[f][2].record(stream)
        torch.cuda.synchronize()
        scene.check()
        upd = [e[0].elapsed_time(e[1]) for e in ev[1:]]
        frm = [e[0].elapsed_time(e[2]) for e in ev[1:]]
        res[mode] = (float(np.mean(upd)), float(np.mean(frm)))
        scene.close()
    rays = W2 * H2 * spp
    return {"frames": frames, "image": f"{W2}x{H2}x{spp}spp", "triangles": anim.mesh0.ntri,
            "refit_update_ms": round(res["refit"][0], 4), "rebuild_update_ms": round(res["rebuild"][0], 4),
            "refit_frame_ms": round(res["refit"][1], 3), "rebuild_frame_ms": round(res["rebuild"][1], 3),
            "refit_mrays_s": round(rays / res["refit"][1] / 1e3, 1),
            "rebuild_mrays_s": round(rays / res["rebuild"][1] / 1e3, 1)}


def run_batched(count=256, reps=3):
    """The batched workload: 256 meshes (log-uniform 1k..500k triangles),
    each with its own camera and light, 256x256 at 4 spp.  Batched = one
    graph replay of the persistent launch(es) that build and render every
    mesh (one launch, or the render in a second one: the autotuner chose the
    faster, and the other form is timed beside it); plain = the 256 meshes built
    and rendered one after another with the plain entry points (scenes
    resident on the device).  Both timed with CUDA events, L2 flushed first;
    the images of both must be identical."""
    import torch

    import crt
    from crt import data
    scs = data.config3(count=count)
    views = [(s.camera, s.light, s.width, s.height, s.spp) for s in scs]
    stream = torch.cuda.current_stream()
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    b = crt.Batch([s.mesh for s in scs], views)
    total_px = int(b.offsets[-1])
    rays = b.rays
    tris = sum(b.ntri)
    img_b = torch.empty((total_px, 3), dtype=torch.uint8, device="cuda")
    tune = b.autotune(stream=stream)
    for _ in range(2):
        b.run(img_b, graph=True, stream=stream)
    torch.cuda.synchronize()
    b.check()

    def timed(fn):
        ts = []
        for _ in range(reps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return float(np.median(ts))

    t_batch = timed(lambda: b.run(img_b, graph=True, stream=stream))
    # the other launch form with the same shape (one launch: build and render
    # in one persistent kernel; two: the render in its own launch)
    other = 3 - tune["launches"]
    b.set_tuning(tune["block_size"], tune["lanes_per_pixel"], tune["stack"], other)
    img_o = torch.empty_like(img_b)
    b.run(img_o, graph=True, stream=stream)
    t_other = timed(lambda: b.run(img_o, graph=True, stream=stream))
    same_forms = bool(torch.equal(img_o, img_b))
    b.set_tuning(tune["block_size"], tune["lanes_per_pixel"], tune["stack"], tune["launches"])
    scenes = [crt.Scene(s.mesh) for s in scs]
    img_p = torch.empty((total_px, 3), dtype=torch.uint8, device="cuda")
    outs = [{"rgb8": img_p[b.offsets[m]:b.offsets[m + 1]]} for m in range(count)]

    def plain():
        for m, s in enumerate(scs):
            scenes[m].build(stream=stream)
            scenes[m].render(s.camera, s.light, s.width, s.height, s.spp, out=outs[m], stream=stream)

    plain()
    torch.cuda.synchronize()
    t_plain = timed(plain)
    same = bool(torch.equal(img_b, img_p))
    # traversal work per primary ray of this workload (the same walks as the
    # batched render's), from instrumented plain renders, untimed
    stats = torch.zeros(2, dtype=torch.int64, device="cuda")
    total = torch.zeros(2, dtype=torch.int64, device="cuda")
    for m, s in enumerate(scs):  # (each render clears the counters it is given)
        scenes[m].render(s.camera, s.light, s.width, s.height, s.spp, out={"rgb8": img_p[b.offsets[m]:b.offsets[m + 1]],
                                                                           "traversal_stats": stats}, stream=stream)
        total += stats
    torch.cuda.synchronize()
    nodes, tested = (int(x) for x in total.cpu())
    for s in scenes:
        s.check()
        s.close()
    b.close()
    return {"meshes": count, "triangles": tris, "rays": rays, "image": "256x256x4spp per mesh",
            "batched_ms": round(t_batch, 3), "plain_ms": round(t_plain, 3),
            "batched_mrays_s": round(rays / t_batch / 1e3, 1), "plain_mrays_s": round(rays / t_plain / 1e3, 1),
            "speedup": round(t_plain / t_batch, 3), "tuning": tune, "images_identical": same and same_forms,
            "plain_launches": sum(build_launches(t) + 1 for t in b.ntri), "batched_launches": tune["launches"],
            "nodes_per_ray": round(nodes / rays, 2), "tris_per_ray": round(tested / rays, 2),
            f"{other}_launch_form_ms": round(t_other, 3)}


def run_adjoint(reps=5):
    """The differentiable workload: the 200,000-face icosphere with per-triangle
    albedo, 512x512 at 4 spp, pinhole; L2 loss against the image of the
    perturbed mesh.  Times one forward render (mean colour in double) and one
    adjoint (d loss / d vertices, light, albedo) with CUDA events; the adjoint
    re-traces every sample (nothing is stored between the two)."""
    import torch

    import crt
    from crt import data
    W = H = 512
    spp = 4
    sc = data.config4(width=W, height=H, spp=spp)
    tgt = data.config4(width=W, height=H, spp=spp, perturbed=True)
    stream = torch.cuda.current_stream()
    g = crt.Scene(sc.mesh)
    t_img = torch.empty((W * H, 3), dtype=torch.float64, device="cuda")
    crt.Scene(tgt.mesh).render(tgt.camera, tgt.light, W, H, spp, out={"rgb_f64": t_img}, stream=stream)
    img = torch.empty_like(t_img)
    out = dict(vertices=torch.zeros((g.nv, 3), dtype=torch.float64, device="cuda"),
               light=torch.zeros(3, dtype=torch.float64, device="cuda"),
               kd=torch.zeros((g.nmat, 3), dtype=torch.float64, device="cuda"))

    def fwd():
        g.render(sc.camera, sc.light, W, H, spp, out={"rgb_f64": img}, stream=stream)

    def bwd():
        g.adjoint(sc.camera, sc.light, W, H, spp, 2.0 * (img - t_img), out=out, stream=stream)

    fwd()
    bwd()
    torch.cuda.synchronize()
    res = {}
    for name, fn in (("forward", fwd), ("adjoint", bwd)):
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        res[name] = float(np.median(ts))
    g.check()
    rays = W * H * spp
    return {"triangles": sc.mesh.ntri, "image": f"{W}x{H}x{spp}spp", "forward_ms": round(res["forward"], 3),
            "adjoint_ms": round(res["adjoint"], 3), "forward_mrays_s": round(rays / res["forward"] / 1e3, 1),
            "adjoint_mrays_s": round(rays / res["adjoint"] / 1e3, 1),
            "loss": round(float(((img - t_img) ** 2).sum()), 6)}


def run_next_rows(reps=3):
    """The rows next to the path, each timed: (1) OBJ/MTL ingestion of the
    200,000-face icosphere written as an OBJ (crt_obj_load, host); (2) full
    shade -- Phong highlights and an area light (radius 0.3, three draws per
    hit) against Lambert with a point light, 1280x720x4, on the mirror/glass
    scene with an 81,920-face glass sphere; (3) reflections and refractions
    to depth 3 on that scene (crt_render_recursive) against depth 0; (4) the
    drop-in CLI end to end (process start, OBJ load, build, 1024x1024x20
    thin-lens render, BMP write) on the OBJ of (1)."""
    import shutil
    import tempfile

    import torch

    import crt
    from crt import build as cbuild
    from crt import data
    res = {}
    tmp = tempfile.mkdtemp(prefix="crt_next_")
    try:
        # (1) ingestion
        m = data.config4().mesh
        obj = os.path.join(tmp, "ico.obj")
        with open(os.path.join(tmp, "ico.mtl"), "w") as f:
            f.write("newmtl lambert\nKd 0.8 0.8 0.8\n")
        with open(obj, "w") as f:
            f.write("mtllib ico.mtl\n")
            np.savetxt(f, m.verts, fmt="v %.9g %.9g %.9g")
            np.savetxt(f, m.normals, fmt="vn %.9g %.9g %.9g")
            f.write("usemtl lambert\n")
            np.savetxt(f, np.stack([m.vidx + 1, m.nidx + 1], 2).reshape(-1, 6), fmt="f %d//%d %d//%d %d//%d")
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            crt.load_obj_native(obj)
            ts.append(time.perf_counter() - t0)
        t = float(np.median(ts))
        res["obj_ingest"] = {"triangles": m.ntri, "mbytes": round(os.path.getsize(obj) / 1e6, 1),
                             "ms": round(t * 1e3, 1), "mtris_s": round(m.ntri / t / 1e6, 2)}
        # (2), (3) shading and recursion
        W2, H2, spp = 1280, 720, 4
        stream = torch.cuda.current_stream()
        rgb = torch.empty((W2 * H2, 3), dtype=torch.uint8, device="cuda")

        def timed(fn):
            fn()
            torch.cuda.synchronize()
            out = []
            for _ in range(reps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                fn()
                e1.record(stream)
                torch.cuda.synchronize()
                out.append(e0.elapsed_time(e1))
            return float(np.median(out))

        cam = data.Camera(fov=50.0, focal_point=3.0, fstop=1.0 / (2 * 0.02))
        lt = data.light_for((2.0, 2.5, -2.0), (0.0, 0.0, -3.0))
        point = data.Light(position=lt, linear_term=0.02, quadratic_term=0.01)
        area = data.Light(position=lt, radius=0.3, linear_term=0.02, quadratic_term=0.01)
        lam_mesh, optics = data.optics_scene(nu=64)
        spec_mesh, _ = data.optics_scene(nu=64, specular=True)
        g_lam, g_spec = crt.Scene(lam_mesh), crt.Scene(spec_mesh)
        t_lam = timed(lambda: g_lam.render(cam, point, W2, H2, spp, out={"rgb8": rgb}, stream=stream))
        t_full = timed(lambda: g_spec.render(cam, area, W2, H2, spp, out={"rgb8": rgb}, stream=stream))
        rays = W2 * H2 * spp
        res["full_shade"] = {"triangles": spec_mesh.ntri, "image": f"{W2}x{H2}x{spp}spp",
                             "lambert_point_ms": round(t_lam, 3), "phong_area_ms": round(t_full, 3),
                             "phong_area_mrays_s": round(rays / t_full / 1e3, 1)}
        d_optics = torch.tensor(optics, dtype=torch.float64, device="cuda")
        t_d0 = timed(lambda: g_spec.render_recursive(cam, area, W2, H2, spp, 0, d_optics, out={"rgb8": rgb},
                                                     stream=stream))
        t_d3 = timed(lambda: g_spec.render_recursive(cam, area, W2, H2, spp, 3, d_optics, out={"rgb8": rgb},
                                                     stream=stream))
        counts = torch.zeros(2, dtype=torch.int64, device="cuda")
        g_spec.render_recursive(cam, area, W2, H2, spp, 3, d_optics, out={"rgb8": rgb, "traversal_stats": counts},
                                stream=stream)
        n_rays, n_shadow = (int(x) for x in counts.cpu().tolist())
        g_lam.check()
        g_spec.check()
        res["recursive"] = {"triangles": spec_mesh.ntri, "image": f"{W2}x{H2}x{spp}spp", "depth": 3,
                            "depth0_ms": round(t_d0, 3), "depth3_ms": round(t_d3, 3),
                            "primary_mrays_s": round(rays / t_d3 / 1e3, 1), "rays_traced": n_rays,
                            "shadow_rays": n_shadow, "all_rays_mrays_s": round((n_rays + n_shadow) / t_d3 / 1e3, 1)}
        # (4) the CLI
        cli = cbuild.build_cli()
        bmp = os.path.join(tmp, "out.bmp")
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            subprocess.run([cli, "-i", obj, "-o", bmp, "-w", "1024", "-h", "1024", "-R", "0"], check=True,
                           capture_output=True, timeout=300)
            ts.append(time.perf_counter() - t0)
        res["cli"] = {"triangles": m.ntri, "image": "1024x1024x20spp thin lens", "seconds": round(float(np.median(ts)), 3)}
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    return res


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu model")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def _cpu_impl():
    from oracle import oracle as orc
    kind = "port"
    try:
        if orc.ref_available():
            import ctypes
            ctypes.CDLL(orc.REF_LIB)
            kind = "reference"
    except OSError:
        kind = "port"
    return kind


def cpu_baseline(sc, seconds):
    """The reference algorithm on the host cores for a band of rows of the
    same frame; Mrays/s of primary rays (each with its shadow ray)."""
    from oracle.oracle import OracleScene
    kind = _cpu_impl()
    cores = os.cpu_count() or 1
    o = OracleScene(sc.mesh, "ref" if kind == "reference" else "oracle")
    spp = 20 if kind == "reference" else SPP  # the reference's kernel always takes 20
    # bands of 96 rows, as in the reference arm: large enough that the per-call
    # setup (the reference's full-frame buffers) is negligible; one untimed band first
    rows, done, t_used = 96, 0, 0.0
    r0 = H // 2 - rows // 2
    o.render(sc.camera, sc.light, W, H, spp=None if kind == "reference" else spp, rows=(r0, r0 + rows))
    while t_used < seconds:
        a = max(0, min(r0, H - rows))
        t0 = time.perf_counter()
        o.render(sc.camera, sc.light, W, H, spp=None if kind == "reference" else spp, rows=(a, a + rows))
        t_used += time.perf_counter() - t0
        done += rows
        r0 = (r0 + 97) % (H - rows)
    value = done * W * spp / t_used / 1e6
    return {"value": round(value, 4), "unit": "Mrays/s", "cores": cores, "cpu_model": cpu_model(), "kind": kind,
            "sample": f"{done} rows of {W} px x {spp} spp (bands of {rows} rows) of the {W}x{H} frame, "
                      f"BVH built once untimed, {t_used:.1f} s"}


def run_reference(args, dist, rank, ws):
    from crt import data
    from oracle.oracle import OracleScene
    if rank != 0:
        return None
    kind = _cpu_impl()
    sc = data.config1()
    o = OracleScene(sc.mesh, "ref" if kind == "reference" else "oracle")
    spp = 20 if kind == "reference" else SPP
    rows = 96  # a band large enough that the per-call setup is negligible (~0.1 s of work per step)
    times = []
    for k in range(args.warmup + args.steps):
        a = (H // 2 - rows // 2 + 37 * k) % (H - rows)
        t0 = time.perf_counter()
        o.render(sc.camera, sc.light, W, H, spp=None if kind == "reference" else spp, rows=(a, a + rows))
        if k >= args.warmup:
            times.append(time.perf_counter() - t0)
    t = sum(times)
    value = rows * W * spp * len(times) / t / 1e6
    cores = os.cpu_count() or 1
    sample = f"{rows} rows x {W} px x {spp} spp per step of the {W}x{H} frame, BVH built once untimed"
    return {"metric": METRIC, "value": round(value, 4), "unit": "Mrays/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(t / len(times) * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded icosphere, PCG64)",
            "config": {"workload": "large plain: nu=224 icosphere 1,003,520 tris FP32, 1920x1080 thin-lens render, "
                                   "Lambert + 1 shadow ray/hit (row-band sample)", "triangles": sc.mesh.ntri},
            "impl": "reference",
            "cpu_baseline": {"value": round(value, 4), "unit": "Mrays/s", "cores": cores,
                             "cpu_model": cpu_model(), "kind": kind, "sample": sample},
            "e2e": {"value": round(value, 4), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="crt", choices=["crt", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the refit-vs-rebuild, batched-vs-plain, adjoint and next-row figures")
    ap.add_argument("--batched-only", type=int, default=0, metavar="MESHES",
                    help="build and render the first MESHES meshes of the batched workload twice, two launches "
                         "each (block 256, 1 lane per pixel, stack 16), and time the second run: for profiling")
    ap.add_argument("--render-only", type=int, nargs=2, default=None, metavar=("WIDTH", "HEIGHT"),
                    help="time crt_render of the large mesh alone at WIDTH x HEIGHT, 16 spp: for profiling it")
    ap.add_argument("--build-only", action="store_true",
                    help="time the LBVH build of the large mesh alone (no render, no lens tables): for profiling it")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "crt" else args.warmup
    dist, rank, ws = dist_setup()
    if args.impl == "reference":
        line = run_reference(args, dist, rank, ws)
    else:
        import __graft_entry__
        if rank == 0:
            __graft_entry__.build()
        barrier(dist)
        if args.build_only:
            line = run_build_only(args)
        elif args.render_only:
            line = run_render_only(args, *args.render_only)
        elif args.batched_only:
            line = run_batched_only(args.batched_only)
        else:
            line = run_crt(args, dist, rank, ws)
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
