#!/usr/bin/env python
"""Benchmark of the LBVH build + traversal hot path on GB300.

Workload: the largest single-GPU case of the LBVH build + traversal
microbenchmark -- 16 Mi random triangles (centroids uniform in [0,1]^3, edge
length ~ Exp(mean 0.5 N^-1/3), fp32 SoA, unindexed), 30-bit Morton keys
(10 bits per axis); 16 Mi closest-hit rays and 16 Mi shadow segments.  Seeded
synthetic data (the reference ships no scenes for this path).

One step = one LBVH build of the 16 Mi triangles.  The headline metric is the
build time per million triangles (lower is better).  Inputs (576 MB of
vertices) exceed the 129 MB L2, so no flush is needed between steps.

Reported with it:
  e2e        the same metric through the C ABI from pinned HOST vertex arrays
             (clr_lbvh_build_host): each step copies the vertices host->device,
             builds, and reads the root box (the scene bounds) back to the
             host; a step's copy overlaps the previous step's build
             (serial_value: copy and build back to back on one stream);
  roofline   the build's dominant kernel: algorithmic bytes / its CUDA-event
             duration vs the measured HBM copy bandwidth;
  traversal  closest-hit and shadow throughput (Mrays/s) on the built tree;
  cpu_baseline  the oracle's restatement of the reference LBVH build on the
             same 16 Mi triangles, run data-parallel on every host core.

--impl reference times the reference's algorithm on the host CPU instead, on
the same workload and metric (the reference's own code is OpenCL and cannot
run here; its restatement in oracle/ runs stage by stage on all host cores, as
the reference's kernels would on a CPU OpenCL device).

Multi-GPU: the build does not shard; --gpus N runs N independent replicas
(one process per GPU, started through torchrun by this script itself when no
launcher started it), value = total triangles / max time.  With more than one
process the terrain render is also split into row bands, one per GPU, and
gathered on rank 0 (render_bands).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_TRIS = 1 << 24
N_RAYS = 1 << 24
BITS = 10
METRIC = "LBVH build ms per 1M triangles"
UNIT = "ms/Mtri"
WORKLOAD = "lbvh-build+traversal, 16Mi random triangles (30-bit Morton), 16Mi closest + 16Mi shadow rays"

# Algorithmic bytes per unit (triangle, or internal node ~ triangle) of each
# build kernel: the bytes the algorithm must read and write, counted once.
ALGO_BYTES = {
    "scene_box": 36.0,          # read 9 floats per triangle
    "morton": 40.0,             # read 9 floats; write a 4-byte key
    "sort_pass_first": 12.0,    # read key, write key + index
    "sort_pass": 16.0,          # read key + index, write key + index
    # per triangle: sorted index 4, its key 4, its 3 vertices 36, its 48-byte record,
    # and one 64-byte internal node (n - 1 of them); child slots of nodes inside
    # a block live in shared memory
    "build_tree": 156.0,
}
# Bytes the kernels of this design move beyond the algorithmic ones: the Morton
# pass also writes each triangle's 48-byte staging record (read back in sorted
# order by the tree pass instead of three 12-byte vertex gathers) and its
# 4-byte arrival counter.
DESIGN_BYTES = {"morton": 92.0}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--tris", type=int, default=N_TRIS)
    ap.add_argument("--rays", type=int, default=N_RAYS)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--render", type=int, default=1, help="also time the path tracer (0 = skip)")
    ap.add_argument("--render-only", action="store_true", help="time only the path tracer (for profiling)")
    ap.add_argument("--adjoint-only", action="store_true", help="time only the adjoint renderer (for profiling)")
    ap.add_argument("--batched-only", action="store_true", help="time only the batched form (for profiling)")
    ap.add_argument("--terrain-only", action="store_true",
                    help="time only the wavefront (ordered) render of the terrain scene (for profiling)")
    ap.add_argument("--terrain-spp", type=int, default=64)
    ap.add_argument("--loader-only", action="store_true",
                    help="time only the .obj loader on a generated 1 M-triangle mesh (host code)")
    ap.add_argument("--batched-scenes", type=int, default=512)
    ap.add_argument("--batched-graph", type=int, default=1,
                    help="0: launch the batched frame loop kernel by kernel (profiling)")
    ap.add_argument("--adjoint-res", type=int, default=512)
    ap.add_argument("--adjoint-spp", type=int, default=32)
    ap.add_argument("--band-spp", type=int, default=16,
                    help="samples per pixel of the row-band terrain render (more than one process)")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class ClockSampler:
    """nvidia-smi clock / throttle sampling while the timed loops run."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as fh:
            for line in fh:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        top = max(sm)
        loaded = [s for s in sm if s >= 0.5 * top] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(kernel: str):
    """DRAM bytes per launch of `kernel` from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as fh:
        d = json.load(fh)
    v = d.get(kernel)
    return None if v is None else float(v["bytes_per_launch"])


def host_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_build_ms(vx, vy, vz, n: int, steps: int, warmup: int, threads: int) -> list[float]:
    """Milliseconds per build of the n triangles by the restatement of the
    reference's LBVH construction run data-parallel on `threads` host threads
    (oracle/lbvh_oracle.c, orc_lbvh_build_mt; the C code releases the
    interpreter lock)."""
    import oracle

    out = []
    for i in range(warmup + steps):
        t0 = time.perf_counter()
        oracle.lbvh_build_mt(vx, vy, vz, None, n, BITS, threads)
        if i >= warmup:
            out.append(1e3 * (time.perf_counter() - t0))
    return out


def cpu_trace_mrays(vx, vy, vz, n: int, rays, threads: int) -> float:
    """Closest-hit rays per second of the restated reference traversal
    (orc_trace_closest, reference order) over the CPU-built tree, the rays
    split into one chunk per host thread."""
    import oracle
    from concurrent.futures import ThreadPoolExecutor

    ob = oracle.lbvh_build_mt(vx, vy, vz, None, n, BITS, threads)
    chunks = np.array_split(rays, threads)
    with ThreadPoolExecutor(max_workers=threads) as ex:
        t0 = time.perf_counter()
        list(ex.map(lambda c: oracle.trace_closest(vx, vy, vz, None, ob, c), chunks))
        dt = time.perf_counter() - t0
    return rays.shape[0] / dt / 1e6


CPU_NOTE = ("the reference's LBVH construction (OpenCL/lbvh_construction.cl driven as LBVHBuilder.cpp:160-375) "
            "restated in C and run stage by stage on all host cores, as its kernels would run on a CPU OpenCL "
            "device; the reference's own kernels and CPU code cannot run on this host (no OpenCL driver; its "
            "sources are not on the GPU host and x86 builds of them do not run on its aarch64 cores)")


def cpu_baseline(n: int, budget_s: float = 20.0) -> dict:
    """The CPU build of the same 16 Mi-triangle workload on every host core,
    a few builds within `budget_s`."""
    from clear_gb300 import workloads as W

    threads = host_threads()
    vx, vy, vz = W.triangle_soup(n, seed=1)
    first = cpu_build_ms(vx, vy, vz, n, 1, 0, threads)[0]
    reps = max(1, min(5, int(budget_s * 1e3 / max(first, 1.0))))
    ms = statistics.median(cpu_build_ms(vx, vy, vz, n, reps, 0, threads))
    return {"value": ms / (n / 1e6), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{reps} builds of the full {n}-triangle workload (median), {CPU_NOTE}"}


def gpu_time_us(fn, stream, reps: int = 20) -> float:
    """Device time of one call of `fn` (a short kernel launch): the stream is
    first held by a GPU-side sleep while the host enqueues `reps` calls, so
    the CUDA events around them measure the kernels back to back, not the
    host's launch overhead."""
    import torch

    fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda._sleep(40_000_000)  # ~20 ms of device time to queue behind
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return 1e3 * e0.elapsed_time(e1) / reps


def path_traffic(ds, spp: int, max_depth: int, msamples_s: float, peak: float) -> dict:
    """Bytes a path sample moves, from the counted megakernel (the same
    paths as the timed wavefront): per node loaded 64 B (both child boxes),
    per triangle tested 48 B (its record), per ray 32 B in + 8 B out, per
    shaded hit 64 B of face and vertex data, per sample 16 B of accumulation;
    applied to `msamples_s` against the HBM peak.  Most of it is served by
    L1/L2, so the fraction measures demand, not DRAM traffic."""
    rng, pix = ds.new_frame()
    c = ds.render_counted(rng, pix, spp, max_depth=max_depth, ordered=True)
    n = c["samples"]
    b = (64 * c["nodes"] + 48 * c["tris"] + 40 * (c["rays"] + c["shadow_rays"]) + 64 * c["hits"] + 16 * n) / n
    gbs = b * msamples_s * 1e6 / 1e9
    return {"per_sample": {k: c[k] / n for k in ("rays", "shadow_rays", "nodes", "tris", "hits")},
            "counted_spp": spp, "bytes_per_sample": b, "gbs_at_wavefront_ordered": gbs, "frac_of_hbm": gbs / peak}


def bench_loader(reps: int = 3) -> dict:
    """The .obj loader on a generated 1 M-triangle heightfield (93 MB, v/t/n
    faces): the native parse alone and load_model (parse + scene encoding),
    best of `reps`, with the host threads it used."""
    from clear_gb300 import model_loader
    from clear_gb300 import scene as S
    from clear_gb300 import workloads as W
    from clear_gb300.build import build

    build()
    with tempfile.TemporaryDirectory() as d:
        path = W.write_grid_obj(d)
        size = os.path.getsize(path)
        parse_s, load_s = [], []
        for _ in range(reps):
            t0 = time.perf_counter()
            model_loader.parse_obj(path)
            parse_s.append(time.perf_counter() - t0)
            sc = S.Scene()
            t0 = time.perf_counter()
            model_loader.load_model(path, sc)
            load_s.append(time.perf_counter() - t0)
        faces = len(sc.faces)
    return {"file_mb": size / 1e6, "triangles": faces, "parse_s": min(parse_s), "parse_mb_s": size / 1e6 / min(parse_s),
            "load_model_s": min(load_s), "mtri_s": faces / 1e6 / min(load_s), "host_threads": host_threads()}


def bench_render(dev, args) -> dict:
    """Path tracing throughput on the procedural Cornell box (996 triangles,
    coat-over-diffuse sphere, quad light): 256 x 256 pixels, 16 samples per
    pixel, depth 5, pinhole camera -- Msamples/s for the exact-order and the
    nearer-child-first traversal."""
    import torch

    from clear_gb300 import scenes
    from clear_gb300.render import DeviceScene

    w = h = 256
    spp = 16
    ds = DeviceScene(scenes.cornell_box(w, h), dev)
    out = {"workload": "cornell box 996 tris, 256x256, 16 spp, depth 5", "samples": w * h * spp}
    stream = torch.cuda.current_stream(dev)
    for name, ordered, wf in (("exact", False, False), ("ordered", True, False), ("wavefront_exact", False, True),
                              ("wavefront_ordered", True, True)):
        rng, pix = ds.new_frame()
        ds.render(rng, pix, 2, max_depth=5, ordered=ordered, wavefront=wf)  # warm-up
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = 3
        e0.record(stream)
        for _ in range(reps):
            ds.render(rng, pix, spp, max_depth=5, ordered=ordered, wavefront=wf)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        out[f"{name}_ms"] = ms
        out[f"{name}_msamples_s"] = w * h * spp / ms / 1e3
    out["traffic"] = path_traffic(ds, spp, 5, out["wavefront_ordered_msamples_s"], measured_peaks()[0])
    return out


def bench_render_terrain(dev, spp=64, forms=("megakernel_ordered", "wavefront_exact", "wavefront_ordered")) -> dict:
    """Wavefront vs megakernel on the large scene: 2.23 M triangles
    (1024^2 heightfield + 256 spheres), 1024 x 512 sky, 8 bump-mapped
    materials, thin lens 0.02 / 1.5, 1920 x 1080, depth 8; `spp` samples per
    pixel per timed render."""
    import torch

    from clear_gb300 import scenes
    from clear_gb300.render import DeviceScene

    sc = scenes.terrain_scene()
    ds = DeviceScene(sc, dev)
    w, h = sc.width, sc.height
    out = {"workload": f"terrain 2.23M tris, 1920x1080, {spp} spp, depth 8, thin lens", "spp": spp,
           "samples": w * h * spp}
    stream = torch.cuda.current_stream(dev)
    for name, ordered, wf in (("megakernel_ordered", True, False), ("wavefront_exact", False, True),
                              ("wavefront_ordered", True, True)):
        if name not in forms:
            continue
        rng, pix = ds.new_frame()
        ds.render(rng, pix, 1, max_depth=8, ordered=ordered, wavefront=wf)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ds.render(rng, pix, spp, max_depth=8, ordered=ordered, wavefront=wf)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        out[f"{name}_ms"] = ms
        out[f"{name}_msamples_s"] = w * h * spp / ms / 1e3
    if "wavefront_ordered_msamples_s" in out:
        out["traffic"] = path_traffic(ds, 2, 8, out["wavefront_ordered_msamples_s"], measured_peaks()[0])
    # the steps either side of the path on the same scene: the 8-bit tone map
    # of the image (16 B read + 3 B written per pixel) and the rebuild of the
    # sky's importance distribution (8 B read + 8 B written per texel)
    from clear_gb300 import postprocess as PP

    peak, _ = measured_peaks()
    tm_us = gpu_time_us(lambda: PP.to_ldr(pix, w, h, spp), stream)
    env_us = gpu_time_us(ds.update_env_distribution, stream)
    ew, eh = ds.env_dist["width"], ds.env_dist["height"]
    out["tonemap"] = {"us": tm_us, "gbs": 19 * w * h / tm_us / 1e3, "frac_of_hbm": 19 * w * h / tm_us / 1e3 / peak}
    out["env_distribution"] = {"texels": ew * eh, "us": env_us, "gbs": 16 * ew * eh / env_us / 1e3,
                               "frac_of_hbm": 16 * ew * eh / env_us / 1e3 / peak}
    return out


def bench_render_bands(dev, spp: int) -> dict:
    """The terrain image split into row bands, one per process (each GPU
    renders its band with the wavefront form, clr_render_wavefront_rows), and
    gathered on rank 0; the timed region holds the renders and the gather.
    Whole-job Msamples/s over all processes."""
    import torch

    from clear_gb300 import scenes, shard
    from clear_gb300.render import DeviceScene

    sc = scenes.terrain_scene()
    ds = DeviceScene(sc, dev)
    w, h = sc.width, sc.height
    rng_all, _ = ds.new_frame()

    def render_band(y0, y1):
        rng = rng_all.view(h * w, 4)[y0 * w:y1 * w].clone()
        pix = torch.zeros(((y1 - y0) * w, 4), dtype=torch.float32, device=dev)
        ds.render(rng, pix, spp, max_depth=8, ordered=True, rows=(y0, y1))
        return pix

    shard.timed_band_render(render_band, h, w, steps=1)  # warm-up
    dt, img = shard.timed_band_render(render_band, h, w, steps=1)
    return {"workload": f"terrain 2.23M tris, 1920x1080, {spp} spp, depth 8, row bands + gather to rank 0",
            "samples": w * h * spp, "s_per_frame": dt, "msamples_s": w * h * spp / dt / 1e6,
            "gathered_pixels": None if img is None else int(img.shape[0])}


def bench_adjoint(dev, spp=32, res=512) -> dict:
    """Differentiable render: the 8-material Cornell box with a 64 x 32
    environment, 512 x 512, `spp` samples per pixel, depth 5.  Times the
    forward wavefront render and the adjoint pass (path replay; gradients of
    an L2 image loss against a target rendered with perturbed parameters for
    8 RGB albedos, 8 roughness values and 2048 x 3 environment texels), both
    with nearer-child-first traversal."""
    import numpy as np
    import torch

    from clear_gb300 import scenes
    from clear_gb300.render import DeviceScene

    w = h = res
    sc, info = scenes.cornell_adjoint(w, h)
    ds = DeviceScene(sc, dev)
    r = np.random.default_rng(11)
    alb = np.clip(info["albedo"] + r.normal(0, 0.1, info["albedo"].shape), 0.01, 0.99)
    rough = info["roughness"].copy()
    rough[:7] = np.maximum(rough[:7] + r.normal(0, 0.05, 7), 0.02)
    env = info["env"] * np.exp(r.normal(0, 0.3, info["env"].shape))
    tsc, _ = scenes.cornell_adjoint(w, h, albedo=alb, roughness=rough, env=env)
    tds = DeviceScene(tsc, dev)
    rng, target = tds.new_frame()
    tds.render(rng, target, spp, max_depth=5, wavefront=True)
    tex = torch.tensor(info["albedo_tex"] + info["rough_tex"], dtype=torch.int32, device=dev)
    kind = torch.tensor([0] * 8 + [1] * 8, dtype=torch.uint8, device=dev)
    grad = torch.zeros((16, 4), dtype=torch.float32, device=dev)
    genv = torch.zeros((info["env"].shape[0] * info["env"].shape[1], 4), dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    seeds, pix = ds.new_frame()
    ds.render(seeds.clone(), pix, 2, max_depth=5, wavefront=True)  # warm-up
    ds.render_adjoint(seeds.clone(), torch.zeros_like(pix), 2, 5, tex, kind, grad, info["env_tex"], genv)
    torch.cuda.synchronize()
    pix.zero_()
    reps = 2
    ev[0].record(stream)
    for _ in range(reps):
        pix.zero_()
        ds.render(seeds.clone(), pix, spp, max_depth=5, wavefront=True)
    ev[1].record(stream)
    dloss = torch.zeros_like(pix)
    dloss[:, :3] = 2.0 * (pix[:, :3] - target[:, :3]) / (spp * spp)
    grad.zero_()
    genv.zero_()
    ev[2].record(stream)
    for _ in range(reps):
        ds.render_adjoint(seeds.clone(), dloss, spp, 5, tex, kind, grad, info["env_tex"], genv)
    ev[3].record(stream)
    torch.cuda.synchronize()
    fwd = ev[0].elapsed_time(ev[1]) / reps
    adj = ev[2].elapsed_time(ev[3]) / reps
    # The same adjoint with every replayed ray traced again (no hit records
    # carried from the primal pass).
    g2, ge2 = torch.zeros_like(grad), torch.zeros_like(genv)
    ev[0].record(stream)
    for _ in range(reps):
        ds.render_adjoint(seeds.clone(), dloss, spp, 5, tex, kind, g2, info["env_tex"], ge2, retrace=True)
    ev[1].record(stream)
    torch.cuda.synchronize()
    adj_rt = ev[0].elapsed_time(ev[1]) / reps
    return {"workload": f"adjoint cornell 8 materials + 64x32 env, {w}x{h}, {spp} spp, depth 5",
            "params": 16 * 3 + genv.shape[0] * 3, "forward_ms": fwd, "adjoint_ms": adj,
            "adjoint_over_forward": adj / fwd, "adjoint_retrace_ms": adj_rt,
            "adjoint_retrace_over_forward": adj_rt / fwd,
            "retrace_grad_rel_diff": float((torch.linalg.norm(g2 - grad) / torch.linalg.norm(grad)).item()),
            "forward_msamples_s": w * h * spp / fwd / 1e3,
            "adjoint_msamples_s": w * h * spp / adj / 1e3,
            "grad_norm": float(torch.linalg.norm(grad).item()), "env_grad_norm": float(torch.linalg.norm(genv).item())}


def bench_batched(dev, num_scenes=512, spp=8, depth=5, graph=True) -> dict:
    """Many scenes per launch: `num_scenes` scenes with log-uniform 1k-200k
    random triangles plus a quad light, square resolutions from {128, 256,
    384, 512}, `spp` samples, depth `depth`.  Batched form: one segmented LBVH
    build and one CUDA-graph wavefront over all scenes, configured by the
    autotuner.  Plain form: a standalone build and a wavefront render per
    scene.  Both produce bit-identical images (compared here)."""
    import time as _t

    import torch

    from clear_gb300 import autotune
    from clear_gb300.batch import BatchRenderer, PerSceneLoop, batch_workload, random_scene

    t0 = _t.perf_counter()
    wl = batch_workload(num_scenes)
    scenes = [random_scene(n, w, h, seed) for n, w, h, seed in wl]
    gen_s = _t.perf_counter() - t0
    total_tris = sum(w[0] + 2 for w in wl)
    stream = torch.cuda.current_stream(dev)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(8)]

    br = BatchRenderer(scenes, dev)
    tuned = autotune.tune(br, depth, use_cache=False, graph=graph)
    seeds, pix = br.new_frame()
    # warm-up (also captures the graph for this spp)
    rng = seeds.clone()
    br.render(rng, pix, spp, depth, graph=graph)
    torch.cuda.synchronize()
    pix.zero_()
    rng.copy_(seeds)
    ev[0].record(stream)
    br.rebuild_into_current()
    ev[1].record(stream)
    br.render(rng, pix, spp, depth, graph=graph)
    ev[2].record(stream)
    torch.cuda.synchronize()
    b_build, b_render = ev[0].elapsed_time(ev[1]), ev[1].elapsed_time(ev[2])
    batched_img = pix[:, :3].clone()
    del pix, rng
    br.close()
    del br
    torch.cuda.empty_cache()

    loop = PerSceneLoop(scenes, dev)
    rngs0, pixs = loop.new_frame()
    rngs = [r.clone() for r in rngs0]
    loop.render(rngs, pixs, 1, depth)  # warm-up (allocates the workspaces)
    torch.cuda.synchronize()
    for p_ in pixs:
        p_.zero_()
    for r, r0 in zip(rngs, rngs0):
        r.copy_(r0)
    torch.cuda.synchronize()
    ev[3].record(stream)
    loop.build_all()
    ev[4].record(stream)
    loop.render(rngs, pixs, spp, depth)
    ev[5].record(stream)
    torch.cuda.synchronize()
    l_build, l_render = ev[3].elapsed_time(ev[4]), ev[4].elapsed_time(ev[5])
    loop_img = torch.cat([p_[:, :3] for p_ in pixs])
    diff = float((loop_img - batched_img).abs().max().item())
    samples = int(loop_img.shape[0]) * spp
    return {"workload": f"{num_scenes} scenes, {total_tris} triangles, {loop_img.shape[0]} pixels, {spp} spp, "
                        f"depth {depth}", "host_scene_generation_s": gen_s,
            "batched": {"build_ms": b_build, "render_ms": b_render,
                        "msamples_s": samples / b_render / 1e3,
                        "build_plus_render_msamples_s": samples / (b_build + b_render) / 1e3,
                        "config": tuned["config"], "radix_bits": tuned["radix_bits"]},
            "per_scene_loop": {"build_ms": l_build, "render_ms": l_render, "msamples_s": samples / l_render / 1e3,
                               "build_plus_render_msamples_s": samples / (l_build + l_render) / 1e3},
            "speedup_render": l_render / b_render, "speedup_build_plus_render": (l_build + l_render) /
            (b_build + b_render), "max_abs_image_diff": diff,
            "autotune_trials": len(tuned["render_trials"]), "autotune_build_ms": tuned["build_ms"]}


def run_reference(args):
    """The reference's build on the host CPU, on this arm's workload: the same
    16 Mi random triangles (seed 1) and 10 bits per axis, one build per step on
    every host core.  For information it also times the restated reference
    traversal on a ray sample and the reference's own CPU builder (the
    midpoint-split BVH of BVH.hpp, single-threaded as the reference runs it)
    restated, on a 1 Mi sample."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import oracle
    from clear_gb300 import workloads as W

    n = args.tris
    threads = host_threads()
    vx, vy, vz = W.triangle_soup(n, seed=1)
    oracle.lbvh_build(vx[:9], vy[:9], vz[:9], None, 3, BITS)  # loads (and if needed builds) the C library
    ms = cpu_build_ms(vx, vy, vz, n, args.steps, args.warmup, threads)
    ms_step = statistics.mean(ms)
    value = ms_step / (n / 1e6)
    rays = W.closest_rays(1 << 18, seed=11)
    mrays = cpu_trace_mrays(vx, vy, vz, n, rays, threads)
    m = 1 << 20
    t0 = time.perf_counter()
    oracle.midbvh_build(vx[:3 * m], vy[:3 * m], vz[:3 * m], None, m)
    mid_ms = 1e3 * (time.perf_counter() - t0)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "tris_per_gpu": n, "bits_per_dim": BITS, "host_threads": threads,
                   "same_config": True, "note": CPU_NOTE},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"one build of the full {n}-triangle workload per step on {threads} threads"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "traversal": {"closest_mrays_s": mrays, "rays": int(rays.shape[0]), "threads": threads,
                      "form": "restated reference order (bvh_traversal.cl:182-215) over the CPU-built tree"},
        "midpoint_bvh_build": {"ms_per_mtri": mid_ms / (m / 1e6), "tris": m, "threads": 1,
                               "form": "restated BVH::build (BVH.hpp:140-175), the reference's CPU builder"},
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    import torch.distributed as dist

    from clear_gb300 import _lib, lbvh, shard
    from clear_gb300 import workloads as W
    from clear_gb300.build import build

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        dist.init_process_group("nccl", device_id=dev)
    if rank == 0:
        build()
    if world > 1:
        dist.barrier()
    else:
        build()

    def barrier():
        if world > 1:
            dist.barrier()

    n = args.tris
    vx, vy, vz = W.triangle_soup(n, seed=1 + rank)
    host = [torch.from_numpy(a).pin_memory() for a in (vx, vy, vz)]
    verts = [h.to(dev) for h in host]
    builder = lbvh.LBVHBuilder(n, dev)
    bvh = lbvh.BVH(n, dev)
    stream = torch.cuda.current_stream(dev)

    clocks = ClockSampler(local)
    clocks.start()
    for _ in range(args.warmup):
        builder.perform(verts, None, n, BITS, out=bvh)
    torch.cuda.synchronize()

    # ---- headline: K builds, device-resident inputs
    barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        builder.perform(verts, None, n, BITS, out=bvh)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    ms_step = e0.elapsed_time(e1) / args.steps

    # ---- per-kernel durations (CUDA events around each launch) over K builds
    builder.set_profiling(True)
    per = {}
    for _ in range(args.steps):
        builder.perform(verts, None, n, BITS, out=bvh)
        for i, (name, ms) in enumerate(builder.pass_times()):
            key = "sort_pass_first" if name == "sort_pass" and i == 2 else name
            per.setdefault(key, []).append(ms)
    builder.set_profiling(False)
    kern_ms = {k: statistics.mean(v) for k, v in per.items()}
    # kernels per build: one per timed pass, two for the tree pass (k_build_tree
    # and k_build_tree_top)
    launches_per_build = sum(len(v) * (2 if k == "build_tree" else 1) for k, v in per.items()) // args.steps

    # ---- e2e through the C ABI from pinned host memory: every step uploads
    # its vertices (clr_lbvh_build_host) and reads the root record back; a
    # step's upload overlaps the previous step's build
    root_host = torch.empty(8, dtype=torch.float32).pin_memory()
    # the same steps with the upload and the build back to back on one stream
    torch.cuda.synchronize()
    barrier()
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s0.record(stream)
    for _ in range(args.steps):
        for d, h in zip(verts, host):
            d.copy_(h, non_blocking=True)
        builder.perform(verts, None, n, BITS, out=bvh)
        root_host.copy_(bvh.root_box, non_blocking=True)
    s1.record(stream)
    torch.cuda.synchronize()
    e2e_serial_ms = s0.elapsed_time(s1) / args.steps
    for _ in range(2):
        builder.perform_host(host, None, n, BITS, out=bvh, root_host=root_host)
    torch.cuda.synchronize()
    barrier()
    e2, e3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e2.record(stream)
    builder.host_copy_after_stream()  # no upload starts before the timed region opens
    for _ in range(args.steps):
        builder.perform_host(host, None, n, BITS, out=bvh, root_host=root_host)
    e3.record(stream)
    torch.cuda.synchronize()
    barrier()
    e2e_ms = e2.elapsed_time(e3) / args.steps

    # ---- the same build at the other sizes of the microbenchmark (1 Mi, 4 Mi)
    sizes = {}
    for ns in (1 << 20, 1 << 22):
        sx, sy, sz = W.triangle_soup(ns, seed=1 + rank)
        sv = [torch.from_numpy(a).to(dev) for a in (sx, sy, sz)]
        sb = lbvh.LBVHBuilder(ns, dev)
        sbvh = lbvh.BVH(ns, dev)
        for _ in range(3):
            sb.perform(sv, None, ns, BITS, out=sbvh)
        torch.cuda.synchronize()
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record(stream)
        for _ in range(args.steps):
            sb.perform(sv, None, ns, BITS, out=sbvh)
        a1.record(stream)
        torch.cuda.synchronize()
        sms = a0.elapsed_time(a1) / args.steps
        sb.set_profiling(True)
        sb.perform(sv, None, ns, BITS, out=sbvh)
        sizes[str(ns)] = {"ms_per_build": sms, "ms_per_mtri": sms / (ns / 1e6),
                          "kernels_ms": {f"{i}:{k}": v for i, (k, v) in enumerate(sb.pass_times())}}
        sb.close()
        del sv, sbvh

    # ---- traversal throughput on the built tree
    m = args.rays
    crays = torch.from_numpy(W.closest_rays(m, seed=11 + rank)).to(dev)
    srays = torch.from_numpy(W.shadow_rays(m, seed=12 + rank)).to(dev)
    hid = torch.empty(m, dtype=torch.int32, device=dev)
    ht = torch.empty(m, dtype=torch.float32, device=dev)
    occ = torch.empty(m, dtype=torch.uint8, device=dev)
    trav_steps = max(3, args.steps // 4)
    for _ in range(2):
        lbvh.trace_closest(bvh, crays, hid, ht, ordered=False)
        lbvh.trace_shadow(bvh, srays, occ)
    torch.cuda.synchronize()
    hid2 = torch.empty(m, dtype=torch.int32, device=dev)
    ht2 = torch.empty(m, dtype=torch.float32, device=dev)
    lbvh.trace_replays(clear=True)
    lbvh.trace_closest(bvh, crays, hid2, ht2, ordered=True)
    replayed = lbvh.trace_replays(clear=True)
    t0, t1, t2, t3 = (torch.cuda.Event(enable_timing=True) for _ in range(4))
    t0.record(stream)
    for _ in range(trav_steps):
        lbvh.trace_closest(bvh, crays, hid, ht, ordered=False)
    t1.record(stream)
    for _ in range(trav_steps):
        lbvh.trace_shadow(bvh, srays, occ)
    t2.record(stream)
    for _ in range(trav_steps):
        lbvh.trace_closest(bvh, crays, hid2, ht2, ordered=True)
    t3.record(stream)
    # the same searches with the rays sorted by origin first (the sort inside
    # the timed region)
    hid3 = torch.empty(m, dtype=torch.int32, device=dev)
    ht3 = torch.empty(m, dtype=torch.float32, device=dev)
    occ3 = torch.empty(m, dtype=torch.uint8, device=dev)
    lbvh.trace_closest(bvh, crays, hid3, ht3, sort=True)
    lbvh.trace_shadow(bvh, srays, occ3, sort=True)
    t4, t5, t6 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    t4.record(stream)
    for _ in range(trav_steps):
        lbvh.trace_closest(bvh, crays, hid3, ht3, sort=True)
    t5.record(stream)
    for _ in range(trav_steps):
        lbvh.trace_shadow(bvh, srays, occ3, sort=True)
    t6.record(stream)
    torch.cuda.synchronize()
    lbvh.trace_replays(clear=True)
    refo_ms = t0.elapsed_time(t1) / trav_steps
    shadow_ms = t1.elapsed_time(t2) / trav_steps
    closest_ms = t2.elapsed_time(t3) / trav_steps
    closest_sorted_ms = t4.elapsed_time(t5) / trav_steps
    shadow_sorted_ms = t5.elapsed_time(t6) / trav_steps
    sorted_mismatches = int((hid3 != hid2).sum().item() + (ht3.view(torch.int32) != ht2.view(torch.int32)).sum().item()
                            + (occ3 != occ).sum().item())
    del hid3, ht3, occ3
    # visiting statistics of the reference-order query: the bytes that search
    # gathers per ray, 64 per node loaded and 48 per triangle tested, plus the
    # 32-byte ray and its 8-byte result
    _, cnt = lbvh.trace_closest_counted(bvh, crays)
    nodes_per_ray = float(cnt[:, 0].double().mean().item())
    tris_per_ray = float(cnt[:, 1].double().mean().item())
    del cnt
    fetch_bytes = m * (32 + 8 + 64 * nodes_per_ray + 48 * tris_per_ray)
    ordered_id_mismatch = int((hid != hid2).sum().item())
    ordered_t_mismatch = int((ht != ht2).sum().item())
    render = bench_render(dev, args) if args.render else None
    render_terrain = bench_render_terrain(dev) if args.render else None
    adjoint = bench_adjoint(dev) if args.render else None
    batched = bench_batched(dev, args.batched_scenes) if args.render else None
    bands = bench_render_bands(dev, args.band_spp) if args.render and world > 1 else None
    hit_frac = float((hid >= 0).float().mean().item())
    occ_frac = float(occ.float().mean().item())
    clk = clocks.stop()
    dev_err = _lib.device_status()

    # ---- max over ranks
    ms_step, e2e_ms, e2e_serial_ms, closest_ms, shadow_ms, closest_sorted_ms, shadow_sorted_ms = shard.max_over_ranks(
        [ms_step, e2e_ms, e2e_serial_ms, closest_ms, shadow_ms, closest_sorted_ms, shadow_sorted_ms], dev)
    if rank != 0:
        dist.destroy_process_group()
        return

    mtris_total = world * n / 1e6
    value = ms_step / mtris_total
    peak, peak_kind = measured_peaks()
    dom = max(kern_ms, key=kern_ms.get)
    dom_ms = kern_ms[dom]
    achieved = ALGO_BYTES.get(dom, 0.0) * n / (dom_ms * 1e-3) / 1e9
    traffic = ncu_traffic(dom)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "tris_per_gpu": n, "rays_per_gpu": m, "bits_per_dim": BITS,
                   "parallelism": f"replicas x{world}", "l2": "inputs (576 MB) larger than L2, no flush"},
        "e2e": {"value": e2e_ms / mtris_total, "unit": UNIT, "h2d_bytes_per_step": 3 * 4 * 3 * n,
                "d2h_bytes_per_step": 32, "ms_per_step": e2e_ms,
                "path": "clr_lbvh_build_host per step (upload of step k+1 overlaps the build of step k)",
                "serial_value": e2e_serial_ms / mtris_total, "serial_ms_per_step": e2e_serial_ms,
                "h2d_gbs": 3 * 4 * 3 * n / e2e_ms / 1e6},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                     "peak_source": f"{peak_kind} hbm_gbs", "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "algo_bytes_per_tri": ALGO_BYTES.get(dom),
                     "kernel_ms": dom_ms},
        "build_kernels_ms": kern_ms,
        "build_other_sizes": sizes,
        # every build pass against the same measured copy bandwidth
        "build_kernels_roofline": {k: {"gbs": ALGO_BYTES[k] * n / (v * 1e-3) / 1e9,
                                       "frac": ALGO_BYTES[k] * n / (v * 1e-3) / 1e9 / peak}
                                   for k, v in kern_ms.items() if k in ALGO_BYTES},
        "build_kernels_design_bytes": {k: {"bytes_per_tri": b, "gbs": b * n / (kern_ms[k] * 1e-3) / 1e9,
                                           "frac": b * n / (kern_ms[k] * 1e-3) / 1e9 / peak}
                                       for k, b in DESIGN_BYTES.items() if k in kern_ms},
        "traversal": {"closest_mrays_s": m / closest_ms / 1e3, "shadow_mrays_s": m / shadow_ms / 1e3,
                      "closest_form": "nearer-first with replay of order-dependent rays (bit-exact)",
                      "closest_replayed_frac": replayed / m,
                      "closest_reference_order_mrays_s": m / refo_ms / 1e3,
                      "fast_vs_reference_order_id_mismatches": ordered_id_mismatch,
                      "fast_vs_reference_order_t_mismatches": ordered_t_mismatch,
                      "closest_ms": closest_ms, "closest_reference_order_ms": refo_ms, "shadow_ms": shadow_ms,
                      "closest_sorted_mrays_s": m / closest_sorted_ms / 1e3,
                      "shadow_sorted_mrays_s": m / shadow_sorted_ms / 1e3,
                      "sorted_form": "rays sorted by the Morton code of their origin first (sort timed); "
                                     "the same answers as the given order",
                      "sorted_vs_given_order_mismatches": sorted_mismatches,
                      "closest_hit_frac": hit_frac,
                      "reference_order_nodes_per_ray": nodes_per_ray, "reference_order_tris_per_ray": tris_per_ray,
                      "reference_order_gather_gbs": fetch_bytes / (refo_ms * 1e-3) / 1e9,
                      "reference_order_gather_frac_of_hbm": fetch_bytes / (refo_ms * 1e-3) / 1e9 / peak,
                      "shadow_occluded_frac": occ_frac},
        "render": render,
        "render_terrain": render_terrain,
        "adjoint": adjoint,
        "batched": batched,
        "render_bands": bands,
        "gpu_launches": launches_per_build * args.steps,
        "clocks": clk,
        "device_error_bits": dev_err,
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(n)
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def main():
    args = parse()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # started without a launcher: one process per GPU of this node
        from clear_gb300 import shard

        sys.exit(shard.launch_local(args.gpus, os.path.abspath(__file__), sys.argv[1:]))
    if args.render_only:
        import torch

        from clear_gb300.build import build

        build()
        dev = torch.device("cuda", 0)
        print(json.dumps({"render": bench_render(dev, args), "render_terrain": bench_render_terrain(dev)}), flush=True)
        return
    if args.loader_only:
        print(json.dumps({"obj_loader": bench_loader()}), flush=True)
        return
    if args.terrain_only:
        import torch

        from clear_gb300.build import build

        build()
        print(json.dumps({"render_terrain": bench_render_terrain(torch.device("cuda", 0), args.terrain_spp,
                                                                 forms=("wavefront_ordered",))}), flush=True)
        return
    if args.batched_only:
        import torch

        from clear_gb300.build import build

        build()
        print(json.dumps({"batched": bench_batched(torch.device("cuda", 0), args.batched_scenes,
                                                   graph=bool(args.batched_graph))}), flush=True)
        return
    if args.adjoint_only:
        import torch

        from clear_gb300.build import build

        build()
        print(json.dumps({"adjoint": bench_adjoint(torch.device("cuda", 0), args.adjoint_spp, args.adjoint_res)}),
              flush=True)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
