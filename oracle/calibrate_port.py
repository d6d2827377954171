"""The reference's own CPU code timed beside the oracle's restatement of it,
on the same inputs and the same host (test infrastructure; needs the
reference checkout, so it runs where oracle/_ref can be built, not on the
GPU host).

The benchmark's CPU baseline is the restatement (the reference's code cannot
run on the GPU host); these ratios say how far that restatement is from the
reference's own code in speed:

* LBVH build: the reference's OpenCL construction kernels run on the CPU by
  the shim of oracle/ref_lbvh_cl.cpp (work-groups as coroutines, one
  thread) against orc_lbvh_build (one thread) and orc_lbvh_build_mt;
* midpoint BVH: BVH::build (OpenCL_PathTracer/BVH.hpp) compiled in place
  against orc_midbvh_build;
* closest-hit traversal: sim::rayIntersection (Equivalent/
  sim_bvh_traversal.hpp, LBVH variant; its face ids are 16-bit, so the scene
  has fewer than 65,536 triangles) against orc_trace_closest;
* path tracing: sim::pathtracing on the path-tracing benchmark's Cornell box
  (256 x 256, 16 samples per pixel, depth 5), one process per host thread
  rendering a band of rows (the renderer keeps its work-item ids in process
  globals), in Msamples/s.

    python oracle/calibrate_port.py
"""
from __future__ import annotations

import json
import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import oracle  # noqa: E402
from clear_gb300 import scenes  # noqa: E402
from clear_gb300 import workloads as W  # noqa: E402


def _best(fn, reps=3) -> float:
    best = float("inf")
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        best = min(best, time.perf_counter() - t0)
    return best


def _band(args):
    y0, y1, w, h, spp, depth = args
    sc = scenes.cornell_box(w, h)
    b = sc.blobs()
    vx, vy, vz, tri = sc.soa()
    ob = oracle.lbvh_build(vx, vy, vz, tri, len(sc.faces), 10)
    rng = scenes.pixel_seeds(w, h)
    pix = np.zeros((w * h, 4), dtype=np.float32)
    t0 = time.perf_counter()
    oracle.ref_render(b, ob.inodes, ob.lnodes, rng, pix, w, h, y0, y1, spp, max_depth=depth)
    return time.perf_counter() - t0


def main() -> None:
    if not oracle.ref_available():
        raise SystemExit("reference checkout not available")
    out = {"host_threads": os.cpu_count()}
    n = 1 << 16
    vx, vy, vz = W.triangle_soup(n, seed=5)
    t_ref = _best(lambda: oracle.ref_cl_lbvh_build(vx, vy, vz, None, n, 10), 1)
    t_port = _best(lambda: oracle.lbvh_build(vx, vy, vz, None, n, 10))
    out["lbvh_build_65536"] = {"reference_kernels_on_cpu_ms": 1e3 * t_ref, "port_1_thread_ms": 1e3 * t_port}
    m = 1 << 20
    vx, vy, vz = W.triangle_soup(m, seed=6)
    tri = np.arange(3 * m, dtype=np.uint32)
    t_ref = _best(lambda: oracle.ref_midbvh_build(vx, vy, vz, tri, m), 1)
    t_port = _best(lambda: oracle.midbvh_build(vx, vy, vz, None, m), 1)
    t_mt = _best(lambda: oracle.lbvh_build_mt(vx, vy, vz, None, m, 10, 0))
    out["build_1Mi"] = {"reference_midpoint_bvh_ms": 1e3 * t_ref, "port_midpoint_bvh_ms": 1e3 * t_port,
                        "port_lbvh_all_threads_ms": 1e3 * t_mt}
    k = 60000
    vx, vy, vz = W.triangle_soup(k, seed=7)
    ob = oracle.lbvh_build(vx, vy, vz, None, k, 10)
    rays = W.closest_rays(100000, seed=8)
    t_ref = _best(lambda: oracle.ref_trace_closest_lbvh(vx, vy, vz, None, k, ob, rays), 1)
    t_port = _best(lambda: oracle.trace_closest(vx, vy, vz, None, ob, rays), 1)
    out["closest_hit_60k_tris_100k_rays"] = {"reference_mrays_s": 0.1 / t_ref, "port_mrays_s": 0.1 / t_port}
    w = h = 256
    spp, depth = 16, 5
    procs = os.cpu_count() or 1
    bands = [(h * i // procs, h * (i + 1) // procs, w, h, spp, depth) for i in range(procs)]
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(procs) as pool:
        pool.map(_band, bands)
    wall = time.perf_counter() - t0
    t1 = _band((0, h // 8, w, h, spp, depth))
    out["pathtracing_cornell_256_16spp_depth5"] = {
        "reference_msamples_s_all_threads": w * h * spp / wall / 1e6, "processes": procs,
        "reference_msamples_s_1_thread": (w * (h // 8) * spp) / t1 / 1e6}
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
