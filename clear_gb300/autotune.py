"""Autotuner of the batched form.

Picks, for one batch on one GPU, the path-slot pool size (the queue
capacity), the block sizes of the tracing and shading kernels and the radix
width of the segmented LBVH sort, by timing candidates on the batch itself
(CUDA events, a 1-sample frame per render candidate) in coordinate-descent
order: pool size, then trace block, then shade block; radix width for the
build.  Results are cached in a JSON file keyed by the GPU and the batch's
shape (scenes, pixels, triangles, depth), so a later run of the same
workload skips the search.
"""
from __future__ import annotations

import json
import os
from pathlib import Path

import torch

CACHE_ENV = "CLEAR_GB300_TUNE_CACHE"
POOL_CANDIDATES = (0, 8 << 20, 4 << 20, 2 << 20, 1 << 20)  # 0 = one slot per pixel
TRACE_BLOCKS = (64, 128, 256)
SHADE_BLOCKS = (64, 96, 128)
RADIX_BITS = (6, 7, 8)


def cache_path() -> Path:
    p = os.environ.get(CACHE_ENV)
    return Path(p) if p else Path.home() / ".cache" / "clear_gb300" / "autotune.json"


def signature(br, max_depth: int) -> str:
    name = torch.cuda.get_device_name(br.device)
    return f"{name}|scenes={len(br.scenes)}|pixels={br.total_pixels}|tris={br.offsets[-1]}|depth={max_depth}"


def _events(n):
    return [torch.cuda.Event(enable_timing=True) for _ in range(n)]


def time_render(br, config: dict, max_depth: int, seeds: torch.Tensor, spp: int = 1, graph: bool = True) -> float:
    """ms of one `spp`-sample render of the whole batch with `config` (after a
    warm-up render that also captures the graph); graph=False times the
    frame loop launched kernel by kernel."""
    br.set_config(config)
    pix = torch.zeros((br.total_pixels, 4), dtype=torch.float32, device=br.device)
    rng = seeds.clone()
    br.render(rng, pix, spp, max_depth, graph=graph)
    rng.copy_(seeds)
    e0, e1 = _events(2)
    stream = torch.cuda.current_stream(br.device)
    e0.record(stream)
    br.render(rng, pix, spp, max_depth, graph=graph)
    e1.record(stream)
    torch.cuda.synchronize(br.device)
    return e0.elapsed_time(e1)


def time_build(br, radix_bits: int, reps: int = 3) -> float:
    br.rebuild_into_current(radix_bits)
    e0, e1 = _events(2)
    stream = torch.cuda.current_stream(br.device)
    e0.record(stream)
    for _ in range(reps):
        br.rebuild_into_current(radix_bits)
    e1.record(stream)
    torch.cuda.synchronize(br.device)
    return e0.elapsed_time(e1) / reps


def tune(br, max_depth: int = 5, use_cache: bool = True, graph: bool = True) -> dict:
    """Tunes `br` (a BatchRenderer), applies the best configuration and
    returns it with the trial timings (renders timed as graphs, or kernel by
    kernel with graph=False)."""
    key = signature(br, max_depth)
    path = cache_path()
    cache = {}
    if use_cache and path.exists():
        try:
            cache = json.loads(path.read_text())
        except (OSError, ValueError):
            cache = {}
    if use_cache and key in cache:
        best = cache[key]
        br.set_config(best["config"])
        br.radix_bits = best["radix_bits"]
        return dict(best, cached=True)
    seeds, _ = br.new_frame()
    trials = []
    cfg = {"trace_block": 128, "shade_block": 128, "pool_slots": 0}
    for field, values in (("pool_slots", POOL_CANDIDATES), ("trace_block", TRACE_BLOCKS),
                          ("shade_block", SHADE_BLOCKS)):
        best_v, best_ms = cfg[field], None
        for v in values:
            c = dict(cfg, **{field: v})
            ms = time_render(br, c, max_depth, seeds, graph=graph)
            trials.append({"config": c, "ms": ms})
            if best_ms is None or ms < best_ms:
                best_v, best_ms = v, ms
        cfg[field] = best_v
    br.set_config(cfg)
    build = {r: time_build(br, r) for r in RADIX_BITS}
    radix = min(build, key=build.get)
    br.radix_bits = radix
    br.rebuild_into_current(radix)
    best = {"config": br.config(), "radix_bits": radix, "render_trials": trials,
            "build_ms": {str(k): v for k, v in build.items()}}
    if use_cache:
        cache[key] = best
        try:
            path.parent.mkdir(parents=True, exist_ok=True)
            path.write_text(json.dumps(cache, indent=1))
        except OSError:
            pass
    return dict(best, cached=False)
