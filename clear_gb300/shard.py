"""The path across GPUs: one process per GPU, no exchange inside the path.

The reference renders an image on one OpenCL device, tile by tile
(main.cpp:477-494).  Its work falls into independent units: pixels, each with
its own XORShift128 stream, and the scenes of a batch.  So the GPUs of a node
split the work without any exchange until the end:

* an image is split into contiguous row bands (``row_bands``); each process
  renders its band (``DeviceScene.render(..., rows=band)``), bit-identical to
  the same rows of a whole-image render, and ``gather_rows`` collects the
  bands' accumulation buffers on one rank -- the single collective of the
  path;
* a batch of scenes is split into contiguous runs of about equal pixel count
  (``scene_partition``); each process renders its run as one batch;
* each process builds its own BVH (the build is a small fraction of a
  render).

``max_over_ranks`` is the timing reduction (the slowest rank sets the time);
``timed_band_render`` times one band render per rank plus the gather, with
barriers and device synchronisation around the timed region;
``launch_local`` starts one process per GPU of this node for a script that
was run without a launcher.  Every collective works with any
``torch.distributed`` backend: NCCL between GPUs, gloo on the host.
"""
from __future__ import annotations

import os
import socket
import subprocess
import sys
import time
from typing import Callable

import torch
import torch.distributed as dist


def row_bands(height: int, world: int) -> list[tuple[int, int]]:
    """Contiguous bands [y0, y1) covering [0, height), one per rank, sizes
    differing by at most one row (the first height % world bands are one row
    taller)."""
    if world < 1:
        raise ValueError("world must be at least 1")
    base, extra = divmod(height, world)
    out, y = [], 0
    for r in range(world):
        n = base + (1 if r < extra else 0)
        out.append((y, y + n))
        y += n
    return out


def scene_partition(pixels: list[int], world: int) -> list[range]:
    """Contiguous runs of scenes, one per rank, cut where the running pixel
    count crosses k * total / world (each run's pixel count is within one
    scene of the ideal share)."""
    total = sum(pixels)
    cuts, run, k = [0], 0, 1
    for i, n in enumerate(pixels):
        run += n
        while k < world and run >= k * total / world:
            cuts.append(i + 1)
            k += 1
    while len(cuts) < world:
        cuts.append(len(pixels))
    cuts.append(len(pixels))
    return [range(cuts[r], cuts[r + 1]) for r in range(world)]


def gather_rows(band: torch.Tensor, bands: list[tuple[int, int]], width: int, dst: int = 0,
                group=None) -> torch.Tensor | None:
    """Collects every rank's band (rows x width pixel rows of `band`, any
    trailing shape) on rank `dst`, which receives the whole image in row
    order; other ranks receive None.  One gather of equal-size (padded)
    buffers."""
    rank = dist.get_rank(group)
    world = dist.get_world_size(group)
    if len(bands) != world:
        raise ValueError(f"{len(bands)} bands for {world} ranks")
    rows = [y1 - y0 for y0, y1 in bands]
    per_row = band.shape[1:] if band.dim() > 1 else ()
    pad_rows = max(rows)
    mine = rows[rank]
    if band.shape[0] != mine * width:
        raise ValueError(f"rank {rank}: band of {band.shape[0]} pixels, expected {mine * width}")
    send = torch.zeros((pad_rows * width, *per_row), dtype=band.dtype, device=band.device)
    send[:mine * width] = band
    recv = [torch.empty_like(send) for _ in range(world)] if rank == dst else None
    dist.gather(send, recv, dst=dst, group=group)
    if rank != dst:
        return None
    return torch.cat([recv[r][:rows[r] * width] for r in range(world)])


def max_over_ranks(values: list[float], device: torch.device | str = "cpu", group=None) -> list[float]:
    """Element-wise maximum of `values` over the ranks (all ranks get it)."""
    t = torch.tensor(values, dtype=torch.float64, device=device)
    if dist.is_initialized() and dist.get_world_size(group) > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return t.tolist()


def timed_band_render(render_band: Callable[[int, int], torch.Tensor], height: int, width: int,
                      steps: int = 1, group=None) -> tuple[float, torch.Tensor | None]:
    """Each rank renders its row band `steps` times (render_band(y0, y1)
    returns the band's accumulation buffer, (y1 - y0) * width pixel rows) and
    rank 0 gathers the last one; the timed region -- between barriers, with
    the device synchronised on both sides -- holds the renders and the
    gather.  Returns (seconds per step, the slowest rank's; the whole image on
    rank 0, else None)."""
    world = dist.get_world_size(group) if dist.is_initialized() else 1
    rank = dist.get_rank(group) if dist.is_initialized() else 0
    bands = row_bands(height, world)
    y0, y1 = bands[rank]
    cuda = torch.cuda.is_available()

    def sync():
        if cuda:
            torch.cuda.synchronize()
        if world > 1:
            dist.barrier(group=group)

    sync()
    t0 = time.perf_counter()
    band = None
    for _ in range(steps):
        band = render_band(y0, y1)
    img = gather_rows(band, bands, width, group=group) if world > 1 else band
    sync()
    dt = (time.perf_counter() - t0) / max(steps, 1)
    dev = band.device if band is not None else "cpu"
    return max_over_ranks([dt], dev, group)[0], img


def _free_port() -> int:
    with socket.socket() as s_:
        s_.bind(("127.0.0.1", 0))
        return s_.getsockname()[1]


def launch_local(nprocs: int, script: str, args: list[str], timeout: float | None = None) -> int:
    """Runs `script` with `args` as `nprocs` processes of one node through
    torch.distributed.run (rendezvous on 127.0.0.1, a free port); each
    process reads RANK / LOCAL_RANK / WORLD_SIZE from its environment.
    Returns the launcher's exit status."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={int(nprocs)}",
           "--master-addr=127.0.0.1", f"--master-port={_free_port()}", script, *args]
    env = dict(os.environ)
    env.setdefault("OMP_NUM_THREADS", "1")
    return subprocess.run(cmd, env=env, timeout=timeout).returncode
