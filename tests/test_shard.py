"""Multi-GPU partition of the path (clear_gb300/shard.py): row bands and
scene runs cover the work exactly once; the rank-0 gather of the bands and
the max-over-ranks timing reduction across real processes on the gloo
backend (world sizes 2 and 3, CPU); and, on one GPU, band renders that equal
the whole-image render bit for bit."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from clear_gb300 import shard


def test_row_bands_cover_the_image_once():
    for h in (1, 2, 7, 64, 1080):
        for world in (1, 2, 3, 8):
            b = shard.row_bands(h, world)
            assert len(b) == world and b[0][0] == 0 and b[-1][1] == h
            assert all(b[i][1] == b[i + 1][0] for i in range(world - 1))
            sizes = [y1 - y0 for y0, y1 in b]
            assert max(sizes) - min(sizes) <= 1 and sizes == sorted(sizes, reverse=True)
    with pytest.raises(ValueError):
        shard.row_bands(4, 0)


def test_scene_partition_is_contiguous_and_balanced():
    rng = np.random.default_rng(3)
    for world in (1, 2, 3, 8):
        px = rng.choice([128 ** 2, 256 ** 2, 384 ** 2, 512 ** 2], size=512).tolist()
        runs = shard.scene_partition(px, world)
        assert len(runs) == world and runs[0].start == 0 and runs[-1].stop == len(px)
        assert all(runs[i].stop == runs[i + 1].start for i in range(world - 1))
        ideal = sum(px) / world
        for r in runs:
            assert abs(sum(px[i] for i in r) - ideal) <= max(px)
    assert [len(r) for r in shard.scene_partition([5, 5], 3)] == [1, 1, 0]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, width, height, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bands = shard.row_bands(height, world)
        y0, y1 = bands[rank]
        # this rank's "render": each pixel holds its global index in x and the rank in w
        idx = torch.arange(y0 * width, y1 * width, dtype=torch.float32)
        band = torch.stack([idx, idx * 2, idx * 3, torch.full_like(idx, rank)], dim=1)
        img = shard.gather_rows(band, bands, width)
        slowest = shard.max_over_ranks([float(rank), -float(rank)])
        out.put((rank, None if img is None else img.numpy(), slowest))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world,width,height", [(2, 5, 7), (3, 4, 10), (2, 3, 1)])
def test_gather_rows_and_max_over_gloo_ranks(world, width, height):
    ctx = mp.get_context("spawn")
    out = ctx.SimpleQueue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, width, height, out)) for r in range(world)]
    for p in procs:
        p.start()
    res = {}
    for _ in range(world):
        rank, img, slowest = out.get()
        res[rank] = (img, slowest)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    img = res[0][0]
    idx = np.arange(width * height, dtype=np.float32)
    assert img.shape == (width * height, 4)
    assert np.array_equal(img[:, 0], idx) and np.array_equal(img[:, 2], 3 * idx)
    bands = shard.row_bands(height, world)
    owner = np.concatenate([np.full((y1 - y0) * width, r) for r, (y0, y1) in enumerate(bands)])
    assert np.array_equal(img[:, 3], owner)
    for r in range(1, world):
        assert res[r][0] is None
    for r in range(world):
        assert res[r][1] == [float(world - 1), 0.0]


@pytest.mark.gpu
@pytest.mark.parametrize("world", [2, 3])
def test_band_renders_equal_the_whole_image(cuda, world):
    """Row bands rendered separately (as the ranks of a node would) and put
    together are the whole-image wavefront render, bit for bit, RNG states
    included."""
    from clear_gb300 import _lib, scenes
    from clear_gb300.render import DeviceScene

    w, h, spp = 96, 70, 4
    ds = DeviceScene(scenes.cornell_box(w, h), cuda)
    rng, pix = ds.new_frame()
    rng0 = rng.clone()
    ds.render(rng, pix, spp, max_depth=5, ordered=True, wavefront=True)
    r4 = rng0.view(h * w, 4)
    parts_pix, parts_rng = [], []
    for y0, y1 in shard.row_bands(h, world):
        rb = r4[y0 * w:y1 * w].clone()
        pb = torch.zeros(((y1 - y0) * w, 4), dtype=torch.float32, device=cuda)
        ds.render(rb, pb, spp, max_depth=5, ordered=True, rows=(y0, y1))
        parts_pix.append(pb)
        parts_rng.append(rb)
    torch.cuda.synchronize()
    assert torch.equal(torch.cat(parts_pix), pix)
    assert torch.equal(torch.cat(parts_rng).view(-1), rng.view(-1))
    assert _lib.device_status() == 0


def _band_worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        width, height = 6, 11

        def render_band(y0, y1):  # pixel (x, y) holds y * width + x + 1
            idx = torch.arange(y0 * width, y1 * width, dtype=torch.float32) + 1
            return torch.stack([idx, idx, idx, idx], dim=1)

        dt, img = shard.timed_band_render(render_band, height, width, steps=2)
        out.put((rank, dt, None if img is None else img.numpy()))
    finally:
        dist.destroy_process_group()


def test_timed_band_render_over_gloo_ranks():
    """The band-render timing of the multi-process benchmark: every rank gets
    the same (slowest) time, rank 0 the whole image in row order."""
    world = 2
    ctx = mp.get_context("spawn")
    out = ctx.SimpleQueue()
    port = _free_port()
    procs = [ctx.Process(target=_band_worker, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    res = {}
    for _ in range(world):
        rank, dt, img = out.get()
        res[rank] = (dt, img)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0][0] == res[1][0] and res[0][0] > 0
    assert np.array_equal(res[0][1][:, 0], np.arange(66, dtype=np.float32) + 1)
    assert res[1][1] is None


def test_launch_local_starts_one_process_per_rank(tmp_path):
    """launch_local (what `bench.py --gpus N` uses when no launcher started
    it) runs N processes that see their rank and world size and can form a
    process group (gloo here)."""
    script = tmp_path / "probe.py"
    script.write_text(
        "import os, sys, torch.distributed as dist\n"
        "dist.init_process_group('gloo')\n"
        "r, w = dist.get_rank(), dist.get_world_size()\n"
        "open(os.path.join(sys.argv[1], f'rank{r}'), 'w').write(f'{r} {w} {os.environ[\"LOCAL_RANK\"]}')\n"
        "dist.barrier()\n"
        "dist.destroy_process_group()\n")
    rc = shard.launch_local(2, str(script), [str(tmp_path)], timeout=120)
    assert rc == 0
    assert sorted((tmp_path / f"rank{r}").read_text() for r in range(2)) == ["0 2 0", "1 2 1"]
