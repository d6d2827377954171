"""Host side of the batched form (clear_gb300/batch.py), no GPU: the seeded
512-scene workload (triangle counts log-uniform in [1k, 200k], square
resolutions from the four sizes; about 19 M triangles and 61 M pixels) and
the byte concatenation that packs every scene's blobs at 256-byte offsets."""
import numpy as np

from clear_gb300 import batch


def test_workload_is_seeded_and_has_the_benchmark_shape():
    w = batch.batch_workload()
    assert w == batch.batch_workload()
    assert w != batch.batch_workload(seed=8)
    assert len(w) == 512
    tris = np.array([t for t, _, _, _ in w])
    assert tris.min() >= 1000 and tris.max() <= 200_000
    assert 17e6 < tris.sum() < 21e6
    # log-uniform: the median sits near the geometric mean of the bounds
    assert 0.6 < np.median(tris) / np.sqrt(1000 * 200_000) < 1.6
    assert {wd for _, wd, _, _ in w} <= set(batch.RESOLUTIONS)
    assert all(wd == ht for _, wd, ht, _ in w)
    pixels = sum(wd * ht for _, wd, ht, _ in w)
    assert 55e6 < pixels < 70e6
    assert len({s for _, _, _, s in w}) == 512


def test_concat_aligns_every_array_and_keeps_its_bytes():
    rng = np.random.default_rng(3)
    arrays = [rng.integers(0, 255, size=n, dtype=np.uint8) for n in (1, 255, 256, 257, 1000)]
    arrays.append(np.arange(7, dtype=np.float32))
    buf, offs = batch._concat(arrays)
    assert all(o % 256 == 0 for o in offs)
    for a, o in zip(arrays, offs):
        assert bytes(buf[o:o + a.nbytes]) == a.tobytes()
    assert all(offs[i + 1] - offs[i] >= arrays[i].nbytes for i in range(len(offs) - 1))
    empty, eo = batch._concat([])
    assert eo == [] and empty.size == 256
