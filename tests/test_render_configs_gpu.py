"""The benchmarked render configurations against the reference's own CPU
renderer at the benchmarks' path-length caps (tests/golden/render_configs.npz,
made by tests/golden/make_golden_configs.py).

* cornell: the path-tracing benchmark's Cornell box at depth 5, 16 samples
  per pixel (128 x 128 here);
* terrain: the large benchmark scene reduced below the reference's 65,535-face
  limit -- heightfield, spheres, the 1024 x 512 sky with its sun spot, eight
  bump-mapped materials, thin lens 0.02 / 1.5 -- at depth 8, 32 samples.

Every device form renders each: megakernel and wavefront, reference-order
and nearer-first traversal; they must give one identical image.  That image
is held to the bars of the other render tests (relative RMSE <= 1e-4, mean
within 1e-5, >= 99.9 % of pixels within 1e-3 relative), each widened to three
times the reference's own floor where that floor is higher: the distance the
reference's renderer moves when its transcendental functions are rebuilt one
ulp off on an eighth of the inputs (stored with the golden; the sun spot's
5e3 peak makes the terrain's floor 4.3e-4).
"""
import os
import sys

import numpy as np
import pytest
import torch

from clear_gb300 import _lib
from clear_gb300.render import DeviceScene

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden_configs as GC  # noqa: E402
from make_golden_render import blob_hash  # noqa: E402

GOLDEN = os.path.join(HERE, "golden", "render_configs.npz")


@pytest.mark.parametrize("name", sorted(GC.CONFIGS))
def test_config_scene_encoding_matches_golden(name):
    g = np.load(GOLDEN)
    assert blob_hash(GC.build_scene(name).blobs()) == str(g[f"{name}_hash"])
    assert int(g[f"{name}_faces"]) < 65536


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(GC.CONFIGS))
def test_config_render_matches_reference_sim(cuda, name):
    g = np.load(GOLDEN)
    w, h, spp, depth = (int(g[f"{name}_{k}"]) for k in ("width", "height", "spp", "depth"))
    ds = DeviceScene(GC.build_scene(name), cuda)
    images = []
    for wavefront in (False, True):
        for ordered in (False, True):
            rng, pix = ds.new_frame()
            ds.render(rng, pix, spp, max_depth=depth, ordered=ordered, wavefront=wavefront)
            images.append((pix, rng))
    torch.cuda.synchronize()
    for pix, rng in images[1:]:
        assert torch.equal(pix, images[0][0]) and torch.equal(rng, images[0][1])
    img = images[0][0][:, :3].cpu().numpy()
    rel_rmse, mean_err, frac_close = GC.image_metrics(img, g[f"{name}_image"])
    f_rmse, f_mean, f_close = (float(v) for v in g[f"{name}_floor"])
    bar = (max(1e-4, 3 * f_rmse), max(1e-5, 3 * f_mean), min(0.999, 1.0 - 3 * (1.0 - f_close)))
    print(f"{name}: rel RMSE {rel_rmse:.4g}, mean err {mean_err:.4g}, close {frac_close:.5f}; "
          f"reference floor {f_rmse:.3g} / {f_mean:.3g} / {f_close:.5f}; bars {bar}")
    assert rel_rmse <= bar[0] and mean_err <= bar[1] and frac_close >= bar[2], (rel_rmse, mean_err, frac_close)
    assert _lib.device_status() == 0
