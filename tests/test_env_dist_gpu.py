"""The environment light's importance distribution rebuilt on the device
(clr_env_distribution_update) against the host scene encoder
(MaterialCreator.continuous_consts_2d_h, the reference's
createContinuousConsts2D_H_FromImageTexture): bit-identical `others` blobs,
before and after the environment texels change, for a 64 x 32 and a
1024 x 512 map."""
import numpy as np
import pytest
import torch

from clear_gb300 import _lib, scenes
from clear_gb300.render import DeviceScene

pytestmark = pytest.mark.gpu


def _write_env(ds, env):
    """Write (h, w, 3) texels into the device copy of the RGBA16F texture."""
    off = ds.env_dist["tex_offset"]
    rel = int(np.frombuffer(ds.blobs["textures"][off + 12:off + 16].tobytes(), dtype=np.int32)[0])
    h, w = env.shape[:2]
    rgba = np.ones((h, w, 4), dtype=np.float16)
    rgba[..., :3] = env.astype(np.float16)
    t = ds.t["textures"]
    t[off + rel:off + rel + rgba.nbytes] = torch.from_numpy(rgba.view(np.uint8).reshape(-1)).to(t.device)


def _array_spans(ds):
    """Byte ranges in `others` of the distribution's numeric arrays (the
    parent's pdf and cdf; the rows' pdfs and cdfs), between which the
    headers the update reads stay untouched."""
    d = ds.env_dist
    h, w = d["height"], d["width"]
    p0 = d["dist_offset"] + 36
    p1 = p0 + 4 * h + 4 * (h + 1)
    c0 = p1 + 28 * h
    c1 = c0 + 4 * w * h + 4 * (w + 1) * h
    return [(p0, p1), (c0, c1)]


@pytest.mark.parametrize("shape", [(32, 64), (512, 1024)])
def test_env_distribution_matches_encoder(cuda, shape):
    h, w = shape
    env0 = scenes.sky_map(w, h, seed=5) if h > 32 else scenes.adjoint_env()
    ds = DeviceScene(scenes.cornell_box(32, 32, env=env0), cuda)
    ref0 = ds.blobs["others"]
    spans = _array_spans(ds)
    # wipe the distribution's arrays on the device, rebuild, compare
    o = ds.t["others"]
    for a, b in spans:
        o[a:b] = 0
    ds.update_env_distribution()
    torch.cuda.synchronize()
    assert _lib.device_status() == 0
    assert np.array_equal(o.cpu().numpy(), ref0)
    # new texels: the device rebuild equals re-encoding the scene
    env1 = np.minimum(env0 * np.exp(np.random.default_rng(2).normal(0, 0.3, env0.shape)), 6e4).astype(np.float32)
    _write_env(ds, env1)
    ds.update_env_distribution()
    ref1 = scenes.cornell_box(32, 32, env=env1).blobs()["others"]
    torch.cuda.synchronize()
    assert np.array_equal(o.cpu().numpy(), ref1)
    assert not np.array_equal(ref0, ref1)
    # the default row weights, the same float argument through the device's
    # cosf instead of the C library's: equal to a few ulps of the weight
    ds.update_env_distribution(encoder_weights=False)
    got = o.cpu().numpy()
    for lo, hi in spans:
        a, b = got[lo:hi].view(np.float32), ref1[lo:hi].view(np.float32)
        nz = np.abs(b) > 1e-30
        assert np.max(np.abs(a[nz] - b[nz]) / np.abs(b[nz])) < 1e-4
    assert _lib.device_status() == 0
