"""Post-processing (accumulation -> 8-bit BGR BMP pixels) against the
reference's own `clear` / `scaling` / `toneMapping` kernels run on the CPU
(oracle/ref_post_cl.cpp; golden tests/golden/post_ref.npz), against the numpy
restatement oracle/postprocess.py, and the BMP file against the reference's
saveBMP.  Bar (stated here): every byte within 1 and at least 99.9 % of bytes
equal (exp and pow of two math libraries may round differently; the numpy
restatement and the reference kernels agree exactly on small images); the
row padding and the file header exact."""
import struct

import numpy as np
import pytest
import torch

import os
import sys

import oracle
from clear_gb300 import _lib
from clear_gb300 import postprocess as PP
from oracle import postprocess as OP

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
import make_golden_post as GP  # noqa: E402

POST_GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "post_ref.npz")


def _close(got, want, frac=0.999):
    d = np.abs(got.astype(np.int32) - want.astype(np.int32))
    assert d.max() <= 1, d.max()
    assert (d == 0).mean() >= frac, (d == 0).mean()


def _hdr(n, seed=3):
    r = np.random.default_rng(seed)
    a = np.zeros((n, 4), dtype=np.float32)
    a[:, :3] = r.lognormal(0.0, 2.0, size=(n, 3)).astype(np.float32)
    special = [(0.0, 0.0, 0.0),      # black: Y = 0 branch
               (1e6, 1e6, 1e6),      # saturates at the threshold
               (0.0, 5.0, 0.0)]
    for i, v in enumerate(special[:n]):
        a[i, :3] = v
    return a


def test_oracle_layout_and_header():
    w, h = 5, 3
    acc = _hdr(w * h)
    px = OP.tonemap(acc, w, h, 4)
    assert px.size == h * OP.byte_width(w) == h * (3 * w + 1)
    rows = px.reshape(h, -1)
    assert np.all(rows[:, 3 * w:] == 0)
    assert tuple(rows[h - 1, 0:3]) == (0, 0, 0)  # pixel 0 (black) is the first pixel of the last row
    b = PP.bmp_bytes(px, w, h)
    assert b[:2] == b"BM" and len(b) == 54 + px.size
    size, _, _, off, info, ww, hh, planes, bits = struct.unpack_from("<IHHIIIIHH", b, 2)
    assert (size, off, info, ww, hh, planes, bits) == (54 + px.size, 54, 40, w, h, 1, 24)


@pytest.mark.gpu
@pytest.mark.parametrize("w,h,spp", [(1920, 1080, 64), (33, 7, 1), (1, 1, 3)])
def test_postprocess_matches_oracle(cuda, w, h, spp):
    acc = _hdr(w * h, seed=w)
    got = PP.to_ldr(torch.from_numpy(acc).to(cuda), w, h, spp).cpu().numpy()
    want = OP.tonemap(acc, w, h, spp)
    diff = np.abs(got.astype(np.int32) - want.astype(np.int32))
    assert diff.max() <= 1, diff.max()
    assert (diff == 0).mean() >= 0.99
    rows = got.reshape(h, -1)
    assert np.all(rows[:, 3 * w:] == 0)
    assert _lib.device_status() == 0


@pytest.mark.gpu
def test_tone_scales_are_the_double_expressions(cuda):
    """Y and the tone-mapping scale, computed in float-float with a double
    fallback, equal the double-precision expressions exactly (numpy float64),
    over 4 Mi pixels of a wide radiance distribution and the edge cases:
    zeros, saturation, subnormal, negative and NaN channels."""
    w, h, spp = 2048, 2048, 4
    r = np.random.default_rng(11)
    acc = np.zeros((w * h, 4), dtype=np.float32)
    acc[:, :3] = (r.lognormal(0.0, 3.0, size=(w * h, 3)) * spp).astype(np.float32)
    edge = np.array([[0, 0, 0], [1e9, 1e9, 1e9], [1e-40, 0, 0], [1e-30, 1e-30, 1e-30], [-1.0, 2.0, 3.0],
                     [np.nan, 1.0, 1.0], [0.0, 0.0, 1e-7], [4.0, 4.0, 4.0], [120.0, 0.0, 0.0]], dtype=np.float32)
    acc[:len(edge), :3] = edge
    acc[len(edge):len(edge) + 4096, :3] = r.uniform(0, 1e-6, size=(4096, 3)).astype(np.float32)
    got = PP.tone_scales(torch.from_numpy(acc).to(cuda), w, h, spp).cpu().numpy()
    inv = np.float32(1.0) / np.float32(spp)
    v = (acc[:, :3] * inv).astype(np.float32)
    sat = np.where(v > np.float32(30.0), np.float32(30.0), v).astype(np.float32)
    s64 = sat.astype(np.float64)
    Y = (0.2989 * s64[:, 0] + 0.5866 * s64[:, 1] + 0.1144 * s64[:, 2]).astype(np.float32)
    assert np.array_equal(got[:, 0], Y, equal_nan=True)
    e = got[:, 1]
    fin = np.isfinite(Y)
    assert np.all(np.abs(e[fin].astype(np.float64) - np.exp(-Y[fin].astype(np.float64))) <= 3e-7 * e[fin])
    with np.errstate(divide="ignore", invalid="ignore"):
        scale = ((1.0 - e.astype(np.float64)) / Y.astype(np.float64)).astype(np.float32)
    scale = np.where(Y == 0.0, np.float32(1.0), scale)
    assert np.array_equal(got[:, 2], scale, equal_nan=True)
    assert _lib.device_status() == 0


@pytest.mark.skipif(not __import__("oracle").ref_available(), reason="reference checkout not available")
@pytest.mark.parametrize("w,h", [(1, 1), (5, 3), (6, 2), (7, 4), (8, 5)])
def test_bmp_file_matches_reference_writer(tmp_path, w, h):
    """save_bmp writes the same file as the reference's saveBMP, for every
    row-padding case (width % 4 = 0 .. 3)."""
    import oracle

    px = OP.tonemap(_hdr(w * h, seed=w), w, h, 2)
    oracle.ref_save_bmp(tmp_path / "ref.bmp", px, w, h)
    PP.save_bmp(str(tmp_path / "ours.bmp"), px, w, h)
    assert (tmp_path / "ours.bmp").read_bytes() == (tmp_path / "ref.bmp").read_bytes()


def test_oracle_matches_reference_kernels_golden():
    g = np.load(POST_GOLDEN)
    w, h, spp = int(g["width"]), int(g["height"]), int(g["spp"])
    _close(OP.tonemap(GP.accum(w, h), w, h, spp), g["pixels"])


@pytest.mark.skipif(not oracle.ref_available(), reason="reference checkout not available")
@pytest.mark.parametrize("w,h,spp", [(1, 1, 3), (5, 3, 4), (64, 33, 2), (97, 61, 1)])
def test_oracle_matches_reference_kernels_live(w, h, spp):
    acc = _hdr(w * h, seed=w)
    assert np.array_equal(OP.tonemap(acc, w, h, spp), oracle.ref_cl_postprocess(acc, w, h, spp))


@pytest.mark.gpu
def test_device_matches_reference_kernels(cuda):
    """clr_postprocess_ldr against the reference's own kernels (golden)."""
    g = np.load(POST_GOLDEN)
    w, h, spp = int(g["width"]), int(g["height"]), int(g["spp"])
    got = PP.to_ldr(torch.from_numpy(GP.accum(w, h)).to(cuda), w, h, spp).cpu().numpy()
    _close(got, g["pixels"])
    assert _lib.device_status() == 0