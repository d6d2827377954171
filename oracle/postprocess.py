"""Restatement of the reference's post-processing (test infrastructure only):
the `scaling` and `toneMapping` kernels of OpenCL/post_processing.cl (:20-26,
:98-117) in numpy, evaluated in the precisions the OpenCL source gives them
(float channels, double luminance and tone-mapping scale from the double
literals, float exp and pow).  The reference has no CPU version of these
kernels and no golden images, so this restatement is the oracle; exp and pow
of two math libraries may round differently, which can move a byte by one.
"""
from __future__ import annotations

import numpy as np

THRESHOLD = np.float32(30.0)  # post_processing.cl:70


def byte_width(width: int) -> int:
    return 3 * width + width % 4  # BMPExporter.cpp:15


def tonemap(accum: np.ndarray, width: int, height: int, spp: int) -> np.ndarray:
    a = np.asarray(accum, dtype=np.float32).reshape(height * width, -1)[:, :3]
    inv = np.float32(1.0) / np.float32(spp)
    v = (a * inv).astype(np.float32)                                   # scaling
    s = np.where(v > THRESHOLD, THRESHOLD, v).astype(np.float32)       # saturation
    s64 = s.astype(np.float64)
    Y = (0.2989 * s64[:, 0] + 0.5866 * s64[:, 1] + 0.1144 * s64[:, 2]).astype(np.float32)
    with np.errstate(divide="ignore", invalid="ignore"):
        e = np.exp(-Y).astype(np.float32)
        scale = ((1.0 - e.astype(np.float64)) / Y.astype(np.float64)).astype(np.float32)
    scale = np.where(Y == 0.0, np.float32(1.0), scale).astype(np.float32)
    gamma = np.float32(1.0) / np.float32(2.2)
    with np.errstate(invalid="ignore"):
        p = np.power((scale[:, None] * s).astype(np.float32), gamma).astype(np.float32)
    r = (np.float32(255.0) * p).astype(np.float32)
    r = np.where(np.isnan(r), np.float32(0.0), r)
    r = np.clip(r, 0.0, 255.0)
    u8 = r.astype(np.uint8)  # truncation toward zero (convert_uchar3_rtz)
    bw = byte_width(width)
    out = np.zeros((height, bw), dtype=np.uint8)
    img = u8.reshape(height, width, 3)[::-1]  # rows bottom-up
    out[:, :3 * width] = img[:, :, ::-1].reshape(height, 3 * width)  # BGR
    return out.reshape(-1)
