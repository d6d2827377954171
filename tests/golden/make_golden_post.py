"""Golden post-processing output from the reference's own kernels.

Run where the reference checkout is available (compiled in place into
oracle/_ref by oracle/build_oracle.py):

    python tests/golden/make_golden_post.py

post_ref.npz -- the BMP pixel array that the reference's `clear`, `scaling`
and `toneMapping` kernels (OpenCL_PathTracer/OpenCL/post_processing.cl, run
on the CPU by oracle/ref_post_cl.cpp, exp and pow from the C library) make
of the accumulation buffer ``accum(W, H)`` at SPP samples per pixel.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

W, H, SPP = 321, 181, 16


def accum(width: int = W, height: int = H, seed: int = 5) -> np.ndarray:
    """A wide radiance distribution with black, saturated and NaN pixels."""
    r = np.random.default_rng(seed)
    a = np.zeros((width * height, 4), dtype=np.float32)
    a[:, :3] = (r.lognormal(0.0, 2.5, size=(width * height, 3)) * SPP).astype(np.float32)
    a[0, :3] = 0.0
    a[1, :3] = 1e9
    a[2, :3] = (np.nan, 1.0, 1.0)
    a[3, :3] = (0.0, 5.0 * SPP, 0.0)
    return a


def main() -> None:
    import oracle

    if not oracle.ref_available():
        raise SystemExit("reference checkout not available")
    px = oracle.ref_cl_postprocess(accum(), W, H, SPP)
    np.savez_compressed(os.path.join(HERE, "post_ref.npz"), pixels=px, width=W, height=H, spp=SPP)
    print("wrote", os.path.join(HERE, "post_ref.npz"))


if __name__ == "__main__":
    main()
