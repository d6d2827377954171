"""The last step of a render: accumulation buffer -> 8-bit image -> BMP.

``to_ldr`` runs ``clr_postprocess_ldr`` (the reference's ``scaling`` +
``toneMapping`` kernels, OpenCL/post_processing.cl:20-26, 98-117, fused) on
the device; ``save_bmp`` writes the pixel array with the header of the
reference's ``saveBMP`` (OpenCL_PathTracer/BMPExporter.cpp:14-55).
"""
from __future__ import annotations

import ctypes as C
import struct

import numpy as np
import torch

from . import _lib


def byte_width(width: int) -> int:
    """Bytes per BMP row as the reference computes them (BMPExporter.cpp:15)."""
    return 3 * width + width % 4


def to_ldr(accum: torch.Tensor, width: int, height: int, spp: int) -> torch.Tensor:
    """accum: (width * height, 4) float32 on the GPU.  Returns the BMP pixel
    array (height * byte_width(width) uint8, BGR, rows bottom-up)."""
    out = torch.empty(height * byte_width(width), dtype=torch.uint8, device=accum.device)
    a = accum.contiguous()
    with torch.cuda.device(accum.device):
        _lib.call("clr_postprocess_ldr", C.c_void_p(a.data_ptr()), C.c_uint32(width), C.c_uint32(height),
                  C.c_uint32(spp), C.c_void_p(out.data_ptr()),
                  C.c_void_p(torch.cuda.current_stream(accum.device).cuda_stream))
    return out


def tone_scales(accum: torch.Tensor, width: int, height: int, spp: int) -> torch.Tensor:
    """Per pixel {Y, expf(-Y), scale, 0} as ``to_ldr`` computes them
    (``clr_postprocess_scales``): (width * height, 4) float32 on the GPU."""
    out = torch.empty((height * width, 4), dtype=torch.float32, device=accum.device)
    a = accum.contiguous()
    with torch.cuda.device(accum.device):
        _lib.call("clr_postprocess_scales", C.c_void_p(a.data_ptr()), C.c_uint32(width), C.c_uint32(height),
                  C.c_uint32(spp), C.c_void_p(out.data_ptr()),
                  C.c_void_p(torch.cuda.current_stream(accum.device).cuda_stream))
    return out


def bmp_bytes(pixels: np.ndarray, width: int, height: int) -> bytes:
    """The file saveBMP writes: a 14 + 40 byte header (24 bits, uncompressed,
    1 pixel per metre) followed by the pixel array."""
    data_size = byte_width(width) * height
    pix = np.ascontiguousarray(pixels, dtype=np.uint8).reshape(-1)
    if pix.size != data_size:
        raise ValueError(f"pixel array of {pix.size} bytes, expected {data_size}")
    head = b"BM" + struct.pack("<IHHI", data_size + 54, 0, 0, 54)
    info = struct.pack("<IIIHHIIII", 40, width, height, 1, 24, 0, data_size, 1, 1) + b"\0" * 8
    return head + info + pix.tobytes()


def save_bmp(path: str, pixels: np.ndarray, width: int, height: int) -> None:
    with open(path, "wb") as fh:
        fh.write(bmp_bytes(pixels, width, height))
