"""Build recipe for the CPU oracle (test infrastructure only).

* ``oracle/liboracle.so`` -- the C restatement in ``oracle/lbvh_oracle.c``.
  Built everywhere (here and on the GPU host) with ``-ffp-contract=off`` so the
  reference's float expressions round exactly as written.
* ``oracle/_ref/libref_lbvh.so`` and ``oracle/_ref/libref_mid.so`` -- the
  reference's own CPU code (``OpenCL_PathTracer/Equivalent/sim_*.hpp`` and
  ``OpenCL_PathTracer/BVH.hpp``) compiled in place from a reference checkout
  with the stand-in headers of ``oracle/ref_stubs``.
* ``oracle/_ref/libref_lbvh_kbump.so`` -- ``libref_lbvh.so`` with the one
  line where the CPU renderer departs from its OpenCL kernel (the bump frame's
  axis normalisation, ``OpenCL/reflection.cl:210``) as the kernel has it.
* ``oracle/_ref/libref_lbvh_cl.so`` and ``libref_post_cl.so`` -- the
  reference's LBVH construction kernels (``OpenCL/lbvh_construction.cl``,
  ``CommonSources/OpenCL/generic_kernels.cl``) and post-processing kernels
  (``OpenCL/post_processing.cl``) run on the CPU by ``oracle/ref_lbvh_cl.cpp``
  and ``oracle/ref_post_cl.cpp`` (executor ``oracle/ref_cl_exec.cpp``).
* ``oracle/_ref/libref_scene.so`` -- the reference's scene encoders, .obj
  loader and BMP writer (``OpenCL_PathTracer/CreateFunctions.cpp``,
  ``ModelLoader.cpp``, ``BMPExporter.cpp``,
  with ``LinearAlgebra/*.cpp`` for the matrices of ``Scene.h``) behind
  ``oracle/ref_scene.cpp``.

The ``_ref`` libraries are built only when the reference checkout exists:
the directory named by ``CLEAR_REFERENCE_DIR``, else a checkout named
``reference`` beside this repository (``<repo>/../reference``); nothing is
copied out of it.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REF_DIR = Path(os.environ.get("CLEAR_REFERENCE_DIR", HERE.parent.parent / "reference"))
CFLAGS = ["-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math"]


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{res.stderr}")


def _stale(out: Path, srcs: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(s.stat().st_mtime > t for s in srcs if s.exists())


def build_oracle() -> Path:
    out = HERE / "liboracle.so"
    src = HERE / "lbvh_oracle.c"
    if _stale(out, [src, Path(__file__)]):
        _run(["gcc", "-std=c11", *CFLAGS, str(src), "-o", str(out), "-lm"])
    return out


def build_ref() -> list[Path]:
    """Compile the reference's CPU code if its sources are present."""
    eq = REF_DIR / "OpenCL_PathTracer" / "Equivalent"
    if not eq.is_dir():
        return []
    outdir = HERE / "_ref"
    outdir.mkdir(exist_ok=True)
    src = HERE / "ref_harness.cpp"
    stubs = HERE / "ref_stubs"
    deps = [src, *stubs.iterdir(), Path(__file__)]
    built = []
    for name, defs in (("libref_lbvh.so", ["-D__USE_LBVH"]), ("libref_mid.so", [])):
        out = outdir / name
        if _stale(out, deps):
            # sim::pathtracing reads two locals it may never set: lpos.faceID
            # before the path's first light face, and the shadow ray's hit
            # record after a miss (sim_pathtracer.hpp:80, 121-123).  Filling
            # uninitialised locals with the 0xFE pattern gives both a value
            # that matches no face instead of stack leftovers.
            _run(["g++", "-std=c++17", "-w", *CFLAGS, "-ftrivial-auto-var-init=pattern", *defs, f"-I{stubs}", f"-I{eq}",
                  f"-I{REF_DIR / 'OpenCL_PathTracer'}", str(src), "-o", str(out)])
        built.append(out)
    out = outdir / "libref_scene.so"
    scene_src = HERE / "ref_scene.cpp"
    if _stale(out, [scene_src, *stubs.iterdir(), Path(__file__)]):
        pt, la = REF_DIR / "OpenCL_PathTracer", REF_DIR / "LinearAlgebra"
        srcs = [scene_src, pt / "CreateFunctions.cpp", pt / "ModelLoader.cpp", pt / "BMPExporter.cpp",
                *(la / f for f in ("LinearAlgebra.cpp", "Matrix4f.cpp", "Vector4f.cpp", "Vector3f.cpp",
                                 "Point3f.cpp"))]
        # the encoders copy stack structs whose padding they never set:
        # zero-initialised locals make those bytes zeros instead of garbage
        _run(["g++", "-std=c++17", "-w", *CFLAGS, "-ftrivial-auto-var-init=zero", f"-I{stubs}", f"-I{pt}",
              f"-I{la}", *map(str, srcs), "-o", str(out), "-Wl,--no-undefined"])
    built.append(out)
    out = outdir / "libref_lbvh_kbump.so"
    if _stale(out, deps):
        build_ref_kernel_bump(out, src, stubs, eq)
    built.append(out)
    cl_dir = REF_DIR / "OpenCL_PathTracer" / "OpenCL"
    for lib, harness, kernels in (
            ("libref_lbvh_cl.so", "ref_lbvh_cl.cpp",
             [cl_dir / "lbvh_construction.cl", REF_DIR / "CommonSources" / "OpenCL" / "generic_kernels.cl"]),
            ("libref_post_cl.so", "ref_post_cl.cpp", [cl_dir / "post_processing.cl"])):
        out = outdir / lib
        if _stale(out, [HERE / harness, HERE / "ref_cl_exec.cpp", *stubs.iterdir(), Path(__file__)]):
            build_ref_kernels(out, HERE / harness, kernels, stubs)
        built.append(out)
    return built


def build_ref_kernel_bump(out: Path, harness: Path, stubs: Path, eq: Path) -> None:
    """The LBVH harness over the reference's CPU renderer with the one line
    where that renderer departs from its OpenCL kernel put back as the kernel
    has it: the bump frame's rotation axis is normalised before use
    (OpenCL/reflection.cl:210; Equivalent/sim_reflection.hpp omits it, which
    turns the frame by the wrong matrix).  sim_reflection.hpp is read from the
    checkout, changed in memory and piped to the compiler ahead of the
    harness, whose own #include of it is then a no-op (include guard);
    nothing is written."""
    text = (eq / "sim_reflection.hpp").read_text()
    anchor = "float sinTH = fminf(length(ax), 1.0f);\n            if (sinTH > 0.0001f) {\n"
    if text.count(anchor) != 1:
        raise RuntimeError("oracle build: the bump block of sim_reflection.hpp is not where expected")
    text = text.replace(anchor, anchor + "                ax = normalize(ax);\n")
    src = "#include <cstdint>\n#include <cstring>\n#include <vector>\n" + text + '\n#include "ref_harness.cpp"\n'
    res = subprocess.run(["g++", "-std=c++17", "-w", *CFLAGS, "-ftrivial-auto-var-init=pattern", "-D__USE_LBVH",
                          f"-I{stubs}", f"-I{eq}", f"-I{REF_DIR / 'OpenCL_PathTracer'}", f"-I{harness.parent}",
                          "-x", "c++", "-", "-o", str(out)], input=src, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed: kernel-bump renderer\n{res.stderr}")


def build_ref_kernels(out: Path, harness: Path, kernels: list[Path], stubs: Path) -> None:
    """Reference OpenCL kernels compiled as C++ with the OpenCL C subset of
    ref_stubs/opencl_c.hpp and linked with `harness` and the executor
    (ref_cl_exec.cpp).  The kernel text is read from the checkout and piped to
    the compiler with two spellings changed: a work-group `local` declaration
    at the start of a line becomes `static` (work-groups run one at a time, so
    a function static is the group's local memory), and a vector literal
    `(T)(...)` becomes the functional cast `T(...)`; nothing else changes and
    nothing is written."""
    import re
    import tempfile

    def rewrite(text: str) -> str:
        text = re.sub(r"(?m)^(\s+)local\s", r"\1static ", text)
        return re.sub(r"\((float3|point3|vector3|uint3|int3|uchar3)\)\(", r"\1(", text)

    src = "\n".join(rewrite(k.read_text()) for k in kernels)
    cl_dir = kernels[0].parent
    flags = ["-std=c++17", "-w", "-O2", "-fPIC", "-fsigned-char", "-ffp-contract=off", "-fno-fast-math",
             f"-I{stubs}"]
    with tempfile.TemporaryDirectory() as tmp:
        obj = Path(tmp) / "kernels.o"
        res = subprocess.run(["g++", *flags, "-include", str(stubs / "opencl_c.hpp"), f"-I{cl_dir}", "-x", "c++",
                              "-", "-c", "-o", str(obj)], input=src, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"oracle build failed: reference LBVH kernels\n{res.stderr}")
        _run(["g++", *flags, "-shared", str(harness), str(HERE / "ref_cl_exec.cpp"), str(obj), "-o", str(out),
              "-Wl,--no-undefined"])


if __name__ == "__main__":
    print(build_oracle())
    for p in build_ref():
        print(p)
    sys.exit(0)
