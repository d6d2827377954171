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
  axis normalisation, ``OpenCL/reflection.cl:210``) as the kernel has it, and
  its path-length cap settable (``ref_set_max_depth``);
  ``libref_lbvh_kbump_ulp.so`` the same with the transcendental functions'
  results one ulp off on an eighth of the inputs (the reference's own
  sensitivity to its math library, the floor of the image bars).
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
        # OpenMP runs orc_lbvh_build_mt on all host cores; without it (no
        # libgomp) the same function runs on one thread
        try:
            _run(["gcc", "-std=c11", *CFLAGS, "-fopenmp", str(src), "-o", str(out), "-lm"])
        except RuntimeError:
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
    for lib, perturb in (("libref_lbvh_kbump.so", False), ("libref_lbvh_kbump_ulp.so", True)):
        out = outdir / lib
        if _stale(out, deps):
            build_ref_kernel_bump(out, src, stubs, eq, perturb_math=perturb)
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


# Wrappers that move the results of the transcendental functions the
# reference's renderer calls by one ulp on about an eighth of the inputs
# (chosen by a hash of the argument): the reference rebuilt with them shows how
# far its own images move when only the math library's rounding changes.
MATH_ULP_PRELUDE = r"""
#include <cmath>
#include <cstdint>
#include <cstring>
static inline float clr_ulp_off(float r, float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    u ^= u >> 15; u *= 0x2c1b3c6du; u ^= u >> 12; u *= 0x297a2d39u; u ^= u >> 15;
    if ((u & 7u) != 0u) return r;
    return std::nextafter(r, (u & 8u) ? INFINITY : -INFINITY);
}
static inline float clr_sinf(float x) { return clr_ulp_off(::sinf(x), x); }
static inline float clr_cosf(float x) { return clr_ulp_off(::cosf(x), x); }
static inline float clr_asinf(float x) { return clr_ulp_off(::asinf(x), x); }
static inline float clr_acosf(float x) { return clr_ulp_off(::acosf(x), x); }
static inline float clr_atanf(float x) { return clr_ulp_off(::atanf(x), x); }
static inline float clr_atan2f(float y, float x) { return clr_ulp_off(::atan2f(y, x), x + y); }
static inline float clr_expf(float x) { return clr_ulp_off(::expf(x), x); }
static inline float clr_logf(float x) { return clr_ulp_off(::logf(x), x); }
static inline float clr_powf(float x, float y) { return clr_ulp_off(::powf(x, y), x * y); }
#define sinf clr_sinf
#define cosf clr_cosf
#define asinf clr_asinf
#define acosf clr_acosf
#define atanf clr_atanf
#define atan2f clr_atan2f
#define expf clr_expf
#define logf clr_logf
#define powf clr_powf
"""


def build_ref_kernel_bump(out: Path, harness: Path, stubs: Path, eq: Path, perturb_math: bool = False) -> None:
    """The LBVH harness over the reference's CPU renderer with two changes:
    * the one line where that renderer departs from its OpenCL kernel is put
      back as the kernel has it: the bump frame's rotation axis is normalised
      before use (OpenCL/reflection.cl:210; Equivalent/sim_reflection.hpp
      omits it, which turns the frame by the wrong matrix);
    * the path-length cap (ray.depth > 99, sim_pathtracer.hpp:167; the
      kernel's pathtracer.cl:166) reads a variable, set by ref_set_max_depth,
      so that the renderer can run at the benchmarked depths (5 and 8);
      it starts at the reference's 99.
    sim_reflection.hpp and sim_pathtracer.hpp are read from the checkout,
    changed in memory and piped to the compiler ahead of the harness (whose
    own include of sim_pathtracer.hpp is then skipped, and whose include of
    sim_reflection.hpp is a no-op by its include guard); nothing is written.
    perturb_math prepends MATH_ULP_PRELUDE (the floor measurement build)."""
    text = (eq / "sim_reflection.hpp").read_text()
    anchor = "float sinTH = fminf(length(ax), 1.0f);\n            if (sinTH > 0.0001f) {\n"
    if text.count(anchor) != 1:
        raise RuntimeError("oracle build: the bump block of sim_reflection.hpp is not where expected")
    text = text.replace(anchor, anchor + "                ax = normalize(ax);\n")
    pt = (eq / "sim_pathtracer.hpp").read_text()
    cap = "if (ray.depth > 99) {"
    if pt.count(cap) != 1:
        raise RuntimeError("oracle build: the depth cap of sim_pathtracer.hpp is not where expected")
    pt = pt.replace(cap, "if (ray.depth > clr_ref_depth_cap) {")
    src = ((MATH_ULP_PRELUDE if perturb_math else "") +
           "#include <cstdint>\n#include <cstring>\n#include <vector>\n"
           "static int clr_ref_depth_cap = 99;\n#define CLR_REF_PIPED_PATHTRACER 1\n" + text + "\n" + pt +
           '\n#include "ref_harness.cpp"\n')
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
