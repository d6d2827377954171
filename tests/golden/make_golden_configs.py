"""Golden images of the benchmarked render configurations, from the
reference's own CPU renderer at the benchmarks' path-length caps.

Run where the reference checkout is available (compiled in place into
oracle/_ref by oracle/build_oracle.py):

    python tests/golden/make_golden_configs.py

Writes render_configs.npz with two scenes, each rendered by
``sim::pathtracing`` (OpenCL_PathTracer/Equivalent/sim_pathtracer.hpp) built
as the OpenCL kernel has it (bump-frame axis normalised, reflection.cl:210)
and with its depth cap (ray.depth > 99, sim_pathtracer.hpp:167; the kernel's
pathtracer.cl:166) set to the benchmark's depth (oracle/_ref/
libref_lbvh_kbump.so), over the oracle-built LBVH, per-pixel XORShift128
streams seeded with pixel index + 1:

* ``cornell`` -- the Cornell box of the path-tracing benchmark (five walls,
  two rotated boxes, the 32 x 16 sphere under a Beckmann coat, the quad lamp),
  at 128 x 128 (the benchmark renders 256 x 256), 16 samples per pixel,
  depth 5;
* ``terrain`` -- the large benchmark scene reduced below the reference's
  65,535-face limit (its traversal stores face ids as ushort,
  bvh_traversal.cl:43,56): a 128 x 128-cell heightfield with 6-octave value
  noise, 32 spheres, the 1024 x 512 lognormal sky with its sun spot, eight
  bump-mapped materials, thin lens 0.02 / 1.5, at 160 x 90, 32 samples per
  pixel, depth 8.

For each it also stores the reference's own floor: relative RMSE, relative
error of the mean and fraction of pixels within 1e-3 between this image and
the same renderer rebuilt with its transcendental functions one ulp off on
an eighth of the inputs (libref_lbvh_kbump_ulp.so) -- how far the reference
moves when only its math library's rounding changes.  A
SHA-256 of the blobs pins each scene's encoding.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

CONFIGS = {
    "cornell": {"width": 128, "height": 128, "spp": 16, "depth": 5},
    "terrain": {"width": 160, "height": 90, "spp": 32, "depth": 8},
}


def build_scene(name: str):
    from clear_gb300 import scenes

    c = CONFIGS[name]
    if name == "cornell":
        return scenes.cornell_box(c["width"], c["height"])
    return scenes.terrain_scene(width=c["width"], height=c["height"], grid=128, n_spheres=32)


def reference_image(sc, c: dict, perturb_math: bool = False) -> np.ndarray:
    import oracle
    from clear_gb300 import scenes

    b = sc.blobs()
    vx, vy, vz, tri = sc.soa()
    ob = oracle.lbvh_build(vx, vy, vz, tri, len(sc.faces), 10)
    w, h = c["width"], c["height"]
    pix = np.zeros((w * h, 4), dtype=np.float32)
    oracle.ref_render(b, ob.inodes, ob.lnodes, scenes.pixel_seeds(w, h), pix, w, h, 0, h, c["spp"],
                      bump_as_kernel=True, max_depth=c["depth"], perturb_math=perturb_math)
    return pix[:, :3].copy()


def image_metrics(img: np.ndarray, ref: np.ndarray) -> tuple[float, float, float]:
    """Relative RMSE, relative error of the mean, and the fraction of pixels
    whose three channels are all within 1e-3 relative (floor 1e-3)."""
    rmse = float(np.sqrt(((img - ref) ** 2).mean()))
    close = np.abs(img - ref) <= 1e-3 * np.maximum(np.abs(ref), 1e-3)
    return (rmse / float(ref.mean()), abs(float(img.mean()) - float(ref.mean())) / float(ref.mean()),
            float(close.all(axis=1).mean()))


def main() -> None:
    import oracle
    from make_golden_render import blob_hash

    if not oracle.ref_available():
        raise SystemExit("reference checkout not available")
    out = {}
    for name, c in CONFIGS.items():
        sc = build_scene(name)
        img = reference_image(sc, c)
        alt = reference_image(sc, c, perturb_math=True)
        floor = image_metrics(alt, img)
        for k, v in c.items():
            out[f"{name}_{k}"] = v
        out[f"{name}_image"] = img
        out[f"{name}_hash"] = blob_hash(sc.blobs())
        out[f"{name}_floor"] = np.array(floor, dtype=np.float64)
        out[f"{name}_faces"] = len(sc.faces)
        print(f"{name}: {len(sc.faces)} faces, mean {img.mean():.5g}, reference floor (rel RMSE, mean error, "
              f"pixels within 1e-3) {floor}")
    np.savez_compressed(os.path.join(HERE, "render_configs.npz"), **out)
    print("wrote render_configs.npz")


if __name__ == "__main__":
    main()
