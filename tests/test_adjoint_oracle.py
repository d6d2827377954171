"""The float64 path re-evaluator (oracle/adjoint_fd.py) on hand-made tapes:
record decoding, path assembly order, and central differences against
closed forms (CPU only)."""
import numpy as np

from clear_gb300 import scenes
from oracle import adjoint_fd as FD


def _rec(pixel, sample, depth, kind, **f):
    w = np.zeros(32, dtype=np.uint32)
    w[0], w[1], w[2], w[3] = pixel, sample, depth, kind
    fl = w.view(np.float32)
    for k, v in f.items():
        i = int(k[1:])
        v = np.atleast_1d(np.asarray(v))
        if v.dtype.kind in "ui":
            w[i:i + v.size] = v.astype(np.uint32)
        else:
            fl[i:i + v.size] = v.astype(np.float32)
    return w


def _scene():
    sc, info = scenes.cornell_adjoint(8, 8)
    b = sc.blobs()
    return sc, info, b


def _mat(sc, name):
    return sc.mat_ref["m_" + name]


def test_decode_materials():
    sc, info, b = _scene()
    left = FD.decode_material(b["materials"], _mat(sc, "left"))
    assert [c["id"] for c in left] == [FD.ME_DIFFUSE]
    assert left[0]["c0"] == info["albedo_tex"][0] and left[0]["a"] == info["rough_tex"][0]
    floor = FD.decode_material(b["materials"], _mat(sc, "floor"))
    assert [c["id"] for c in floor] == [FD.ME_DIFFUSE, FD.ME_NEWWARD]
    assert floor[1]["a"] == floor[1]["b"] == info["rough_tex"][2]
    sph = FD.decode_material(b["materials"], _mat(sc, "sphere"))
    assert [c["id"] for c in sph] == [FD.ME_ASH_S, FD.ME_ASH_D]
    assert sph[1]["c0"] == info["albedo_tex"][7]  # Rd
    P = FD.Params(b["textures"])
    assert np.allclose(P.color(info["albedo_tex"][0]), (0.63, 0.06, 0.06), atol=1e-7)
    assert abs(P.scalar(info["rough_tex"][7]) - 40.0) < 1e-6


def test_lambert_limit_and_reciprocity():
    sc, info, b = _scene()
    P = FD.Params(b["textures"])
    rng = np.random.default_rng(1)
    vo = rng.normal(size=(64, 3))
    vi = rng.normal(size=(64, 3))
    vo[:, 2], vi[:, 2] = np.abs(vo[:, 2]), np.abs(vi[:, 2])
    vo /= np.linalg.norm(vo, axis=1, keepdims=True)
    vi /= np.linalg.norm(vi, axis=1, keepdims=True)
    for name in ("left", "floor", "sphere"):
        for c in FD.decode_material(b["materials"], _mat(sc, name)):
            if c["id"] == FD.ME_ASH_S:
                continue  # Ashikhmin-Shirley's max(|cos|) denominator is symmetric, its Fresnel is not
            assert np.allclose(FD.comp_f(c, P, vo, vi), FD.comp_f(c, P, vi, vo), rtol=1e-12)
    # sigma = 0: Oren-Nayar is Lambert
    c = dict(FD.decode_material(b["materials"], _mat(sc, "left"))[0])
    P.values[c["a"]] = np.array([0.0])
    f = FD.comp_f(c, P, vo, vi)
    assert np.allclose(f, np.array([0.63, 0.06, 0.06]) / np.pi, rtol=1e-6)
    # opposite hemispheres reflect nothing
    assert np.all(FD.comp_f(c, P, vo, -vi) == 0)


def test_path_assembly_and_differences():
    sc, info, b = _scene()
    left, floor = _mat(sc, "left"), _mat(sc, "floor")
    vo0, vi0 = np.array([0.3, 0.1, 0.9]), np.array([-0.2, 0.4, 0.8])
    vo0 /= np.linalg.norm(vo0)
    vi0 /= np.linalg.norm(vi0)
    vo0, vi0 = vo0.astype(np.float32).astype(np.float64), vi0.astype(np.float32).astype(np.float64)  # as taped
    refl = FD.TY_REFLECTION | FD.TY_DIFFUSE | FD.TY_GLOSSY | FD.TY_SPECULAR  # transmission masked off
    recs = [  # shuffled: the evaluator orders by pixel, sample, depth, kind
        _rec(3, 0, 1, FD.NEE | FD.VISIBLE, f4=0.5, f5=[1.0, 2.0, 3.0], w8=np.uint32(FD.NONE32), w10=np.uint32(floor),
             f13=vo0, f16=vi0, w19=np.uint32(refl)),
        _rec(3, 0, 0, FD.CAM, f4=[1.0, 1.0, 1.0]),
        _rec(3, 0, 1, FD.EMIT, f4=0.25, f5=[4.0, 4.0, 4.0], w8=np.uint32(FD.NONE32)),
        _rec(3, 0, 0, FD.SAMPLE, f4=2.0, w10=np.uint32(left), f13=vo0, f16=vi0, w19=np.uint32(refl)),
        _rec(3, 0, 1, FD.RR, f4=1.25),
        _rec(5, 1, 0, FD.CAM, f4=[0.5, 0.5, 0.5]),
        _rec(5, 1, 0, FD.NEE, f4=9.0, f5=[1.0, 1.0, 1.0], w8=np.uint32(FD.NONE32), w10=np.uint32(left),
             f13=vo0, f16=vi0, w19=np.uint32(refl)),  # not visible: no term
        _rec(5, 1, 0, FD.EMIT, f4=1.0, f5=[0.0, 1.0, 0.0], w8=np.uint32(FD.NONE32)),
    ]
    tape = np.stack(recs)
    dloss = np.zeros((8, 4))
    dloss[3, :3] = (1.0, 0.5, 0.25)
    dloss[5, :3] = (2.0, 2.0, 2.0)
    fp = FD.FrozenPaths(tape, b, dloss)
    P = FD.Params(b["textures"])
    ctop = FD.decode_material(b["materials"], left)
    cfl = FD.decode_material(b["materials"], floor)
    f_left = FD.comp_f(ctop[0], P, vo0[None], vi0[None])[0]
    f_floor = sum(FD.comp_f(c, P, vo0[None], vi0[None])[0] for c in cfl)
    a1 = 2.0 * f_left
    term3 = a1 * 0.25 * 4.0 + a1 * 1.25 * 0.5 * np.array([1.0, 2.0, 3.0]) * f_floor
    term5 = 0.5 * np.array([0.0, 1.0, 0.0])
    want = float(dloss[3, :3] @ term3 + dloss[5, :3] @ term5)
    assert abs(fp.loss(P) - want) <= 1e-12 * abs(want)
    img = fp.image(P, 8)
    assert np.allclose(img[3], term3) and np.allclose(img[5], term5)
    # the loss is linear in the left wall's albedo: the central difference is exact
    off = info["albedo_tex"][0]
    R = P.color(off)
    for c in range(3):
        d = fp.fd_texture(P, off, c, 1e-4)
        assert abs(d - want_dR(dloss, a1, f_left, f_floor, R, c)) <= 1e-7 * max(1.0, abs(d))


def want_dR(dloss, a1, f_left, f_floor, R, c):
    # term3 is proportional to f_left, which is proportional to R (channel-wise)
    t = 0.25 * 4.0 + 1.25 * 0.5 * np.array([1.0, 2.0, 3.0])[c] * f_floor[c]
    return float(dloss[3, c] * 2.0 * f_left[c] / R[c] * t)
