"""FP64 re-evaluation of recorded paths: the finite-difference check of the
adjoint renderer (test infrastructure only; the shipped library never
imports it).

The adjoint renderer differentiates the path-tracing estimator with its
sampling decisions held fixed (directions, pdfs, MIS weights, light choice
and roulette probabilities).  Its optional tape records, for every replayed
sample, each factor of that estimator:

  CAM    alpha0                      throughput starts at the camera weight
  EMIT   term += alpha * w * Le      (Le = env texel * multiplier for the
                                      differentiated environment texture)
  RR     alpha *= 1 / q
  NEE    term += alpha * s * Le * fs(vout, vin)   (if the light was visible)
  SAMPLE alpha *= fs(vout, vin) * |cos| / pdf

``FrozenPaths.loss(params)`` evaluates sum_p dLoss/dAccum_p . Accum_p over
those records in float64 with the material and environment parameters of
``params``; central differences of it with respect to one parameter give the
derivative that the adjoint renderer must reproduce.

The BSDF values are a float64 restatement of the reference's BxDF functions
(OpenCL/reflection.cl): fx :500-583 (Oren-Nayar diffuse, NewWard,
Ashikhmin-Shirley specular and diffuse), the specular samples of sample_fx
:404-438, the Fresnel terms :345-390, and fs's sum over the components that
match the reflection / transmission side :679-702.  Only constant textures
(texture.cl:58-74, 147-150) are parameters; every material of a recorded
path must read constant textures.
"""
from __future__ import annotations

import struct

import numpy as np

CAM, EMIT, RR, NEE, SAMPLE = range(5)
VISIBLE = 0x100
SPECULAR_SAMPLE = 0x80000000
NONE32 = 0xFFFFFFFF

ME_DIFFUSE, ME_SPEC_R, ME_SPEC_T, ME_NEWWARD, ME_ASH_S, ME_ASH_D = range(6)
TY_REFLECTION, TY_TRANSMISSION, TY_DIFFUSE, TY_GLOSSY, TY_SPECULAR = 1, 2, 4, 8, 16
TEX_COLOR_CONSTANT, TEX_FLOAT_CONSTANT = 0, 6
FRESNEL_NOOP, FRESNEL_CONDUCTOR, FRESNEL_DIELECTRIC = 0, 1, 2

_TYPE = {ME_DIFFUSE: TY_REFLECTION | TY_DIFFUSE, ME_SPEC_R: TY_REFLECTION | TY_SPECULAR,
         ME_SPEC_T: TY_TRANSMISSION | TY_SPECULAR, ME_NEWWARD: TY_REFLECTION | TY_GLOSSY,
         ME_ASH_S: TY_REFLECTION | TY_GLOSSY, ME_ASH_D: TY_REFLECTION | TY_DIFFUSE}
_SIZE = {ME_SPEC_T: 20, ME_NEWWARD: 16, ME_ASH_S: 16}


def _u32(b: np.ndarray, off: int) -> int:
    return struct.unpack_from("<I", b, off)[0]


def _f32(b: np.ndarray, off: int) -> float:
    return struct.unpack_from("<f", b, off)[0]


def decode_material(materials: np.ndarray, off: int) -> list[dict]:
    """Components of the material at `off` (MaterialInfo, then 4-byte
    aligned elements; reflection.cl:185-342)."""
    m = memoryview(materials.tobytes())
    num = m[off]
    comps, o = [], off + 8
    for _ in range(num):
        o = (o + 3) & ~3
        cid = m[o]
        c = {"id": cid, "type": _TYPE.get(cid, TY_REFLECTION | TY_DIFFUSE), "c0": None, "c1": None, "a": None,
             "b": None}
        if cid == ME_DIFFUSE:
            c["c0"], c["a"] = _u32(m, o + 4), _u32(m, o + 8)
        elif cid == ME_SPEC_R:
            c["c0"], c["fresnel"] = _u32(m, o + 4), _u32(m, o + 8)
        elif cid == ME_SPEC_T:
            c["c0"], c["eta"] = _u32(m, o + 4), (_f32(m, o + 8), _f32(m, o + 12))
            c["fresnel"] = _u32(m, o + 16)
        elif cid in (ME_NEWWARD, ME_ASH_S):
            c["c0"], c["a"], c["b"] = _u32(m, o + 4), _u32(m, o + 8), _u32(m, o + 12)
        elif cid == ME_ASH_D:
            c["c0"], c["c1"] = _u32(m, o + 8), _u32(m, o + 4)  # Rd, Rs
        else:
            raise NotImplementedError(f"material element id {cid}")
        comps.append(c)
        o += _SIZE.get(cid, 12)
    return comps


class Params:
    """Parameter values: constant textures by textures-blob offset (colour:
    3 floats, float: 1) and the environment's texels (texels x 3)."""

    def __init__(self, textures: np.ndarray, env: np.ndarray | None = None):
        self.textures = memoryview(np.ascontiguousarray(textures).tobytes())
        self.values: dict[int, np.ndarray] = {}
        self.env = None if env is None else np.asarray(env, dtype=np.float64).reshape(-1, 3)

    def copy(self) -> "Params":
        p = Params.__new__(Params)
        p.textures = self.textures
        p.values = {k: v.copy() for k, v in self.values.items()}
        p.env = None if self.env is None else self.env.copy()
        return p

    def color(self, off: int) -> np.ndarray:
        if off not in self.values:
            if self.textures[off] != TEX_COLOR_CONSTANT:
                raise NotImplementedError(f"colour texture {off} is not constant")
            self.values[off] = np.array(struct.unpack_from("<3f", self.textures, off + 16), dtype=np.float64)
        return self.values[off]

    def scalar(self, off: int) -> float:
        if off not in self.values:
            if self.textures[off] != TEX_FLOAT_CONSTANT:
                raise NotImplementedError(f"float texture {off} is not constant")
            self.values[off] = np.array([_f32(self.textures, off + 4)], dtype=np.float64)
        return float(self.values[off][0])


def _fresnel(others: memoryview, off: int, cosi: np.ndarray) -> np.ndarray:
    """reflection.cl:345-390 in float64; (n, 3)."""
    kind = others[off]
    n = cosi.shape[0]
    if kind == FRESNEL_NOOP:
        return np.ones((n, 3))
    if kind == FRESNEL_CONDUCTOR:
        eta = np.array(struct.unpack_from("<3f", others, off + 16), dtype=np.float64)
        k = np.array(struct.unpack_from("<3f", others, off + 32), dtype=np.float64)
        c = np.abs(cosi)[:, None]
        tmp = (eta * eta + k * k) * c * c
        r_parl2 = (tmp - 2 * eta * c + 1) / (tmp + 2 * eta * c + 1)
        tmp_f = eta * eta + k * k
        r_perp2 = (tmp_f - 2 * eta * c + c * c) / (tmp_f + 2 * eta * c + c * c)
        return (r_parl2 + r_perp2) / 2
    if kind == FRESNEL_DIELECTRIC:
        ei0, et0 = _f32(others, off + 4), _f32(others, off + 8)
        c = np.clip(cosi, -1.0, 1.0)
        entering = c > 0
        ei = np.where(entering, ei0, et0)
        et = np.where(entering, et0, ei0)
        sint = ei / et * np.sqrt(np.maximum(0.0, 1 - c * c))
        cost = np.sqrt(np.maximum(0.0, 1 - sint * sint))
        c = np.abs(c)
        r_parl = (et * c - ei * cost) / (et * c + ei * cost)
        r_perp = (ei * c - et * cost) / (ei * c + et * cost)
        v = np.where(sint >= 1.0, 1.0, (r_parl * r_parl + r_perp * r_perp) / 2)
        return np.repeat(v[:, None], 3, axis=1)
    return np.zeros((n, 3))


def _sin_theta(v):
    return np.sqrt(np.maximum(1 - v[:, 2] ** 2, 0.0))


def _cos_phi(v, s):
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.where(s == 0, 1.0, np.clip(v[:, 0] / np.where(s == 0, 1, s), -1, 1))


def _sin_phi(v, s):
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.where(s == 0, 0.0, np.clip(v[:, 1] / np.where(s == 0, 1, s), -1, 1))


def _normalize(v):
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def comp_f(c: dict, P: Params, vo: np.ndarray, vi: np.ndarray) -> np.ndarray:
    """fx of one component, reflection.cl:500-583, float64, (n, 3)."""
    n = vo.shape[0]
    same = (vi[:, 2] * vo[:, 2] > 0)[:, None]
    cid = c["id"]
    if cid == ME_DIFFUSE:
        R, sigma = P.color(c["c0"]), P.scalar(c["a"])
        s2 = sigma * sigma
        A = 1 - s2 / (2 * (s2 + 0.33))
        B = 0.45 * s2 / (s2 + 0.09)
        sti, sto = _sin_theta(vi), _sin_theta(vo)
        dcos = _cos_phi(vi, sti) * _cos_phi(vo, sto) + _sin_phi(vi, sti) * _sin_phi(vo, sto)
        max_cos = np.where((sti > 1e-4) & (sto > 1e-4), np.maximum(0.0, dcos), 0.0)
        big_in = np.abs(vi[:, 2]) > np.abs(vo[:, 2])
        sin_a = np.where(big_in, sto, sti)
        with np.errstate(divide="ignore", invalid="ignore"):
            tan_b = np.where(big_in, sti / np.abs(vi[:, 2]), sto / np.abs(vo[:, 2]))
        f = R[None, :] / np.pi * (A + B * max_cos * sin_a * tan_b)[:, None]
        return np.where(same, f, 0.0)
    if cid in (ME_SPEC_R, ME_SPEC_T):
        return np.zeros((n, 3))
    if cid == ME_NEWWARD:
        R, ax, ay = P.color(c["c0"]), P.scalar(c["a"]), P.scalar(c["b"])
        h = _normalize(vo + vi)
        hx, hy, dn = h[:, 0] / ax, h[:, 1] / ay, np.abs(h[:, 2])
        di = np.sum(h * vi, axis=1)
        k = np.exp(-(hx * hx + hy * hy) / (dn * dn)) / (4 * np.pi * ax * ay * di * di * dn ** 4)
        return np.where(same, R[None, :] * k[:, None], 0.0)
    if cid == ME_ASH_S:
        Rs, nu, nv = P.color(c["c0"]), P.scalar(c["a"]), P.scalar(c["b"])
        h = _normalize(vo + vi)
        dv = np.sum(h * vo, axis=1)
        e = (nu * h[:, 0] ** 2 + nv * h[:, 1] ** 2) / (1 - h[:, 2] ** 2)
        g = np.sqrt((nu + 1) * (nv + 1)) / (8 * np.pi) * np.abs(h[:, 2]) ** e / (
            dv * np.maximum(np.abs(vo[:, 2]), np.abs(vi[:, 2])))
        fr = Rs[None, :] + (1 - Rs[None, :]) * ((1 - dv) ** 5)[:, None]
        return np.where(same, g[:, None] * fr, 0.0)
    if cid == ME_ASH_D:
        Rd, Rs = P.color(c["c0"]), P.color(c["c1"])
        go = 1 - (1 - np.abs(vo[:, 2]) / 2) ** 5
        gi = 1 - (1 - np.abs(vi[:, 2]) / 2) ** 5
        f = (28 * Rd / (23 * np.pi) * (1 - Rs))[None, :] * (go * gi)[:, None]
        return np.where(same, f, 0.0)
    raise NotImplementedError(cid)


def comp_specular(c: dict, P: Params, others: memoryview, vo: np.ndarray, vi: np.ndarray) -> np.ndarray:
    """Value a sampled specular component returns, reflection.cl:404-438."""
    F = _fresnel(others, c["fresnel"], vo[:, 2])
    col = P.color(c["c0"])[None, :]
    if c["id"] == ME_SPEC_R:
        return col * F / np.abs(vi[:, 2])[:, None]
    return (1 - F) * col / np.abs(vi[:, 2])[:, None]


def _textures_of(comps: list[dict]) -> set[int]:
    return {c[k] for c in comps for k in ("c0", "c1", "a", "b") if c.get(k) is not None}


class FrozenPaths:
    """A tape (records x 32 uint32) with the scene blobs and dLoss/dAccum
    (pixels x 4)."""

    def __init__(self, tape: np.ndarray, blobs: dict, dloss: np.ndarray):
        t = np.ascontiguousarray(tape, dtype=np.uint32)
        f = t.view(np.float32).astype(np.float64)
        self.n = t.shape[0]
        self.pixel = t[:, 0].astype(np.int64)
        self.sample = t[:, 1].astype(np.int64)
        self.depth = t[:, 2].astype(np.int64)
        self.kind = (t[:, 3] & 0xFF).astype(np.int64)
        self.visible = (t[:, 3] & VISIBLE) != 0
        self.f = f
        self.texel = np.where(t[:, 8] == NONE32, -1, t[:, 8].astype(np.int64))
        self.mat = t[:, 10].astype(np.int64)
        self.flags = t[:, 19].astype(np.uint64)
        self.others = memoryview(np.ascontiguousarray(blobs["others"]).tobytes())
        self.materials = np.ascontiguousarray(blobs["materials"])
        self.dloss = np.asarray(dloss, dtype=np.float64)[:, :3]
        # path order: (pixel, sample), then depth, then record kind
        key = ((self.pixel * (self.sample.max(initial=0) + 1) + self.sample) * 4096 + self.depth) * 8 + self.kind
        self.order = np.argsort(key, kind="stable")
        path = (self.pixel * (self.sample.max(initial=0) + 1) + self.sample)[self.order]
        start = np.ones(self.n, dtype=bool)
        start[1:] = path[1:] != path[:-1]
        first = np.maximum.accumulate(np.where(start, np.arange(self.n), 0))
        self.pos = np.arange(self.n) - first  # position of each sorted record within its path
        self.max_pos = int(self.pos.max(initial=0))
        self.comps = {m: decode_material(self.materials, int(m)) for m in np.unique(self.mat[self.kind >= NEE])}
        self.tex_records = {}
        for m, comps in self.comps.items():
            rec = np.nonzero(((self.kind == NEE) | (self.kind == SAMPLE)) & (self.mat == m))[0]
            for off in _textures_of(comps):
                self.tex_records.setdefault(off, []).append(rec)
        self.tex_records = {k: np.concatenate(v) for k, v in self.tex_records.items()}

    # -- factors ---------------------------------------------------------
    def _le(self, idx: np.ndarray, P: Params) -> np.ndarray:
        le = self.f[idx, 5:8].copy()
        tx = self.texel[idx]
        env = tx >= 0
        if np.any(env):
            if P.env is None:
                raise ValueError("records read the environment texture but no texels were given")
            le[env] = P.env[tx[env]] * self.f[idx[env], 9][:, None]
        return le

    def _bsdf(self, idx: np.ndarray, P: Params) -> np.ndarray:
        out = np.zeros((idx.size, 3))
        for m in np.unique(self.mat[idx]):
            sel = np.nonzero(self.mat[idx] == m)[0]
            r = idx[sel]
            vo, vi = self.f[r, 13:16], self.f[r, 16:19]
            flags = self.flags[r]
            comps = self.comps[int(m)]
            spec = (flags & SPECULAR_SAMPLE) != 0
            val = np.zeros((r.size, 3))
            for k, c in enumerate(comps):
                match = ((c["type"] & flags) == c["type"]) & ~spec
                if np.any(match):
                    val[match] += comp_f(c, P, vo[match], vi[match])
                pick = spec & ((flags & 0xFF) == k)
                if np.any(pick):
                    val[pick] = comp_specular(c, P, self.others, vo[pick], vi[pick])
            out[sel] = val
        return out

    def factors(self, P: Params, idx: np.ndarray | None = None):
        """(mul, val) of records idx: the throughput factor (CAM, RR,
        SAMPLE) and the emitted term before the throughput (EMIT, NEE)."""
        idx = np.arange(self.n) if idx is None else idx
        mul = np.ones((idx.size, 3))
        val = np.zeros((idx.size, 3))
        k = self.kind[idx]
        s = k == CAM
        mul[s] = self.f[idx[s], 4:7]
        s = k == RR
        mul[s] = self.f[idx[s], 4][:, None]
        s = np.nonzero(k == EMIT)[0]
        val[s] = self.f[idx[s], 4][:, None] * self._le(idx[s], P)
        s = np.nonzero((k == NEE) & self.visible[idx])[0]
        if s.size:
            val[s] = self.f[idx[s], 4][:, None] * self._le(idx[s], P) * self._bsdf(idx[s], P)
        s = np.nonzero(k == SAMPLE)[0]
        if s.size:
            mul[s] = self.f[idx[s], 4][:, None] * self._bsdf(idx[s], P)
        return mul, val

    def assemble(self, mul: np.ndarray, val: np.ndarray) -> float:
        """sum_p dLoss_p . sum of the terms of pixel p's paths."""
        o = self.order
        m, v = mul[o], val[o]
        alpha = np.ones((self.n, 3))  # throughput before each record
        for j in range(1, self.max_pos + 1):
            s = np.nonzero(self.pos == j)[0]
            alpha[s] = alpha[s - 1] * m[s - 1]
        contrib = alpha * v
        return float(np.sum(self.dloss[self.pixel[o]] * contrib))

    def loss(self, P: Params) -> float:
        return self.assemble(*self.factors(P))

    def image(self, P: Params, npix: int) -> np.ndarray:
        """Accumulated radiance per pixel (npix x 3) of the recorded paths."""
        mul, val = self.factors(P)
        o = self.order
        m, v = mul[o], val[o]
        alpha = np.ones((self.n, 3))
        for j in range(1, self.max_pos + 1):
            s = np.nonzero(self.pos == j)[0]
            alpha[s] = alpha[s - 1] * m[s - 1]
        img = np.zeros((npix, 3))
        np.add.at(img, self.pixel[o], alpha * v)
        return img

    # -- central differences ------------------------------------------
    def fd_texture(self, P: Params, off: int, channel: int, h: float, base=None) -> float:
        """d loss / d (texture `off`, channel) by central differences; only
        the records of materials reading that texture are re-evaluated."""
        mul0, val0 = base if base is not None else self.factors(P)
        idx = self.tex_records.get(off)
        if idx is None:
            return 0.0
        out = []
        for sgn in (1.0, -1.0):
            Q = P.copy()
            if Q.textures[off] == TEX_COLOR_CONSTANT:
                Q.color(off)
            else:
                Q.scalar(off)
            Q.values[off][channel] += sgn * h
            mul, val = mul0.copy(), val0.copy()
            mul[idx], val[idx] = self.factors(Q, idx)
            out.append(self.assemble(mul, val))
        return (out[0] - out[1]) / (2 * h)

    def fd_env(self, P: Params, texel: int, channel: int, h: float, base=None) -> float:
        mul0, val0 = base if base is not None else self.factors(P)
        idx = np.nonzero(self.texel == texel)[0]
        if idx.size == 0:
            return 0.0
        out = []
        for sgn in (1.0, -1.0):
            Q = P.copy()
            Q.env[texel, channel] += sgn * h
            mul, val = mul0.copy(), val0.copy()
            mul[idx], val[idx] = self.factors(Q, idx)
            out.append(self.assemble(mul, val))
        return (out[0] - out[1]) / (2 * h)
