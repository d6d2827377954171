"""Adjoint (path-replay backpropagation) renderer against float64 finite
differences.

The scene is the differentiable Cornell box: 8 materials with an albedo
(colour) and a roughness (float) constant texture each, plus a 64 x 32
environment image.  The loss is L2 between the image (accumulation / spp) and
a target rendered with perturbed parameters.  The adjoint call records a tape
of every replayed path; oracle/adjoint_fd.py re-evaluates the same paths in
float64 and takes central differences (h = 1e-4) with the sampling decisions
frozen -- the estimator the adjoint differentiates.  Bar (stated here): per
parameter group (albedo, roughness, environment texels), the relative L2
error of the gradient over 64 sampled parameters is <= 1e-3.

``AdjointRender`` is the torch.autograd.Function wrapper of the adjoint entry
point (test harness only).
"""
import numpy as np
import pytest
import torch

from clear_gb300 import _lib, scenes
from clear_gb300.render import DeviceScene
from oracle import adjoint_fd as FD

W = H = 64
SPP = 4
DEPTH = 5
H_FD = 1e-4
TAPE_CAP = 1 << 20


def _setup(dev, width=W, height=H, **kw):
    sc, info = scenes.cornell_adjoint(width, height, **kw)
    ds = DeviceScene(sc, dev)
    tex = torch.tensor(info["albedo_tex"] + info["rough_tex"], dtype=torch.int32, device=dev)
    kind = torch.tensor([0] * 8 + [1] * 8, dtype=torch.uint8, device=dev)
    return sc, info, ds, tex, kind


def _target(dev, info, width=W, height=H, seed=11, spp=SPP):
    """Image rendered with perturbed parameters (albedo + N(0, 0.1) clamped to
    [0.01, 0.99], roughness + N(0, 0.05) (x lognormal(0, 0.05) for the
    Ashikhmin exponent), env x lognormal(0, 0.3))."""
    r = np.random.default_rng(seed)
    alb = np.clip(info["albedo"] + r.normal(0, 0.1, info["albedo"].shape), 0.01, 0.99)
    rough = info["roughness"].copy()
    rough[:7] = np.maximum(rough[:7] + r.normal(0, 0.05, 7), 0.02)
    rough[7] = rough[7] * np.exp(r.normal(0, 0.05))
    env = info["env"] * np.exp(r.normal(0, 0.3, info["env"].shape))
    sc, _ = scenes.cornell_adjoint(width, height, albedo=alb, roughness=rough, env=env)
    ds = DeviceScene(sc, dev)
    rng, pix = ds.new_frame()
    ds.render(rng, pix, spp, DEPTH, wavefront=True)
    return pix[:, :3] / spp


def _dloss(pix, target, spp=SPP):
    d = torch.zeros_like(pix)
    d[:, :3] = 2.0 * (pix[:, :3] / spp - target) / spp
    return d


def _check_groups(fp, P, info, g, ge, base, seed=2024):
    """Adjoint against FP64 central differences per parameter group: all 24
    albedo channels, all 8 roughness values and 32 environment texel channels
    drawn by a seeded generator among the texels the recorded paths read
    (chosen from the tape alone, so a texel whose adjoint gradient is wrongly
    zero is as likely to be drawn as any)."""
    groups = {"albedo": [], "roughness": [], "env": []}
    for i, off in enumerate(info["albedo_tex"]):
        for c in range(3):
            groups["albedo"].append((g[i, c], fp.fd_texture(P, off, c, H_FD, base)))
    for i, off in enumerate(info["rough_tex"]):
        groups["roughness"].append((g[8 + i, 0], fp.fd_texture(P, off, 0, H_FD, base)))
    read = np.unique(fp.texel[fp.texel >= 0])
    assert read.size >= 32
    pick = np.random.default_rng(seed).choice(read.size * 3, size=32, replace=False)
    for k in pick:
        texel, c = int(read[k // 3]), int(k % 3)
        groups["env"].append((ge[texel, c], fp.fd_env(P, texel, c, H_FD, base)))
    assert sum(len(v) for v in groups.values()) == 64
    for name, pairs in groups.items():
        a = np.array([p[0] for p in pairs])
        b = np.array([p[1] for p in pairs])
        rel = np.linalg.norm(a - b) / np.linalg.norm(b)
        print(f"{name}: relative gradient error {rel:.3e} over {len(pairs)} parameters (|fd| {np.linalg.norm(b):.3e})")
        assert np.linalg.norm(b) > 0
        assert rel <= 1e-3, (name, rel)


class AdjointRender(torch.autograd.Function):
    """image = render(albedo (8,3), roughness (8,), env texels (T,3));
    backward runs the adjoint entry point on the same RNG streams."""

    @staticmethod
    def forward(ctx, albedo, roughness, env, ds, info, tex, kind):
        _write_params(ds, info, albedo, roughness, env)
        rng, pix = ds.new_frame()
        ctx.seeds = rng.clone()
        ds.render(rng, pix, SPP, DEPTH, wavefront=True)
        ctx.ds, ctx.info, ctx.tex, ctx.kind = ds, info, tex, kind
        return pix[:, :3].clone()

    @staticmethod
    def backward(ctx, g):
        ds, info = ctx.ds, ctx.info
        dloss = torch.zeros((g.shape[0], 4), dtype=torch.float32, device=g.device)
        dloss[:, :3] = g
        grad = torch.zeros((16, 4), dtype=torch.float32, device=g.device)
        genv = torch.zeros((info["env"].shape[0] * info["env"].shape[1], 4), dtype=torch.float32, device=g.device)
        ds.render_adjoint(ctx.seeds.clone(), dloss, SPP, DEPTH, ctx.tex, ctx.kind, grad, info["env_tex"], genv)
        return grad[:8, :3], grad[8:, 0], genv[:, :3], None, None, None, None


def _write_params(ds, info, albedo, roughness, env):
    """Writes parameter values into the device textures blob (constant
    textures; the environment's RGBA16F texels)."""
    t = ds.t["textures"]
    for i, off in enumerate(info["albedo_tex"]):
        t[off + 16:off + 28].view(torch.float32)[:] = albedo[i].detach().float()
    for i, off in enumerate(info["rough_tex"]):
        t[off + 4:off + 8].view(torch.float32)[:] = roughness[i].detach().float()
    off = info["env_tex"]
    rel = int(np.frombuffer(ds.blobs["textures"][off + 12:off + 16].tobytes(), dtype=np.int32)[0])
    n = env.shape[0]
    texels = t[off + rel:off + rel + 8 * n].view(torch.float16).view(n, 4)
    texels[:, :3] = env.detach().to(torch.float16)


@pytest.mark.gpu
# depth 12: the replay pass takes the primal's hit records and next-event
# visibilities for a path's first 8 vertices and traces the deeper ones
@pytest.mark.parametrize("depth", [DEPTH, 12])
def test_adjoint_matches_fp64_finite_differences(cuda, depth):
    sc, info, ds, tex, kind = _setup(cuda)
    target = _target(cuda, info)
    rng, pix = ds.new_frame()
    seeds = rng.clone()
    ds.render(rng, pix, SPP, depth, wavefront=True)
    dloss = _dloss(pix, target)
    grad = torch.zeros((16, 4), dtype=torch.float32, device=cuda)
    T = info["env"].shape[0] * info["env"].shape[1]
    genv = torch.zeros((T, 4), dtype=torch.float32, device=cuda)
    tape = torch.zeros((TAPE_CAP, 32), dtype=torch.int32, device=cuda)
    count = torch.zeros(1, dtype=torch.int32, device=cuda)
    rng_adj = seeds.clone()
    ds.render_adjoint(rng_adj, dloss, SPP, depth, tex, kind, grad, info["env_tex"], genv, tape, count)
    torch.cuda.synchronize()
    assert _lib.device_status() == 0
    assert torch.equal(rng_adj, rng), "the adjoint must consume the forward render's random numbers"
    n = int(count.item())
    assert 0 < n <= TAPE_CAP
    assert torch.isfinite(grad).all() and torch.isfinite(genv).all()
    blobs = sc.blobs()
    fp = FD.FrozenPaths(tape[:n].cpu().numpy().view(np.uint32), blobs, dloss.cpu().numpy())
    P = FD.Params(blobs["textures"], env=info["env"])
    # the recorded paths are the rendered ones: same image up to float rounding
    img = fp.image(P, W * H)
    ref = pix[:, :3].double().cpu().numpy()
    assert abs(img.sum() - ref.sum()) <= 1e-5 * ref.sum()
    assert np.sqrt(((img - ref) ** 2).mean()) <= 1e-5 * ref.mean()

    base = fp.factors(P)
    _check_groups(fp, P, info, grad.double().cpu().numpy(), genv.double().cpu().numpy(), base)


@pytest.mark.gpu
def test_adjoint_at_the_benchmark_configuration(cuda):
    """The differentiable-render benchmark's configuration: 512 x 512, 32
    samples per pixel, depth 5, the target from parameters perturbed as the
    benchmark perturbs them.  The loss is kept on a seeded 24 x 24 window of
    pixels (the weight elsewhere is zero, so only the window's 18,432 samples
    are replayed and taped; the others still run their forward pass and
    advance their random numbers)."""
    w = h = 512
    spp = 32
    sc, info, ds, tex, kind = _setup(cuda, w, h)
    target = _target(cuda, info, w, h, spp=spp)
    rng, pix = ds.new_frame()
    seeds = rng.clone()
    ds.render(rng, pix, spp, DEPTH, wavefront=True)
    full = _dloss(pix, target, spp)
    r = np.random.default_rng(17)
    x0, y0 = (int(v) for v in r.integers(0, w - 24, size=2))
    win = torch.zeros((h, w), dtype=torch.bool, device=cuda)
    win[y0:y0 + 24, x0:x0 + 24] = True
    dloss = torch.where(win.view(-1, 1), full, torch.zeros_like(full))
    grad = torch.zeros((16, 4), dtype=torch.float32, device=cuda)
    T = info["env"].shape[0] * info["env"].shape[1]
    genv = torch.zeros((T, 4), dtype=torch.float32, device=cuda)
    tape = torch.zeros((TAPE_CAP, 32), dtype=torch.int32, device=cuda)
    count = torch.zeros(1, dtype=torch.int32, device=cuda)
    rng_adj = seeds.clone()
    ds.render_adjoint(rng_adj, dloss, spp, DEPTH, tex, kind, grad, info["env_tex"], genv, tape, count)
    torch.cuda.synchronize()
    assert _lib.device_status() == 0
    assert torch.equal(rng_adj, rng)
    n = int(count.item())
    assert 0 < n <= TAPE_CAP
    blobs = sc.blobs()
    fp = FD.FrozenPaths(tape[:n].cpu().numpy().view(np.uint32), blobs, dloss.cpu().numpy())
    P = FD.Params(blobs["textures"], env=info["env"])
    img = fp.image(P, w * h)[win.view(-1).cpu().numpy()]
    ref = pix[:, :3][win.view(-1)].double().cpu().numpy()
    assert np.sqrt(((img - ref) ** 2).mean()) <= 1e-5 * ref.mean()
    _check_groups(fp, P, info, grad.double().cpu().numpy(), genv.double().cpu().numpy(), fp.factors(P))


@pytest.mark.gpu
def test_adjoint_without_tape_and_global_sums_agree(cuda):
    """The same gradients with and without a tape, and with a parameter table
    too large for shared memory (sums go straight to the caller's buffer)."""
    sc, info, ds, tex, kind = _setup(cuda)
    target = _target(cuda, info)
    rng, pix = ds.new_frame()
    seeds = rng.clone()
    ds.render(rng, pix, SPP, DEPTH, wavefront=True)
    dloss = _dloss(pix, target)
    T = info["env"].shape[0] * info["env"].shape[1]

    def run(tex_, kind_):
        grad = torch.zeros((tex_.numel(), 4), dtype=torch.float32, device=cuda)
        genv = torch.zeros((T, 4), dtype=torch.float32, device=cuda)
        ds.render_adjoint(seeds.clone(), dloss, SPP, DEPTH, tex_, kind_, grad, info["env_tex"], genv)
        return grad[:16].double(), genv.double()

    g0, e0 = run(tex, kind)
    assert torch.isfinite(g0).all() and torch.isfinite(e0).all()
    assert torch.linalg.norm(g0) > 0 and torch.linalg.norm(e0) > 0
    # 40 entries: shared-memory atomics; 1100: global atomics (unused offsets pad the table)
    for k in (40, 1100):
        pad = torch.full((k - 16,), 0x7FFFFFF0, dtype=torch.int32, device=cuda)
        g1, e1 = run(torch.cat([tex, pad]), torch.cat([kind, torch.zeros(k - 16, dtype=torch.uint8, device=cuda)]))
        assert torch.linalg.norm(g1 - g0) <= 1e-5 * torch.linalg.norm(g0), k
        assert torch.linalg.norm(e1 - e0) <= 1e-5 * torch.linalg.norm(e0), k
    assert _lib.device_status() == 0


@pytest.mark.gpu
def test_autograd_function_matches_adjoint(cuda):
    sc, info, ds, tex, kind = _setup(cuda)
    target = _target(cuda, info)
    albedo = torch.tensor(info["albedo"], dtype=torch.float32, device=cuda, requires_grad=True)
    rough = torch.tensor(info["roughness"], dtype=torch.float32, device=cuda, requires_grad=True)
    env = torch.tensor(info["env"].reshape(-1, 3), dtype=torch.float32, device=cuda, requires_grad=True)
    img = AdjointRender.apply(albedo, rough, env, ds, info, tex, kind)
    loss = ((img / SPP - target) ** 2).sum()
    loss.backward()
    # the same through the entry point directly
    rng, pix = ds.new_frame()
    seeds = rng.clone()
    ds.render(rng, pix, SPP, DEPTH, wavefront=True)
    assert torch.equal(pix[:, :3], img.detach())
    dloss = _dloss(pix, target)
    grad = torch.zeros((16, 4), dtype=torch.float32, device=cuda)
    genv = torch.zeros((env.shape[0], 4), dtype=torch.float32, device=cuda)
    ds.render_adjoint(seeds, dloss, SPP, DEPTH, tex, kind, grad, info["env_tex"], genv)
    assert torch.allclose(albedo.grad, grad[:8, :3], rtol=1e-4, atol=1e-9)
    assert torch.allclose(rough.grad, grad[8:, 0], rtol=1e-4, atol=1e-9)
    assert torch.allclose(env.grad, genv[:, :3], rtol=1e-4, atol=1e-9)
    assert _lib.device_status() == 0


@pytest.mark.gpu
def test_adjoint_rejects_bad_arguments(cuda):
    sc, info, ds, tex, kind = _setup(cuda, 16, 16)
    rng, _ = ds.new_frame()
    dloss = torch.zeros((256, 4), dtype=torch.float32, device=cuda)
    grad = torch.zeros((16, 4), dtype=torch.float32, device=cuda)
    with pytest.raises(_lib.ClrError):  # grad_env missing for an environment parameter
        ds.render_adjoint(rng, dloss, 1, DEPTH, tex, kind, grad, info["env_tex"], None)
    tape = torch.zeros((8, 32), dtype=torch.int32, device=cuda)
    with pytest.raises(_lib.ClrError):  # tape without a counter
        ds.render_adjoint(rng, dloss, 1, DEPTH, tex, kind, grad, None, None, tape, None)
    # a tape too small keeps counting and drops the rest (a nonzero loss
    # weight: pixels with weight zero are not replayed, hence not taped)
    count = torch.zeros(1, dtype=torch.int32, device=cuda)
    dloss[:, :3] = 1.0
    ds.render_adjoint(rng, dloss, 1, DEPTH, tex, kind, grad, None, None, tape, count)
    torch.cuda.synchronize()
    assert int(count.item()) > 8
    assert _lib.device_status() == 0


@pytest.mark.gpu
def test_adjoint_cached_and_retraced_replay_agree(cuda):
    """The replay pass takes the primal pass's hit records and next-event
    visibilities for a path's first 8 vertices, or traces those rays again
    (CLR_ADJOINT_RETRACE): the same paths, so the same gradients (up to the
    order of their atomic sums) and the same random-number states."""
    sc, info, ds, tex, kind = _setup(cuda)
    target = _target(cuda, info)
    rng, pix = ds.new_frame()
    seeds = rng.clone()
    ds.render(rng, pix, SPP, 12, wavefront=True)
    dloss = _dloss(pix, target)
    T = info["env"].shape[0] * info["env"].shape[1]
    out = []
    for retrace in (False, True):
        grad = torch.zeros((16, 4), dtype=torch.float32, device=cuda)
        genv = torch.zeros((T, 4), dtype=torch.float32, device=cuda)
        r = seeds.clone()
        ds.render_adjoint(r, dloss, SPP, 12, tex, kind, grad, info["env_tex"], genv, retrace=retrace)
        torch.cuda.synchronize()
        out.append((grad.double(), genv.double(), r))
    assert torch.equal(out[0][2], out[1][2]) and torch.equal(out[0][2], rng)
    for k in (0, 1):
        a, b = out[0][k], out[1][k]
        assert torch.allclose(a, b, rtol=1e-5, atol=1e-6 * float(a.abs().max())), k
    assert _lib.device_status() == 0
