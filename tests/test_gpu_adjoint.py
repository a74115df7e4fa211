"""Path-replay adjoint on the GPU (mrg_pt_adjoint): against the oracle's
FP64 replay on a small case, and against central finite differences of the
GPU's own renders on the differentiable-rendering workload (box + 65k-triangle
displaced sphere with a 512^2 f32 albedo texture, L2 loss over a 512^2
image, 32 spp, depth 6, finite-difference step 1e-3 on 64 seeded texels
drawn uniformly, within 2%, and the host replay at that full size); the same
for the area light's radiance (d(loss)/d(emission)).
Russian roulette is off (rr_start = max_depth): with it on, its
throughput-dependent probability is treated as a constant by the adjoint."""
import numpy as np
import pytest
import torch

import oracle
from mray_gb300 import scenes
from mray_gb300.pt import PathTracer, load_box_scene

pytestmark = pytest.mark.gpu


def _tracer(tex_dev, n_theta, n_phi):
    surf = scenes.adjoint_scene(None, n_theta=n_theta, n_phi=n_phi)
    pt = PathTracer(0)
    sphere = None
    for k, s in enumerate(surf):
        inst = pt.add_surface(s["pos"], s["idx"], s["m34"], cull=s.get("cull", True), uv=s.get("uv"))
        if s["kind"] == "light":
            pt.set_area_light(inst, s["radiance"])
        else:
            pt.set_lambert(inst, s["albedo"])
        if "uv" in s:
            sphere = inst
    tid = pt.add_texture(tex_dev)
    pt.set_albedo_texture(sphere, tid)
    pt.build()
    return pt, tid, sphere


def _img(t):
    return t[..., :3] / t[..., 3:]


@pytest.mark.parametrize("spp_pass", [0, 1])
def test_adjoint_matches_oracle_small(spp_pass):
    """spp_pass 1: four passes, primal + replay each, on two pipelines."""
    tex = scenes.value_noise_texture(8, seed=0, dtype=np.float32)
    tgt_tex = scenes.value_noise_texture(8, seed=1, dtype=np.float32)
    dev = torch.from_numpy(tex.copy()).cuda()
    pt, tid, sphere = _tracer(dev, 12, 24)
    cam = scenes.box_camera()
    p = PathTracer.params(16, 16, 4, cam, max_depth=4, rr_start=4, seed=5, samples_per_pass=spp_pass)
    img = _img(pt.render(p))
    dev.copy_(torch.from_numpy(tgt_tex))
    tgt = _img(pt.render(p))
    dev.copy_(torch.from_numpy(tex))
    npix = 16 * 16
    delta = torch.zeros((16, 16, 4), dtype=torch.float32, device="cuda")
    delta[..., :3] = 2.0 * (img - tgt) / npix
    g = pt.adjoint(p, tid, delta).cpu().numpy().astype(np.float64)
    S = oracle.PtScene(scenes.adjoint_scene(tex, n_theta=12, n_phi=24))
    go = S.adjoint(oracle.PtScene.params(16, 16, 4, cam, max_depth=4, rr_start=4, seed=5), sphere,
                   delta.cpu().numpy())
    scale = np.abs(go[..., :3]).max()
    assert scale > 0
    err = np.abs(g[..., :3] - go[..., :3]).max() / scale
    print("adjoint vs oracle: max |diff| / max |grad| = %.3g" % err)
    assert err <= 1e-3
    pt.close()


def test_adjoint_finite_differences_full_size():
    rng = np.random.default_rng(11)
    tex = scenes.value_noise_texture(512, seed=0, dtype=np.float32)
    tgt_tex = scenes.value_noise_texture(512, seed=1, dtype=np.float32)
    dev = torch.from_numpy(tex.copy()).cuda()
    pt, tid, _ = _tracer(dev, 128, 256)
    cam = scenes.box_camera()
    p = PathTracer.params(512, 512, 32, cam, max_depth=6, rr_start=6, seed=7)
    img = _img(pt.render(p)).double()
    dev.copy_(torch.from_numpy(tgt_tex))
    tgt = _img(pt.render(p)).double()
    dev.copy_(torch.from_numpy(tex))
    npix = 512 * 512
    delta = torch.zeros((512, 512, 4), dtype=torch.float32, device="cuda")
    delta[..., :3] = (2.0 * (img - tgt) / npix).float()
    grad = pt.adjoint(p, tid, delta).cpu().numpy().astype(np.float64)
    # the same gradient through torch.autograd (backward = the adjoint)
    from mray_gb300.adjoint import render_albedo
    dev.requires_grad_(True)
    ag_loss = torch.sum((render_albedo(dev, pt, tid, p).double() - tgt) ** 2) / npix
    ag_loss.backward()
    assert np.array_equal(dev.grad.cpu().numpy(), grad.astype(np.float32)[..., :dev.shape[-1]]) or \
        np.abs(dev.grad.cpu().numpy() - grad[..., :dev.shape[-1]]).max() <= 1e-6 * np.abs(grad).max()
    dev.requires_grad_(False)
    dev.grad = None

    def loss():
        return float(torch.sum((_img(pt.render(p)).double() - tgt) ** 2) / npix)

    # 64 seeded texel channels drawn uniformly over the whole texture (those
    # the camera never sees must come out zero on both sides)
    dev = dev.detach()
    picks = rng.choice(512 * 512 * 3, 64, replace=False)
    gscale = float(np.abs(grad[..., :3]).max())
    h = 1e-3
    bad, rel, fds = [], [], []
    for flat in picks:
        y, x, k = np.unravel_index(flat, (512, 512, 3))
        v = float(tex[y, x, k])
        dev[y, x, k] = v + h
        lp = loss()
        dev[y, x, k] = v - h
        lm = loss()
        dev[y, x, k] = v
        fd = (lp - lm) / (2 * h)
        fds.append(fd)
        g = grad[y, x, k]
        if g != 0.0:
            rel.append(abs(fd - g) / abs(g))
        # 2% of the gradient, with a floor of 1e-6 of the largest gradient
        # for channels whose gradient is (near) zero
        if abs(fd - g) > 0.02 * abs(g) + 1e-6 * gscale:
            bad.append((int(y), int(x), int(k), fd, g))
    live = int(np.sum(grad[..., :3].ravel()[picks] != 0.0))
    print("finite differences: %d of 64 outside 2%% (%d with a nonzero gradient); relative error median %.2g, "
          "max %.2g" % (len(bad), live, float(np.median(rel)), float(np.max(rel))), bad[:4])
    assert live >= 16
    assert len(bad) <= 1, bad[:8]

    # the project's FP64-accumulated host replay at the full size, on the
    # same texels and over the whole texture
    S = oracle.PtScene(scenes.adjoint_scene(tex))
    sphere = [k for k, s_ in enumerate(scenes.adjoint_scene(None)) if "uv" in s_][0]
    go = S.adjoint(oracle.PtScene.params(512, 512, 32, cam, max_depth=6, rr_start=6, seed=7), sphere,
                   delta.cpu().numpy())
    err_all = float(np.linalg.norm(grad[..., :3] - go[..., :3]) / np.linalg.norm(go[..., :3]))
    yy, xx, kk = np.unravel_index(picks, (512, 512, 3))
    err_picks = float(np.abs(grad[yy, xx, kk] - go[yy, xx, kk]).max() / gscale)
    print("full size against the host replay: relative L2 %.3g over the texture, max %.3g on the 64 texels"
          % (err_all, err_picks))
    assert err_all <= 1e-2 and err_picks <= 1e-3
    pt.close()


def _light(n_theta, n_phi):
    surf = scenes.adjoint_scene(None, n_theta=n_theta, n_phi=n_phi)
    lights = [k for k, s in enumerate(surf) if s["kind"] == "light"]
    assert len(lights) == 1
    return len(surf), lights[0], np.array(surf[lights[0]]["radiance"], np.float64)


def test_emission_gradient_matches_oracle_small():
    """d(loss)/d(area-light radiance) beside the texture gradient, and alone
    (no texture parameter), against the oracle's FP64 replay."""
    tex = scenes.value_noise_texture(8, seed=0, dtype=np.float32)
    dev = torch.from_numpy(tex.copy()).cuda()
    pt, tid, sphere = _tracer(dev, 12, 24)
    n, light, _ = _light(12, 24)
    cam = scenes.box_camera()
    p = PathTracer.params(16, 16, 4, cam, max_depth=4, rr_start=4, seed=5, samples_per_pass=1)
    img = _img(pt.render(p))
    tgt = 0.8 * torch.flip(img, dims=[0])
    delta = torch.zeros((16, 16, 4), dtype=torch.float32, device="cuda")
    delta[..., :3] = 2.0 * (img - tgt) / (16 * 16)
    ge = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    g = pt.adjoint(p, tid, delta, grad_emission=ge).cpu().numpy().astype(np.float64)
    ge_only = torch.zeros_like(ge)
    assert pt.adjoint(p, None, delta, grad_emission=ge_only) is None
    ge, ge_only = ge.cpu().numpy().astype(np.float64), ge_only.cpu().numpy().astype(np.float64)
    S = oracle.PtScene(scenes.adjoint_scene(tex, n_theta=12, n_phi=24))
    go, geo = S.adjoint(oracle.PtScene.params(16, 16, 4, cam, max_depth=4, rr_start=4, seed=5), sphere,
                        delta.cpu().numpy(), emission=True)
    assert np.abs(geo[light, :3]).min() > 0
    assert not np.delete(ge, light, axis=0).any()
    err = np.abs(ge[:, :3] - geo[:, :3]).max() / np.abs(geo[:, :3]).max()
    print("emission gradient vs oracle: max |diff| / max |grad| = %.3g" % err, ge[light], geo[light])
    assert err <= 1e-3
    assert np.allclose(ge_only, ge, rtol=1e-5, atol=0)
    terr = np.abs(g[..., :3] - go[..., :3]).max() / np.abs(go[..., :3]).max()
    assert terr <= 1e-3
    pt.close()


def test_emission_gradient_full_size():
    """On the differentiable-rendering workload (512^2, 32 spp, depth 6): the
    image is linear in the light's radiance, so radiance * gradient equals
    sum(delta * image) per channel, and central differences of the GPU's own
    renders (radiance +- 1%) agree within 0.5%."""
    tex = scenes.value_noise_texture(512, seed=0, dtype=np.float32)
    dev = torch.from_numpy(tex.copy()).cuda()
    pt, tid, _ = _tracer(dev, 128, 256)
    n, light, rad = _light(128, 256)
    cam = scenes.box_camera()
    p = PathTracer.params(512, 512, 32, cam, max_depth=6, rr_start=6, seed=7)
    img = _img(pt.render(p)).double()
    tgt = 0.8 * torch.flip(img, dims=[0])
    npix = 512 * 512
    delta = torch.zeros((512, 512, 4), dtype=torch.float32, device="cuda")
    delta[..., :3] = (2.0 * (img - tgt) / npix).float()
    ge = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    assert pt.adjoint(p, None, delta, grad_emission=ge) is None
    ge = ge.cpu().numpy().astype(np.float64)
    lin = (delta[..., :3].double() * img).sum(dim=(0, 1)).cpu().numpy()
    print("radiance * gradient", ge[light, :3] * rad, "sum(delta * image)", lin)
    assert np.allclose(ge[light, :3] * rad, lin, rtol=1e-4, atol=0)
    # the same gradients through torch.autograd (backward = the adjoint)
    from mray_gb300.adjoint import render_scene
    dev.requires_grad_(True)
    em = torch.tensor(rad[None, :], dtype=torch.float64, requires_grad=True)
    ag_loss = torch.sum((render_scene(dev, em, pt, tid, [light], p).double() - tgt) ** 2) / npix
    ag_loss.backward()
    assert np.allclose(em.grad.numpy()[0], ge[light, :3], rtol=1e-5, atol=0)
    assert float(dev.grad.abs().max()) > 0
    dev.requires_grad_(False)

    def loss(r):
        pt.set_area_light(light, r)
        out = float(torch.sum((_img(pt.render(p)).double() - tgt) ** 2) / npix)
        pt.set_area_light(light, rad)
        return out

    for k in range(3):
        h = 1e-2 * rad[k]
        rp, rm = rad.copy(), rad.copy()
        rp[k] += h
        rm[k] -= h
        fd = (loss(rp) - loss(rm)) / (2 * h)
        print("channel %d: finite difference %.6g, adjoint %.6g" % (k, fd, ge[light, k]))
        assert abs(fd - ge[light, k]) <= 5e-3 * abs(ge[light, k])
    pt.close()


def test_emission_gradient_many_lights_with_sky():
    """The production scene (eight quad lights, a skysphere, Lambert / GGX /
    glass surfaces, RGBA8 textures) at 64x36, RGB, 2 spp, depth 5: every
    light's gradient against the oracle's; skysphere NEE samples add none."""
    from mray_gb300.pt import load_box_scene
    surf, cam = scenes.c2_scene(0, texture_size=64)
    env = dict(texels=scenes.sky_map(64, 32, seed=0))
    pt = PathTracer(0)
    load_box_scene(pt, surf)
    pt.set_env(env["texels"])
    p = PathTracer.params(64, 36, 2, cam, max_depth=5, rr_start=5, seed=3, samples_per_pass=1)
    img = _img(pt.render(p))
    delta = torch.zeros((36, 64, 4), dtype=torch.float32, device="cuda")
    delta[..., :3] = 2.0 * (img - 0.8 * torch.flip(img, dims=[0])) / (64 * 36)
    ge = torch.zeros((pt.n_instances, 4), dtype=torch.float32, device="cuda")
    assert pt.adjoint(p, None, delta, grad_emission=ge) is None
    ge = ge.cpu().numpy().astype(np.float64)
    S = oracle.PtScene(surf, env=env)
    _, geo = S.adjoint(oracle.PtScene.params(64, 36, 2, cam, max_depth=5, rr_start=5, seed=3), None,
                       delta.cpu().numpy(), emission=True)
    lights = [k for k, s in enumerate(surf) if s["kind"] == "light"]
    assert len(lights) == 8
    assert not np.delete(geo, lights, axis=0).any() and not np.delete(ge, lights, axis=0).any()
    assert np.count_nonzero(np.abs(geo[lights, :3]).max(axis=1)) >= 6
    err = np.abs(ge[:, :3] - geo[:, :3]).max() / np.abs(geo[:, :3]).max()
    print("8 lights: emission gradient vs oracle, max |diff| / max |grad| = %.3g" % err)
    assert err <= 1e-3
    # per light, against that light's own scale (gradients span four decades)
    for k in lights:
        scale = np.abs(geo[k, :3]).max()
        assert np.abs(ge[k, :3] - geo[k, :3]).max() <= 1e-3 * scale + 1e-6 * np.abs(geo).max(), (k, ge[k], geo[k])
    pt.close()
