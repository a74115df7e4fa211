"""Path-replay adjoint on the GPU (mrg_pt_adjoint): against the oracle's
FP64 replay on a small case, and against central finite differences of the
GPU's own renders on the differentiable-rendering workload (box + 65k-triangle
displaced sphere with a 512^2 f32 albedo texture, L2 loss over a 512^2
image, 32 spp, depth 6, finite-difference step 1e-3 on 64 seeded texels,
within 2%).
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

    # 64 seeded texels among those the adjoint says matter
    dev = dev.detach()
    g3 = np.abs(grad[..., :3]).ravel()
    live = np.nonzero(g3 > np.quantile(g3[g3 > 0], 0.5))[0]
    picks = rng.choice(live, 64, replace=False)
    h = 1e-3
    bad, rel = [], []
    for flat in picks:
        y, x, k = np.unravel_index(flat, (512, 512, 3))
        v = float(tex[y, x, k])
        dev[y, x, k] = v + h
        lp = loss()
        dev[y, x, k] = v - h
        lm = loss()
        dev[y, x, k] = v
        fd = (lp - lm) / (2 * h)
        g = grad[y, x, k]
        rel.append(abs(fd - g) / max(abs(g), 1e-30))
        if abs(fd - g) > 0.02 * abs(g) + 1e-9:
            bad.append((int(y), int(x), int(k), fd, g))
    print("finite differences: %d of 64 outside 2%%; relative error median %.2g, max %.2g"
          % (len(bad), float(np.median(rel)), float(np.max(rel))), bad[:4])
    assert len(bad) <= 3, bad[:8]
    pt.close()
