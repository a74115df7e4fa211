"""Path-replay adjoint, CPU: the oracle's FP64-accumulated gradient against
central finite differences of the same (deterministic, counter-based RNG)
renders.  Lambert albedos are linear along every path and no sampling
decision depends on them with Russian roulette off, so the estimator is a
polynomial in the texels and finite differences are exact up to rounding."""
import numpy as np

import oracle
from mray_gb300 import scenes


def _render(tex, p):
    S = oracle.PtScene(scenes.adjoint_scene(tex, n_theta=12, n_phi=24))
    img = S.render(p)
    return img[..., :3] / img[..., 3:], S


def test_adjoint_matches_finite_differences():
    tex = scenes.value_noise_texture(8, seed=0, dtype=np.float32)
    target_tex = scenes.value_noise_texture(8, seed=1, dtype=np.float32)
    cam = scenes.box_camera()
    p = oracle.PtScene.params(16, 16, 4, cam, max_depth=4, rr_start=4, seed=5)
    img, S = _render(tex, p)
    tgt, _ = _render(target_tex, p)
    npix = img.shape[0] * img.shape[1]
    delta = np.zeros(img.shape[:2] + (4,), np.float32)
    delta[..., :3] = 2.0 * (img - tgt) / npix
    surf = len(S.surf) - 2                    # the sphere
    grad = S.adjoint(p, surf, delta)

    def loss(t):
        im, _ = _render(t, p)
        return float(np.sum((im.astype(np.float64) - tgt) ** 2) / npix)

    rng = np.random.default_rng(3)
    h = 1e-2
    checked = 0
    # the six largest gradients (texels the camera sees) and six seeded ones
    top = np.argsort(-np.abs(grad[..., :3]).ravel())[:6]
    picks = [np.unravel_index(i, (8, 8, 3)) for i in top]
    picks += [(rng.integers(0, 8), rng.integers(0, 8), rng.integers(0, 3)) for _ in range(6)]
    for (y, x, k) in picks:
        tp, tm = tex.copy(), tex.copy()
        tp[y, x, k] += h
        tm[y, x, k] -= h
        fd = (loss(tp) - loss(tm)) / (2 * h)
        g = grad[y, x, k]
        assert abs(fd - g) <= 0.02 * abs(g) + 1e-7, (y, x, k, fd, g)
        checked += abs(g) > 1e-6
    assert checked >= 6


def _scene_with_light(tex, radiance):
    surf = scenes.adjoint_scene(tex, n_theta=12, n_phi=24)
    light = [k for k, s in enumerate(surf) if s["kind"] == "light"]
    assert len(light) == 1
    surf[light[0]]["radiance"] = list(radiance)
    return surf, light[0]


def test_emission_gradient_matches_finite_differences():
    """d(loss)/d(area-light radiance): every contribution of an area light
    (a hit, or a visible NEE sample) is linear in its radiance and no
    sampling decision depends on it, so the image is linear in it and central
    differences are exact up to rounding."""
    tex = scenes.value_noise_texture(8, seed=0, dtype=np.float32)
    cam = scenes.box_camera()
    p = oracle.PtScene.params(16, 16, 4, cam, max_depth=4, rr_start=4, seed=5)
    surf = scenes.adjoint_scene(tex, n_theta=12, n_phi=24)
    light = [k for k, s in enumerate(surf) if s["kind"] == "light"][0]
    base = np.array(surf[light]["radiance"], np.float64)
    S = oracle.PtScene(surf)
    img = S.render(p)
    img = img[..., :3] / img[..., 3:]
    tgt = 0.8 * img[::-1, :, :].astype(np.float64)        # a different image of the same scale
    npix = img.shape[0] * img.shape[1]
    delta = np.zeros(img.shape[:2] + (4,), np.float32)
    delta[..., :3] = 2.0 * (img - tgt) / npix
    tgrad, egrad = S.adjoint(p, len(surf) - 2, delta, emission=True)
    # the texture gradient is unchanged by asking for the emission one too,
    # and emission only (no texture parameter) gives the same emission
    # gradient (up to the order in which worker threads' sums are added)
    assert np.allclose(tgrad, S.adjoint(p, len(surf) - 2, delta), rtol=1e-9, atol=1e-15)
    _, e2 = S.adjoint(p, None, delta, emission=True)
    assert np.allclose(e2, egrad, rtol=1e-9, atol=0)
    # only the light's entry is written
    others = np.delete(egrad, light, axis=0)
    assert not others.any()
    # linearity: radiance * gradient = sum(delta * image) per channel
    lin = np.sum(delta[..., :3].astype(np.float64) * img, axis=(0, 1))
    assert np.allclose(egrad[light, :3] * base, lin, rtol=1e-4, atol=0), (egrad[light, :3] * base, lin)

    def loss(rad):
        sr, _ = _scene_with_light(tex, rad)
        im = oracle.PtScene(sr).render(p)
        im = im[..., :3] / im[..., 3:]
        return float(np.sum((im.astype(np.float64) - tgt) ** 2) / npix)

    for k in range(3):
        h = 1e-2 * base[k]
        rp, rm = base.copy(), base.copy()
        rp[k] += h
        rm[k] -= h
        fd = (loss(rp) - loss(rm)) / (2 * h)
        g = egrad[light, k]
        assert abs(g) > 0
        assert abs(fd - g) <= 0.02 * abs(g), (k, fd, g)
