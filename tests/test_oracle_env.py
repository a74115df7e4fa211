"""Skysphere light oracle: the piecewise-constant 2D distribution against the
properties MRay's own tests check (Source/Tests/Tracer/T_Distributions.cu,
Dist_PiecewiseConstant2D Uniform / ZeroVariance), the spherical mapping and
the bilinear texel read.  CPU only."""
import numpy as np
import pytest

import oracle
from mray_gb300 import scenes


def _xi(n, seed):
    rng = np.random.default_rng(seed)
    xi = rng.random((n, 2), dtype=np.float32)
    xi[0] = 0.0
    xi[1] = np.nextafter(np.float32(1.0), np.float32(0.0))
    return xi


def test_pwc2d_uniform():
    """Constant function: pdf 1, sample = xi, pdf_uv(sample) == pdf."""
    w, h = 384, 216
    d = oracle.Pwc2D(np.full((h, w), 12.0, np.float32))
    xi = _xi(1024, 332)
    uv, pdf = d.sample_uv(xi)
    assert np.all(np.abs(pdf - 1.0) <= 1e-3)
    np.testing.assert_allclose(uv * [w, h], xi * [w, h], atol=1e-3 * max(w, h))
    np.testing.assert_allclose(d.pdf_uv(uv), pdf, rtol=4 * np.finfo(np.float32).eps)
    assert np.all((uv >= 0.0) & (uv < 1.0))


def test_pwc2d_zero_variance():
    """f / pdf equals the integral for every sample (piecewise-constant
    importance sampling of a piecewise-constant function), with a four-texel
    'sun' of 2e4 on a [0, 10] noise floor."""
    w, h = 960, 540
    rng = np.random.default_rng(332)
    f = (rng.random((h, w), dtype=np.float32) * 10.0).astype(np.float32)
    f[h // 2:h // 2 + 2, w // 2:w // 2 + 2] = 2.0e4
    d = oracle.Pwc2D(f)
    xi = _xi(4096, 7)
    uv, pdf = d.sample_uv(xi)
    idx = np.minimum((uv * [w, h]).astype(np.int64), [w - 1, h - 1])
    est = f[idx[:, 1], idx[:, 0]] / pdf
    integral = float(f.astype(np.float64).sum()) / (w * h)
    assert np.all(np.abs(est - integral) <= 0.06), np.abs(est - integral).max()
    assert abs(est.mean() - integral) <= 0.06
    np.testing.assert_allclose(d.pdf_uv(uv), pdf, rtol=4 * np.finfo(np.float32).eps)


def test_pwc2d_cdf_shape():
    f = np.abs(np.random.default_rng(3).standard_normal((17, 33))).astype(np.float32)
    d = oracle.Pwc2D(f)
    assert np.all(np.diff(d.cdf_x, axis=1) >= 0) and np.all(np.diff(d.cdf_y) >= 0)
    assert np.all(d.cdf_x[:, -1] == 1.0) and d.cdf_y[-1] == 1.0
    rows = f.astype(np.float64).sum(1)
    np.testing.assert_allclose(d.cdf_y, np.cumsum(rows) / rows.sum(), rtol=1e-5)


def test_sphere_mapping_round_trip():
    rng = np.random.default_rng(5)
    uv = rng.random((500, 2), dtype=np.float32) * 0.98 + 0.01
    d = oracle.env_uv_to_dir(uv)
    np.testing.assert_allclose(np.linalg.norm(d, axis=1), 1.0, atol=1e-6)
    np.testing.assert_allclose(oracle.env_dir_to_uv(d), uv, atol=2e-6)
    # v = 1 is straight up (+y), v = 0 straight down; u = 0.5 faces +z
    up = oracle.env_uv_to_dir(np.array([[0.3, 1.0], [0.3, 0.0], [0.5, 0.5]], np.float32))
    np.testing.assert_allclose(up[0], [0, 1, 0], atol=1e-6)
    np.testing.assert_allclose(up[1], [0, -1, 0], atol=1e-6)
    np.testing.assert_allclose(up[2], [0, 0, 1], atol=1e-6)


def test_solid_angle_pdf_integrates_to_4pi():
    """E[1 / pdf_solid_angle] over importance samples of the sky = 4 pi."""
    tex = scenes.sky_map(64, 32, seed=2)
    d = oracle.Pwc2D(oracle.env_luminance(tex))
    uv, pdf = d.sample_uv(np.random.default_rng(9).random((20000, 2), dtype=np.float32))
    sin_phi = np.sin((1.0 - uv[:, 1].astype(np.float64)) * np.pi)
    ok = sin_phi > 0
    inv = 2.0 * np.pi ** 2 * sin_phi[ok] / pdf[ok]
    assert abs(inv.mean() - 4 * np.pi) < 0.05 * 4 * np.pi


def test_bilinear_read():
    tex = scenes.sky_map(16, 8, seed=1)
    h, w = tex.shape[:2]
    # texel centres return the texel (up to the rounding of the centre uv)
    y, x = np.meshgrid(np.arange(1, h - 1), np.arange(1, w - 1), indexing="ij")
    uv = np.stack([(x.ravel() + 0.5) / w, (y.ravel() + 0.5) / h], 1).astype(np.float32)
    np.testing.assert_allclose(oracle.env_read(tex, uv), tex[y.ravel(), x.ravel(), :3], rtol=1e-5)
    # u = 0 wraps: half the last column, half the first
    got = oracle.env_read(tex, np.array([[0.0, (3 + 0.5) / h]], np.float32))[0]
    np.testing.assert_allclose(got, 0.5 * (tex[3, -1, :3] + tex[3, 0, :3]), rtol=1e-6)


def test_luminance_of_constant_map():
    tex = np.zeros((4, 8, 4), np.float32)
    tex[..., :3] = [1.0, 1.0, 1.0]
    lum = oracle.env_luminance(tex)
    np.testing.assert_allclose(lum, 0.2126729 + 0.7151522 + 0.0721750, rtol=1e-6)


def test_sky_scene_shape():
    s = scenes.sky_scene(0)
    assert [x["kind"] for x in s].count("light") == 1
    tex = scenes.sky_map()
    assert tex.shape == (32, 64, 4) and np.all(tex[..., :3] > 0)


def test_albedo_texture_read_rgba8():
    """UNORM8 albedo texels read back as v / 255 at texel centres; uv wraps."""
    import ctypes as C
    tex = scenes.value_noise_texture(16, seed=3)
    L = oracle.lib()
    out = np.zeros(3, np.float32)
    for (x, y) in [(0, 0), (5, 7), (15, 15), (3, 12)]:
        uv = np.array([(x + 0.5) / 16 + 2.0, (y + 0.5) / 16 - 1.0], np.float32)    # wrapped twice
        L.orc_tex_read(tex.ctypes.data_as(C.c_void_p), 16, 16, 0, uv.ctypes.data_as(C.c_void_p),
                       out.ctypes.data_as(C.c_void_p))
        np.testing.assert_allclose(out, tex[y, x, :3] / 255.0, rtol=1e-4, atol=1e-6)


def test_textured_box_renders():
    S = oracle.PtScene(scenes.box_scene_textured(0, size=64))
    img = S.render(S.params(24, 24, 8, scenes.box_camera(), seed=1))
    assert np.all(np.isfinite(img)) and img[..., :3].mean() > 0
