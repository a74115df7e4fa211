"""Spectral oracle (Jakob-Hanika RGB -> 4-wavelength spectrum, hyperbolic
wavelength sampling, spectrum -> XYZ -> RGB) over the committed fixtures
written by MRay's own LUT generator and colour tables
(tests/golden/make_spectral.py).  CPU only."""
import os

import numpy as np
import pytest

import oracle
from mray_gb300 import scenes, spectral

GOLD = os.path.join(os.path.dirname(__file__), "golden")
LUT = os.path.join(GOLD, "REC_709_r32.mrspectra")
TABLES = os.path.join(GOLD, "spectral_rec709.npz")


@pytest.fixture(scope="module")
def S():
    return oracle.Spectral(LUT, TABLES)


def test_fixture_format():
    res, lut = spectral.read_mrspectra(LUT)
    assert res == 32 and lut.size == 9 * 32 ** 3 and np.all(np.isfinite(lut))
    t = spectral.load_tables(TABLES)
    assert t["cie_xyz"].shape == (471, 3) and int(t["cie_start"]) == 360
    # the rows of RGB -> XYZ and XYZ -> RGB are inverse
    m = t["rgb_to_xyz"].reshape(3, 3).astype(np.float64) @ t["xyz_to_rgb"].reshape(3, 3).astype(np.float64)
    np.testing.assert_allclose(m, np.eye(3), atol=1e-5)


def _xi(n=1024):
    # equally spaced like MRay's own spectrum test (Tests/Tracer/T_Spectrum.cu:107-116)
    return (np.arange(n) * ((1 << 24) // n)) / float(1 << 24)


def test_wavelength_pdf(S):
    w = np.array([S.sample_waves(x)[0] for x in _xi()])
    p = np.array([S.sample_waves(x)[1] for x in _xi()])
    assert w.min() >= 360.0 and w.max() <= 830.0
    # E[1 / pdf] = length of the sampled range (PBRT's visible-wavelength density)
    assert abs(np.mean(1.0 / p) - 470.0) < 0.01 * 470.0


COLORS = [(0.00368, 0.00304, 0.01033), (0, 0, 0), (0.5, 0.5, 0.5), (1, 1, 1), (0.85, 0.15, 0.15),
          (0.15, 0.85, 0.15), (0.15, 0.15, 0.85), (15, 15, 15)]


@pytest.mark.parametrize("col", COLORS + [tuple(np.random.default_rng(0).random(3))])
def test_radiance_round_trip(S, col):
    """An emitter's RGB survives RGB -> spectrum (with the illuminant) ->
    XYZ -> RGB, averaged over the wavelength samples."""
    acc = np.zeros(3)
    for x in _xi():
        w, p = S.sample_waves(x)
        acc += S.to_rgb(S.convert_radiance(col, w), w, p)
    acc /= len(_xi())
    np.testing.assert_allclose(acc, col, rtol=0.03, atol=0.01)    # the reference test allows 0.1


@pytest.mark.parametrize("col", [(0.5, 0.5, 0.5), (0.8, 0.3, 0.1), (0.1, 0.6, 0.3), (0.2, 0.2, 0.7)])
def test_albedo_under_white_light(S, col):
    """A reflectance lit by an RGB-white emitter reads back as itself."""
    acc = np.zeros(3)
    for x in _xi():
        w, p = S.sample_waves(x)
        s = S.convert_albedo(col, w) * S.convert_radiance((1.0, 1.0, 1.0), w)
        acc += S.to_rgb(s, w, p)
    acc /= len(_xi())
    np.testing.assert_allclose(acc, col, rtol=0.05, atol=0.02)


def test_albedo_in_unit_range(S):
    rng = np.random.default_rng(4)
    for _ in range(200):
        w, _ = S.sample_waves(rng.random())
        s = S.convert_albedo(rng.random(3), w)
        assert np.all((s >= 0.0) & (s <= 1.0))


def test_spectral_box_render_matches_rgb_mean(S):
    """The spectral box scene's image mean is within a few percent of the RGB
    render's (same scene, different colour model)."""
    pts = oracle.PtScene(scenes.box_scene(0))
    ptr = oracle.PtScene(scenes.box_scene(0), spectral=S)
    cam = scenes.box_camera()
    a = pts.render(pts.params(32, 32, 32, cam, seed=1))
    b = ptr.render(ptr.params(32, 32, 32, cam, seed=1))
    ma = (a[..., :3] / a[..., 3:]).mean(axis=(0, 1))
    mb = (b[..., :3] / b[..., 3:]).mean(axis=(0, 1))
    np.testing.assert_allclose(mb, ma, rtol=0.08)
