"""GPU guided path tracer (MRay's GuidedPTRenderer) against the CPU oracle's
wavefront restatement of it.

Both run the same schedule: per bounce, every slot's hash-grid work in the
same stage order, irradiance records applied per cell in (path, NEE, light),
then slot, order, chain locks won by the smallest slot.  They can part only
where CUDA's atan / sin / cos / exp / log and the host C library's differ by
an ulp and a decision (a grid cell, a lobe choice, a path) flips.  Bars:
  - images: |gpu - oracle| <= 1e-4 * (1 + oracle) on >= 95% of pixels and
    relMSE <= 1e-3;
  - grid: the sets of codes differ in <= 1% of the oracle's entries; on the
    shared codes, chain weights and irradiance averages agree within
    1e-4 * (1 + |oracle|) on >= 95% of them;
  - a render is bit-for-bit reproducible run to run.
"""
import numpy as np
import pytest

import oracle
from mray_gb300 import scenes
from mray_gb300.pt import PathTracer, load_box_scene
from mray_gb300 import _native as N

pytestmark = pytest.mark.gpu

EMPTY = np.uint64(0xFFFFFFFFFFFFFFFF)


def _img(a):
    a = a.cpu().numpy() if hasattr(a, "cpu") else a
    return a[..., :3] / np.maximum(a[..., 3:], 1e-30)


def relmse(a, b):
    return float(np.mean((a - b) ** 2 / (b ** 2 + 1e-2)))


def _table(codes, chain, irr):
    m = codes != EMPTY
    return {int(c): (chain[i], irr[i]) for i, c in zip(np.nonzero(m)[0], codes[m])}


@pytest.fixture(scope="module")
def box():
    pt = PathTracer(0)
    surf = load_box_scene(pt, 0)
    return pt, oracle.PtScene(surf)


def _render_both(pt, S, calls, w=32, h=32, spp=4, sampler="independent", seed=3, cam=None, depth=8, **kw):
    cam = cam or scenes.box_camera()
    pt.guide_create(**kw)
    G = S.guide(**kw)
    gi, oi = None, None
    for c in range(calls):
        pg = PathTracer.params(w, h, spp, cam, max_depth=depth, rr_start=2, seed=seed, sample_start=spp * c,
                               samples_per_pass=spp, sampler=sampler)
        po = S.params(w, h, spp, cam, max_depth=depth, rr_start=2, seed=seed, sample_start=spp * c,
                      sampler=3 if sampler == "pcg32" else 0)
        gi = pt.render_guided(pg, image=gi)
        oi = S.render_guided(po, G, spp, image=oi)
    return gi.cpu().numpy(), oi, pt.guide_read(), G.read()


def _check_images(g, o):
    g, o = _img(g), _img(o)
    close = np.abs(g - o) <= 1e-4 * (1.0 + np.abs(o))
    frac = close.all(axis=-1).mean()
    assert frac >= 0.95, frac
    assert relmse(g, o) <= 1e-3, relmse(g, o)
    return frac


def _check_grids(gs, os_):
    tg, to = _table(*gs), _table(*os_)
    assert len(to) > 0
    diff = len(set(tg) ^ set(to))
    assert diff <= 0.01 * len(to), (diff, len(to))
    shared = sorted(set(tg) & set(to))
    cg = np.array([tg[c][0] for c in shared]); co = np.array([to[c][0] for c in shared])
    ig = np.array([tg[c][1] for c in shared]); io = np.array([to[c][1] for c in shared])
    ok_w = np.abs(cg[:, 4] - co[:, 4]) <= 1e-4 * (1.0 + np.abs(co[:, 4]))
    ok_i = np.abs(ig[:, 0] - io[:, 0]) <= 1e-4 * (1.0 + np.abs(io[:, 0]))
    assert ok_w.mean() >= 0.95, ok_w.mean()
    assert ok_i.mean() >= 0.95, ok_i.mean()
    assert np.array_equal(cg[:, 5], co[:, 5]) or (cg[:, 5] == co[:, 5]).mean() >= 0.95
    return len(to), diff, float(ok_w.mean()), float(ok_i.mean())


def test_guided_box_matches_oracle(box):
    """Three calls of 4 spp (the grid learns across them), counter sampler."""
    pt, S = box
    g, o, gs, os_ = _render_both(pt, S, 3)
    frac = _check_images(g, o)
    stats = _check_grids(gs, os_)
    print("pixels close %.4f; entries %d, code differences %d, weights %.4f, irradiance %.4f" % ((frac,) + stats))


def test_guided_pcg32_matches_oracle(box):
    """MRay's independent sampler (per-pixel PCG32 streams) for the paths."""
    pt, S = box
    g, o, gs, os_ = _render_both(pt, S, 2, sampler="pcg32", seed=7)
    _check_images(g, o)
    _check_grids(gs, os_)


def test_guided_mixed_materials_matches_oracle():
    """Lambert, mirror, glass and GGX surfaces: specular vertices take no
    mixture and no NEE; the Unreal material's specularity scales the lobe
    probability."""
    pt = PathTracer(0)
    surf = load_box_scene(pt, scenes.box_scene_mixed(0))
    S = oracle.PtScene(surf)
    g, o, gs, os_ = _render_both(pt, S, 2, seed=5)
    _check_images(g, o)
    _check_grids(gs, os_)


def test_guided_mipmapped_textures_match_oracle():
    """Textured walls with mip chains: the guided shade kernel reads the
    albedo at the ray cone's level of detail like the plain one."""
    pt = PathTracer(0)
    surf = load_box_scene(pt, scenes.mipmapped(scenes.box_scene_textured(0, size=128)))
    S = oracle.PtScene(surf)
    g, o, gs, os_ = _render_both(pt, S, 2, seed=5)
    _check_images(g, o)
    _check_grids(gs, os_)
    pt.close()


def test_guided_unreal_parameter_textures_match_oracle():
    pt = PathTracer(0)
    surf = load_box_scene(pt, scenes.mipmapped(scenes.box_scene_unreal_textured(0, size=64)))
    S = oracle.PtScene(surf)
    g, o, gs, os_ = _render_both(pt, S, 2, seed=7)
    _check_images(g, o)
    _check_grids(gs, os_)
    pt.close()


def test_guided_fix_zero_weight_matches_oracle():
    """The opt-in correction of MRay's zero-weight mixture sample: GPU and
    oracle agree, and the images differ from the reproduced defect's."""
    pt = PathTracer(0)
    surf = load_box_scene(pt, 0)
    S = oracle.PtScene(surf)
    g, o, gs, os_ = _render_both(pt, S, 2, seed=5, fix_zero_weight=True)
    _check_images(g, o)
    _check_grids(gs, os_)
    g0, _, _, _ = _render_both(pt, S, 2, seed=5)
    assert not np.allclose(_img(g), _img(g0))
    pt.close()


def _spectral_pair(surf, env=None):
    import os
    from mray_gb300 import spectral
    gold = os.path.join(os.path.dirname(__file__), "golden")
    res, lut = spectral.read_mrspectra(os.path.join(gold, "REC_709_r32.mrspectra"))
    tables = spectral.load_tables(os.path.join(gold, "spectral_rec709.npz"))
    pt = PathTracer(0)
    load_box_scene(pt, surf)
    if env is not None:
        pt.set_env(env["texels"])
    pt.set_spectral(res, lut, tables)
    S = oracle.PtScene(surf, env=env, spectral=oracle.Spectral(os.path.join(gold, "REC_709_r32.mrspectra"),
                                                               os.path.join(gold, "spectral_rec709.npz")))
    return pt, S


def test_guided_spectral_sky_matches_oracle():
    """MRay's guided renderer is spectral (GuidedPathTracerSpectral): 4
    wavelengths per path, and a skysphere whose misses feed the light records
    with MIS against the uniform light sampler."""
    env = dict(texels=scenes.sky_map(64, 32, seed=0))
    pt, S = _spectral_pair(scenes.sky_scene(0), env)
    g, o, gs, os_ = _render_both(pt, S, 2, seed=4)
    _check_images(g, o)
    _check_grids(gs, os_)
    pt.close()


def test_guided_c2_scene_small():
    """The production scene (textured Lambert, GGX metal, glass, 8 area
    lights, sky, 4 wavelengths) at a small film, depth 12: the same bar as
    the plain tracer's test of that scene (98% of pixels, the rest may take
    another path after a flipped decision)."""
    surf, cam = scenes.c2_scene(0, texture_size=256)
    env = dict(texels=scenes.sky_map(128, 64, seed=0))
    pt, S = _spectral_pair(surf, env)
    g, o, gs, os_ = _render_both(pt, S, 2, w=96, h=54, spp=2, seed=2, cam=cam, depth=12)
    g, o = _img(g), _img(o)
    close = (np.abs(g - o) <= 1e-4 * (1.0 + np.abs(o))).all(axis=-1).mean()
    d = np.abs(g - o).max(axis=-1).ravel()
    keep = d <= np.quantile(d, 0.98)
    rel_kept = float(np.mean(((g - o).reshape(-1, 3)[keep]) ** 2 / (o.reshape(-1, 3)[keep] ** 2 + 1e-2)))
    print("c2 guided: close %.4f relMSE %.3g kept %.3g" % (close, relmse(g, o), rel_kept))
    assert close >= 0.95 and rel_kept <= 1e-5
    stats = _check_grids(gs, os_)
    print("c2 guided grid: entries %d, code differences %d, weights %.4f, irradiance %.4f" % stats)
    pt.close()


def test_guided_reproducible(box):
    pt, _ = box
    cam = scenes.box_camera()
    outs = []
    for _ in range(2):
        pt.guide_create()
        img = None
        for c in range(3):
            img = pt.render_guided(PathTracer.params(40, 24, 4, cam, max_depth=8, rr_start=2, seed=2,
                                                     sample_start=4 * c, samples_per_pass=4), image=img)
        outs.append((img.cpu().numpy(), _table(*pt.guide_read())))
    assert np.array_equal(outs[0][0], outs[1][0])
    a, b = outs[0][1], outs[1][1]
    assert a.keys() == b.keys()
    assert all(np.array_equal(a[k][0], b[k][0]) and np.array_equal(a[k][1], b[k][1]) for k in a)


def test_guided_learns_and_stays_near_reference(box):
    """After a few hundred samples per pixel of learning, the guided image's
    mean is within 3% of a high-spp plain render and the chains carry
    weight."""
    pt, _ = box
    cam = scenes.box_camera()
    pt.guide_create()
    img = None
    for c in range(32):
        img = pt.render_guided(PathTracer.params(64, 64, 8, cam, max_depth=8, rr_start=2, seed=1,
                                                 sample_start=8 * c, samples_per_pass=8), image=img)
    ref = pt.render(PathTracer.params(64, 64, 1024, cam, max_depth=8, rr_start=2, seed=9))
    g, r = _img(img), _img(ref)
    assert np.isfinite(g).all()
    rel = np.abs(g.mean(axis=(0, 1)) - r.mean(axis=(0, 1))) / r.mean(axis=(0, 1))
    assert (rel <= 0.03).all(), rel
    used, size = pt.guide_stats()
    codes, chain, irr = pt.guide_read()
    m = codes != EMPTY
    assert m.sum() == used and 0 < used <= 0.6 * size
    assert (chain[m, 4] > 0).sum() > 0.05 * used
    assert (chain[m, 5] <= 1024).all() and (irr[m, 1] <= 128).all()
    print("entries %d, weighted %d, relative mean error %s" % (used, int((chain[m, 4] > 0).sum()), rel))


def test_guided_errors(box):
    pt, _ = box
    cam = scenes.box_camera()
    h = pt.acc._h
    N.check(N.lib().mrg_guide_destroy(h))
    p = PathTracer.params(16, 16, 1, cam)
    import torch
    img = torch.zeros((16, 16, 4), dtype=torch.float32, device="cuda")
    import ctypes as C
    st = N.lib().mrg_pt_render_guided(h, C.byref(p), C.c_void_p(img.data_ptr()), None)
    assert st == N.MRG_ERR_NOT_BUILT
    g = N.MrgGuideParams()
    N.check(N.lib().mrg_guide_defaults(C.byref(g)))
    g.normalBits = 4
    assert N.lib().mrg_guide_create(h, C.byref(g)) == N.MRG_ERR_INVALID_ARG
    pt.guide_create()
    pz = PathTracer.params(16, 16, 1, cam, sampler="zsobol")
    assert N.lib().mrg_pt_render_guided(h, C.byref(pz), C.c_void_p(img.data_ptr()), None) == N.MRG_ERR_INVALID_ARG
