"""The oracle's guided path tracer (wavefront restatement of MRay's
GuidedPTRenderer) on the CPU: reproducible, learning (the grid fills, chains
gain weight, counts stay within MRay's caps) and converging near the plain
tracer's image.  Its building blocks are pinned to MRay's compiled code in
test_oracle_pt_golden.py; the GPU renderer is compared with it in
test_gpu_guided.py."""
import numpy as np

import oracle
from mray_gb300 import scenes

EMPTY = np.uint64(0xFFFFFFFFFFFFFFFF)


def _render(S, G, calls, w=24, h=24, spp=4, seed=3, sampler=0):
    cam = scenes.box_camera()
    img = None
    for c in range(calls):
        p = S.params(w, h, spp, cam, max_depth=8, rr_start=2, seed=seed, sample_start=spp * c, sampler=sampler)
        img = S.render_guided(p, G, spp, image=img)
    return img


def test_guided_oracle_reproducible():
    S = oracle.PtScene(scenes.box_scene(0))
    a = _render(S, S.guide(), 3)
    G = S.guide()
    b = _render(S, G, 3)
    assert np.array_equal(a, b)
    # clearing restarts the grid and the backup streams
    G.clear()
    assert np.array_equal(_render(S, G, 3), a)


def test_guided_oracle_learns_within_caps():
    S = oracle.PtScene(scenes.box_scene(0))
    G = S.guide(entry_limit=100000)
    _render(S, G, 6)
    used, size = G.stats()
    assert size == 262144                       # NextPowerOfTwo(100000 / 0.6)
    codes, chain, irr = G.read()
    m = codes != EMPTY
    assert m.sum() == used and 0 < used <= 0.6 * size
    assert (chain[m, 4] > 0).any() and (chain[m, 4] >= 0).all()
    assert (chain[m, 5] <= 1024).all() and (irr[m, 1] <= 128).all()
    assert np.isfinite(chain[m]).all() and np.isfinite(irr[m]).all()
    # an entry's cosine never exceeds its weight (MCState::EMA clamps it)
    assert (chain[m, 3] <= chain[m, 4]).all()
    # SpatioDirCode: levels are in [0, 15], normal texels of a 4 x 4 grid
    lv = (codes[m] >> np.uint64(60)).astype(np.int64)
    nc = ((codes[m] >> np.uint64(54)) & np.uint64(63)).astype(np.int64)
    assert lv.min() >= 0 and lv.max() <= 14 and nc.max() < 16


def test_guided_oracle_pcg32_streams():
    S = oracle.PtScene(scenes.box_scene(0))
    a = _render(S, S.guide(), 2, sampler=3, seed=9)
    b = _render(S, S.guide(), 2, sampler=0, seed=9)
    assert np.isfinite(a).all() and not np.array_equal(a, b)


def test_guided_oracle_learning_reduces_the_zero_weight_bias():
    """MRay's mixture sample of a zero-weight lobe is the +Y axis with pdf 0
    and the path goes on with a finite weight, so guided images of a young
    grid are biased.  As the chains gain weight, later frames come closer to
    the plain tracer's high-spp image than early ones, and end within 5 %."""
    S = oracle.PtScene(scenes.box_scene(0))
    cam = scenes.box_camera()
    G = S.guide()
    frames = []
    for c in range(24):
        p = S.params(16, 16, 8, cam, max_depth=8, rr_start=2, seed=3, sample_start=8 * c)
        frames.append(S.render_guided(p, G, 8))
    early = sum(frames[:8])
    late = sum(frames[16:])
    ref = S.render(S.params(16, 16, 512, cam, max_depth=8, rr_start=2, seed=11))
    mean = lambda im: (im[..., :3] / im[..., 3:]).mean(axis=(0, 1))
    rm = mean(ref)
    e, l = np.abs(mean(early) - rm) / rm, np.abs(mean(late) - rm) / rm
    assert e.max() > l.max(), (e, l)
    assert np.all(l < 0.05), l


def test_guided_oracle_fix_zero_weight_removes_the_young_grid_bias():
    """With the opt-in correction a vertex whose chosen lobe has no weight
    samples the material only, so even the first frames of an empty grid
    are unbiased: their mean is closer to the plain tracer's than MRay's."""
    S = oracle.PtScene(scenes.box_scene(0))
    cam = scenes.box_camera()
    ref = S.render(S.params(16, 16, 512, cam, max_depth=8, rr_start=2, seed=11))
    mean = lambda im: (im[..., :3] / im[..., 3:]).mean(axis=(0, 1))
    rm = mean(ref)
    errs = []
    for fix in (False, True):
        G = S.guide(fix_zero_weight=fix)
        img = None
        for c in range(4):
            p = S.params(16, 16, 16, cam, max_depth=8, rr_start=2, seed=3, sample_start=16 * c)
            img = S.render_guided(p, G, 16, image=img)
        errs.append(np.abs(mean(img) - rm) / rm)
    assert errs[1].max() < errs[0].max(), errs
    assert np.all(errs[1] < 0.05), errs[1]
