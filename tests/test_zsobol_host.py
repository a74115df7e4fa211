"""ZSobol oracle (oracle/zsobol_oracle.c), CPU: the MT19937 restatement
against the C++ standard's known answer, the generated Sobol matrices and
digit permutations against MRay's own tables (read from its source when the
source tree is present), the product's seeds against the oracle's, and
properties of the generator's outputs."""
import os
import re

import numpy as np
import pytest

import oracle
from oracle.build import reference_source_dir

_REF = reference_source_dir()
REF_RANDOM = os.path.join(_REF, "Tracer", "Random.cu") if _REF else None


def test_mt19937_known_answer():
    # [rand.predef]: the 10000th consecutive output of a default-seeded
    # std::mt19937 (seed 5489) is 4123659995
    assert int(oracle.mt19937(5489, 10000)[-1]) == 4123659995


@pytest.mark.skipif(REF_RANDOM is None or not os.path.exists(REF_RANDOM), reason="MRay source tree not present")
def test_tables_match_reference_source():
    m, p = oracle.zsobol_tables()
    src = open(REF_RANDOM).read()
    for d in range(3):
        blk = re.search(r"SOBOL_32_JOE_KUO_DIM_%d\s*=\s*\{(.*?)\};" % d, src, re.S).group(1)
        ref = np.array([int(x, 16) for x in re.findall(r"0x([0-9A-Fa-f]+)u", blk)], np.uint32)
        assert np.array_equal(ref, m[d]), d
    blk = re.search(r"TABLE\s*=\s*\{(.*?)\};", src, re.S).group(1)
    rows = re.findall(r"COMPOSE_48x2\((.*?)\),?\s*(?://|\})", blk + "}", re.S)
    table = np.array([[int(v) for v in re.findall(r"(\d+)ull", r)] for r in rows])
    assert table.shape == (4, 24)
    assert np.array_equal(table.T, p)


def test_seeds_are_the_mt19937_stream():
    s = oracle.zsobol_seeds(7, 5, (3 << 32) | 11)
    assert np.array_equal(s, oracle.mt19937(3 ^ 11, 35))


def test_product_seeds_match_oracle():
    from mray_gb300 import zsobol
    try:
        got = zsobol.seeds(33, 17, 0x123456789)
    except OSError:
        pytest.skip("library not built")
    assert np.array_equal(got, oracle.zsobol_seeds(33, 17, 0x123456789))


@pytest.mark.parametrize("spp", [4, 8])
def test_samples_of_a_pixel_are_distinct(spp):
    """For a fixed dimension the samples of one pixel read distinct Sobol
    indices of the pixel's block, and the scramble is a bijection, so their
    numbers are distinct."""
    w, h = 16, 12
    seeds = oracle.zsobol_seeds(w, h, 7)
    for dim in (0, 5):
        vals = np.stack([oracle.zsobol_generate(w, h, seeds, spp, s, dim, [2])
                         for s in range(spp)])            # (spp, 2, pixels)
        for k in range(2):
            for px in range(0, w * h, 37):
                assert len(set(vals[:, k, px].tolist())) == spp


def test_request_layout():
    """Request r reads dimension dim_start + (numbers before it); a 2D request
    equals the first two numbers of a 3D request only in its first number's
    Sobol dimension, so check the layout through 1D requests: request list
    [1, 1] at dim_start d gives Next(d), Next(d + 1)."""
    w, h = 8, 8
    seeds = oracle.zsobol_seeds(w, h, 1)
    a = oracle.zsobol_generate(w, h, seeds, 16, 3, 4, [1, 1])
    b0 = oracle.zsobol_generate(w, h, seeds, 16, 3, 4, [1])
    b1 = oracle.zsobol_generate(w, h, seeds, 16, 3, 5, [1])
    assert np.array_equal(a[0], b0[0]) and np.array_equal(a[1], b1[0])
    c = oracle.zsobol_generate(w, h, seeds, 16, 3, 4, [2, 3, 1])
    assert c.shape == (6, 64)


@pytest.mark.parametrize("sampler", [1, 3])
def test_oracle_render_with_sampler_is_statistically_equal(sampler):
    """The box scene at 24x24, 64 spp: the ZSobol (sampler 1) or MRay's PCG32
    (sampler 3) renders and the counter-hash renders agree in mean radiance within 2.5% (averaged over eight seeds: one
    seed's noise is about 1.4% of the mean, so the bar is about 3.5 standard
    deviations of the difference) and per pixel in
    relMSE (the 1% largest pixel errors, fireflies, left out)."""
    from mray_gb300 import scenes
    S = oracle.PtScene(scenes.box_scene(0))
    cam = scenes.box_camera()
    ma, mb = [], []
    for seed in range(3, 11):
        a = S.render(S.params(24, 24, 64, cam, seed=seed))
        b = S.render(S.params(24, 24, 64, cam, seed=seed, sampler=sampler))
        a, b = a[..., :3] / a[..., 3:], b[..., :3] / b[..., 3:]
        assert not np.array_equal(a, b)
        e = ((a - b) ** 2 / (a ** 2 + 1e-2)).ravel()
        assert float(np.mean(np.sort(e)[: int(e.size * 0.99)])) <= 0.05     # fireflies trimmed
        ma.append(a.mean())
        mb.append(b.mean())
    assert abs(np.mean(ma) - np.mean(mb)) <= 0.025 * np.mean(ma)


def test_owen_variant_keeps_stratification():
    """16 samples of one pixel, a 2D request: with the scramble's reversal
    undone every cell of the 4x4 grid (and of the 16x1 and 1x16 grids) holds
    one point, as a scrambled (0, 2)-sequence must; MRay's form does not keep
    that for every pixel."""
    def points(owen, px, py, seed):
        return np.array([[oracle.zsobol_number(px, py, seed, s, 16, 6, 0, 2, c, owen) for c in range(2)]
                         for s in range(16)], np.uint64)

    strat_mray = 0
    for px, py, seed in ((3, 5, 11), (40, 7, 12345), (0, 0, 99), (63, 63, 7)):
        p = points(True, px, py, seed)
        for bx, by in ((2, 2), (4, 0), (0, 4)):
            cells = (p[:, 0] >> np.uint64(32 - bx)) * (1 << by) + (p[:, 1] >> np.uint64(32 - by))
            assert len(set(cells.tolist())) == 16, (px, py, bx, by)
        q = points(False, px, py, seed)
        cells = (q[:, 0] >> np.uint64(30)) * 4 + (q[:, 1] >> np.uint64(30))
        strat_mray += len(set(cells.tolist())) == 16
    assert strat_mray < 4
