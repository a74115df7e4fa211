"""The oracle's texture pipeline on the CPU: MRay's mip generation
(TextureFilter.cu:126-210, KCGenerateMipmaps in its accumulate mode: an 8 x 8
stratified grid of samples over the filter's support, Gaussian weights of
sigma 0.285714 R, each sample reading the nearest parent texel found by
Graphics::ConvertPixelIndices) and the ray-cone level of detail the path
tracer reads the chain with.  The building blocks (ConvertPixelIndices, the
Gaussian filter, the cone steps) are pinned to MRay's compiled code in
test_oracle_pt_golden.py; the GPU chain and renders are compared with these
in test_gpu_pt.py."""
import numpy as np
import pytest

import oracle
from mray_gb300 import scenes


def _levels(w, h):
    return max(w, h).bit_length()


def _np_mips(tex, radius):
    """A plain numpy restatement of one chain, float32 arithmetic in the
    oracle's order, for small textures."""
    f32 = np.float32
    sigma = f32(radius) * f32(0.285714)
    xi = (f32(0.5) / f32(8)) + (f32(1) / f32(8)) * np.arange(8, dtype=f32)
    off = (xi * f32(2) * f32(radius) - f32(radius)).astype(f32)
    si = f32(1) / sigma
    g = (f32(1 / np.sqrt(2 * np.pi)) * si * np.exp(f32(-0.5) * (off * si) ** 2)).astype(f32)
    levels = []
    src = tex.astype(np.float32)
    ph, pw = src.shape[:2]
    h, w = tex.shape[:2]
    m = 1
    while pw > 1 or ph > 1:
        cw, ch = max(w >> m, 1), max(h >> m, 1)
        out = np.zeros((ch, cw, 4), np.float32)
        rx, ry = f32(pw) / f32(cw), f32(ph) / f32(ch)
        for y in range(ch):
            for x in range(cw):
                acc = np.zeros(4, np.float32)
                ws = f32(0)
                for sy in range(8):
                    py = min(max(f32(0), (f32(y) + off[sy] + f32(0.5)) * ry - f32(0.5)), f32(ph - 1))
                    iy = int(np.floor(py + f32(0.5)))
                    for sx in range(8):
                        px = min(max(f32(0), (f32(x) + off[sx] + f32(0.5)) * rx - f32(0.5)), f32(pw - 1))
                        ix = int(np.floor(px + f32(0.5)))
                        wg = f32(g[sx] * g[sy])
                        acc = (acc + wg * src[iy, ix]).astype(np.float32)
                        ws = f32(ws + wg)
                out[y, x] = acc / ws
        if tex.dtype == np.uint8:
            out = np.clip(np.floor(out + 0.5), 0, 255)
        levels.append(out.astype(tex.dtype))
        src = out.astype(np.float32)
        ph, pw = ch, cw
        m += 1
    return levels


@pytest.mark.parametrize("w,h", [(8, 16), (13, 7), (1, 5), (64, 64), (1, 1)])
def test_chain_sizes(w, h):
    tex = np.zeros((h, w, 4), np.uint8)
    chain, count = oracle.gen_mips(tex, 2.0)
    assert count == _levels(w, h)
    dims, m = [], 1
    while len(dims) + 1 < count:
        dims.append((max(w >> m, 1), max(h >> m, 1)))
        m += 1
    assert chain.size == 4 * sum(a * b for a, b in dims) == 4 * oracle.mip_chain_texels(w, h)


@pytest.mark.parametrize("dtype", [np.uint8, np.float32])
def test_constant_texture_stays_constant(dtype):
    tex = np.empty((24, 40, 4), dtype)
    tex[...] = np.array([200, 17, 0, 255] if dtype == np.uint8 else [0.7, 0.25, 0.0, 1.0], dtype)
    chain, count = oracle.gen_mips(tex, 2.0)
    assert count == 6
    assert np.array_equal(chain.reshape(-1, 4), np.broadcast_to(tex[0, 0], (chain.size // 4, 4)))


def test_mean_is_kept_and_detail_smoothed():
    tex = np.random.default_rng(3).uniform(0.0, 1.0, (64, 64, 4)).astype(np.float32)
    chain, count = oracle.gen_mips(tex, 2.0)
    lv1 = chain[:32 * 32 * 4].reshape(32, 32, 4)
    assert abs(lv1[..., :3].mean() - tex[..., :3].mean()) < 0.02 * tex[..., :3].mean()
    # a low-pass filter: white noise loses most of its variance
    assert lv1[..., :3].var() < 0.25 * tex[..., :3].var()
    # the 1 x 1 top level is near the texture's mean
    top = chain[-4:]
    assert np.allclose(top[:3], tex[..., :3].mean(axis=(0, 1)), rtol=0.05)


@pytest.mark.parametrize("dtype", [np.float32, np.uint8])
def test_chain_matches_numpy_restatement(dtype):
    rng = np.random.default_rng(4)
    tex = (rng.uniform(0, 255, (7, 13, 4)) if dtype == np.uint8 else rng.uniform(0, 1, (7, 13, 4))).astype(dtype)
    chain, count = oracle.gen_mips(tex, 1.5)
    ref = np.concatenate([l.ravel() for l in _np_mips(tex, 1.5)])
    if dtype == np.uint8:
        assert np.abs(chain.astype(int) - ref.astype(int)).max() <= 1
        assert (chain == ref).mean() > 0.95
    else:
        assert np.allclose(chain, ref, rtol=2e-6, atol=1e-7)


def _textured(mip):
    surf = scenes.box_scene_textured(0, size=128)
    return scenes.mipmapped(surf) if mip else surf


def test_ray_cone_lod_changes_the_textured_image():
    """With a chain the walls' albedo is read at the cone's level; without one
    at level 0 (MRay's LOD query on a single-level texture), so the two images
    differ on the textured walls and nowhere else much."""
    cam = scenes.box_camera()
    imgs = []
    for mip in (False, True):
        S = oracle.PtScene(_textured(mip))
        imgs.append(S.render(S.params(32, 32, 4, cam, seed=5)))
    a, b = (im[..., :3] / im[..., 3:] for im in imgs)
    assert np.isfinite(b).all()
    assert not np.allclose(a, b)
    # filtering keeps the average reflectance: whole-image means within 5%
    assert np.all(np.abs(a.mean(axis=(0, 1)) - b.mean(axis=(0, 1))) < 0.05 * a.mean(axis=(0, 1)))
    # the noise the filter removes: neighbouring pixels vary less
    assert np.abs(np.diff(b, axis=1)).mean() < np.abs(np.diff(a, axis=1)).mean()


def test_guided_oracle_reads_mips():
    cam = scenes.box_camera()
    S = oracle.PtScene(_textured(True))
    G = S.guide()
    img = S.render_guided(S.params(24, 24, 4, cam, max_depth=8, rr_start=2, seed=3), G, 4)
    assert np.isfinite(img).all() and G.stats()[0] > 0


def test_given_levels_are_kept_and_filtered_from():
    """PushTextureData of a mip level: the level is kept and the levels
    below it are filtered from it (MRay's validMips); without a generation
    filter the chain ends at the last given level."""
    rng = np.random.default_rng(8)
    tex = rng.uniform(0, 1, (16, 16, 4)).astype(np.float32)
    lv2 = np.full((4, 4, 4), 0.25, np.float32)
    full, n = oracle.gen_mips(tex, 2.0)
    chain, n2 = oracle.gen_mips(tex, 2.0, {2: lv2})
    assert n == n2 == 5
    o1, o2, o3 = (4 * oracle.mip_chain_texels(16, 16, m) for m in (1, 2, 3))
    assert np.array_equal(chain[:o2], full[:o2])               # level 1 from level 0
    assert np.array_equal(chain[o2:o3], lv2.ravel())          # level 2 as given
    assert np.allclose(chain[o3:], 0.25)                       # levels 3, 4 from the constant level 2
    only, n3 = oracle.gen_mips(tex, 0.0, {1: full[:o2].reshape(8, 8, 4), 2: lv2})
    assert n3 == 3 and np.array_equal(only, chain[:o3])
    with pytest.raises(ValueError):
        oracle.gen_mips(tex, 0.0, {2: lv2})                    # level 1 missing, no filter
    with pytest.raises(ValueError):
        oracle.gen_mips(tex, 2.0, {5: lv2})                    # past the 1 x 1 level


def test_unreal_parameter_textures_change_the_image():
    """Unreal's textured roughness / metallic / specular replace the
    constants at each hit: the image differs from the constant-parameter
    one, and textures holding constant values reproduce those constants'
    image."""
    cam = scenes.box_camera()
    surf = scenes.box_scene_unreal_textured(0, size=32)
    flat = [dict(s) for s in surf]
    for s in flat:
        for k in ("roughness_texture", "metallic_texture", "specular_texture"):
            s.pop(k, None)
    const = [dict(s) for s in flat]
    for s in const:
        if s.get("material") == "unreal":
            for k, v in (("roughness", 0.2), ("metallic", 0.6), ("specular", 0.4)):
                s[k + "_texture"] = np.full((8, 8, 4), v, np.float32)
                s[k] = v
    imgs = []
    for sc in (surf, flat, const):
        S = oracle.PtScene(sc)
        imgs.append(S.render(S.params(24, 24, 4, cam, seed=5)))
    a, b, c = (im[..., :3] / im[..., 3:] for im in imgs)
    assert np.isfinite(a).all() and not np.allclose(a, b)
    ref = [dict(s) for s in const]
    for s in ref:
        for k in ("roughness_texture", "metallic_texture", "specular_texture"):
            s.pop(k, None)
    S2 = oracle.PtScene(ref)
    d = S2.render(S2.params(24, 24, 4, cam, seed=5))
    # a bilinear read of a constant texture is the constant to an ulp, which
    # can flip a rare sampling decision: nearly every pixel agrees
    close = (np.abs(imgs[2] - d) <= 1e-4 * (1.0 + np.abs(d))).all(axis=-1).mean()
    assert close >= 0.97, close
