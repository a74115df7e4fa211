"""CPU oracle self-consistency: the restated two-level LBVH (MRay host-backend
stack traversal) agrees bit for bit with brute force over every triangle
(AcceleratorLinear semantics) on small seeded scenes, for closest and any hit,
with and without back-face culling and ray-index indirection."""
import numpy as np
import pytest

import oracle
from mray_gb300 import scenes

MISS = 0xFFFFFFFF


def small_scene(level=3, ninst=8, cull=True, corrected=False, seed=0):
    pos, idx = scenes.icosphere(level, 1.0, 0.05, 4.0, seed)
    m = scenes.instance_field(ninst, seed, box=6.0, jitter=0.3)
    S = oracle.Scene()
    mid = S.add_mesh(pos, idx, prim_key_base=0x10000000)
    for i in range(ninst):
        S.add_instance(mid, m[i], cull=cull, lm_key=100 + i, trans_key=(1 << 24) | i,
                       accel_key=(2 << 20) | i, corrected_inverse=corrected)
    S.build()
    return S, pos, idx, m


@pytest.mark.parametrize("cull", [True, False])
@pytest.mark.parametrize("corrected", [False, True])
def test_lbvh_equals_linear(built_libs, cull, corrected):
    S, *_ = small_scene(cull=cull, corrected=corrected)
    rays = scenes.primary_rays(48, 48, 1, eye=(0, 0, -12), tan_half_fov=0.4)
    a = S.cast_closest(rays, threads=2)
    b = S.cast_closest(rays, linear=True, threads=2)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    assert (a[3] != MISS).sum() > 300


def test_hit_keys_and_misses_untouched(built_libs):
    S, *_ = small_scene()
    rays = scenes.primary_rays(32, 32, 2, eye=(0, 0, -12), tan_half_fov=0.6)
    pre = np.full((rays.shape[0], 4), 0xABCDEF, np.uint32)
    r, h, m, inst = S.cast_closest(rays, hits=pre)
    miss = inst == MISS
    assert miss.any() and (~miss).any()
    assert (h[miss] == 0xABCDEF).all()
    assert np.array_equal(r[miss], rays[miss])
    hit = ~miss
    assert (h[hit, 0] >= 0x10000000).all()
    assert np.array_equal(h[hit, 1], 100 + inst[hit])
    assert np.array_equal(h[hit, 2], (1 << 24) | inst[hit])
    assert np.array_equal(h[hit, 3], (2 << 20) | inst[hit])
    assert (r[hit, 7] < rays[hit, 7]).all()


def test_local_cast(built_libs):
    """CastLocalRays: given the instance of its closest hit, a ray finds the
    same hit locally; given another instance, a hit is never closer than the
    scene's closest and carries that instance's keys; misses stay untouched."""
    S, *_ = small_scene(ninst=8)
    rays = scenes.primary_rays(40, 40, 5, eye=(0, 0, -12), tan_half_fov=0.5)
    r, h, m, inst = S.cast_closest(rays)
    hit = inst != MISS
    own = np.where(hit, inst, 0).astype(np.uint32)
    r2, h2, m2 = S.cast_local(rays, own, threads=2)
    assert np.array_equal(h2[hit], h[hit]) and np.array_equal(r2[hit], r[hit]) and np.array_equal(m2[hit], m[hit])
    rng = np.random.default_rng(1)
    other = rng.integers(0, 8, rays.shape[0]).astype(np.uint32)
    pre = np.full((rays.shape[0], 4), 0xABCDEF, np.uint32)
    r3, h3, m3 = S.cast_local(rays, other, hits=pre, threads=2)
    got = h3[:, 0] != 0xABCDEF
    assert got.any() and (~got).any()
    assert np.array_equal(r3[~got], rays[~got])
    assert np.array_equal(h3[got, 1], 100 + other[got])
    assert np.array_equal(h3[got, 3], (2 << 20) | other[got])
    closer = got & hit
    assert (r3[closer, 7] >= r[closer, 7]).all()
    # out-of-range instance ids skip the ray
    bad = np.full(rays.shape[0], 8, np.uint32)
    r4, h4, _ = S.cast_local(rays, bad, hits=pre, threads=2)
    assert (h4 == 0xABCDEF).all() and np.array_equal(r4, rays)


def test_indirection_and_visibility(built_libs):
    S, *_ = small_scene()
    rays = scenes.primary_rays(40, 40, 3, eye=(0, 0, -12), tan_half_fov=0.5)
    rng = np.random.default_rng(0)
    sel = rng.permutation(rays.shape[0])[:700].astype(np.uint32)
    full = S.cast_closest(rays)
    part = S.cast_closest(rays, ray_idx=sel)
    assert np.array_equal(part[1][sel], full[1][sel])
    others = np.setdiff1d(np.arange(rays.shape[0]), sel)
    assert (part[3][others] == MISS).all()
    bits = S.cast_visibility(rays)
    vis = ((bits[np.arange(rays.shape[0]) >> 5] >> (np.arange(rays.shape[0]) & 31)) & 1).astype(bool)
    assert np.array_equal(vis, full[3] == MISS)
    # segment rays: shorten tMax to just before the closest hit -> visible
    short = rays.copy()
    hitm = full[3] != MISS
    short[hitm, 7] = full[0][hitm, 7] * np.float32(0.999)
    bits2 = S.cast_visibility(short)
    vis2 = ((bits2[np.arange(rays.shape[0]) >> 5] >> (np.arange(rays.shape[0]) & 31)) & 1).astype(bool)
    assert vis2[hitm].mean() > 0.95


def test_single_triangle_and_degenerate(built_libs):
    pos = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [2, 0, 0]], np.float32)
    idx = np.array([[0, 1, 2], [0, 1, 3]], np.uint32)   # second one is degenerate
    S = oracle.Scene()
    mid = S.add_mesh(pos, idx)
    S.add_instance(mid, np.array([1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 5], np.float32))
    S.build()
    rays = np.array([[0.2, 0.2, 10, 0, 0, 0, -1, 3e38], [0.9, 0.9, 10, 0, 0, 0, -1, 3e38],
                     [0.2, 0.2, 0, 0, 0, 0, 1, 3e38]], np.float32)   # last one sees the back face
    r, h, m, inst = S.cast_closest(rays)
    assert inst[0] == 0 and h[0, 0] == 0 and r[0, 7] == np.float32(5.0)
    assert inst[1] == MISS and inst[2] == MISS
