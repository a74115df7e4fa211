"""Pins the CPU oracle (oracle/mrg_oracle.c) to the reference.

- against golden fixtures produced by the reference's own compiled core math
  (tests/golden/core_math.npz, see tests/golden/make_golden.py);
- against the reference's known-answer tests for 64-bit Morton codes
  (Source/Tests/Core/T_GraphicsFunctions.cpp:263-284);
- against the reference library itself when it is built here (oracle/_ref).
Bit-exact comparisons throughout (integer / IEEE float work).
"""
import ctypes as C
import os

import numpy as np
import pytest

import oracle

GOLD = os.path.join(os.path.dirname(__file__), "golden", "core_math.npz")


@pytest.fixture(scope="module")
def g(built_libs):
    return np.load(GOLD)


def _vp(a):
    return a.ctypes.data_as(C.c_void_p)


def test_mt_matches_reference_fixture(g):
    rays, tris = g["mt_rays"], g["mt_tris"]
    for cull in (0, 1):
        hit, bary, t = g["mt_hit_c%d" % cull], g["mt_bary_c%d" % cull], g["mt_t_c%d" % cull]
        bad = 0
        for i in range(rays.shape[0]):
            h, b, tt, bf = oracle.intersect_triangle(rays[i, :3], rays[i, 3:], tris[i, :3],
                                                     tris[i, 3:6], tris[i, 6:], cull)
            if h != bool(hit[i] & 1):
                bad += 1
                continue
            if h and (bf != bool(hit[i] & 2) or np.float32(tt).view(np.uint32) != t[i].view(np.uint32)
                      or not np.array_equal(b.view(np.uint32), bary[i].view(np.uint32))):
                bad += 1
        assert bad == 0, "cull=%d: %d mismatches" % (cull, bad)
        assert hit.sum() > 100


def test_aabb_matches_reference_fixture(g):
    L = oracle.lib()
    rays, boxes, tmm = g["aabb_rays"], g["aabb_boxes"], g["aabb_tmm"]
    for i in range(rays.shape[0]):
        tout = np.zeros(2, np.float32)
        d = np.ascontiguousarray(rays[i, :3]); p = np.ascontiguousarray(rays[i, 3:])
        bmin = np.ascontiguousarray(boxes[i, :3]); bmax = np.ascontiguousarray(boxes[i, 3:])
        tm = np.ascontiguousarray(tmm[i])
        h = L.orc_intersect_aabb(_vp(d), _vp(p), _vp(bmin), _vp(bmax), _vp(tm), _vp(tout))
        assert bool(h) == bool(g["aabb_hit"][i]), i
        assert np.array_equal(tout.view(np.uint32), g["aabb_tout"][i].view(np.uint32)), i


def test_matrix_inverse_transform_match_reference_fixture(g):
    L = oracle.lib()
    for i in range(g["mats"].shape[0]):
        m = np.ascontiguousarray(g["mats"][i])
        inv = np.zeros(12, np.float32)
        L.orc_mat34_inverse(_vp(m), _vp(inv))
        assert np.array_equal(inv.view(np.uint32), g["inv"][i].view(np.uint32)), i
        d = np.ascontiguousarray(g["tr_rays"][i, :3]); p = np.ascontiguousarray(g["tr_rays"][i, 3:])
        od = np.zeros(3, np.float32); op = np.zeros(3, np.float32)
        L.orc_transform_ray(_vp(m), _vp(d), _vp(p), _vp(od), _vp(op))
        assert np.array_equal(np.concatenate([od, op]).view(np.uint32), g["tr_out"][i].view(np.uint32)), i
        bmin = np.ascontiguousarray(g["taabb_in"][i, :3]); bmax = np.ascontiguousarray(g["taabb_in"][i, 3:])
        omin = np.zeros(3, np.float32); omax = np.zeros(3, np.float32)
        L.orc_transform_aabb(_vp(m), _vp(bmin), _vp(bmax), _vp(omin), _vp(omax))
        assert np.array_equal(np.concatenate([omin, omax]).view(np.uint32),
                              g["taabb_out"][i].view(np.uint32)), i


def test_reference_inverse_sign_defect_and_corrected_mode(g):
    """MRay's Matrix3x4::Inverse is wrong in element [6] for general rotations;
    the corrected mode fixes exactly that element."""
    L = oracle.lib()
    worst_ref, worst_fix = 0.0, 0.0
    for i in range(g["mats"].shape[0]):
        m = np.ascontiguousarray(g["mats"][i])
        M = np.vstack([m.reshape(3, 4).astype(np.float64), [0, 0, 0, 1]])
        inv = np.zeros(12, np.float32)
        L.orc_mat34_inverse_corrected(_vp(m), _vp(inv))
        ref = g["inv"][i]
        same = np.arange(12) != 6
        assert np.array_equal(inv[same].view(np.uint32), ref[same].view(np.uint32))
        assert inv[6] == -ref[6]
        I = np.vstack([inv.reshape(3, 4).astype(np.float64), [0, 0, 0, 1]])
        Ir = np.vstack([ref.reshape(3, 4).astype(np.float64), [0, 0, 0, 1]])
        worst_fix = max(worst_fix, np.abs(M @ I - np.eye(4)).max())
        worst_ref = max(worst_ref, np.abs(M @ Ir - np.eye(4)).max())
    assert worst_fix < 1e-4
    assert worst_ref > 1e-2


def test_morton_reference_kats_and_fixture(g):
    L = oracle.lib()
    # Source/Tests/Core/T_GraphicsFunctions.cpp:263-284
    assert L.orc_morton3d_u64(0b11111111111111111111, 0, 0) == 0x249249249249249
    assert L.orc_morton3d_u64(0, 0b11111111111111111111, 0) == 0x492492492492492
    assert L.orc_morton3d_u64(0, 0, 0b11111111111111111111) == 0x924924924924924
    xyz, codes = g["morton_xyz"], g["morton_code"]
    for i in range(xyz.shape[0]):
        assert L.orc_morton3d_u64(int(xyz[i, 0]), int(xyz[i, 1]), int(xyz[i, 2])) == int(codes[i])


def test_nudge_matches_reference_fixture(g):
    L = oracle.lib()
    for i in range(g["nudge_pos"].shape[0]):
        p = np.ascontiguousarray(g["nudge_pos"][i]); d = np.ascontiguousarray(g["nudge_dir"][i])
        o = np.zeros(3, np.float32)
        L.orc_nudge(_vp(p), _vp(d), _vp(o))
        assert np.array_equal(o.view(np.uint32), g["nudge_out"][i].view(np.uint32)), i


def test_oracle_against_live_reference_library(built_libs):
    """Random MT cases through the reference library built here (skips on
    hosts without the MRay source tree)."""
    try:
        R = oracle.RefCore()
    except FileNotFoundError:
        pytest.skip("reference source tree not present")
    rng = np.random.default_rng(7)
    n = 4000
    rays = rng.normal(size=(n, 6)).astype(np.float32)
    tris = rng.normal(size=(n, 9)).astype(np.float32)
    h, b, t = R.intersect_triangles(rays, tris, 0)
    for i in range(n):
        hh, bb, tt, _ = oracle.intersect_triangle(rays[i, :3], rays[i, 3:], tris[i, :3], tris[i, 3:6],
                                                  tris[i, 6:], 0)
        assert hh == bool(h[i] & 1)
        if hh:
            assert np.float32(tt) == t[i] and np.array_equal(bb, b[i])
