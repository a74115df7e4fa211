"""Generates the golden fixtures in this directory from the REFERENCE's own
compiled core math (oracle/_ref/libmray_ref_core.so, built from the MRay
source tree by oracle/build.py) and records digests of the seeded workloads.

Run where the MRay source tree is present:
    python tests/golden/make_golden.py
Fixtures written:
    core_math.npz       Moller-Trumbore (cull on/off), slab AABB, Matrix3x4
                        inverse / TransformRay / TransformAABB, Morton 64-bit,
                        Nudge -- inputs and the reference's outputs
    scene_digests.json  sha256 of the seeded scene / ray generators' outputs
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from mray_gb300 import build as B  # noqa: E402
from mray_gb300 import scenes  # noqa: E402


def mt_cases(rng, n):
    rays = rng.normal(size=(n, 6)).astype(np.float32)
    tris = rng.normal(size=(n, 9)).astype(np.float32)
    # aim half of the rays at a point inside the triangle (more hits)
    k = n // 2
    w = rng.dirichlet([1, 1, 1], size=k).astype(np.float32)
    p = (tris[:k, 0:3] * w[:, 0:1] + tris[:k, 3:6] * w[:, 1:2] + tris[:k, 6:9] * w[:, 2:3])
    rays[:k, 0:3] = (p - rays[:k, 3:6]).astype(np.float32)
    # edge cases: rays through a vertex / along an edge, parallel rays,
    # degenerate triangles, hits just beyond the epsilon
    m = 64
    e = np.zeros((m, 6), np.float32)
    et = np.zeros((m, 9), np.float32)
    et[:, :] = [0, 0, 0, 1, 0, 0, 0, 1, 0]
    e[:, 3:6] = [0.25, 0.25, -1.0]
    e[:, 0:3] = [0, 0, 1]
    e[1, 3:6] = [0, 0, -1]                # through vertex 0
    e[2, 3:6] = [0.5, 0.5, -1]            # on the hypotenuse
    e[3, 3:6] = [1.0, 0.0, -1]            # through vertex 1
    e[4, 0:3] = [1, 0, 0]                 # parallel to the plane
    e[5, 3:6] = [0.25, 0.25, 1.0]         # from the back
    e[5, 0:3] = [0, 0, -1]
    e[6, 3:6] = [0.25, 0.25, -1e-7]       # t at the epsilon
    e[7, 3:6] = [0.25, 0.25, -2e-7]
    et[8] = [0, 0, 0, 1, 0, 0, 2, 0, 0]   # degenerate (collinear)
    et[9] = [0, 0, 0, 0, 0, 0, 0, 0, 0]   # degenerate (point)
    e[10, 0:3] = [0, 0, 0]                # zero direction
    for i in range(11, m):
        e[i, 3:6] = [rng.uniform(-0.1, 1.1), rng.uniform(-0.1, 1.1), -1.0]
    return np.vstack([rays, e]), np.vstack([tris, et])


def aabb_cases(rng, n):
    rays = rng.normal(size=(n, 6)).astype(np.float32)
    lo = rng.normal(size=(n, 3)).astype(np.float32)
    hi = lo + np.abs(rng.normal(size=(n, 3))).astype(np.float32)
    boxes = np.hstack([lo, hi]).astype(np.float32)
    tmm = np.stack([np.zeros(n), np.where(rng.random(n) < 0.5, np.float32(3.4028235e38),
                                          rng.uniform(0.1, 5, n))], 1).astype(np.float32)
    # axis-parallel directions (zero components -> infinite inverse)
    rays[: n // 8, 0] = 0.0
    rays[n // 8: n // 4, 0:2] = 0.0
    return rays, boxes, tmm


def main():
    R = oracle.RefCore()
    rng = np.random.default_rng(20261203)
    out = {}
    rays, tris = mt_cases(rng, 4096)
    out["mt_rays"], out["mt_tris"] = rays, tris
    for cull in (0, 1):
        h, b, t = R.intersect_triangles(rays, tris, cull)
        out["mt_hit_c%d" % cull], out["mt_bary_c%d" % cull], out["mt_t_c%d" % cull] = h, b, t
    ar, ab, at = aabb_cases(rng, 4096)
    h, tout = R.intersect_aabbs(ar, ab, at)
    out.update(aabb_rays=ar, aabb_boxes=ab, aabb_tmm=at, aabb_hit=h, aabb_tout=tout)
    mats = []
    for i in range(64):
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        w, x, y, z = q
        Rm = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                       [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                       [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])
        if i % 4 == 1:
            Rm = Rm * rng.uniform(0.5, 2.0)
        M = np.hstack([Rm, rng.normal(size=(3, 1)) * 10]).astype(np.float32)
        mats.append(M.reshape(12))
    mats = np.array(mats, np.float32)
    out["mats"] = mats
    out["inv"] = np.array([R.mat34_inverse(m) for m in mats], np.float32)
    tr_rays = rng.normal(size=(64, 6)).astype(np.float32)
    out["tr_rays"] = tr_rays
    out["tr_out"] = np.array([R.transform_rays(mats[i], tr_rays[i:i + 1])[0] for i in range(64)],
                             np.float32)
    boxes = np.hstack([-np.abs(rng.normal(size=(64, 3))), np.abs(rng.normal(size=(64, 3)))]).astype(np.float32)
    out["taabb_in"] = boxes
    out["taabb_out"] = np.array([R.transform_aabb(mats[i], boxes[i]) for i in range(64)], np.float32)
    xyz = rng.integers(0, 1 << 21, size=(1024, 3), dtype=np.uint32)
    xyz[0] = [0xFFFFF, 0, 0]
    xyz[1] = [0, 0xFFFFF, 0]
    xyz[2] = [0, 0, 0xFFFFF]
    out["morton_xyz"] = xyz
    out["morton_code"] = R.morton3d(xyz)
    npos = (rng.normal(size=(1024, 3)) * np.where(rng.random((1024, 1)) < 0.2, 0.01, 10)).astype(np.float32)
    ndir = rng.normal(size=(1024, 3)).astype(np.float32)
    ndir /= np.linalg.norm(ndir, axis=1, keepdims=True)
    out["nudge_pos"], out["nudge_dir"] = npos, ndir
    out["nudge_out"] = R.nudge(npos, ndir)
    np.savez_compressed(os.path.join(HERE, "core_math.npz"), **out)

    B.build_scenes()
    dig = {}
    pos, idx = scenes.icosphere(5, 1.0, 0.05, 4.0, 0)
    dig["icosphere_l5"] = [hashlib.sha256(pos.tobytes()).hexdigest(), hashlib.sha256(idx.tobytes()).hexdigest()]
    m = scenes.instance_field(64, 0)
    dig["instance_field_64"] = hashlib.sha256(m.tobytes()).hexdigest()
    r = scenes.primary_rays(64, 48, 0)
    dig["primary_64x48"] = hashlib.sha256(r.tobytes()).hexdigest()
    with open(os.path.join(HERE, "scene_digests.json"), "w") as f:
        json.dump(dig, f, indent=1)
    print("wrote fixtures")


if __name__ == "__main__":
    main()
